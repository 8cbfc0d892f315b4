/*
 * mpm3d_gpu_main.c -- command-line driver: the MPM3D.f90 time loop
 * (MPM3D.f90:62-160) over the C ABI of libmpm3d_gpu.
 *
 *   mpm3d_gpu deck.mpm [--precision fp64|native|mixed] [--steps N] [--report K] [--no-output]
 *             [--pinned] [--dump FILE]
 *
 * It writes the reference's result files next to the deck (job = the deck
 * path without its extension): <job>_curv.dat, EnergyPlot.dat and
 * MomentumPlot.dat every step (OutCurve, fed by a gather of the curve
 * particles' values behind each step), and with 'tecp' / 'para' the
 * animation frames at t = 0 and every OutTime (OutAnim / OutAnimPV, from full
 * field downloads).
 *
 * Without --steps it runs until the reference's exit test is met (CurrentTime >
 * EndTime, or for quasi-static decks CurrentTime > EndTime, KE/(KE+IE) < 0.005
 * and CurrentTime > 100; MPM3D.f90:152-158). It reports per K steps like the
 * reference's progress line and ends with the "time per particle cycle" of
 * MPM3D.f90:267, measured around the device step loop.
 *
 * --pinned follows the Fortran shim's memory sequence: the deck's particle
 * arrays page-locked around mpm_create (mpm_deck_pin on, create, pin off)
 * and the final read-back into a page-locked buffer from mpm_host_alloc,
 * released with mpm_host_free. --dump FILE writes the final Xp (3), VXp (3),
 * SM and SD (6) as raw doubles, component-major, in the input particle
 * order.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "mpm3d_gpu.h"
#include "mpm_output.h"

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* OutAnim / OutAnimPV frame from the device state (only with 'tecp' / 'para') */
static int anim_frame(mpm_ctx* c, const mpm_deck* d, mpm_output* out, const double* s) {
  if (!(d->flags & (MPM_F_TECPLOT | MPM_F_PARAVIEW))) return 0;
  const int64_t np = d->nb_particle;
  static const struct {
    int field, ncomp;
  } want[] = {{MPM_P_XP, 3},   {MPM_P_VXP, 3},  {MPM_P_FXP, 3},     {MPM_P_MASS, 1}, {MPM_P_SEQV, 1},
              {MPM_P_EPEFF, 1}, {MPM_P_SM, 1},   {MPM_P_VOL, 1},     {MPM_P_IE, 1},   {MPM_P_CELSIUS, 1},
              {MPM_P_CP, 1},    {MPM_P_DMG, 1},  {MPM_P_SD, 6},      {MPM_P_FAILURE, 1}, {MPM_P_ICELL, 1},
              {MPM_P_SPRE, 1}};
  enum { NW = sizeof want / sizeof want[0] };
  double* a[NW];
  for (int k = 0; k < NW; ++k) {
    a[k] = (double*)malloc(sizeof(double) * (size_t)(want[k].ncomp * np));
    if (!a[k] || mpm_download(c, want[k].field, a[k])) { /* a form without this field */
      free(a[k]);
      a[k] = NULL;
    }
  }
  mpm_particle_view v = {a[0], a[1], a[2],  a[3],  a[4],  a[5],  a[6], a[7],
                         a[8], a[9], a[10], a[11], a[12], a[13], a[14], a[15]};
  int st = mpm_output_anim(out, s, &v);
  for (int k = 0; k < NW; ++k) free(a[k]);
  if (st) fprintf(stderr, "animation output error %d\n", st);
  return st;
}

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s deck.mpm [--precision fp64|native|mixed] [--steps N] [--report K]\n", argv[0]);
    return 2;
  }
  int precision = MPM_FP64_STRICT;
  long steps = -1, report = 100;
  int write_output = 1, pinned = 0;
  const char* dump = NULL;
  for (int i = 2; i < argc; ++i) {
    if (!strcmp(argv[i], "--precision") && i + 1 < argc) {
      ++i;
      precision = !strcmp(argv[i], "mixed") ? MPM_MIXED : (!strcmp(argv[i], "native") ? MPM_FP64_NATIVE : 0);
    } else if (!strcmp(argv[i], "--steps") && i + 1 < argc) {
      steps = atol(argv[++i]);
    } else if (!strcmp(argv[i], "--report") && i + 1 < argc) {
      report = atol(argv[++i]);
    } else if (!strcmp(argv[i], "--no-output")) {
      write_output = 0;
    } else if (!strcmp(argv[i], "--pinned")) {
      pinned = 1;
    } else if (!strcmp(argv[i], "--dump") && i + 1 < argc) {
      dump = argv[++i];
    }
  }
  char err[256] = {0};
  mpm_deck* d = NULL;
  int st = mpm_deck_load(argv[1], &d, err, sizeof err);
  if (st) {
    fprintf(stderr, "deck error %d: %s\n", st, err);
    return 1;
  }
  mpm_ctx* c = NULL;
  if (pinned && (st = mpm_deck_pin(d, 1))) {
    fprintf(stderr, "deck pin error %d: %s\n", st, mpm_last_error(NULL));
    return 1;
  }
  st = mpm_create(d, precision, -1, &c);
  if (pinned) {
    int st2 = mpm_deck_pin(d, 0);
    if (!st && st2) st = st2;
  }
  if (st) {
    fprintf(stderr, "create error %d: %s\n", st, mpm_last_error(NULL));
    return 1;
  }
  double s[MPM_NSCALARS];
  mpm_get_scalars(c, s);
  /* result files (InputPara / OutCurve / OutAnim) */
  mpm_output* out = NULL;
  int ncur = 0;
  int64_t cp_[64];
  int cf_[64], cc_[64];
  double cv_[64];
  char job[1024];
  snprintf(job, sizeof job, "%s", argv[1]);
  {
    char* base = strrchr(job, '/');
    char* dot = strchr(base ? base + 1 : job, '.');
    if (dot) *dot = 0;
  }
  if (write_output) {
    if ((st = mpm_output_open(d, job, NULL, &out))) {
      fprintf(stderr, "cannot open the result files of %s\n", job);
      return 1;
    }
    ncur = mpm_output_curve_items(out, cp_, cf_, cc_, 64);
    if (anim_frame(c, d, out, s)) return 1;
  }
  float plt = (float)d->outtime; /* plt is a default REAL (MPM3D.f90:34, 45) */
  printf("particles %lld  grid nodes %lld  DT = %10.3e\nsolving...\n", (long long)mpm_nb_particle(c),
         (long long)mpm_nb_gridnode(c), s[2]);
  const int quasi = (d->flags & MPM_F_QUASILOAD) != 0;
  double t0 = now_s();
  long n = 0;
  for (;;) {
    if (steps >= 0 && n >= steps) break;
    if ((st = mpm_step(c))) break;
    ++n;
    if (out && ncur > 0 && (st = mpm_gather_async(c, ncur, cp_, cf_, cc_))) break;
    if ((st = mpm_get_scalars(c, s))) break; /* exit test needs CurrentTime */
    if (out) {
      if (ncur > 0 && (st = mpm_gather_wait(c, cv_))) break;
      if ((st = mpm_output_curve(out, s, cv_))) break;
      if (d->flags & MPM_F_CONTACT) {
        double cf[3];
        if ((st = mpm_contact_force(c, cf)) || (st = mpm_output_contact(out, s[1], cf))) break;
      }
      if (s[1] >= (double)plt) {
        plt = plt + (float)d->outtime;
        if ((st = anim_frame(c, d, out, s))) break;
      }
    }
    if (report > 0 && n % report == 0)
      printf(" Step=%6ld   T=%10.3e   DT=%10.3e   K.E.=%10.3e  T.E.=%10.3e\n", n, s[1], s[2], s[3], s[3] + s[4]);
    if (steps < 0) {
      if (quasi) {
        if (s[1] > d->endtime && s[3] / (s[3] + s[4]) < 0.005 && s[1] > 100) break;
      } else if (s[1] > d->endtime) {
        break;
      }
    }
  }
  if (!st) st = mpm_sync(c);
  double t = now_s() - t0;
  if (st) {
    fprintf(stderr, "step error %d: %s\n", st, mpm_last_error(c));
    return 1;
  }
  const double np = (double)mpm_nb_particle(c);
  printf("** steps %ld  elapsed %.4f s\n** Time per particle cycle: %12.4f nanoseconds\n", n, t,
         1e9 * t / np / (double)(n > 0 ? n : 1));
  if (dump) {
    static const int fields[4] = {MPM_P_XP, MPM_P_VXP, MPM_P_SM, MPM_P_SD};
    const int64_t npi = mpm_nb_particle(c);
    const int64_t bytes = (int64_t)sizeof(double) * 6 * npi; /* the largest field */
    double* buf = pinned ? (double*)mpm_host_alloc(bytes) : (double*)malloc((size_t)bytes);
    FILE* f = buf ? fopen(dump, "wb") : NULL;
    if (!f) {
      fprintf(stderr, "cannot write %s\n", dump);
      return 1;
    }
    for (int k = 0; k < 4 && !st; ++k) {
      const int64_t cnt = (int64_t)mpm_field_components(fields[k]) * npi;
      st = mpm_download(c, fields[k], buf);
      if (!st && fwrite(buf, sizeof(double), (size_t)cnt, f) != (size_t)cnt) st = MPM_ERR_IO;
    }
    fclose(f);
    if (pinned) mpm_host_free(buf);
    else free(buf);
    if (st) {
      fprintf(stderr, "dump error %d: %s\n", st, mpm_last_error(c));
      return 1;
    }
  }
  mpm_output_close(out);
  mpm_destroy(c);
  mpm_deck_free(d);
  return 0;
}
