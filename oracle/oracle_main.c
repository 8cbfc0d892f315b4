/*
 * oracle_main.c -- command-line front end of the CPU oracle (test
 * infrastructure; see mpm_oracle.h).
 *
 *   mpm3d_oracle deck.mpm [--steps N] [--libm system|project] [--every K]
 *
 * Runs the time loop of MPM3D.f90:69-160 for N steps (default: until
 * CurrentTime > EndTime, the non-quasi-static exit of MPM3D.f90:157) and
 * prints the per-step scalars every K steps plus the wall time of the step
 * loop in the reference's "time per particle cycle" form (MPM3D.f90:267).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "mpm3d_gpu.h"
#include "mpm_oracle.h"

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s deck.mpm [--steps N] [--libm system|project] [--every K]\n", argv[0]);
    return 2;
  }
  long steps = -1, every = 0;
  int libm = ORC_LIBM_SYSTEM;
  for (int i = 2; i < argc; ++i) {
    if (!strcmp(argv[i], "--steps") && i + 1 < argc) steps = atol(argv[++i]);
    else if (!strcmp(argv[i], "--every") && i + 1 < argc) every = atol(argv[++i]);
    else if (!strcmp(argv[i], "--libm") && i + 1 < argc) libm = !strcmp(argv[++i], "project");
  }
  char err[256] = {0};
  mpm_deck* d = NULL;
  int st = mpm_deck_load(argv[1], &d, err, sizeof err);
  if (st) {
    fprintf(stderr, "deck error %d: %s\n", st, err);
    return 1;
  }
  orc* o = NULL;
  st = orc_create(d, libm, &o);
  if (st) {
    fprintf(stderr, "oracle error %d: %s\n", st, orc_error(o));
    return 1;
  }
  double s[MPM_NSCALARS];
  orc_get_scalars(o, s);
  printf("particles %lld  grid nodes %lld  DT %.17g\n", (long long)orc_nb_particle(o),
         (long long)orc_nb_gridnode(o), s[2]);
  double t0 = now_s();
  long n = 0;
  for (;;) {
    if (steps >= 0 && n >= steps) break;
    st = orc_step(o);
    if (st) {
      fprintf(stderr, "step error %d: %s\n", st, orc_error(o));
      return 1;
    }
    ++n;
    orc_get_scalars(o, s);
    if (every > 0 && n % every == 0)
      printf("step %6ld  t %.10e  DT %.10e  KE %.10e  IE %.10e\n", n, s[1], s[2], s[3], s[4]);
    if (steps < 0) {
      /* exit tests of MPM3D.f90:152-158 */
      if (d->flags & MPM_F_QUASILOAD) {
        if (s[1] > d->endtime && s[3] / (s[3] + s[4]) < 0.005 && s[1] > 100) break;
      } else if (s[1] > d->endtime) {
        break;
      }
    }
  }
  double t = now_s() - t0;
  printf("steps %ld  wall %.6f s  time per particle cycle %.4f ns  particle-steps/s %.6e\n", n, t,
         1e9 * t / (double)orc_nb_particle(o) / (double)(n > 0 ? n : 1),
         (double)orc_nb_particle(o) * (double)n / (t > 0 ? t : 1e-30));
  /* displacement of the curve particles (the 'disx/disy/disz' curves) */
  int64_t np = orc_nb_particle(o);
  double* xp = (double*)malloc(sizeof(double) * 3 * (size_t)np);
  orc_download(o, MPM_P_XP, xp);
  for (int c = 0; c < d->n_curves; ++c) {
    int64_t p = d->curve_point[c] - 1;
    if (p < 0 || p >= np) continue;
    printf("curve %d particle %lld displacement %.10e %.10e %.10e\n", c + 1, (long long)p + 1,
           xp[p] - d->xp[p], xp[np + p] - d->xp[np + p], xp[2 * np + p] - d->xp[2 * np + p]);
  }
  free(xp);
  orc_destroy(o);
  mpm_deck_free(d);
  return 0;
}
