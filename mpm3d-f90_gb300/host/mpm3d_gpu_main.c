/*
 * mpm3d_gpu_main.c -- command-line driver: the MPM3D.f90 time loop
 * (MPM3D.f90:62-160) over the C ABI of libmpm3d_gpu.
 *
 *   mpm3d_gpu deck.mpm [--precision fp64|native|mixed] [--steps N] [--report K]
 *
 * Without --steps it runs until the reference's exit test is met (CurrentTime >
 * EndTime, or for quasi-static decks CurrentTime > EndTime, KE/(KE+IE) < 0.005
 * and CurrentTime > 100; MPM3D.f90:152-158). It reports per K steps like the
 * reference's progress line and ends with the "time per particle cycle" of
 * MPM3D.f90:267, measured around the device step loop.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "mpm3d_gpu.h"

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s deck.mpm [--precision fp64|native|mixed] [--steps N] [--report K]\n", argv[0]);
    return 2;
  }
  int precision = MPM_FP64_STRICT;
  long steps = -1, report = 100;
  for (int i = 2; i < argc; ++i) {
    if (!strcmp(argv[i], "--precision") && i + 1 < argc) {
      ++i;
      precision = !strcmp(argv[i], "mixed") ? MPM_MIXED : (!strcmp(argv[i], "native") ? MPM_FP64_NATIVE : 0);
    } else if (!strcmp(argv[i], "--steps") && i + 1 < argc) {
      steps = atol(argv[++i]);
    } else if (!strcmp(argv[i], "--report") && i + 1 < argc) {
      report = atol(argv[++i]);
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
  st = mpm_create(d, precision, -1, &c);
  if (st) {
    fprintf(stderr, "create error %d: %s\n", st, mpm_last_error(NULL));
    return 1;
  }
  double s[MPM_NSCALARS];
  mpm_get_scalars(c, s);
  printf("particles %lld  grid nodes %lld  DT = %10.3e\nsolving...\n", (long long)mpm_nb_particle(c),
         (long long)mpm_nb_gridnode(c), s[2]);
  const int quasi = (d->flags & MPM_F_QUASILOAD) != 0;
  double t0 = now_s();
  long n = 0;
  for (;;) {
    if (steps >= 0 && n >= steps) break;
    if ((st = mpm_step(c))) break;
    ++n;
    if ((st = mpm_get_scalars(c, s))) break; /* exit test needs CurrentTime */
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
  mpm_destroy(c);
  mpm_deck_free(d);
  return 0;
}
