/*
 * mpm_oracle.h -- CPU restatement of the MPM3D-F90 explicit step.
 *
 * TEST INFRASTRUCTURE ONLY. The oracle is the checker for the GPU library:
 * only tests, the smoke check and the CPU-baseline leg of the benchmark may
 * load it. Nothing in the product links or calls it.
 *
 * Parity status: UNPINNED against the reference binary. The reference is
 * Fortran 90 and no Fortran compiler exists on either build machine, and the
 * reference ships no golden vectors. The oracle follows the reference source
 * routine by routine (file:line cited at each function) including its REAL(4)
 * roundings, and is pinned only coarsely by the published Cook-membrane tip
 * displacements (VolumetricLockingEx/ExamplesResults.pdf, Table 1).
 *
 * It runs the reference's sequential loops over an array-of-structs particle
 * list with the reference's module-level scratch state, so order effects
 * (per-node summation order, the Johnson-Cook depeff value carried from one
 * particle to the next) are reproduced by construction.
 */
#ifndef MPM_ORACLE_H
#define MPM_ORACLE_H

#include <stdint.h>

#include "mpm_deck.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc orc;

enum orc_libm { ORC_LIBM_SYSTEM = 0, ORC_LIBM_PROJECT = 1 };

int orc_create(const mpm_deck* deck, int libm_mode, orc** out);
void orc_destroy(orc* o);
const char* orc_error(const orc* o);

/* One phase (enum mpm_phase of mpm3d_gpu.h) or one full step. */
int orc_phase(orc* o, int phase);
int orc_step(orc* o);
int orc_run(orc* o, int nsteps);

int orc_get_scalars(orc* o, double* out16);
int orc_download(orc* o, int field, double* out);
int orc_upload(orc* o, int field, const double* in);
int64_t orc_nb_particle(const orc* o);
int64_t orc_nb_gridnode(const orc* o);
/* grid components (grid fields hold nb_component * nb_gridnode nodes,
 * component-major) and the total contact force of the last step */
int orc_nb_component(const orc* o);
int orc_contact_force(const orc* o, double f[3]);
int64_t orc_nb_cell(const orc* o);

#ifdef __cplusplus
}
#endif
#endif
