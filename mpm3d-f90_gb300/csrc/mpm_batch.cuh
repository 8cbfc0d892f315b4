// mpm_batch.cuh -- the batched mixed-precision step: many independent scenes
// advanced together by one set of kernels indexed by per-scene offset tables.
//
// Layout (all scenes concatenated; scene s owns the ranges in its Scene entry):
//   particles, kept physically sorted by (scene, cell) at the start of every
//   step (stable sort of the previous order, then a permutation of every
//   field), component-major over the total particle count NP:
//     FP64: x[3], xx[3], v[3], fxp[3], mass, ie
//     FP32: vol, evol (V / V0 - 1), sig_y, sm, seqv, sd[6], fp[9], epeff, celsius,
//     dmg, lt, cp, q
//     per step (written by the permutation): cell (scene-local cell, -1
//     outside), off[3] (offset in the cell, in cells), SGMP dual cell, nearest
//     node, xxn[3], xn[3]; body, scene, orig (scene-local input index)
//   grid nodes concatenated: FP64 mg, px[3], fx[3]; FP32 float4 velocity and
//     acceleration (for the particle gathers); fix, bd, node scene
//   SGMP centre nodes (one per cell) concatenated: 64-bit fixed-point
//     accumulators cacc[13] (mass, momentum[3], external force[3], internal
//     force[6]); FP32 co[6], cw[3], cdefp[9], cvx[3], cax[3]
//   sort keys: scene s owns keys [k0, k0 + nk), the last one collects the
//     particles outside its grid; seg[k] = end of key k's particle range
//     (kept for SGMP scenes). Linear / B-spline: one key per cell; GIMP:
//     one key per node (the particle's nearest node); SGMP: one key per dual
//     cell.
//   P2G accumulators: acc[4][NN] 64-bit fixed point (see the scatter kernels).
//
// Transfers particle -> grid are scatters of FP32 per-cell partial sums
// (one warp per occupied cell, or dual cell for SGMP), summed exactly in
// 64-bit fixed point into the nodes (SGMP: the centre nodes, whose integer
// sums the node kernels add up exactly). They are deterministic and give a
// scene the same results alone or in a batch.
// Transfers grid -> particle are particle-centric with shape functions
// evaluated on the fly in FP32.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_deck.h"
#include "mpm_gpu_internal.cuh"

namespace mpm {
namespace bm {

struct Scene {
  long long p0, np;  // particles
  long long n0, nn;  // grid nodes
  long long k0, nk;  // sort keys (ncell + 1; GIMP nn + 1)
  long long c0, nc;  // SGMP centre nodes
  long long r0, nr;  // reduction chunks
  int NGx, NGy, NGz, NGxy, NCx, NCy, NCz, NCxy, CNCx, CNCy, CNCz, CNCxy, CNC;
  int shape, usf, musl, uvfp, qload, qdamp, gravity, drdamp, has_jc;
  int fixs[6];
  int mat0, nmat;
  double span0[3], span1[3], dcell, idcell, cutoff, iJacobi, iJacobi4;
  double dtscale, qload_time, damp_factor, bq1, bq2;
  // FP32 copies for the mixed-precision kernels (a conversion from FP64 runs
  // on GB300's narrow FP64 pipe, once per thread that makes it)
  float fdcell, fidcell, fbq1, fbq2, fdamp, fiJacobi4, fnp, fspan0[3];
  float fidcell_lo, fspan0_lo[3];  // idcell - fidcell, span0 - fspan0 (FP32 double-float pairs)
  float fspan1[3], fspan1_lo[3];    // span1 as an FP32 pair
  // division by the grid's row and layer sizes: n / d = the high 64 bits of
  // n * m for 0 <= n < 2^32, m = floor(2^64 / d) + 1 (0 for d = 1), see div_by
  unsigned long long mNGx, mNGxy, mNCx, mNCxy, mCNCx, mCNCxy;
  int has_fxp;  // some particle of the scene carries an external force
};

struct SceneState {
  int istep;
  int active;  // 0: the scene is parked (no work this step)
  double time, dt, ke, ie, mom[3], ke_prev, max_vp, depeff_carry;
  unsigned long long active_nodes;
  unsigned status;
  unsigned qmax[4];  // per-step contribution bounds of the P2G scatters (float bits)
  float fdt, ftime;  // FP32 dt and time (written with dt and time)
  unsigned red_done;          // chunks of the energy reduction done this step (reset by the last)
};

// State of the device-resident run loop (mpm_batch_run_loop).
struct LoopCtl {
  int finished;   // scenes that took their last step (counted by kb_begin, never reset)
  int fin0;       // finished when the loop began
  int iters;      // loop iterations taken (two steps each)
  int max_iters;  // iteration budget
  int min_iters;  // iterations before an interrupt is honoured
  int pad_;
};

struct BState {
  long long NP, NN, NK, NC, NR;
  int nscene;
  int any_uvfp, any_sgmp, any_jc;
  // particles (A = current, B = permutation target)
  double *x, *xx, *v, *fxp, *mass, *ie;
  float *vol, *evol, *sig_y, *sm, *seqv, *sd, *fp, *epeff, *celsius, *dmg, *lt, *cp, *q;
  uint8_t* failure;
  uint16_t *body, *scene;
  int* orig;
  int* inv;  // position of a particle by scene p0 + deck index (rebuilt before downloads and probes)
  // per-step derived (written by the permutation)
  int *cell, *dual, *inode;
  float *off, *xxn, *xn;
  float* fs;  // force staging [9][NP]: sigma*vol (xx, yy, zz, xy, yz, xz), fext (3)
  float *m32, *v32;  // FP32 mass and velocity [3][NP] for the momentum transfers (permutation; position update)
  // sort (mpm_sort.cuh)
  unsigned* key;
  int *perm, *seg;
  int *fill, *tiles, *big, *nbig;  // per-key slots taken, scan tile totals, long segments
  LoopCtl* ctl;  // run-loop state (one per batch, outside the layout arena)
  int* task0;  // first particle task (32 sorted particles) of each scene, nscene + 1 entries; SGMP scenes have none
  // grid
  double *mg, *px, *fx;
  float4 *nvel, *nacc;             // FP32 px / mg and fx / mg for the gathers (zero at or below the cut-off)
  unsigned long long* acc;         // [4][NN] fixed-point P2G sums, zero between transfers
  uint8_t *fix, *bd;
  uint16_t* node_scene;
  // SGMP centre grid
  unsigned long long* cacc;            // [CQ_N][NC] fixed-point particle -> centre sums (channels below)
  float *co, *cw, *cdefp, *cvx, *cax;  // derived from node velocities / accelerations (FP32)
  uint16_t* cscene;
  // Johnson-Cook depeff carry (indexed by scene particle range + orig)
  int *setter, *setter_scan;
  double *dep, *jc_aux;
  uint8_t* deferred;
  // reductions
  double* red_part;  // [6][NR]
  uint16_t* rscene;  // chunk -> scene
  Scene* scenes;
  SceneState* sst;
  DevMaterial* mats;
  DevMaterialF* fmats;  // FP32 mirror of mats (the stress update's material constants)
  DevBody* bodies;   // gravp; mat = global material index
};

constexpr int kChunk = 2048;  // particles per reduction chunk

// detonation points of a scene (the lighting time of explosive particles)
struct DetoPoints {
  int n;
  double p[MPM_MAX_DETO][3];
};

// SGMP centre accumulator channels (cacc[channel * NC + cell]): mass and
// momentum (CenterNode Mg / PXg, the MUSL momentum reuses the momentum
// channels), external force, internal force in the reference's Cfint order
// xx, yy, zz, xy, yz, xz
enum : int { CQ_M = 0, CQ_P = 1, CQ_FE = 4, CQ_FI = 7, CQ_N = 13 };

}  // namespace bm
}  // namespace mpm
