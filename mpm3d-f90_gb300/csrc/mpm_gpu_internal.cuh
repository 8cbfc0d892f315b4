// mpm_gpu_internal.cuh -- device data layout and launch interface of the
// GB300 explicit MPM step (internal to libmpm3d_gpu).
//
// Layout in HBM (structure of arrays, one allocation per field):
//   particles, in input order (the reference's particle_list order):
//     FP64 always : xp[3][Np], xx[3][Np], vxp[3][Np], fxp[3][Np], mass[Np], ie[Np]
//     "bulk" type B (double for the FP64 forms, float for the mixed form):
//                   vol, sig_y, sm, seqv, sd[6], fp[9], epeff, celsius, dmg, lt,
//                   cp, q, xn[3], xxn[3]
//     int32       : icell, centericell, inode; uint8 failure; uint16 body
//   shape cache (recomputed every step by the locate kernel, reused by every
//   particle pass of the step; type R = double / float):
//     node[K][Np] int32 (0-based node, -1 = not an influence node),
//     shp / dndx / dndy / dndz [K][Np]
//   node-sorted pair list: key[K*Np] = node, val[K*Np] = (p << 5) | slot,
//     stably radix-sorted by node so that each node's contributions appear in
//     the reference's summation order (ascending particle, then slot);
//     seg[n] = end of node n's slice (inclusive prefix sum of the counts).
//   grid, FP64, flat reference node order: mg[Nn], px[3][Nn], fx[3][Nn],
//     vg[3][Nn] (= px/mg), uint8 fix[Nn] (bit c = DOF c fixed), uint8 bd[Nn];
//     with several grid components (contact) the value arrays hold ncomp
//     grids back to back (Nn = ncomp * nodes), a particle reaching its body's
//     component through the node index of its shape cache
//   SGMP auxiliary grid (one centre node per cell), FP64: cmg, cpx[3],
//     cfext[3], cfint[6], co[6], cw[3], cdefp[9], cvx[3], cax[3].
//   stress smoothing (decks with 'smoo'), FP64: spre[Np], gpre[Nn],
//     cgpre[Nc], cgvall[Nc].
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm3d_gpu.h"

namespace mpm {

constexpr int kMaxMat = 16;
constexpr int kMaxBody = 64;
constexpr int kBlock = 256;
constexpr int kRedVals = 6;  // values reduced per step: ke, ie, momentum x/y/z, max |v| component

// Device status bits (per context status word).
enum StatusBits : unsigned {
  ST_NONFINITE = 1u << 0,
  ST_OUT_OF_GRID = 1u << 1,
  ST_NEGATIVE_VOLUME = 1u << 2,
  ST_BAD_EOS = 1u << 3
};

struct DevMaterial {
  int mat_type, eos_type;
  double density, miu, young, poisson, yield0, tangmod, roomt, melt, specheat;
  double B_jc, n_jc, C_jc, m_jc, epso, epf, D;
  double cEos[10];
  double wavespd, q_fai, k_fai, q_psi, ten_f;
};

// FP32 mirror of DevMaterial for the mixed-precision kernels: the same
// field names, so the material models (templated on the material struct)
// read either; every value is the FP32 rounding of its DevMaterial field,
// which is what each FP32 use of that field converts it to, without a
// conversion on the FP64 pipe per particle.
struct DevMaterialF {
  int mat_type, eos_type;
  float density, miu, young, poisson, yield0, tangmod, roomt, melt, specheat;
  float B_jc, n_jc, C_jc, m_jc, epso, epf, D;
  float cEos[10];
  float wavespd, q_fai, k_fai, q_psi, ten_f;
};

inline DevMaterialF material_f32(const DevMaterial& m) {
  DevMaterialF f;
  f.mat_type = m.mat_type;
  f.eos_type = m.eos_type;
  f.density = (float)m.density; f.miu = (float)m.miu; f.young = (float)m.young; f.poisson = (float)m.poisson;
  f.yield0 = (float)m.yield0; f.tangmod = (float)m.tangmod; f.roomt = (float)m.roomt; f.melt = (float)m.melt;
  f.specheat = (float)m.specheat;
  f.B_jc = (float)m.B_jc; f.n_jc = (float)m.n_jc; f.C_jc = (float)m.C_jc; f.m_jc = (float)m.m_jc;
  f.epso = (float)m.epso; f.epf = (float)m.epf; f.D = (float)m.D;
  for (int k = 0; k < 10; ++k) f.cEos[k] = (float)m.cEos[k];
  f.wavespd = (float)m.wavespd; f.q_fai = (float)m.q_fai; f.k_fai = (float)m.k_fai; f.q_psi = (float)m.q_psi;
  f.ten_f = (float)m.ten_f;
  return f;
}

struct DevBody {
  int mat;   // 0-based material index
  int comp;  // 0-based grid component of the body's particles (comID with contact, else 0)
  double gravp[3];
  float fgravp[3];  // FP32 copy for the mixed-precision kernels
};

// Scalars that stay on the device across steps (MPM3D.f90 loop state).
struct DevScalars {
  int istep;
  int pad_;
  double time;       // CurrentTime
  double dt;         // DT
  double ke, ie, mom[3], ke_prev;
  double depeff_carry;  // MaterialModel's module-level depeff after the last particle
  double max_vp;
  double cont_for[3];  // total contact force of the last step (Lagr_NodContact)
  unsigned long long active_nodes;
  unsigned status;
  unsigned pad2_;
};

// Everything a kernel needs besides the arrays.
struct Geometry {
  long long np;       // particles
  int nn;             // grid nodes (of one grid component)
  int ncomp;          // grid components (nbco); node arrays hold ncomp * nn nodes, component-major
  long long nnt;      // ncomp * nn
  int ncell;          // cells (= SGMP centre nodes)
  int NGx, NGy, NGz, NGxy;
  int NCx, NCy, NCz, NCxy;        // NumCellx..
  int CNCx, CNCy, CNCz, CNCxy, CNC;  // CenterNumCell..
  int K;              // influence slots per particle (8 or 27)
  int shape;          // 0 linear, 1 GIMP, 2 B-spline, 3 SGMP
  double span0[3], span1[3];
  double dcell, cutoff, iJacobi, iJacobi4, iDCell;
  double dtscale, qload_time, damp_factor, bq1, bq2;
  int fixs[6];
  int usf, usl, musl, uvfp, qload, qdamp, gravity;
  int nb_mat, nb_body;
  int has_jc;         // a Johnson-Cook material (types 4, 7) is present
  int contact, contact_type, normbody;  // 'cont': bodies on their own components; type 1 = Lagr_NodContact
  int tlmpm;          // 'TLmp': the total Lagrangian form
  double fricfa;      // friction coefficient of the contact
};

template <class B, class R>
struct DevState {
  // particles
  double *xp, *xx, *vxp, *fxp, *mass, *ie;
  B *vol, *sig_y, *sm, *seqv, *sd, *fp, *epeff, *celsius, *dmg, *lt, *cp, *q, *xn, *xxn;
  int *icell, *centericell, *inode;
  uint8_t* failure;
  uint16_t* body;
  // force inputs prepared per particle before the force transfer
  double *fext, *sdiag;  // fext[3][Np], sdiag[3][Np] = SM - q + SDii
  // shape cache
  int* snode;
  R *shp, *dndx, *dndy, *dndz;
  // pairs
  unsigned *key, *val, *key_sorted, *val_sorted;
  int* seg;
  // grid
  double *mg, *px, *fx, *vg;
  uint8_t *fix, *bd;
  // SGMP centre grid
  double *cmg, *cpx, *cfext, *cfint, *co, *cw, *cdefp, *cvx, *cax;
  // stress smoothing (decks with 'smoo'): Spre per particle, Gpre per node,
  // CGpre / CGV_all per centre node
  double *spre, *gpre, *cgpre, *cgvall;
  // contact: mass-gradient normals [3][ncomp * nn], contact force per node [3][nn]
  double *ndir, *cforce;
  // TLMPM: first Piola-Kirchhoff stress [9][Np] (xx yy zz yz xz xy zy zx yx),
  // initial volume [Np], centre-node PK sums [9][Nc] (SGMP)
  double *pk, *vol0, *cpk;
  // Johnson-Cook depeff carry
  int *setter, *setter_scan;
  double *dep;
  double *jc_aux;  // [5][Np]: vold, ieinc, dvol, smold, vol_ of deferred particles
  uint8_t* deferred;
  // reductions
  double* red_part;  // per-block partial sums
  unsigned* red_count;
  DevMaterial* mats;
  DevBody* bodies;
  DevScalars* sc;
};

// One launch table per arithmetic form; each form is compiled in its own
// translation unit (FP64 forms without FMA contraction).
struct StepOps {
  const char* name;
  size_t bulk_size, real_size;
  void (*begin_step)(void* st, const Geometry& g, cudaStream_t s);
  void (*locate)(void* st, const Geometry& g, cudaStream_t s);
  void (*node_offsets)(void* st, const Geometry& g, long long npairs, cudaStream_t s);
  // P2G of mass + momentum; bc: apply the fixed-DOF zeroing; vel: write vg
  void (*p2g_mass)(void* st, const Geometry& g, int bc, int vel, cudaStream_t s);
  void (*node_velocity)(void* st, const Geometry& g, cudaStream_t s);
  void (*apply_bc)(void* st, const Geometry& g, cudaStream_t s);
  void (*stress)(void* st, const Geometry& g, cudaStream_t s);
  void (*depeff_apply)(void* st, const Geometry& g, cudaStream_t s);
  void (*force_prep)(void* st, const Geometry& g, cudaStream_t s);
  // force transfer; integ: also integrate momentum + BC + vg
  void (*p2g_force)(void* st, const Geometry& g, int integ, cudaStream_t s);
  void (*integrate)(void* st, const Geometry& g, cudaStream_t s);
  void (*position)(void* st, const Geometry& g, cudaStream_t s);
  void (*p2g_momentum)(void* st, const Geometry& g, int vel, cudaStream_t s);
  // mode bit 0: energies and momentum (calcEnergy), bit 1: next DT (UpdateDT)
  void (*reduce)(void* st, const Geometry& g, int mode, int nblocks, cudaStream_t s);
  void (*dr_damping)(void* st, const Geometry& g, cudaStream_t s);
  // SmoothStressbyGrid (after fixed_locate and the pair sort): the maps to
  // the grid and back
  void (*smooth)(void* st, const Geometry& g, cudaStream_t s);
  // Lagr_NodContact after IntegrateMomentum, with the total contact force
  void (*contact)(void* st, const Geometry& g, cudaStream_t s);
  // shapes and pair keys from the cells the particles hold (smoothing: with_comp 0)
  void (*fixed_locate)(void* st, const Geometry& g, int with_comp, cudaStream_t s);
  // TLMPM: initial cells, momentum transfer, stress, force (+ integrate)
  void (*tl_initial)(void* st, const Geometry& g, cudaStream_t s);
  void (*tl_momentum)(void* st, const Geometry& g, int vel, cudaStream_t s);
  void (*tl_stress)(void* st, const Geometry& g, cudaStream_t s);
  void (*tl_force)(void* st, const Geometry& g, int integ, cudaStream_t s);
};

extern const StepOps kOpsStrict;   // MPM_FP64_STRICT
extern const StepOps kOpsNative;   // MPM_FP64_NATIVE

// Kernel launch bookkeeping for per-kernel event timing.
void prof_begin(int kernel_id, cudaStream_t s);
void prof_end(int kernel_id, cudaStream_t s);

enum KernelId {
  K_BEGIN = 0, K_LOCATE, K_SORT, K_SEG, K_P2G_MASS, K_NODE_VEL, K_BC, K_STRESS, K_DEPEFF,
  K_FORCE_PREP, K_P2G_FORCE, K_INTEGRATE, K_POSITION, K_P2G_MOM, K_REDUCE, K_DR, K_PERMUTE,
  K_SCATTER_MASS, K_SCATTER_FORCE, K_SCATTER_MOM, K_SG_CLEAR, K_SG_GRADIENT, K_SG_VELOCITY, K_SMOOTH,
  K_CONTACT, K_COUNT
};
extern const char* const kKernelNames[K_COUNT];

// Per-kernel CUDA-event timing shared by contexts and batches: while a
// Profiler is current on the calling thread and enabled, every launch
// bracketed by prof_begin / prof_end records an event pair on its stream
// (event-record nodes when the stream is being captured into a graph).
struct Profiler {
  bool on = false;
  bool capturing = false;
  struct Rec {
    int kernel;
    cudaEvent_t a, b;
  };
  Rec* recs = nullptr;
  int nrec = 0, cap = 0;
  cudaEvent_t* pool = nullptr;
  int npool = 0, next = 0;
  double ms[K_COUNT] = {};
  long long n[K_COUNT] = {};
};
void prof_set_current(Profiler* p);
Profiler* prof_current();
int prof_harvest(Profiler* p, cudaStream_t s);
void prof_reset(Profiler* p);
void prof_free(Profiler* p);

}  // namespace mpm
