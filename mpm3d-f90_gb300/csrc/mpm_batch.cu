// mpm_batch.cu -- host side of the batched mixed-precision step (C ABI in
// include/mpm3d_gpu.h, kernels in mpm_batch_kernels.cuh).
//
// A batch holds the scenes of one composition laid out back to back in device
// memory. Changing the composition (mpm_batch_commit) builds a new layout:
// resident scenes are moved on the device by a relocation kernel, new scenes
// are uploaded, retired scenes are dropped. Every step sorts the particles of
// all scenes by (scene, cell) and runs one launch per kernel for the batch.
#include <cuda_runtime.h>


#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "mpm3d_gpu.h"
#include "mpm_batch_host.h"
#include "mpm_batch_kernels.cuh"
#include "mpm_sort.cuh"
#include "mpm_setup.h"

using namespace mpm;
using namespace mpm::bm;

namespace mpm {

// a scene staged on the host: its set-up and input state (copied from the
// deck, so the deck may be freed once the scene is staged)
struct HostScene {
  int id = 0;
  int steps = 0;  // step count to run (INT_MAX = unlimited)
  SceneSetup su;
  long long np = 0, nn = 0, ncell = 0;
  std::vector<double> mass, x, v, fxp;  // input state, component-major, input order
  // borrowed input state (the deck's arrays) when the scene is committed
  // before its deck may be freed; otherwise null and the copies above are used
  const double *bmass = nullptr, *bx = nullptr, *bv = nullptr, *bfxp = nullptr;
  std::vector<uint16_t> body_local;     // body index per particle
  const double* in_mass() const { return bmass ? bmass : mass.data(); }
  const double* in_x() const { return bx ? bx : x.data(); }
  const double* in_v() const { return bv ? bv : v.data(); }
  const double* in_fxp() const { return bfxp ? bfxp : fxp.data(); }
  // the input state is on the device: drop the host copies
  void release_inputs() {
    std::vector<double>().swap(mass);
    std::vector<double>().swap(x);
    std::vector<double>().swap(v);
    std::vector<double>().swap(fxp);
    std::vector<uint16_t>().swap(body_local);
    std::vector<double>().swap(su.vol);
    std::vector<double>().swap(su.sig_y);
    std::vector<double>().swap(su.ie);
    std::vector<double>().swap(su.cp);
    std::vector<double>().swap(su.lt);
    bmass = bx = bv = bfxp = nullptr;
  }
  bool resident = false;
  long long p0 = 0, n0 = 0, k0 = 0, c0 = 0, r0 = 0, nr = 0;
  int mat0 = 0, body0 = 0, index = 0;
  SceneState st{};
  int drdamp = 0;
  int smooth = 0;  // 'smoo': Spre is computed when read
  int any_fxp = 1;  // some particle carries an external force (FXP)
  DetoPoints deto{};  // detonation points (lighting time of explosives)
};

}  // namespace mpm

namespace {

// particle state of a newly admitted scene from its uploaded inputs:
// scr = vol, sig_y, cp, lt (FP64, np each); the rest of the state starts at
// zero, the temperature at 293 (Particle.f90:131)
// Initial (DataIn.f90:1211-1267) for the particles of a new scene, from
// their mass and position and their body's material: volume, yield stress,
// internal energy, sound speed, lighting time (sqrt(...)/D a default-REAL
// temporary); bodies of material type 12 keep zeros
__global__ void kb_init_scene(BState s, int scene, int body0, DetoPoints deto) {
  const Scene& sc = s.scenes[scene];
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= sc.np) return;
  const long long NP = s.NP, i = sc.p0 + k;
  const DevMaterial& m = s.mats[s.bodies[body0 + s.body[i]].mat];
  double vol = 0.0, sig_y = 0.0, ie = 0.0, cp = 0.0, lt = 0.0;
  if (m.mat_type != 12) {
    vol = s.mass[i] / m.density;
    sig_y = m.yield0;
    ie = m.cEos[9] * vol;
    if (m.mat_type == 1 || m.mat_type == 11) {
      const double E = m.young, nu = m.poisson, ro = m.density;
      cp = sqrt(E * (1 - nu) / (1 + nu) / (1 - 2 * nu) / ro);
    }
    if (m.mat_type == 9) cp = m.wavespd;
    lt = (double)10e6f;
    for (int j = 0; j < deto.n; ++j) {
      const double dx = s.x[i] - deto.p[j][0], dy = s.x[NP + i] - deto.p[j][1], dz = s.x[2 * NP + i] - deto.p[j][2];
      const float t = (float)(sqrt(dx * dx + dy * dy + dz * dz) / m.D);
      if ((double)t < lt) lt = (double)t;
    }
  }
  s.vol[i] = (float)vol;
  s.sig_y[i] = (float)sig_y;
  s.ie[i] = ie;
  s.cp[i] = (float)cp;
  s.lt[i] = (float)lt;
  s.celsius[i] = 293.0f;
  s.sm[i] = 0.f;
  s.evol[i] = 0.f;
  s.seqv[i] = 0.f;
  s.epeff[i] = 0.f;
  s.dmg[i] = 0.f;
  s.q[i] = 0.f;
  for (int a = 0; a < 6; ++a) s.sd[a * NP + i] = 0.f;
  if (s.any_uvfp)
    for (int a = 0; a < 18; ++a) s.fp[a * NP + i] = 0.f;
  s.failure[i] = 0;
  s.body[i] = (uint16_t)(body0 + s.body[i]);
  s.scene[i] = (uint16_t)scene;
  s.orig[i] = (int)k;
}

__global__ void kb_inverse(BState s) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.NP) return;
  s.inv[s.scenes[s.scene[i]].p0 + s.orig[i]] = (int)i;
}


// relocation of resident particles into a new layout
__global__ void kb_relocate(BState src, BState dst, const int* map, const uint16_t* scene_map,
                            const uint16_t* body_map) {
  long long i = btid();
  if (i >= dst.NP) return;
  long long j = map[i];
  if (j < 0) return;
  const long long NP = dst.NP, SP = src.NP;
  for (int a = 0; a < 3; ++a) {
    dst.x[a * NP + i] = src.x[a * SP + j];
    dst.xx[a * NP + i] = src.xx[a * SP + j];
    dst.v[a * NP + i] = src.v[a * SP + j];
    dst.fxp[a * NP + i] = src.fxp[a * SP + j];
  }
  dst.mass[i] = src.mass[j];
  dst.ie[i] = src.ie[j];
  dst.vol[i] = src.vol[j];
  dst.evol[i] = src.evol[j];
  dst.sig_y[i] = src.sig_y[j];
  dst.sm[i] = src.sm[j];
  dst.seqv[i] = src.seqv[j];
  for (int a = 0; a < 6; ++a) dst.sd[a * NP + i] = src.sd[a * SP + j];
  if (src.any_uvfp && dst.any_uvfp)
    for (int a = 0; a < 18; ++a) dst.fp[a * NP + i] = src.fp[a * SP + j];
  dst.epeff[i] = src.epeff[j];
  dst.celsius[i] = src.celsius[j];
  dst.dmg[i] = src.dmg[j];
  dst.lt[i] = src.lt[j];
  dst.cp[i] = src.cp[j];
  dst.q[i] = src.q[j];
  dst.failure[i] = src.failure[j];
  dst.body[i] = body_map[src.body[j]];
  dst.scene[i] = scene_map[src.scene[j]];
  dst.orig[i] = src.orig[j];
}

}  // namespace

struct mpm_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<HostScene*> order;  // composition order
  std::map<int, HostScene*> by_id;
  int next_id = 1;
  bool dirty = false;
  // current layout
  BState A{}, B{};
  // device arenas: the current layout's, and a spare one kept for the next
  // re-layout (the relocation copies from one to the other), so that a new
  // composition does not allocate when its layout fits the spare
  char* arena = nullptr;
  size_t arena_cap = 0;
  char* spare = nullptr;
  size_t spare_cap = 0;
  double* dl = nullptr;  // particle-field download buffer (all components of one field)
  size_t dl_cap = 0;
  bool inv_stale = false;  // steps ran since the inverse permutation was last built
  long long bytes = 0;
  int* d_target = nullptr;
  // second stream: the energy / DT reduction of a step runs there while the
  // next step's keys are sorted (the two touch disjoint arrays)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int any_sgmp = 0, any_nonsgmp = 0, any_usf = 0, any_later = 0, any_musl = 0, any_jc = 0, any_dr = 0, any_uvfp = 0;
  int any_nonuvfp = 0;
  int any_prep = 0;  // scenes whose force input is not staged by their stress kernel (USL / MUSL, Johnson-Cook)
  unsigned stress_types = 0;  // stress instantiations to launch: bit MT per specialised type, bit 0 for the rest
  cudaGraphExec_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // one step, per buffer parity and
                                                                      // without / with the previous step's reduction
  const double* set0_x = nullptr;                   // identifies particle buffer set 0
  int pblock = 256, nblock = 256;
  int scatter_blocks = 9728;  // scatter grid cap (64 blocks per SM; warps stride over the occupied cells)
  int sort_blocks = 152;      // grid of the long-segment sort (one block per SM)
  int sms = 152;              // multiprocessors of the device
  int loop_min_steps = 0;     // steps a device loop takes before it honours an interrupt
  long long ntask = 0;        // particle tasks of the linear / GIMP / B-spline scenes (32 particles each)
  // device-resident run loop (mpm_batch_run_loop): its state, the host's
  // request flag (page-locked, mapped into the device's address space) and
  // one loop graph per buffer parity
  LoopCtl* ctl = nullptr;
  volatile int* loop_flag_h = nullptr;
  int* loop_flag_d = nullptr;
  cudaGraphExec_t loop_graph[2] = {nullptr, nullptr};
  Profiler prof;
  // particle value gather (curve output)
  GatherItem *g_items_h = nullptr, *g_items_d = nullptr;
  double *g_out_h = nullptr, *g_out_d = nullptr;
  cudaEvent_t g_done = nullptr;
  int g_n = 0;
  std::string err;
};

namespace {

int berr(mpm_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  return code;
}

#define BCK(call)                                                                        \
  do {                                                                                   \
    cudaError_t e__ = (call);                                                            \
    if (e__ != cudaSuccess) return berr(b, MPM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e__)); \
  } while (0)

// Carves the arrays of one layout out of one device arena (256-byte aligned);
// with a null base it only measures the arena size.
struct Alloc {
  char* base = nullptr;
  size_t off = 0;
  template <class T>
  T* get(long long n) {
    if (n <= 0) n = 1;
    off = (off + 255) & ~(size_t)255;
    T* p = base ? (T*)(base + off) : nullptr;
    off += (size_t)n * sizeof(T);
    return p;
  }
};

void alloc_particles(Alloc& al, BState& s, long long NP, bool uvfp) {
  s.x = al.get<double>(3 * NP);
  s.xx = al.get<double>(3 * NP);
  s.v = al.get<double>(3 * NP);
  s.fxp = al.get<double>(3 * NP);
  s.mass = al.get<double>(NP);
  s.ie = al.get<double>(NP);
  s.vol = al.get<float>(NP);
  s.evol = al.get<float>(NP);
  s.sig_y = al.get<float>(NP);
  s.sm = al.get<float>(NP);
  s.seqv = al.get<float>(NP);
  s.sd = al.get<float>(6 * NP);
  s.fp = al.get<float>(uvfp ? 18 * NP : 1);
  s.epeff = al.get<float>(NP);
  s.celsius = al.get<float>(NP);
  s.dmg = al.get<float>(NP);
  s.lt = al.get<float>(NP);
  s.cp = al.get<float>(NP);
  s.q = al.get<float>(NP);
  s.failure = al.get<uint8_t>(NP);
  s.body = al.get<uint16_t>(NP);
  s.scene = al.get<uint16_t>(NP);
  s.orig = al.get<int>(NP);
}

long long scene_bytes(long long np, long long nn, long long ncell, bool sgmp, bool uvfp, bool jc) {
  long long per_p = 2 * (16 * 8 + 17 * 4 + (uvfp ? 72 : 0) + 1 + 2 + 2 + 4);  // two particle buffer sets
  per_p += 4 * 3 + 4 * 9 + 4 * 6 + 4 * 9 + 4 * 4;                          // derived + force staging + FP32 m, v
  per_p += 4 * 3;                                                         // sort key, permutation, inverse
  if (jc) per_p += 4 * 2 + 8 * 6 + 1;
  long long per_n = 8 * 13 + 4 + 8 * 4;
  long long per_k = 4 * 2;                                                // segment ends, fill counters
  long long per_c = sgmp ? 8 * 39 + 2 : 0;
  return np * per_p + nn * per_n + (std::max(nn, ncell) + 1) * per_k + ncell * per_c + 4096;
}

// multiplier of div_by for the divisor d (>= 1): floor(2^64 / d) + 1, exact
// for every 32-bit dividend since n * (m - 2^64 / d) < 2^64 / d; 0 for d = 1
unsigned long long div_magic(long long d) {
  return d > 1 ? ~0ull / (unsigned long long)d + 1ull : 0ull;
}

void layout_flags(mpm_batch* b) {
  b->any_sgmp = b->any_nonsgmp = b->any_usf = b->any_later = b->any_musl = b->any_jc = b->any_dr = b->any_uvfp = 0;
  b->any_nonuvfp = 0;
  b->any_prep = 0;
  for (HostScene* h : b->order) {
    const Geometry& g = h->su.g;
    if (g.shape == 3) b->any_sgmp = 1; else b->any_nonsgmp = 1;
    if (g.usf) b->any_usf = 1; else b->any_later = 1;
    if (g.musl) b->any_musl = 1;
    if (g.has_jc) b->any_jc = 1;
    if (!g.usf || g.has_jc) b->any_prep = 1;
    if (g.uvfp) b->any_uvfp = 1;
    else b->any_nonuvfp = 1;
    if (h->drdamp) b->any_dr = 1;
  }
  b->stress_types = 0;
  for (HostScene* h : b->order)
    for (const DevMaterial& m : h->su.mats) b->stress_types |= 1u << (stress_specialised(m.mat_type) ? m.mat_type : 0);
}

int upload_scene_particles(mpm_batch* b, HostScene* h, BState& s) {
  const long long NP = s.NP, np = h->np, p0 = h->p0;
  cudaStream_t st = b->stream;
  auto upd = [&](double* dst, const double* src, long long n) {
    return cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice, st);
  };
  const double *x = h->in_x(), *v = h->in_v(), *fxp = h->in_fxp();
  for (int a = 0; a < 3; ++a) {
    BCK(upd(s.x + a * NP + p0, x + a * np, np));
    BCK(cudaMemcpyAsync(s.xx + a * NP + p0, s.x + a * NP + p0, sizeof(double) * np, cudaMemcpyDeviceToDevice, st));
    BCK(upd(s.v + a * NP + p0, v + a * np, np));
    BCK(upd(s.fxp + a * NP + p0, fxp + a * np, np));
  }
  BCK(upd(s.mass + p0, h->in_mass(), np));
  BCK(cudaMemcpyAsync(s.body + p0, h->body_local.data(), sizeof(uint16_t) * np, cudaMemcpyHostToDevice, st));
  kb_init_scene<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(s, h->index, h->body0, h->deto);
  BCK(cudaGetLastError());
  BCK(cudaStreamSynchronize(st));  // the host arrays may go away after this
  return MPM_OK;
}

// sort keys of a scene: one per cell (linear, B-spline), per node (GIMP: a
// particle is binned with its nearest node, see kb_keys) or per dual cell
// (SGMP, ncell of them), plus the bucket of the particles outside the grid
long long scene_keys(const Geometry& g) { return (g.shape == 1 ? (long long)g.nn : (long long)g.ncell) + 1; }

inline unsigned gridn(long long n, int blk) { return (unsigned)((n + blk - 1) / blk); }

// inclusive scan in three passes over tiles (mpm_sort.cuh); tiles holds
// scan_tiles(src.n) values of the source's type
template <class S>
void scan_tiles_enqueue(const S& src, typename S::T* tiles, cudaStream_t st) {
  const long long nt = scan_tiles(src.n);
  if (nt <= 0) return;
  ks_tile_total<S><<<(unsigned)nt, kScanThreads, 0, st>>>(src, tiles);
  if (nt <= kFusedTiles) {
    ks_tile_scan<S, true><<<(unsigned)nt, kScanThreads, 0, st>>>(src, tiles);
  } else {
    ks_tile_prefix<typename S::T, typename S::Op><<<1, kScanThreads, 0, st>>>(tiles, nt);
    ks_tile_scan<S, false><<<(unsigned)nt, kScanThreads, 0, st>>>(src, tiles);
  }
}

// one step of every live scene (MPM3D.f90:69-118 for each scene)
// The step in three parts. The front (sort keys, sort, per-key counts,
// occupied keys) reads the positions and scene ids only; the back (begin,
// permutation, transfers, stress, position) does the rest; the reduction
// (calcEnergy, UpdateDT, damping) reads the final velocities, masses and
// energies. The front does not depend on the begin kernel (which advances
// the step count and time), so it runs first.
int enqueue_front(mpm_batch* b) {
  cudaStream_t st = b->stream;
  BState& a = b->A;
  const int pb = b->pblock;
  prof_begin(K_LOCATE, st);
  cudaMemsetAsync(a.seg, 0, sizeof(int) * (size_t)(a.NK + 1), st);
  kb_keys<<<gridn(a.NP, pb), pb, 0, st>>>(a);
  prof_end(K_LOCATE, st);
  // counting sort by key (mpm_sort.cuh): segment ends and the occupied
  // keys, placement, then the stable order inside each segment
  prof_begin(K_SORT, st);
  scan_tiles_enqueue(SegScan{a.seg, a.fill, a.NK}, a.tiles, st);  // (zeroes the fill counters; kb_keys the long-segment count)
  ks_place<<<gridn(a.NP, 256), 256, 0, st>>>(a.key, a.seg, a.fill, a.perm, a.NP);
  ks_segments<<<gridn(a.NK, 256), 256, 0, st>>>(a.seg, a.NK, a.perm, a.big, a.nbig);
  ks_long_segments<<<b->sort_blocks, kSegThreads, 0, st>>>(a.seg, a.perm, a.big, a.nbig);
  prof_end(K_SORT, st);
  return MPM_OK;
}

int enqueue_back(mpm_batch* b) {
  cudaStream_t st = b->stream;
  BState& a = b->A;
  const int pb = b->pblock, nb = b->nblock;
  prof_begin(K_BEGIN, st);
  kb_begin<<<gridn(a.nscene, 128), 128, 0, st>>>(a, b->d_target);
  prof_end(K_BEGIN, st);
  prof_begin(K_PERMUTE, st);
  kb_permute<<<gridn(a.NP, pb), pb, 0, st>>>(a, b->B);
  prof_end(K_PERMUTE, st);
  // swap the particle buffer sets (node and scene arrays are shared)
  std::swap(b->A, b->B);
  BState& s = b->A;
  auto pgrid = [&](int warps) {
    return (unsigned)std::max<long long>(1, std::min<long long>(b->scatter_blocks, (b->ntask + warps - 1) / warps));
  };
  // particle -> grid transfers: particle tasks of every scene
  auto scatter = [&](int mode) {
    constexpr int w0 = PartShape<0>::WARPS, w1 = PartShape<1>::WARPS, w2 = PartShape<2>::WARPS;
    if (mode == 0) kb_part_scatter<0><<<pgrid(w0), 32 * w0, 0, st>>>(s);
    else if (mode == 1) kb_part_scatter<1><<<pgrid(w1), 32 * w1, 0, st>>>(s);
    else kb_part_scatter<2><<<pgrid(w2), 32 * w2, 0, st>>>(s);
  };
  if (b->any_sgmp) {
    prof_begin(K_SG_CLEAR, st);
    kb_sg_clear<<<gridn(s.NC, nb), nb, 0, st>>>(s);
    prof_end(K_SG_CLEAR, st);
  }
  prof_begin(K_SCATTER_MASS, st);
  scatter(0);
  prof_end(K_SCATTER_MASS, st);
  prof_begin(K_P2G_MASS, st);
  kb_p2g_mass<<<gridn(s.NN, nb), nb, 0, st>>>(s, 1, 1);
  prof_end(K_P2G_MASS, st);
  auto stress = [&](int usf_pass) -> int {
    if (b->any_sgmp) {
      prof_begin(K_SG_GRADIENT, st);
      kb_sg_centre_gradient<<<gridn(s.NC, nb), nb, 0, st>>>(s, usf_pass);
      prof_end(K_SG_GRADIENT, st);
    }
    prof_begin(K_STRESS, st);
    // one launch per material instantiation present (each takes its own
    // particles); usually a single one
    // (and per volume update: by Fp or not)
    const unsigned ty = b->stress_types;
    const int f = __builtin_popcount(ty) > 1, uvf = b->any_uvfp && b->any_nonuvfp;
    auto launch = [&](auto kern) { kern<<<gridn(s.NP, pb), pb, 0, st>>>(s, usf_pass, f, uvf); };
    if (b->any_nonuvfp) {
      if (ty & (1u << 1)) launch(kb_stress<1, 0>);
      if (ty & (1u << 9)) launch(kb_stress<9, 0>);
      if (ty & (1u << 10)) launch(kb_stress<10, 0>);
      if (ty & (1u << 11)) launch(kb_stress<11, 0>);
      if (ty & 1u) launch(kb_stress<0, 0>);
    }
    if (b->any_uvfp) {
      if (ty & (1u << 1)) launch(kb_stress<1, 1>);
      if (ty & (1u << 9)) launch(kb_stress<9, 1>);
      if (ty & (1u << 10)) launch(kb_stress<10, 1>);
      if (ty & (1u << 11)) launch(kb_stress<11, 1>);
      if (ty & 1u) launch(kb_stress<0, 1>);
    }
    prof_end(K_STRESS, st);
    if (b->any_jc) {
      prof_begin(K_DEPEFF, st);
      scan_tiles_enqueue(IntScan<ScanMax>{s.setter, s.setter_scan, s.NP}, s.tiles, st);
      kb_depeff_apply<<<gridn(s.NP, pb), pb, 0, st>>>(s, usf_pass);
      kb_depeff_carry<<<gridn(s.nscene, 128), 128, 0, st>>>(s, usf_pass);
      prof_end(K_DEPEFF, st);
    }
    return MPM_OK;
  };
  int r;
  if (b->any_usf && (r = stress(1))) return r;
  if (b->any_prep) {  // (USF scenes without Johnson-Cook tails are staged by their stress kernel)
    prof_begin(K_FORCE_PREP, st);
    kb_force_prep<<<gridn(s.NP, pb), pb, 0, st>>>(s);
    prof_end(K_FORCE_PREP, st);
  }
  prof_begin(K_SCATTER_FORCE, st);
  scatter(2);
  prof_end(K_SCATTER_FORCE, st);
  prof_begin(K_P2G_FORCE, st);
  kb_p2g_force<<<gridn(s.NN, nb), nb, 0, st>>>(s);
  prof_end(K_P2G_FORCE, st);
  if (b->any_sgmp) {
    prof_begin(K_SG_VELOCITY, st);
    kb_sg_centre_velocity<<<gridn(s.NC, nb), nb, 0, st>>>(s);
    prof_end(K_SG_VELOCITY, st);
  }
  prof_begin(K_POSITION, st);
  kb_position<<<gridn(s.NP, pb), pb, 0, st>>>(s);
  prof_end(K_POSITION, st);
  if (b->any_musl) {
    prof_begin(K_SCATTER_MOM, st);
    scatter(1);
    prof_end(K_SCATTER_MOM, st);
    prof_begin(K_P2G_MOM, st);
    kb_p2g_momentum<<<gridn(s.NN, nb), nb, 0, st>>>(s);
    prof_end(K_P2G_MOM, st);
  }
  if (b->any_later && (r = stress(0))) return r;
  return MPM_OK;
}

// calcEnergy + UpdateDT (+ dynamic relaxation) of the step that just ran,
// on stream st
int enqueue_reduce(mpm_batch* b, cudaStream_t st) {
  BState& s = b->A;
  const int pb = b->pblock;
  prof_begin(K_REDUCE, st);
  kb_reduce_chunks<<<(unsigned)s.NR, 256, 0, st>>>(s, 3);
  prof_end(K_REDUCE, st);
  if (b->any_dr) {
    prof_begin(K_DR, st);
    kb_dr_damping<<<gridn(s.NP, pb), pb, 0, st>>>(s);
    kb_dr_finish<<<gridn(s.nscene, 128), 128, 0, st>>>(s);
    prof_end(K_DR, st);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return berr(b, MPM_ERR_CUDA, "launch: %s", cudaGetErrorString(e));
  return MPM_OK;
}

// one whole step, in order
int enqueue_step(mpm_batch* b) {
  int r = enqueue_front(b);
  if (!r) r = enqueue_back(b);
  if (!r) r = enqueue_reduce(b, b->stream);
  return r;
}

// one step whose front overlaps the previous step's reduction (lead), which
// then runs on the side stream; without lead the step ends before its own
// reduction, which the caller enqueues (the next step's lead, or the tail of
// a run)
int enqueue_step_overlapped(mpm_batch* b, bool lead) {
  if (lead) {
    BCK(cudaEventRecord(b->ev_fork, b->stream));
    BCK(cudaStreamWaitEvent(b->side, b->ev_fork, 0));
    if (int r = enqueue_reduce(b, b->side)) return r;
    BCK(cudaEventRecord(b->ev_join, b->side));
  }
  int r = enqueue_front(b);
  if (lead) BCK(cudaStreamWaitEvent(b->stream, b->ev_join, 0));
  if (!r) r = enqueue_back(b);
  if (!r) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return berr(b, MPM_ERR_CUDA, "launch: %s", cudaGetErrorString(e));
  }
  return r;
}

void drop_graph(mpm_batch* b) {
  for (auto& gp : b->graph)
    for (auto& g : gp) {
      if (g) cudaGraphExecDestroy(g);
      g = nullptr;
    }
  for (auto& g : b->loop_graph) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
}

// capture nsteps steps into an executable graph; the host-side buffer handles
// end swapped nsteps times, as after running the steps eagerly. lead < 0:
// whole steps in order; otherwise one overlapped step (with or without the
// previous step's reduction)
int capture(mpm_batch* b, int nsteps, cudaGraphExec_t* out, int lead = -1) {
  cudaGraph_t g;
  BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  b->prof.capturing = true;
  int r = MPM_OK;
  if (lead >= 0) r = enqueue_step_overlapped(b, lead != 0);
  else
    for (int i = 0; i < nsteps && r == MPM_OK; ++i) r = enqueue_step(b);
  b->prof.capturing = false;
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (r) {
    if (e == cudaSuccess) cudaGraphDestroy(g);
    return r;
  }
  if (e != cudaSuccess) return berr(b, MPM_ERR_CUDA, "end capture: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return berr(b, MPM_ERR_CUDA, "instantiate: %s", cudaGetErrorString(e));
  return MPM_OK;
}

// ------------------------------------------------ device-resident loop
// The loop test: iterate again while no scene has taken its last step since
// the loop began, some scene still has steps to take, the host has not
// asked the loop to return (flag, page-locked host memory read through its
// device mapping) and the iteration budget is not spent. One block.
__device__ __forceinline__ void loop_decide(const BState& b, const int* target, const volatile int* flag,
                                            cudaGraphConditionalHandle h) {
  bool pending = false;
  for (int s = threadIdx.x; s < b.nscene; s += blockDim.x) pending = pending || b.sst[s].istep < target[s];
  pending = __syncthreads_or(pending);
  if (threadIdx.x == 0) {
    const LoopCtl& c = *b.ctl;
    const bool go = pending && c.finished == c.fin0 && (*flag == 0 || c.iters < c.min_iters) && c.iters < c.max_iters;
    cudaGraphSetConditional(h, go ? 1u : 0u);
  }
}

// before the loop's first step: budget, iteration count, finished-scene mark
__global__ void kb_loop_arm(LoopCtl* c, int max_iters, int min_iters) {
  c->fin0 = c->finished;
  c->iters = 0;
  c->max_iters = max_iters;
  c->min_iters = min_iters;
}

__global__ void kb_loop_start(BState b, const int* target, const volatile int* flag, cudaGraphConditionalHandle h) {
  loop_decide(b, target, flag, h);
}

__global__ void kb_loop_test(BState b, const int* target, const volatile int* flag, cudaGraphConditionalHandle h) {
  if (threadIdx.x == 0) b.ctl->iters = b.ctl->iters + 1;
  __syncthreads();
  loop_decide(b, target, flag, h);
}

// The loop graph of the current buffer parity: a test kernel, then a WHILE
// node whose body is two overlapped steps (each with the previous step's
// reduction beside its sort) and the test again. Two steps per iteration
// bring the particle buffer sets back to the parity the graph was built
// for.
int build_loop(mpm_batch* b, cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  BCK(cudaGraphCreate(&g, 0));
  int r = MPM_OK;
  cudaGraphConditionalHandle h{};
  cudaGraphNode_t kn = nullptr, cn = nullptr;
  BState s0 = b->A;
  const int* tgt = b->d_target;
  const volatile int* flag = b->loop_flag_d;
  void* args[] = {&s0, &tgt, &flag, &h};
  cudaKernelNodeParams kp{};
  kp.func = (void*)kb_loop_start;
  kp.gridDim = dim3(1);
  kp.blockDim = dim3(256);
  kp.kernelParams = args;
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0, 0);
  if (e == cudaSuccess) e = cudaGraphAddKernelNode(&kn, g, nullptr, 0, &kp);
  if (e == cudaSuccess) {
    cp.conditional.handle = h;
    e = cudaGraphAddNode(&cn, g, &kn, nullptr, 1, &cp);
  }
  if (e == cudaSuccess)
    e = cudaStreamBeginCaptureToGraph(b->stream, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return berr(b, MPM_ERR_CUDA, "loop graph: %s", cudaGetErrorString(e));
  }
  r = enqueue_step_overlapped(b, true);
  if (!r) r = enqueue_step_overlapped(b, true);
  if (!r) kb_loop_test<<<1, 256, 0, b->stream>>>(b->A, tgt, flag, h);
  cudaGraph_t body = nullptr;
  e = cudaStreamEndCapture(b->stream, &body);
  if (!r && e != cudaSuccess) r = berr(b, MPM_ERR_CUDA, "loop body capture: %s", cudaGetErrorString(e));
  if (!r) {
    e = cudaGraphInstantiate(out, g, 0);
    if (e != cudaSuccess) r = berr(b, MPM_ERR_CUDA, "loop graph instantiate: %s", cudaGetErrorString(e));
  }
  cudaGraphDestroy(g);
  return r;
}

// one step replayed from the graph of the current buffer parity (captured on
// first use); lead: with the previous step's reduction beside the sort
int replay_step(mpm_batch* b, int lead) {
  const int par = b->A.x == b->set0_x ? 0 : 1;
  if (!b->graph[par][lead]) {
    cudaGraphExec_t ge = nullptr;
    if (int r = capture(b, 1, &ge, lead)) return r;
    b->graph[par][lead] = ge;
    std::swap(b->A, b->B);  // capture swapped the host handles; the launch below does the step
  }
  BCK(cudaGraphLaunch(b->graph[par][lead], b->stream));
  std::swap(b->A, b->B);
  return MPM_OK;
}

struct BProfScope {
  Profiler* prev;
  explicit BProfScope(mpm_batch* b) : prev(prof_current()) { prof_set_current(&b->prof); }
  ~BProfScope() { prof_set_current(prev); }
};

int commit(mpm_batch* b) {
  cudaStream_t st = b->stream;
  if (b->order.empty()) {
    drop_graph(b);
    if (b->arena) cudaFree(b->arena);
    if (b->spare) cudaFree(b->spare);
    b->arena = b->spare = nullptr;
    b->arena_cap = b->spare_cap = 0;
    b->bytes = 0;
    b->A = BState{};
    b->B = BState{};
    b->set0_x = nullptr;
    b->dirty = false;
    return MPM_OK;
  }
  // scene states of resident scenes, read back before the layout changes
  if (b->A.nscene > 0) {
    std::vector<SceneState> old((size_t)b->A.nscene);
    BCK(cudaMemcpy(old.data(), b->A.sst, sizeof(SceneState) * old.size(), cudaMemcpyDeviceToHost));
    for (HostScene* h : b->order)
      if (h->resident) h->st = old[h->index];
  }
  // new layout
  long long NP = 0, NN = 0, NK = 0, NC = 0, NR = 0;
  int nmat = 0, nbody = 0;
  std::vector<int> old_index;
  for (size_t k = 0; k < b->order.size(); ++k) {
    HostScene* h = b->order[k];
    old_index.push_back(h->resident ? h->index : -1);
  }
  std::vector<long long> old_p0, old_body0;
  for (HostScene* h : b->order) {
    old_p0.push_back(h->p0);
    old_body0.push_back(h->body0);
  }
  for (size_t k = 0; k < b->order.size(); ++k) {
    HostScene* h = b->order[k];
    const Geometry& g = h->su.g;
    h->index = (int)k;
    h->p0 = NP;
    h->n0 = NN;
    h->k0 = NK;
    h->c0 = NC;
    h->r0 = NR;
    h->nr = (h->np + kChunk - 1) / kChunk;
    if (h->nr == 0) h->nr = 1;
    h->mat0 = nmat;
    h->body0 = nbody;
    NP += h->np;
    NN += h->nn;
    NK += scene_keys(h->su.g);
    if (g.shape == 3) NC += h->ncell;
    NR += h->nr;
    nmat += (int)h->su.mats.size();
    nbody += (int)h->su.bodies.size();
  }
  if (b->order.size() > 65535 || nbody > 65535) return berr(b, MPM_ERR_UNSUPPORTED, "too many scenes / bodies");
  if (NP >= (1LL << 31) || NK >= (1LL << 31) || NN >= (1LL << 31))
    return berr(b, MPM_ERR_UNSUPPORTED, "batch too large for 32-bit indices");
  layout_flags(b);
  BState A{}, B{}, shared{};
  int* d_target = nullptr;
  int* d_map = nullptr;
  uint16_t *d_smap = nullptr, *d_bmap = nullptr;
  auto carve = [&](Alloc& al) {
  A = BState{};
  B = BState{};
  shared = BState{};
  A.NP = B.NP = NP;
  A.NN = B.NN = NN;
  A.NK = B.NK = NK;
  A.NC = B.NC = NC;
  A.NR = B.NR = NR;
  A.nscene = B.nscene = (int)b->order.size();
  A.any_uvfp = B.any_uvfp = b->any_uvfp;
  A.any_sgmp = B.any_sgmp = b->any_sgmp;
  A.any_jc = B.any_jc = b->any_jc;
  alloc_particles(al, A, NP, b->any_uvfp);
  alloc_particles(al, B, NP, b->any_uvfp);
  shared.cell = al.get<int>(NP);
  shared.dual = al.get<int>(NP);
  shared.inode = al.get<int>(NP);
  shared.off = al.get<float>(3 * NP);
  shared.xxn = al.get<float>(3 * NP);
  shared.xn = al.get<float>(3 * NP);
  shared.fs = al.get<float>(9 * NP);
  shared.m32 = al.get<float>(NP);
  shared.v32 = al.get<float>(3 * NP);
  shared.key = al.get<unsigned>(NP);
  shared.perm = al.get<int>(NP);
  shared.seg = al.get<int>(NK + 1);
  shared.inv = al.get<int>(NP);
  shared.fill = al.get<int>(NK);
  shared.tiles = al.get<int>(std::max(scan_tiles(NK), scan_tiles(NP)) + 1);
  shared.big = al.get<int>(NP / (kRegSeg + 1) + 1);
  shared.nbig = al.get<int>(1);
  shared.mg = al.get<double>(NN);
  shared.px = al.get<double>(3 * NN);
  shared.fx = al.get<double>(3 * NN);
  shared.nvel = al.get<float4>(NN);
  shared.nacc = al.get<float4>(NN);
  shared.acc = al.get<unsigned long long>(4 * NN);
  shared.fix = al.get<uint8_t>(NN);
  shared.bd = al.get<uint8_t>(NN);
  shared.node_scene = al.get<uint16_t>(NN);
  shared.cacc = al.get<unsigned long long>(CQ_N * NC);
  shared.co = al.get<float>(6 * NC);
  shared.cw = al.get<float>(3 * NC);
  shared.cdefp = al.get<float>(9 * NC);
  shared.cvx = al.get<float>(3 * NC);
  shared.cax = al.get<float>(3 * NC);
  shared.cscene = al.get<uint16_t>(NC);
  if (b->any_jc) {
    shared.setter = al.get<int>(NP);
    shared.setter_scan = al.get<int>(NP);
    shared.dep = al.get<double>(NP);
    shared.jc_aux = al.get<double>(5 * NP);
    shared.deferred = al.get<uint8_t>(NP);
  }
  shared.red_part = al.get<double>(6 * NR);
  shared.rscene = al.get<uint16_t>(NR);
  shared.scenes = al.get<Scene>((long long)b->order.size());
  shared.task0 = al.get<int>((long long)b->order.size() + 1);
  shared.sst = al.get<SceneState>((long long)b->order.size());
  shared.mats = al.get<DevMaterial>(nmat);
  shared.fmats = al.get<DevMaterialF>(nmat);
  shared.bodies = al.get<DevBody>(nbody);
  d_target = al.get<int>((long long)b->order.size());
  d_map = al.get<int>(NP);
  d_smap = al.get<uint16_t>(b->A.nscene + 1);
  d_bmap = al.get<uint16_t>(65536);
  };
  Alloc measure;
  carve(measure);
  const size_t need = measure.off + 256;
  // reuse the spare arena when the layout fits it (and it is not far larger)
  if (b->spare && (b->spare_cap < need || b->spare_cap > 3 * need)) {
    cudaFree(b->spare);
    b->spare = nullptr;
    b->spare_cap = 0;
  }
  if (!b->spare) {
    const size_t cap = need + need / 4;
    void* p = nullptr;
    if (cudaMalloc(&p, cap) != cudaSuccess) {
      cudaGetLastError();
      return berr(b, MPM_ERR_OOM, "device memory for a batch of %lld particles (%zu bytes)", NP, cap);
    }
    b->spare = (char*)p;
    b->spare_cap = cap;
  }
  Alloc al;
  al.base = b->spare;
  carve(al);
  auto share = [&](BState& s) {
    s.cell = shared.cell; s.dual = shared.dual; s.inode = shared.inode; s.off = shared.off; s.xxn = shared.xxn;
    s.xn = shared.xn; s.fs = shared.fs; s.key = shared.key; s.m32 = shared.m32; s.v32 = shared.v32;
    s.perm = shared.perm; s.seg = shared.seg; s.inv = shared.inv;
    s.fill = shared.fill; s.tiles = shared.tiles; s.big = shared.big; s.nbig = shared.nbig; s.mg = shared.mg; s.px = shared.px; s.fx = shared.fx;
    s.nvel = shared.nvel; s.nacc = shared.nacc; s.acc = shared.acc; s.fix = shared.fix; s.bd = shared.bd; s.node_scene = shared.node_scene;
    s.cacc = shared.cacc; s.co = shared.co;
    s.cw = shared.cw; s.cdefp = shared.cdefp; s.cvx = shared.cvx; s.cax = shared.cax; s.cscene = shared.cscene;
    s.setter = shared.setter; s.setter_scan = shared.setter_scan; s.dep = shared.dep; s.jc_aux = shared.jc_aux;
    s.deferred = shared.deferred; s.red_part = shared.red_part; s.rscene = shared.rscene; s.scenes = shared.scenes;
    s.task0 = shared.task0;
    s.sst = shared.sst; s.mats = shared.mats; s.fmats = shared.fmats; s.bodies = shared.bodies;
  };
  share(A);
  share(B);
  // move resident scenes on the device
  bool any_resident = false;
  for (HostScene* h : b->order) any_resident |= h->resident;
  if (any_resident) {
    std::vector<int> map((size_t)NP, -1);
    std::vector<uint16_t> smap((size_t)b->A.nscene + 1, 0);
    std::vector<uint16_t> bmap(65536, 0);
    for (size_t k = 0; k < b->order.size(); ++k) {
      HostScene* h = b->order[k];
      if (!h->resident) continue;
      for (long long i = 0; i < h->np; ++i) map[h->p0 + i] = (int)(old_p0[k] + i);
      smap[old_index[k]] = (uint16_t)h->index;
      for (size_t q = 0; q < h->su.bodies.size(); ++q) bmap[old_body0[k] + q] = (uint16_t)(h->body0 + q);
    }
    BCK(cudaMemcpyAsync(d_map, map.data(), sizeof(int) * NP, cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(d_smap, smap.data(), 2 * smap.size(), cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(d_bmap, bmap.data(), 2 * bmap.size(), cudaMemcpyHostToDevice, st));
    kb_relocate<<<gridn(NP, 256), 256, 0, st>>>(b->A, A, d_map, d_smap, d_bmap);
    BCK(cudaGetLastError());
    BCK(cudaStreamSynchronize(st));
  }
  // static per-scene tables
  std::vector<Scene> scenes;
  std::vector<DevMaterial> mats;
  std::vector<DevBody> bodies;
  std::vector<uint16_t> nscene((size_t)NN), cscene((size_t)NC), rscene((size_t)NR);
  std::vector<uint8_t> fix((size_t)NN), bd((size_t)NN);
  std::vector<int> target;
  std::vector<SceneState> sst;
  std::vector<int> task0;  // first particle task of each scene (32 particles)
  long long ntask = 0;
  for (HostScene* h : b->order) {
    const Geometry& g = h->su.g;
    task0.push_back((int)ntask);
    ntask += (h->np + 31) / 32;
    Scene sc;
    memset(&sc, 0, sizeof sc);
    sc.p0 = h->p0; sc.np = h->np; sc.n0 = h->n0; sc.nn = h->nn; sc.k0 = h->k0; sc.nk = scene_keys(g);
    sc.c0 = h->c0; sc.nc = g.shape == 3 ? h->ncell : 0; sc.r0 = h->r0; sc.nr = h->nr;
    sc.NGx = g.NGx; sc.NGy = g.NGy; sc.NGz = g.NGz; sc.NGxy = g.NGxy;
    sc.NCx = g.NCx; sc.NCy = g.NCy; sc.NCz = g.NCz; sc.NCxy = g.NCxy;
    sc.CNCx = g.CNCx; sc.CNCy = g.CNCy; sc.CNCz = g.CNCz; sc.CNCxy = g.CNCxy; sc.CNC = g.CNC;
    sc.shape = g.shape; sc.usf = g.usf; sc.musl = g.musl; sc.uvfp = g.uvfp; sc.qload = g.qload;
    sc.qdamp = g.qdamp; sc.gravity = g.gravity; sc.drdamp = h->drdamp; sc.has_jc = g.has_jc;
    for (int k = 0; k < 6; ++k) sc.fixs[k] = g.fixs[k];
    sc.mat0 = h->mat0; sc.nmat = (int)h->su.mats.size();
    for (int k = 0; k < 3; ++k) { sc.span0[k] = g.span0[k]; sc.span1[k] = g.span1[k]; }
    sc.dcell = g.dcell; sc.idcell = g.iDCell; sc.cutoff = g.cutoff; sc.iJacobi = g.iJacobi; sc.iJacobi4 = g.iJacobi4;
    sc.dtscale = g.dtscale; sc.qload_time = g.qload_time; sc.damp_factor = g.damp_factor; sc.bq1 = g.bq1; sc.bq2 = g.bq2;
    sc.fdcell = (float)g.dcell; sc.fidcell = (float)g.iDCell; sc.fbq1 = (float)g.bq1; sc.fbq2 = (float)g.bq2;
    sc.fdamp = (float)g.damp_factor; sc.fiJacobi4 = (float)g.iJacobi4; sc.fnp = (float)h->np;
    sc.has_fxp = h->any_fxp;
    for (int k = 0; k < 3; ++k) {
      sc.fspan0[k] = (float)g.span0[k];
      sc.fspan0_lo[k] = (float)(g.span0[k] - (double)sc.fspan0[k]);
      sc.fspan1[k] = (float)g.span1[k];
      sc.fspan1_lo[k] = (float)(g.span1[k] - (double)sc.fspan1[k]);
    }
    sc.fidcell_lo = (float)(g.iDCell - (double)sc.fidcell);
    sc.mNGx = div_magic(g.NGx); sc.mNGxy = div_magic(g.NGxy); sc.mNCx = div_magic(g.NCx);
    sc.mNCxy = div_magic(g.NCxy); sc.mCNCx = div_magic(g.CNCx); sc.mCNCxy = div_magic(g.CNCxy);
    scenes.push_back(sc);
    for (auto m : h->su.mats) mats.push_back(m);
    for (auto bo : h->su.bodies) {
      bo.mat += h->mat0;
      bodies.push_back(bo);
    }
    for (long long n = 0; n < h->nn; ++n) {
      nscene[h->n0 + n] = (uint16_t)h->index;
      fix[h->n0 + n] = h->su.fix[n];
      bd[h->n0 + n] = h->su.bd[n];
    }
    if (g.shape == 3)
      for (long long c = 0; c < h->ncell; ++c) cscene[h->c0 + c] = (uint16_t)h->index;
    for (long long r = 0; r < h->nr; ++r) rscene[h->r0 + r] = (uint16_t)h->index;
    target.push_back(h->steps);
    SceneState s0;
    if (h->resident) {
      s0 = h->st;
    } else {
      memset(&s0, 0, sizeof s0);
      s0.dt = set_dt(h->su.mats, g.dcell, g.dtscale);
    }
    s0.fdt = (float)s0.dt;
    s0.ftime = (float)s0.time;
    s0.active = h->resident ? 0 : 1;  // the initial energy pass below runs for new scenes only
    sst.push_back(s0);
  }
  task0.push_back((int)ntask);
  b->ntask = ntask;
  BCK(cudaMemcpyAsync(shared.task0, task0.data(), sizeof(int) * task0.size(), cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(shared.scenes, scenes.data(), sizeof(Scene) * scenes.size(), cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(shared.mats, mats.data(), sizeof(DevMaterial) * mats.size(), cudaMemcpyHostToDevice, st));
  std::vector<DevMaterialF> fmats;
  for (const DevMaterial& m : mats) fmats.push_back(material_f32(m));
  BCK(cudaMemcpyAsync(shared.fmats, fmats.data(), sizeof(DevMaterialF) * fmats.size(), cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(shared.bodies, bodies.data(), sizeof(DevBody) * bodies.size(), cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(shared.node_scene, nscene.data(), 2 * NN, cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(shared.fix, fix.data(), NN, cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(shared.bd, bd.data(), NN, cudaMemcpyHostToDevice, st));
  if (NC) BCK(cudaMemcpyAsync(shared.cscene, cscene.data(), 2 * NC, cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(shared.rscene, rscene.data(), 2 * NR, cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(d_target, target.data(), sizeof(int) * target.size(), cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(shared.sst, sst.data(), sizeof(SceneState) * sst.size(), cudaMemcpyHostToDevice, st));
  BCK(cudaMemsetAsync(shared.mg, 0, sizeof(double) * NN, st));
  BCK(cudaMemsetAsync(shared.px, 0, sizeof(double) * 3 * NN, st));
  BCK(cudaMemsetAsync(shared.fx, 0, sizeof(double) * 3 * NN, st));
  BCK(cudaMemsetAsync(shared.nvel, 0, sizeof(float4) * NN, st));
  BCK(cudaMemsetAsync(shared.nacc, 0, sizeof(float4) * NN, st));
  BCK(cudaMemsetAsync(shared.acc, 0, sizeof(unsigned long long) * 4 * NN, st));
  if (NC) BCK(cudaMemsetAsync(shared.cacc, 0, sizeof(unsigned long long) * CQ_N * NC, st));
  // every depeff setter entry is -1 or its own index (the max-scan relies on
  // it); only Johnson-Cook scenes rewrite theirs each step
  if (b->any_jc) {
    BCK(cudaMemsetAsync(shared.setter, 0xff, sizeof(int) * NP, st));
    BCK(cudaMemsetAsync(shared.deferred, 0, NP, st));
  }
  for (HostScene* h : b->order)
    if (!h->resident) {
      int r = upload_scene_particles(b, h, A);
      if (r) return r;
    }
  // inverse permutation of the new layout (rebuilt before the first
  // download or probe after later steps)
  kb_inverse<<<gridn(NP, 256), 256, 0, st>>>(A);
  b->inv_stale = false;
  // calcEnergy of the new scenes (MPM3D.f90:42)
  kb_reduce_chunks<<<(unsigned)NR, 256, 0, st>>>(A, 1);
  BCK(cudaGetLastError());
  BCK(cudaStreamSynchronize(st));
  // swap in the new layout: its arena becomes current, the old one spare
  drop_graph(b);
  std::swap(b->arena, b->spare);
  std::swap(b->arena_cap, b->spare_cap);
  b->bytes = (long long)(b->arena_cap + b->spare_cap);
  A.ctl = B.ctl = b->ctl;
  b->A = A;
  b->B = B;
  b->set0_x = A.x;
  b->d_target = d_target;
  for (HostScene* h : b->order) {
    if (!h->resident) h->release_inputs();  // the scene's inputs are on the device now
    h->resident = true;
  }
  b->dirty = false;
  return MPM_OK;
}

int ensure_committed(mpm_batch* b) {
  if (b->dirty) return commit(b);
  return MPM_OK;
}

HostScene* find(mpm_batch* b, int id) {
  auto it = b->by_id.find(id);
  return it == b->by_id.end() ? nullptr : it->second;
}

}  // namespace

extern "C" {

int mpm_batch_create(int device, mpm_batch** out) {
  if (!out) return MPM_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MPM_ERR_CUDA;
  if (device >= ndev) return MPM_ERR_ARG;
  if (device >= 0) cudaSetDevice(device);
  mpm_batch* b = new mpm_batch();
  cudaGetDevice(&b->device);
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device) == cudaSuccess && sms > 0)
  {
    b->scatter_blocks = 64 * sms;
    b->sort_blocks = sms;
    b->sms = sms;
  }
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaMalloc((void**)&b->ctl, sizeof(LoopCtl)) != cudaSuccess ||
      cudaMemset(b->ctl, 0, sizeof(LoopCtl)) != cudaSuccess ||
      cudaHostAlloc((void**)&b->loop_flag_h, sizeof(int), cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess ||
      cudaHostGetDevicePointer((void**)&b->loop_flag_d, (void*)b->loop_flag_h, 0) != cudaSuccess) {
    if (b->ctl) cudaFree(b->ctl);
    if (b->loop_flag_h) cudaFreeHost((void*)b->loop_flag_h);

    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return MPM_ERR_CUDA;
  }
  *out = b;
  return MPM_OK;
}

void mpm_batch_destroy(mpm_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  drop_graph(b);
  if (b->arena) cudaFree(b->arena);
  if (b->spare) cudaFree(b->spare);
  if (b->g_items_h) cudaFreeHost(b->g_items_h);
  if (b->g_out_h) cudaFreeHost(b->g_out_h);
  if (b->g_items_d) cudaFree(b->g_items_d);
  if (b->g_out_d) cudaFree(b->g_out_d);
  if (b->g_done) cudaEventDestroy(b->g_done);
  if (b->dl) cudaFree(b->dl);
  for (auto& kv : b->by_id) delete kv.second;
  prof_free(&b->prof);
  cudaStreamSynchronize(b->side);
  cudaEventDestroy(b->ev_fork);
  cudaEventDestroy(b->ev_join);
  cudaFree(b->ctl);
  cudaFreeHost((void*)b->loop_flag_h);
  cudaStreamDestroy(b->side);
  cudaStreamDestroy(b->stream);
  delete b;
}

const char* mpm_batch_last_error(const mpm_batch* b) { return b ? b->err.c_str() : "null batch"; }

int64_t mpm_scene_device_bytes(const mpm_deck* d) {
  if (!d) return -1;
  SceneSetup su;
  if (scene_setup(d, su)) return -1;
  return scene_bytes(d->nb_particle, su.g.nn, su.g.ncell, su.g.shape == 3, su.g.uvfp, su.g.has_jc);
}

int mpm_batch_add(mpm_batch* b, const mpm_deck* d, int steps, int* scene_id) {
  if (!b || !d) return MPM_ERR_ARG;
  int code = MPM_OK;
  HostScene* h = scene_stage(d, steps, b->err, &code);
  if (!h) return code;
  return batch_insert(b, h, scene_id);
}

int mpm_batch_remove(mpm_batch* b, int id) {
  if (!b) return MPM_ERR_ARG;
  HostScene* h = find(b, id);
  if (!h) return berr(b, MPM_ERR_ARG, "no scene %d", id);
  if (h->resident && b->A.nscene > 0) {
    // keep the other scenes' states: read them now (commit reads by index)
    std::vector<SceneState> old((size_t)b->A.nscene);
    BCK(cudaStreamSynchronize(b->stream));
    BCK(cudaMemcpy(old.data(), b->A.sst, sizeof(SceneState) * old.size(), cudaMemcpyDeviceToHost));
    for (HostScene* o : b->order)
      if (o->resident) o->st = old[o->index];
  }
  b->order.erase(std::find(b->order.begin(), b->order.end(), h));
  b->by_id.erase(id);
  delete h;
  b->dirty = true;
  return MPM_OK;
}

int mpm_batch_commit(mpm_batch* b) {
  if (!b) return MPM_ERR_ARG;
  cudaSetDevice(b->device);
  BCK(cudaStreamSynchronize(b->stream));
  return commit(b);
}

int64_t mpm_batch_device_bytes(const mpm_batch* b) { return b ? b->bytes : -1; }
int mpm_batch_scene_count(const mpm_batch* b) { return b ? (int)b->order.size() : -1; }

int mpm_batch_run(mpm_batch* b, int nsteps, int use_graph) {
  if (!b) return MPM_ERR_ARG;
  if (nsteps <= 0) return MPM_OK;
  cudaSetDevice(b->device);
  int r = ensure_committed(b);
  if (r) return r;
  if (b->order.empty()) return MPM_OK;
  b->inv_stale = true;
  BProfScope ps(b);
  if (!use_graph) {
    // each step's reduction overlaps the next step's sort; the last one ends
    // the run, so nothing is pending between calls
    for (int i = 0; i < nsteps; ++i)
      if ((r = enqueue_step_overlapped(b, i > 0))) return r;
    return enqueue_reduce(b, b->stream);
  }
  if (b->prof.on) {
    // one graph over all the steps, with event nodes around every kernel
    drop_graph(b);
    b->prof.nrec = 0;
    b->prof.next = 0;
    cudaGraphExec_t ge = nullptr;
    if ((r = capture(b, nsteps, &ge))) return r;
    cudaError_t e = cudaGraphLaunch(ge, b->stream);
    cudaGraphExecDestroy(ge);
    if (e != cudaSuccess) return berr(b, MPM_ERR_CUDA, "graph launch: %s", cudaGetErrorString(e));
    return MPM_OK;
  }
  // one graph of one step per buffer parity (the step swaps the two particle
  // buffer sets, so the graph captured from either set is replayed
  // alternately), the steps after the first of the run with the previous
  // step's reduction overlapping their sort; the run's last reduction ends it
  for (int i = 0; i < nsteps; ++i)
    if ((r = replay_step(b, i > 0 ? 1 : 0))) return r;
  return enqueue_reduce(b, b->stream);
}

int mpm_batch_run_loop(mpm_batch* b, int max_steps, int* steps) {
  if (!b || !steps || max_steps < 1) return MPM_ERR_ARG;
  *steps = 0;
  cudaSetDevice(b->device);
  int r = ensure_committed(b);
  if (r) return r;
  if (b->order.empty()) return MPM_OK;
  b->inv_stale = true;
  *b->loop_flag_h = 0;
  // the first step (its reduction overlaps the loop's first step), then the
  // loop's iterations of two steps, then the last step's reduction
  kb_loop_arm<<<1, 1, 0, b->stream>>>(b->ctl, (max_steps - 1) / 2, b->loop_min_steps / 2);
  if ((r = replay_step(b, 0))) return r;
  const int par = b->A.x == b->set0_x ? 0 : 1;
  if (!b->loop_graph[par]) {
    cudaGraphExec_t ge = nullptr;
    if ((r = build_loop(b, &ge))) return r;
    b->loop_graph[par] = ge;
  }
  BCK(cudaGraphLaunch(b->loop_graph[par], b->stream));
  if ((r = enqueue_reduce(b, b->stream))) return r;
  LoopCtl c{};
  BCK(cudaMemcpyAsync(&c, b->ctl, sizeof c, cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  *b->loop_flag_h = 0;  // an interrupt is consumed by the loop it ended (or the next one)
  *steps = 1 + 2 * c.iters;
  return MPM_OK;
}

int mpm_batch_interrupt(mpm_batch* b) {
  if (!b) return MPM_ERR_ARG;
  *b->loop_flag_h = 1;  // read by the loop test through the device mapping
  return MPM_OK;
}

int mpm_batch_sync(mpm_batch* b) {
  if (!b) return MPM_ERR_ARG;
  BCK(cudaStreamSynchronize(b->stream));
  if (b->A.nscene == 0) return MPM_OK;
  std::vector<SceneState> s((size_t)b->A.nscene);
  BCK(cudaMemcpy(s.data(), b->A.sst, sizeof(SceneState) * s.size(), cudaMemcpyDeviceToHost));
  for (auto& x : s)
    if (x.status & ST_NONFINITE) return berr(b, MPM_ERR_NONFINITE, "non-finite particle state");
  return MPM_OK;
}

int mpm_batch_time_steps(mpm_batch* b, int nsteps, int use_graph, double* ms) {
  if (!b || !ms) return MPM_ERR_ARG;
  int r = ensure_committed(b);
  if (r) return r;
  cudaEvent_t e0, e1;
  BCK(cudaEventCreate(&e0));
  BCK(cudaEventCreate(&e1));
  BCK(cudaStreamSynchronize(b->stream));
  BCK(cudaEventRecord(e0, b->stream));
  r = mpm_batch_run(b, nsteps, use_graph);
  BCK(cudaEventRecord(e1, b->stream));
  BCK(cudaEventSynchronize(e1));
  float f = 0;
  cudaEventElapsedTime(&f, e0, e1);
  *ms = f;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (b->prof.on) prof_harvest(&b->prof, b->stream);
  return r;
}

int mpm_batch_scene_scalars(mpm_batch* b, int id, double* o) {
  if (!b || !o) return MPM_ERR_ARG;
  HostScene* h = find(b, id);
  if (!h) return berr(b, MPM_ERR_ARG, "no scene %d", id);
  memset(o, 0, sizeof(double) * MPM_NSCALARS);
  SceneState s = h->st;
  if (h->resident && !b->dirty) {
    BCK(cudaStreamSynchronize(b->stream));
    BCK(cudaMemcpy(&s, b->A.sst + h->index, sizeof s, cudaMemcpyDeviceToHost));
  }
  o[0] = s.istep; o[1] = s.time; o[2] = s.dt; o[3] = s.ke; o[4] = s.ie;
  o[5] = s.mom[0]; o[6] = s.mom[1]; o[7] = s.mom[2]; o[8] = s.ke_prev;
  o[9] = (double)h->nn; o[10] = (double)h->np; o[11] = h->su.g.cutoff; o[12] = h->su.g.dcell;
  o[13] = (double)s.active_nodes; o[14] = s.status;
  return MPM_OK;
}

// Spre of a scene (SmoothStressbyGrid on its state after the last step;
// zero without 'smoo', as in the reference), in its input order
static int scene_spre(mpm_batch* b, HostScene* h, double* out) {
  if (!h->smooth) {
    std::fill(out, out + h->np, 0.0);
    return MPM_OK;
  }
  const BState& s = b->A;
  const long long nodes = h->su.g.shape == 3 ? h->ncell : h->nn;
  const size_t bytes = sizeof(unsigned) * 2 + sizeof(unsigned long long) * 2 * (size_t)nodes +
                       sizeof(double) * ((size_t)h->nn + (size_t)h->ncell + (size_t)h->np);
  char* tmp = nullptr;
  BCK(cudaMalloc(&tmp, bytes));
  unsigned* bnd = reinterpret_cast<unsigned*>(tmp);
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(tmp + 8);
  double* gpre = reinterpret_cast<double*>(acc + 2 * nodes);
  double* cgpre = gpre + h->nn;
  double* spre = cgpre + h->ncell;
  cudaStream_t st = b->stream;
  cudaError_t e = cudaMemsetAsync(tmp, 0, 8 + sizeof(unsigned long long) * 2 * (size_t)nodes, st);
  if (e == cudaSuccess) {
    kb_smooth_bound<<<gridn(h->np, 256), 256, 0, st>>>(s, h->index, bnd);
    kb_smooth_p2g<<<gridn(h->np, 256), 256, 0, st>>>(s, h->index, bnd, acc);
    kb_smooth_node<<<gridn(h->nn, 256), 256, 0, st>>>(s, h->index, bnd, acc, gpre);
    if (h->su.g.shape == 3) kb_smooth_back<<<gridn(h->ncell, 256), 256, 0, st>>>(s, h->index, gpre, cgpre);
    kb_smooth_g2p<<<gridn(h->np, 256), 256, 0, st>>>(s, h->index, gpre, cgpre, spre);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, spre, sizeof(double) * (size_t)h->np, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(tmp);
  if (e != cudaSuccess) return berr(b, MPM_ERR_CUDA, "stress smoothing: %s", cudaGetErrorString(e));
  return MPM_OK;
}

namespace {
// the inverse permutation (deck index -> position) of the current order,
// rebuilt on the batch stream when steps ran since it was last built
void fresh_inverse(mpm_batch* b) {
  if (!b->inv_stale) return;
  kb_inverse<<<gridn(b->A.NP, 256), 256, 0, b->stream>>>(b->A);
  b->inv_stale = false;
}
}  // namespace

int mpm_batch_scene_download(mpm_batch* b, int id, int field, double* out) {
  if (!b || !out) return MPM_ERR_ARG;
  int r = ensure_committed(b);
  if (r) return r;
  HostScene* h = find(b, id);
  if (!h) return berr(b, MPM_ERR_ARG, "no scene %d", id);
  BCK(cudaStreamSynchronize(b->stream));
  const BState& s = b->A;
  const long long NP = s.NP, np = h->np, p0 = h->p0;
  const int nc = mpm_field_components(field);
  if (field == MPM_G_MG || field == MPM_G_PX || field == MPM_G_FX) {
    const double* src = field == MPM_G_MG ? s.mg : (field == MPM_G_PX ? s.px : s.fx);
    for (int a = 0; a < nc; ++a)
      BCK(cudaMemcpy(out + a * h->nn, src + a * s.NN + h->n0, sizeof(double) * h->nn, cudaMemcpyDeviceToHost));
    if (field == MPM_G_MG)  // -0 marks a massless node with a force or momentum (the idle test)
      for (long long k = 0; k < h->nn; ++k) out[k] = out[k] + 0.0;
    return MPM_OK;
  }
  if (field == MPM_P_SPRE) return scene_spre(b, h, out);
  if (field == MPM_C_MG || field == MPM_C_PX) {
    if (h->su.g.shape != 3) return berr(b, MPM_ERR_ARG, "no auxiliary grid (not SGMP)");
    // decoded from the fixed-point sums, one component at a time
    double* tmp = nullptr;
    BCK(cudaMalloc(&tmp, sizeof(double) * (size_t)std::max<long long>(h->ncell, 1)));
    cudaError_t e = cudaSuccess;
    for (int a = 0; a < nc && e == cudaSuccess; ++a) {
      kb_centre_field<<<gridn(h->ncell, 256), 256, 0, b->stream>>>(s, h->index, field == MPM_C_MG ? -1 : a, tmp);
      e = cudaGetLastError();
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(out + a * h->ncell, tmp, sizeof(double) * h->ncell, cudaMemcpyDeviceToHost, b->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    }
    cudaFree(tmp);
    if (e != cudaSuccess) return berr(b, MPM_ERR_CUDA, "centre field: %s", cudaGetErrorString(e));
    return MPM_OK;
  }
  // particle fields: every component un-permuted on the device by one kernel
  // into a download buffer kept by the batch, then one copy
  const bool ok = field >= MPM_P_XP && field <= MPM_P_FAILURE && field != MPM_P_XN && field != MPM_P_XXN &&
                  field != MPM_P_VOL0 && nc > 0 && (field != MPM_P_FP || b->any_uvfp);
  if (!ok) return berr(b, MPM_ERR_ARG, "field %d is not available for batched scenes", field);
  (void)NP;
  (void)p0;
  const size_t bytes = sizeof(double) * (size_t)np * (size_t)nc;
  if (bytes > b->dl_cap) {
    if (b->dl) cudaFree(b->dl);
    b->dl = nullptr;
    b->dl_cap = 0;
    BCK(cudaMalloc(&b->dl, bytes));
    b->dl_cap = bytes;
  }
  fresh_inverse(b);
  kb_unpermute<<<gridn(np * nc, 256), 256, 0, b->stream>>>(s, h->index, field, nc, b->dl);
  BCK(cudaGetLastError());
  mpm::prefault_host(out, bytes);  // while the kernel runs
  BCK(cudaMemcpyAsync(out, b->dl, bytes, cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return MPM_OK;
}

}  // extern "C"

namespace {
// the particle arrays a restart of a scene needs (the rest is rebuilt by the
// next step): device array, bytes per element, components
struct RestartField {
  void* p;
  size_t elem;
  int nc;
};
std::vector<RestartField> restart_fields(const BState& s, bool uvfp) {
  std::vector<RestartField> f = {{s.x, 8, 3},     {s.v, 8, 3},       {s.fxp, 8, 3},   {s.mass, 8, 1},  {s.ie, 8, 1},
                                 {s.vol, 4, 1},   {s.evol, 4, 1},    {s.sig_y, 4, 1}, {s.sm, 4, 1},    {s.seqv, 4, 1},
                                 {s.sd, 4, 6},    {s.epeff, 4, 1},   {s.celsius, 4, 1}, {s.dmg, 4, 1}, {s.lt, 4, 1},
                                 {s.cp, 4, 1},    {s.q, 4, 1},       {s.failure, 1, 1}, {s.body, 2, 1}, {s.scene, 2, 1},
                                 {s.orig, 4, 1}};
  if (uvfp) f.push_back({s.fp, 4, 18});
  return f;
}
}  // namespace

namespace mpm {

long long mpm_batch_scene_restart_bytes(mpm_batch* b, int id) {
  if (!b || ensure_committed(b)) return -1;
  HostScene* h = find(b, id);
  if (!h) return -1;
  long long n = (long long)sizeof(SceneState);
  for (const RestartField& f : restart_fields(b->A, h->su.g.uvfp != 0)) n += (long long)f.nc * h->np * (long long)f.elem;
  return n;
}

int mpm_batch_scene_snapshot(mpm_batch* b, int id, std::vector<unsigned char>& out) {
  if (!b) return MPM_ERR_ARG;
  int r = ensure_committed(b);
  if (r) return r;
  HostScene* h = find(b, id);
  if (!h) return berr(b, MPM_ERR_ARG, "no scene %d", id);
  BCK(cudaStreamSynchronize(b->stream));
  const BState& s = b->A;
  const long long NP = s.NP, np = h->np, p0 = h->p0;
  SceneState st;
  BCK(cudaMemcpy(&st, s.sst + h->index, sizeof st, cudaMemcpyDeviceToHost));
  out.assign(reinterpret_cast<const unsigned char*>(&st), reinterpret_cast<const unsigned char*>(&st) + sizeof st);
  for (const RestartField& f : restart_fields(s, h->su.g.uvfp != 0))
    for (int a = 0; a < f.nc; ++a) {
      const size_t at = out.size(), n = (size_t)np * f.elem;
      out.resize(at + n);
      if (f.p == static_cast<const void*>(s.fxp) && !h->any_fxp) {
        memset(out.data() + at, 0, n);  // (not moved by the permutation: zero in the deck, never read)
        continue;
      }
      BCK(cudaMemcpy(out.data() + at, static_cast<const char*>(f.p) + ((size_t)a * NP + p0) * f.elem, n,
                     cudaMemcpyDeviceToHost));
    }
  return MPM_OK;
}

int mpm_batch_scene_restore(mpm_batch* b, int id, const unsigned char* in, size_t bytes) {
  if (!b || !in) return MPM_ERR_ARG;
  int r = ensure_committed(b);
  if (r) return r;
  HostScene* h = find(b, id);
  if (!h) return berr(b, MPM_ERR_ARG, "no scene %d", id);
  BCK(cudaStreamSynchronize(b->stream));
  const BState& s = b->A;
  const long long NP = s.NP, np = h->np, p0 = h->p0;
  const std::vector<RestartField> fields = restart_fields(s, h->su.g.uvfp != 0);
  size_t need = sizeof(SceneState);
  for (const RestartField& f : fields) need += (size_t)f.nc * (size_t)np * f.elem;
  if (bytes != need) return berr(b, MPM_ERR_STATE, "restart image of %zu bytes, the scene needs %zu", bytes, need);
  SceneState st;
  memcpy(&st, in, sizeof st);
  size_t at = sizeof st;
  for (const RestartField& f : fields)
    for (int a = 0; a < f.nc; ++a) {
      const size_t n = (size_t)np * f.elem;
      BCK(cudaMemcpy(static_cast<char*>(f.p) + ((size_t)a * NP + p0) * f.elem, in + at, n, cudaMemcpyHostToDevice));
      at += n;
    }
  // positions and their copy agree at the end of every step
  for (int a = 0; a < 3; ++a)
    BCK(cudaMemcpy(s.xx + a * NP + p0, s.x + a * NP + p0, sizeof(double) * np, cudaMemcpyDeviceToDevice));
  BCK(cudaMemcpy(s.sst + h->index, &st, sizeof st, cudaMemcpyHostToDevice));
  h->st = st;
  b->inv_stale = true;
  return MPM_OK;
}

}  // namespace mpm

extern "C" {

int mpm_batch_scene_gather_async(mpm_batch* b, int id, int n, const int64_t* particle, const int* field,
                                 const int* component) {
  if (!b || n < 0 || n > MPM_GATHER_MAX || (n > 0 && (!particle || !field || !component))) return MPM_ERR_ARG;
  int r = ensure_committed(b);
  if (r) return r;
  HostScene* h = find(b, id);
  if (!h) return berr(b, MPM_ERR_ARG, "no scene %d", id);
  for (int k = 0; k < n; ++k) {
    const int f = field[k], nc = mpm_field_components(f);
    const bool ok = f >= MPM_P_XP && f <= MPM_P_FAILURE && f != MPM_P_XN && f != MPM_P_XXN && f != MPM_P_VOL0 &&
                    nc > 0 && component[k] >= 0 && component[k] < nc && particle[k] >= 0 && particle[k] < h->np &&
                    (f != MPM_P_FP || b->any_uvfp);
    if (!ok)
      return berr(b, MPM_ERR_ARG, "gather item %d: particle %lld field %d component %d", k, (long long)particle[k], f,
                  component[k]);
  }
  if (!b->g_items_h) {
    BCK(cudaMallocHost((void**)&b->g_items_h, sizeof(GatherItem) * MPM_GATHER_MAX));
    BCK(cudaMallocHost((void**)&b->g_out_h, sizeof(double) * MPM_GATHER_MAX));
    BCK(cudaMalloc((void**)&b->g_items_d, sizeof(GatherItem) * MPM_GATHER_MAX));
    BCK(cudaMalloc((void**)&b->g_out_d, sizeof(double) * MPM_GATHER_MAX));
    BCK(cudaEventCreateWithFlags(&b->g_done, cudaEventDisableTiming));
  }
  BCK(cudaEventSynchronize(b->g_done));
  for (int k = 0; k < n; ++k) b->g_items_h[k] = GatherItem{(long long)particle[k], field[k], component[k]};
  b->g_n = n;
  if (n > 0) {
    BCK(cudaMemcpyAsync(b->g_items_d, b->g_items_h, sizeof(GatherItem) * n, cudaMemcpyHostToDevice, b->stream));
    fresh_inverse(b);
    kb_gather<<<(n + 127) / 128, 128, 0, b->stream>>>(b->A, h->index, b->g_items_d, n, b->g_out_d);
    BCK(cudaGetLastError());
    BCK(cudaMemcpyAsync(b->g_out_h, b->g_out_d, sizeof(double) * n, cudaMemcpyDeviceToHost, b->stream));
  }
  BCK(cudaEventRecord(b->g_done, b->stream));
  return MPM_OK;
}

int mpm_batch_scene_gather_wait(mpm_batch* b, double* out) {
  if (!b || !out) return MPM_ERR_ARG;
  if (!b->g_done) return berr(b, MPM_ERR_STATE, "no gather in flight");
  BCK(cudaEventSynchronize(b->g_done));
  memcpy(out, b->g_out_h, sizeof(double) * (size_t)b->g_n);
  return MPM_OK;
}

int mpm_batch_set_blocks(mpm_batch* b, int pblock, int nblock) {
  if (!b) return MPM_ERR_ARG;
  auto ok = [](int x) { return x == 0 || (x >= 32 && x <= 512 && (x % 32) == 0); };
  if (!ok(pblock) || !ok(nblock)) return berr(b, MPM_ERR_ARG, "block sizes must be multiples of 32 in 32..512");
  if (pblock) b->pblock = pblock;
  if (nblock) b->nblock = nblock;
  drop_graph(b);
  return MPM_OK;
}

int mpm_batch_set_option(mpm_batch* b, int option, int value) {
  if (!b) return MPM_ERR_ARG;
  switch (option) {
    case MPM_BATCH_PARTICLE_BLOCK: return mpm_batch_set_blocks(b, value, 0);
    case MPM_BATCH_NODE_BLOCK: return mpm_batch_set_blocks(b, 0, value);
    case MPM_BATCH_SCATTER_BLOCKS:
      if (value < 1 || value > 64) return berr(b, MPM_ERR_ARG, "scatter blocks per SM %d not in 1..64", value);
      if (b->scatter_blocks != value * b->sms) {
        b->scatter_blocks = value * b->sms;
        drop_graph(b);
      }
      return MPM_OK;
    case MPM_BATCH_LOOP_MIN_STEPS:
      if (value < 0) return berr(b, MPM_ERR_ARG, "loop minimum steps %d < 0", value);
      b->loop_min_steps = value;
      return MPM_OK;
    default: return berr(b, MPM_ERR_ARG, "unknown batch option %d", option);
  }
}

int mpm_batch_get_option(const mpm_batch* b, int option) {
  if (!b) return -1;
  switch (option) {
    case MPM_BATCH_PARTICLE_BLOCK: return b->pblock;
    case MPM_BATCH_NODE_BLOCK: return b->nblock;
    case MPM_BATCH_SCATTER_BLOCKS: return b->scatter_blocks / b->sms;
    case MPM_BATCH_LOOP_MIN_STEPS: return b->loop_min_steps;
    default: return -1;
  }
}

int mpm_batch_profile_enable(mpm_batch* b, int on) {
  if (!b) return MPM_ERR_ARG;
  if (b->prof.on) prof_harvest(&b->prof, b->stream);
  prof_reset(&b->prof);
  b->prof.on = on != 0;
  drop_graph(b);
  return MPM_OK;
}

int mpm_batch_kernel_stats(mpm_batch* b, int k, char* name, int namelen, int64_t* launches, double* total_ms) {
  if (!b || k < 0 || k >= K_COUNT) return MPM_ERR_ARG;
  prof_harvest(&b->prof, b->stream);
  if (name && namelen > 0) snprintf(name, (size_t)namelen, "%s", kKernelNames[k]);
  if (launches) *launches = b->prof.n[k];
  if (total_ms) *total_ms = b->prof.ms[k];
  return MPM_OK;
}

}  // extern "C"

namespace mpm {

HostScene* scene_stage(const mpm_deck* d, int steps, std::string& err, int* code, bool borrow) {
  *code = MPM_OK;
  if (!d) {
    *code = MPM_ERR_ARG;
    err = "deck is NULL";
    return nullptr;
  }
  if (d->flags & (MPM_F_CONTACT | MPM_F_TLMPM)) {
    *code = MPM_ERR_UNSUPPORTED;
    err = "contact and TLMPM are outside the explicit-step path";
    return nullptr;
  }
  if (d->nb_component != 1 || d->nb_particle <= 0 || d->nb_body <= 0) {
    *code = d->nb_component != 1 ? MPM_ERR_UNSUPPORTED : MPM_ERR_ARG;
    err = d->nb_component != 1 ? "only one grid component" : "deck defines no particles / bodies";
    return nullptr;
  }
  HostScene* h = new HostScene();
  int r = scene_setup(d, h->su, false);  // per-particle set-up values are derived on the device
  if (r) {
    *code = r;
    err = h->su.err;
    delete h;
    return nullptr;
  }
  h->deto.n = d->n_deto;
  for (int j = 0; j < d->n_deto; ++j)
    for (int a = 0; a < 3; ++a) h->deto.p[j][a] = d->deto[j][a];
  h->steps = steps > 0 ? steps : 0x7fffffff;
  h->np = d->nb_particle;
  h->nn = h->su.g.nn;
  h->ncell = h->su.g.ncell;
  h->drdamp = !!(d->flags & MPM_F_DRDAMP);
  h->smooth = !!(d->flags & MPM_F_SMOOTH);
  if (borrow) {
    h->bmass = d->mass;
    h->bx = d->xp;
    h->bv = d->vxp;
    h->bfxp = d->fxp;
  } else {
    h->mass.assign(d->mass, d->mass + h->np);
    h->x.assign(d->xp, d->xp + 3 * h->np);
    h->v.assign(d->vxp, d->vxp + 3 * h->np);
    h->fxp.assign(d->fxp, d->fxp + 3 * h->np);
  }
  h->any_fxp = 0;
  for (long long k = 0; d->fxp && k < 3 * h->np && !h->any_fxp; ++k) h->any_fxp = d->fxp[k] != 0.0;
  h->body_local.assign((size_t)h->np, 0);
  for (int bo = 0; bo < d->nb_body; ++bo)
    for (long long p = d->bodies[bo].par_begin; p < d->bodies[bo].par_end; ++p) h->body_local[p] = (uint16_t)bo;
  return h;
}

// Touches every page of a pageable host destination buffer once from the
// CPU: a device-to-host copy into pageable pages that were never touched
// waits for the driver to fault them in one by one, several times slower
// than the CPU does it (a fresh 28 MB array: 28 ms against under 1 ms touched
// first). Page-locked buffers are resident already and are left alone.
void prefault_host(void* p, size_t bytes) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) == cudaSuccess && at.type == cudaMemoryTypeHost) return;  // page-locked
  cudaGetLastError();
  static const size_t page = (size_t)std::max(4096L, sysconf(_SC_PAGESIZE));
  volatile char* c = static_cast<volatile char*>(p);
  for (size_t k = 0; k < bytes; k += page) c[k] = 0;
  if (bytes) c[bytes - 1] = 0;
}

void scene_free(HostScene* h) { delete h; }

const SceneSetup& scene_setup_of(const HostScene* h) { return h->su; }

long long scene_np(const HostScene* h) { return h->np; }

long long scene_device_bytes(const HostScene* h) {
  return scene_bytes(h->np, h->nn, h->ncell, h->su.g.shape == 3, h->su.g.uvfp, h->su.g.has_jc);
}

int batch_insert(mpm_batch* b, HostScene* h, int* scene_id) {
  h->id = b->next_id++;
  h->resident = false;
  b->order.push_back(h);
  b->by_id[h->id] = h;
  b->dirty = true;
  if (scene_id) *scene_id = h->id;
  return MPM_OK;
}

int batch_progress(mpm_batch* b, std::vector<BatchProgress>& out) {
  out.clear();
  int r = ensure_committed(b);
  if (r) return r;
  if (b->order.empty()) return MPM_OK;
  std::vector<SceneState> s((size_t)b->A.nscene);
  BCK(cudaStreamSynchronize(b->stream));
  BCK(cudaMemcpy(s.data(), b->A.sst, sizeof(SceneState) * s.size(), cudaMemcpyDeviceToHost));
  for (HostScene* h : b->order) {
    const SceneState& t = s[h->index];
    out.push_back(BatchProgress{h->id, t.istep, h->steps, h->np, t.status});
  }
  return MPM_OK;
}

long long batch_particles(const mpm_batch* b) {
  long long n = 0;
  for (const HostScene* h : b->order) n += h->np;
  return n;
}

void batch_remaining(mpm_batch*, const std::vector<BatchProgress>& p, int* min_left) {
  int m = 0;
  bool first = true;
  for (const BatchProgress& q : p) {
    int left = q.target - q.istep;
    if (left <= 0) continue;
    if (first || left < m) m = left;
    first = false;
  }
  *min_left = m;
}

}  // namespace mpm
