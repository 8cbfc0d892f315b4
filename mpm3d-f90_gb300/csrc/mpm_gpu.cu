// mpm_gpu.cu -- host side of the C ABI declared in include/mpm3d_gpu.h.
//
// mpm_create derives the reference set-up from a parsed deck
// (Initial, DataIn.f90:1211-1267; SetGridData, Grid.f90:222-418; SetDT,
// DataIn.f90:1269-1297), uploads the structure-of-arrays state and runs the
// initial calcEnergy (MPM3D.f90:42). mpm_step enqueues one time step
// (MPM3D.f90:69-118) on the context's stream without host synchronisation;
// mpm_run replays it from a captured CUDA graph.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <new>
#include <vector>

#include "mpm3d_gpu.h"
#include "mpm_gpu_internal.cuh"
#include "mpm_batch_host.h"
#include "mpm_setup.h"

using namespace mpm;

namespace {

thread_local std::string g_lib_error;

struct MaxOp {
  __host__ __device__ int operator()(int a, int b) const { return a > b ? a : b; }
};

}  // namespace

struct GatherItem {
  long long p;
  int field, comp;
};

struct mpm_ctx {
  int precision = 0;
  const StepOps* ops = nullptr;
  Geometry g{};
  int device = 0;
  int flags = 0;
  int drdamp = 0;
  int smooth = 0;  // SmoothStressbyGrid after every step ('smoo')
  cudaStream_t stream = nullptr;
  DevState<double, double> st{};  // pointer layout is the same for every form
  std::vector<void*> allocs;
  long long bytes = 0;
  int nkeys = 0;
  long long npairs = 0;
  int key_bits = 1;
  int red_blocks = 1;
  void* cub_tmp = nullptr;
  size_t cub_tmp_bytes = 0;
  cudaGraphExec_t graph_exec = nullptr;
  int graph_steps = 0;
  bool graph_prof = false;
  std::vector<DevMaterial> mats;
  std::vector<DevBody> bodies;
  Profiler prof;
  mpm_batch* batch = nullptr;  // the mixed form runs as a batch of one scene
  int batch_scene = -1;
  // particle value gather (curve output): pinned host and device item / value buffers
  GatherItem *g_items_h = nullptr, *g_items_d = nullptr;
  double *g_out_h = nullptr, *g_out_d = nullptr;
  cudaEvent_t g_done = nullptr;
  int g_n = 0;
  std::string err;
};

namespace {

int set_err(mpm_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  else g_lib_error = buf;
  return code;
}

int cuda_err(mpm_ctx* c, cudaError_t e, const char* what) {
  return set_err(c, MPM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call)                                        \
  do {                                                  \
    cudaError_t e__ = (call);                           \
    if (e__ != cudaSuccess) return cuda_err(c, e__, #call); \
  } while (0)

template <class T>
int dalloc(mpm_ctx* c, T** p, long long n) {
  if (n <= 0) n = 1;
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, (size_t)n * sizeof(T));
  if (e != cudaSuccess) return set_err(c, MPM_ERR_OOM, "cudaMalloc(%lld bytes): %s", (long long)(n * sizeof(T)),
                                       cudaGetErrorString(e));
  c->allocs.push_back(q);
  c->bytes += n * (long long)sizeof(T);
  *p = (T*)q;
  return MPM_OK;
}

}  // namespace

namespace mpm {

const char* const kKernelNames[K_COUNT] = {
    "begin_step", "locate", "pair_sort", "segments", "p2g_mass", "node_velocity", "apply_bc",
    "stress_update", "depeff_tail", "force_prep", "p2g_force_integrate", "integrate", "g2p_position",
    "p2g_musl", "reduce_energy_dt", "dr_damping", "permute",
    "p2g_mass_scatter", "p2g_force_scatter", "p2g_musl_scatter", "sgmp_centre_clear",
    "sgmp_centre_gradient", "sgmp_centre_velocity", "stress_smoothing", "contact"};

static thread_local Profiler* t_prof = nullptr;
void prof_set_current(Profiler* p) { t_prof = p; }
Profiler* prof_current() { return t_prof; }

static cudaEvent_t pool_event(Profiler* p) {
  if (p->next == p->npool) {
    int ncap = p->npool ? 2 * p->npool : 256;
    cudaEvent_t* np = (cudaEvent_t*)realloc(p->pool, sizeof(cudaEvent_t) * ncap);
    if (!np) return nullptr;
    p->pool = np;
    for (int k = p->npool; k < ncap; ++k) cudaEventCreate(&p->pool[k]);
    p->npool = ncap;
  }
  return p->pool[p->next++];
}

void prof_begin(int k, cudaStream_t s) {
  Profiler* p = t_prof;
  if (!p || !p->on) return;
  if (p->nrec == p->cap) {
    int ncap = p->cap ? 2 * p->cap : 256;
    Profiler::Rec* nr = (Profiler::Rec*)realloc(p->recs, sizeof(Profiler::Rec) * ncap);
    if (!nr) return;
    p->recs = nr;
    p->cap = ncap;
  }
  Profiler::Rec& r = p->recs[p->nrec++];
  r.kernel = k;
  r.a = pool_event(p);
  r.b = pool_event(p);
  if (p->capturing) cudaEventRecordWithFlags(r.a, s, cudaEventRecordExternal);
  else cudaEventRecord(r.a, s);
}

void prof_end(int k, cudaStream_t s) {
  Profiler* p = t_prof;
  if (!p || !p->on || p->nrec == 0) return;
  Profiler::Rec& r = p->recs[p->nrec - 1];
  if (r.kernel != k) return;
  if (p->capturing) cudaEventRecordWithFlags(r.b, s, cudaEventRecordExternal);
  else cudaEventRecord(r.b, s);
}

int prof_harvest(Profiler* p, cudaStream_t s) {
  if (!p || p->nrec == 0) return MPM_OK;
  if (cudaStreamSynchronize(s) != cudaSuccess) return MPM_ERR_CUDA;
  for (int i = 0; i < p->nrec; ++i) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, p->recs[i].a, p->recs[i].b) == cudaSuccess) {
      p->ms[p->recs[i].kernel] += ms;
      p->n[p->recs[i].kernel] += 1;
    }
  }
  p->nrec = 0;
  p->next = 0;
  return MPM_OK;
}

void prof_reset(Profiler* p) {
  for (int k = 0; k < K_COUNT; ++k) {
    p->ms[k] = 0;
    p->n[k] = 0;
  }
  p->nrec = 0;
  p->next = 0;
}

void prof_free(Profiler* p) {
  for (int k = 0; k < p->npool; ++k) cudaEventDestroy(p->pool[k]);
  free(p->pool);
  free(p->recs);
  p->pool = nullptr;
  p->recs = nullptr;
  p->npool = p->cap = p->nrec = p->next = 0;
}

}  // namespace mpm

namespace {

struct ProfScope {
  Profiler* prev;
  explicit ProfScope(mpm_ctx* c) : prev(prof_current()) { prof_set_current(&c->prof); }
  ~ProfScope() { prof_set_current(prev); }
};

// status of a call delegated to the batched engine, with its message
int batch_status(mpm_ctx* c, int r) {
  if (r) set_err(c, r, "%s", mpm_batch_last_error(c->batch));
  return r;
}

// particle values of a gather request (fields of the FP64 forms: double
// arrays; failure bytes; cell / node ids as integers)
__global__ void k_gather(DevState<double, double> s, long long np, const GatherItem* it, int n, double* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const long long p = it[k].p, c = it[k].comp;
  double v = 0.0;
  switch (it[k].field) {
    case MPM_P_XP: v = s.xp[c * np + p]; break;
    case MPM_P_XX: v = s.xx[c * np + p]; break;
    case MPM_P_VXP: v = s.vxp[c * np + p]; break;
    case MPM_P_FXP: v = s.fxp[c * np + p]; break;
    case MPM_P_XN: v = s.xn[c * np + p]; break;
    case MPM_P_XXN: v = s.xxn[c * np + p]; break;
    case MPM_P_VOL: v = s.vol[p]; break;
    case MPM_P_SIG_Y: v = s.sig_y[p]; break;
    case MPM_P_SM: v = s.sm[p]; break;
    case MPM_P_SEQV: v = s.seqv[p]; break;
    case MPM_P_SD: v = s.sd[c * np + p]; break;
    case MPM_P_FP: v = s.fp[c * np + p]; break;
    case MPM_P_EPEFF: v = s.epeff[p]; break;
    case MPM_P_CELSIUS: v = s.celsius[p]; break;
    case MPM_P_DMG: v = s.dmg[p]; break;
    case MPM_P_LT: v = s.lt[p]; break;
    case MPM_P_IE: v = s.ie[p]; break;
    case MPM_P_MASS: v = s.mass[p]; break;
    case MPM_P_CP: v = s.cp[p]; break;
    case MPM_P_Q: v = s.q[p]; break;
    case MPM_P_FAILURE: v = s.failure[p] ? 1.0 : 0.0; break;
    case MPM_P_ICELL: v = s.icell[p]; break;
    case MPM_P_CENTERICELL: v = s.centericell[p]; break;
    case MPM_P_INODE: v = s.inode[p]; break;
    case MPM_P_SPRE: v = s.spre ? s.spre[p] : 0.0; break;
    default: v = 0.0; break;
  }
  out[k] = v;
}

// ------------------------------------------------------------- set-up

int derive_setup(mpm_ctx* c, const mpm_deck* d, std::vector<double>& host_vol, std::vector<double>& sig_y,
                 std::vector<double>& ie, std::vector<double>& cp, std::vector<double>& lt,
                 std::vector<uint8_t>& fix, std::vector<uint8_t>& bd) {
  SceneSetup su;
  int r = scene_setup(d, su);
  if (r) return set_err(c, r, "%s", su.err.c_str());
  c->g = su.g;
  c->mats = su.mats;
  c->bodies = su.bodies;
  host_vol.swap(su.vol);
  sig_y.swap(su.sig_y);
  ie.swap(su.ie);
  cp.swap(su.cp);
  lt.swap(su.lt);
  fix.swap(su.fix);
  bd.swap(su.bd);
  return MPM_OK;
}

template <class T>
int upload_as(mpm_ctx* c, void* dst, const double* src, long long n, size_t elem) {
  if (elem == sizeof(double)) {
    CK(cudaMemcpyAsync(dst, src, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    return MPM_OK;
  }
  std::vector<float> tmp((size_t)n);
  for (long long i = 0; i < n; ++i) tmp[i] = (float)src[i];
  CK(cudaMemcpyAsync(dst, tmp.data(), (size_t)n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return MPM_OK;
}

// ------------------------------------------------------------ sorting
int sort_pairs(mpm_ctx* c) {
  DevState<double, double>& s = c->st;
  prof_begin(K_SORT, c->stream);
  size_t tmp = c->cub_tmp_bytes;
  cudaError_t e = cub::DeviceRadixSort::SortPairs(c->cub_tmp, tmp, s.key, s.key_sorted, s.val, s.val_sorted,
                                                  (int)c->npairs, 0, c->key_bits, c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "radix sort");
  // per-node pair counts -> inclusive prefix sums (segment ends)
  tmp = c->cub_tmp_bytes;
  e = cub::DeviceScan::InclusiveSum(c->cub_tmp, tmp, s.seg, s.seg, c->nkeys, c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "segment scan");
  prof_end(K_SORT, c->stream);
  return MPM_OK;
}

int depeff_pass(mpm_ctx* c) {
  if (!c->g.has_jc) return MPM_OK;
  DevState<double, double>& s = c->st;
  size_t tmp = c->cub_tmp_bytes;
  cudaError_t e = cub::DeviceScan::InclusiveScan(c->cub_tmp, tmp, s.setter, s.setter_scan, MaxOp(),
                                                 (int)c->g.np, c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "depeff scan");
  c->ops->depeff_apply(&c->st, c->g, c->stream);
  return MPM_OK;
}

int build_pairs(mpm_ctx* c) {
  cudaError_t e = cudaMemsetAsync(c->st.seg, 0, sizeof(int) * ((size_t)c->nkeys + 1), c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "memset seg");
  c->ops->locate(&c->st, c->g, c->stream);
  return sort_pairs(c);
}

// SmoothStressbyGrid: shapes and pairs of the step's cells, then the maps
int smooth_pass(mpm_ctx* c) {
  if (!c->st.spre) return set_err(c, MPM_ERR_ARG, "stress smoothing is off for this deck (no 'smoo')");
  cudaError_t e = cudaMemsetAsync(c->st.seg, 0, sizeof(int) * ((size_t)c->nkeys + 1), c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "memset seg");
  c->ops->fixed_locate(&c->st, c->g, 0, c->stream);
  int r = sort_pairs(c);
  if (r) return r;
  c->ops->smooth(&c->st, c->g, c->stream);
  return MPM_OK;
}

int stress_pass(mpm_ctx* c) {
  c->ops->stress(&c->st, c->g, c->stream);
  return depeff_pass(c);
}

// one step of the total Lagrangian form, MPM3D.f90:164-226
int enqueue_step_tl(mpm_ctx* c) {
  const Geometry& g = c->g;
  const StepOps* o = c->ops;
  void* st = &c->st;
  cudaStream_t s = c->stream;
  int r;
  o->begin_step(st, g, s);
  cudaError_t e = cudaMemsetAsync(c->st.seg, 0, sizeof(int) * ((size_t)c->nkeys + 1), s);
  if (e != cudaSuccess) return cuda_err(c, e, "memset seg");
  o->fixed_locate(st, g, 1, s);
  if ((r = sort_pairs(c))) return r;
  o->tl_momentum(st, g, g.usf, s);
  if (g.usf) o->tl_stress(st, g, s);
  o->force_prep(st, g, s);
  o->tl_force(st, g, 1, s);
  if (g.contact && g.contact_type == 1) o->contact(st, g, s);
  o->position(st, g, s);
  if (g.musl) o->p2g_momentum(st, g, !g.usf, s);
  if (!g.usf) o->tl_stress(st, g, s);
  o->reduce(st, g, 3, c->red_blocks, s);
  if (c->smooth)
    if ((r = smooth_pass(c))) return r;
  if (c->drdamp) o->dr_damping(st, g, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_err(c, e, "kernel launch");
  return MPM_OK;
}

// one full step, MPM3D.f90:69-118, enqueued without synchronisation
int enqueue_step(mpm_ctx* c) {
  if (c->g.tlmpm) return enqueue_step_tl(c);
  const Geometry& g = c->g;
  const StepOps* o = c->ops;
  void* st = &c->st;
  cudaStream_t s = c->stream;
  int r;
  o->begin_step(st, g, s);
  if ((r = build_pairs(c))) return r;
  o->p2g_mass(st, g, g.usf, g.usf, s);
  if (g.usf)
    if ((r = stress_pass(c))) return r;
  o->force_prep(st, g, s);
  o->p2g_force(st, g, 1, s);
  if (g.contact && g.contact_type == 1) o->contact(st, g, s);
  o->position(st, g, s);
  if (g.musl) o->p2g_momentum(st, g, !g.usf, s);
  if (!g.usf)
    if ((r = stress_pass(c))) return r;
  o->reduce(st, g, 3, c->red_blocks, s);
  if (c->smooth)
    if ((r = smooth_pass(c))) return r;
  if (c->drdamp) o->dr_damping(st, g, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_err(c, e, "kernel launch");
  return MPM_OK;
}

void free_ctx(mpm_ctx* c) {
  if (!c) return;
  if (c->g_items_h) cudaFreeHost(c->g_items_h);
  if (c->g_out_h) cudaFreeHost(c->g_out_h);
  if (c->g_items_d) cudaFree(c->g_items_d);
  if (c->g_out_d) cudaFree(c->g_out_d);
  if (c->g_done) cudaEventDestroy(c->g_done);
  if (c->batch) mpm_batch_destroy(c->batch);
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  for (void* p : c->allocs) cudaFree(p);
  prof_free(&c->prof);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int harvest_profile(mpm_ctx* c) { return prof_harvest(&c->prof, c->stream); }

}  // namespace

// =================================================================== ABI

extern "C" {

int mpm_field_components(int f) {
  switch (f) {
    case MPM_P_XP: case MPM_P_XX: case MPM_P_VXP: case MPM_P_FXP: case MPM_P_XN: case MPM_P_XXN:
    case MPM_G_PX: case MPM_G_FX: case MPM_C_PX:
      return 3;
    case MPM_P_SD: return 6;
    case MPM_P_FP: case MPM_P_PK: return 9;
    case MPM_P_VOL: case MPM_P_VOL0: case MPM_P_SIG_Y: case MPM_P_SM: case MPM_P_SEQV: case MPM_P_EPEFF:
    case MPM_P_CELSIUS: case MPM_P_DMG: case MPM_P_LT: case MPM_P_IE: case MPM_P_MASS: case MPM_P_CP:
    case MPM_P_Q: case MPM_P_FAILURE: case MPM_P_ICELL: case MPM_P_CENTERICELL: case MPM_P_INODE: case MPM_P_SPRE:
    case MPM_G_MG: case MPM_C_MG:
      return 1;
    default: return 0;
  }
}

const char* mpm_last_error(const mpm_ctx* c) { return c ? c->err.c_str() : g_lib_error.c_str(); }

int mpm_create(const mpm_deck* d, int precision, int device, mpm_ctx** out) {
  if (!out) return set_err(nullptr, MPM_ERR_ARG, "out is NULL");
  *out = nullptr;
  if (!d) return set_err(nullptr, MPM_ERR_ARG, "deck is NULL");
  if (d->nb_particle <= 0 || d->nb_body <= 0 || d->nb_mat <= 0)
    return set_err(nullptr, MPM_ERR_ARG, "deck defines no particles / bodies / materials");
  if (d->nb_body > 65535) return set_err(nullptr, MPM_ERR_UNSUPPORTED, "more than 65535 bodies");
  mpm_ctx* c = new mpm_ctx();
  c->precision = precision;
  switch (precision) {
    case MPM_FP64_STRICT: c->ops = &kOpsStrict; break;
    case MPM_FP64_NATIVE: c->ops = &kOpsNative; break;
    case MPM_MIXED: c->ops = nullptr; break;  // batched engine, one scene
    default:
      delete c;
      return set_err(nullptr, MPM_ERR_ARG, "unknown precision %d", precision);
  }
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    delete c;
    return set_err(nullptr, MPM_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
  }
  if (device >= 0) {
    if (device >= ndev) {
      delete c;
      return set_err(nullptr, MPM_ERR_ARG, "device %d does not exist", device);
    }
    cudaSetDevice(device);
  }
  cudaGetDevice(&c->device);
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) {
    int r = set_err(nullptr, MPM_ERR_CUDA, "stream: %s", cudaGetErrorString(e));
    delete c;
    return r;
  }
  c->flags = d->flags;
  c->drdamp = !!(d->flags & MPM_F_DRDAMP);
  c->smooth = !!(d->flags & MPM_F_SMOOTH);
  if (precision == MPM_MIXED) {
    // the mixed form is the batched engine running a batch of one scene; the
    // deck's arrays are uploaded in place (committed before returning)
    int r = mpm_batch_create(c->device, &c->batch);
    std::string err;
    int code = MPM_OK;
    mpm::HostScene* h = r ? nullptr : mpm::scene_stage(d, 0, err, &code, true);
    if (!r && !h) r = code;
    if (!r) {
      mpm::batch_insert(c->batch, h, &c->batch_scene);
      c->g = mpm::scene_setup_of(h).g;
      c->mats = mpm::scene_setup_of(h).mats;
      c->bodies = mpm::scene_setup_of(h).bodies;
      r = mpm_batch_commit(c->batch);
      if (r) err = mpm_batch_last_error(c->batch);
    } else if (err.empty() && c->batch) {
      err = "batch create failed";
    }
    if (r) {
      set_err(c, r, "%s", err.c_str());
      g_lib_error = c->err;
      free_ctx(c);
      return r;
    }
    c->bytes = mpm_batch_device_bytes(c->batch);
    *out = c;
    return MPM_OK;
  }
  std::vector<double> vol, sig_y, ie, cp, lt;
  std::vector<uint8_t> fix, bd;
  int r = derive_setup(c, d, vol, sig_y, ie, cp, lt, fix, bd);
  if (r) {
    g_lib_error = c->err;
    free_ctx(c);
    return r;
  }
  Geometry& g = c->g;
  const long long np = g.np, nn = g.nn, nc = g.ncell, nnt = g.nnt;
  const int K = g.K;
  c->nkeys = g.shape == 3 ? (int)nc : (int)nnt;  // pair keys: (component, node) or centre node
  c->npairs = np * K;
  if (c->npairs >= (1LL << 31) || np >= (1LL << 27) || nnt >= (1LL << 31)) {
    // pair values hold particle * 32 + slot in 32 bits, segment ends and the
    // sort's item count are 32-bit ints
    set_err(c, MPM_ERR_UNSUPPORTED, "FP64 forms: %lld particles x %d slots exceed the 32-bit pair indices", np, K);
    g_lib_error = c->err;
    free_ctx(c);
    return MPM_ERR_UNSUPPORTED;
  }
  c->key_bits = 1;
  while ((1LL << c->key_bits) <= (long long)c->nkeys) c->key_bits++;
  c->red_blocks = (int)std::min<long long>(1024, (np + kBlock - 1) / kBlock);
  const size_t B = c->ops->bulk_size, Rz = c->ops->real_size;
  DevState<double, double>& s = c->st;
  // particle arrays
#define AL(ptr, T, n) \
  if ((r = dalloc(c, (T**)&(ptr), (n)))) goto fail;
#define ALB(ptr, n)                                                      \
  if (B == sizeof(double)) { AL(ptr, double, n); } else { AL(ptr, float, n); }
#define ALR(ptr, n)                                                      \
  if (Rz == sizeof(double)) { AL(ptr, double, n); } else { AL(ptr, float, n); }
  {
    AL(s.xp, double, 3 * np); AL(s.xx, double, 3 * np); AL(s.vxp, double, 3 * np); AL(s.fxp, double, 3 * np);
    AL(s.mass, double, np); AL(s.ie, double, np);
    ALB(s.vol, np); ALB(s.sig_y, np); ALB(s.sm, np); ALB(s.seqv, np); ALB(s.sd, 6 * np);
    ALB(s.fp, g.uvfp ? 9 * np : 1); ALB(s.epeff, np); ALB(s.celsius, np); ALB(s.dmg, np); ALB(s.lt, np);
    ALB(s.cp, np); ALB(s.q, np); ALB(s.xn, 3 * np); ALB(s.xxn, 3 * np);
    AL(s.icell, int, np); AL(s.centericell, int, np); AL(s.inode, int, np);
    AL(s.failure, uint8_t, np); AL(s.body, uint16_t, np);
    AL(s.fext, double, 3 * np); AL(s.sdiag, double, 3 * np);
    AL(s.snode, int, (long long)K * np);
    ALR(s.shp, (long long)K * np);
    if (g.shape != 3) { ALR(s.dndx, (long long)K * np); ALR(s.dndy, (long long)K * np); ALR(s.dndz, (long long)K * np); }
    AL(s.key, unsigned, c->npairs); AL(s.val, unsigned, c->npairs);
    AL(s.key_sorted, unsigned, c->npairs); AL(s.val_sorted, unsigned, c->npairs);
    AL(s.seg, int, (long long)c->nkeys + 1);
    AL(s.mg, double, nnt); AL(s.px, double, 3 * nnt); AL(s.fx, double, 3 * nnt); AL(s.vg, double, 3 * nnt);
    AL(s.fix, uint8_t, nn); AL(s.bd, uint8_t, nn);
    if (g.contact) { AL(s.ndir, double, 3 * nnt); AL(s.cforce, double, 3 * nn); }
    if (g.tlmpm) {
      AL(s.pk, double, 9 * np); AL(s.vol0, double, np);
      if (g.shape == 3) AL(s.cpk, double, 9 * nc);
    }
    if (g.shape == 3) {
      AL(s.cmg, double, nc); AL(s.cpx, double, 3 * nc); AL(s.cfext, double, 3 * nc); AL(s.cfint, double, 6 * nc);
      AL(s.co, double, 6 * nc); AL(s.cw, double, 3 * nc); AL(s.cdefp, double, 9 * nc);
      AL(s.cvx, double, 3 * nc); AL(s.cax, double, 3 * nc);
    }
    if (g.has_jc) {
      AL(s.setter, int, np); AL(s.setter_scan, int, np); AL(s.dep, double, np);
      AL(s.jc_aux, double, 5 * np); AL(s.deferred, uint8_t, np);
    }
    if (c->smooth) {
      AL(s.spre, double, np); AL(s.gpre, double, nn);
      if (g.shape == 3) { AL(s.cgpre, double, nc); AL(s.cgvall, double, nc); }
    }
    AL(s.red_part, double, (long long)kRedVals * c->red_blocks); AL(s.red_count, unsigned, 1);
    AL(s.mats, DevMaterial, (long long)c->mats.size()); AL(s.bodies, DevBody, (long long)c->bodies.size());
    AL(s.sc, DevScalars, 1);
  }
#undef AL
#undef ALB
#undef ALR
  {
    // CUB temporary storage: the largest of the three primitives
    size_t t1 = 0, t2 = 0, t3 = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, t1, s.key, s.key_sorted, s.val, s.val_sorted, (int)c->npairs, 0,
                                    c->key_bits, c->stream);
    cub::DeviceScan::InclusiveSum(nullptr, t2, s.seg, s.seg, c->nkeys, c->stream);
    if (g.has_jc) cub::DeviceScan::InclusiveScan(nullptr, t3, s.setter, s.setter_scan, MaxOp(), (int)np, c->stream);
    c->cub_tmp_bytes = std::max(t1, std::max(t2, t3));
    if ((r = dalloc(c, (char**)&c->cub_tmp, (long long)c->cub_tmp_bytes))) goto fail;
  }
  // uploads
  {
#define UPB(dst, src, n) \
  if ((r = upload_as<double>(c, (dst), (src), (n), B))) goto fail;
#define CKF(call)                                              \
  if ((e = (call)) != cudaSuccess) { r = cuda_err(c, e, #call); goto fail; }
    CKF(cudaMemcpyAsync(s.xp, d->xp, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, c->stream));
    // XX (the position at t + DT) is written by ParticlePositionUpdate for
    // the particles inside the grid only (update_step.f90:1477, 1515); the
    // reference's freshly allocated particle list holds 0 until then, which
    // a particle that starts outside the grid keeps
    CKF(cudaMemsetAsync(s.xx, 0, sizeof(double) * 3 * np, c->stream));
    CKF(cudaMemcpyAsync(s.vxp, d->vxp, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, c->stream));
    CKF(cudaMemcpyAsync(s.fxp, d->fxp, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, c->stream));
    CKF(cudaMemcpyAsync(s.mass, d->mass, sizeof(double) * np, cudaMemcpyHostToDevice, c->stream));
    CKF(cudaMemcpyAsync(s.ie, ie.data(), sizeof(double) * np, cudaMemcpyHostToDevice, c->stream));
    std::vector<double> zeros((size_t)9 * np, 0.0), t293((size_t)np, (double)293.0f);
    UPB(s.vol, vol.data(), np);
    UPB(s.sig_y, sig_y.data(), np);
    UPB(s.cp, cp.data(), np);
    UPB(s.lt, lt.data(), np);
    UPB(s.celsius, t293.data(), np);
    UPB(s.sm, zeros.data(), np);
    UPB(s.seqv, zeros.data(), np);
    UPB(s.sd, zeros.data(), 6 * np);
    if (g.uvfp) UPB(s.fp, zeros.data(), 9 * np);
    UPB(s.epeff, zeros.data(), np);
    UPB(s.dmg, zeros.data(), np);
    UPB(s.q, zeros.data(), np);
    UPB(s.xn, zeros.data(), 3 * np);
    UPB(s.xxn, zeros.data(), 3 * np);
    CKF(cudaMemsetAsync(s.failure, 0, np, c->stream));
    std::vector<uint16_t> body((size_t)np, 0);
    for (int b = 0; b < d->nb_body; ++b)
      for (long long p = d->bodies[b].par_begin; p < d->bodies[b].par_end; ++p) body[p] = (uint16_t)b;
    CKF(cudaMemcpyAsync(s.body, body.data(), sizeof(uint16_t) * np, cudaMemcpyHostToDevice, c->stream));
    CKF(cudaMemcpyAsync(s.fix, fix.data(), nn, cudaMemcpyHostToDevice, c->stream));
    CKF(cudaMemcpyAsync(s.bd, bd.data(), nn, cudaMemcpyHostToDevice, c->stream));
    CKF(cudaMemcpyAsync(s.mats, c->mats.data(), sizeof(DevMaterial) * c->mats.size(), cudaMemcpyHostToDevice,
                        c->stream));
    CKF(cudaMemcpyAsync(s.bodies, c->bodies.data(), sizeof(DevBody) * c->bodies.size(), cudaMemcpyHostToDevice,
                        c->stream));
    CKF(cudaMemsetAsync(s.mg, 0, sizeof(double) * nnt, c->stream));
    CKF(cudaMemsetAsync(s.px, 0, sizeof(double) * 3 * nnt, c->stream));
    CKF(cudaMemsetAsync(s.fx, 0, sizeof(double) * 3 * nnt, c->stream));
    CKF(cudaMemsetAsync(s.vg, 0, sizeof(double) * 3 * nnt, c->stream));
    if (s.ndir) CKF(cudaMemsetAsync(s.ndir, 0, sizeof(double) * 3 * nnt, c->stream));
    if (s.cforce) CKF(cudaMemsetAsync(s.cforce, 0, sizeof(double) * 3 * nn, c->stream));
    CKF(cudaMemsetAsync(s.red_count, 0, sizeof(unsigned), c->stream));
    if (s.spre) CKF(cudaMemsetAsync(s.spre, 0, sizeof(double) * np, c->stream));
    DevScalars sc0;
    memset(&sc0, 0, sizeof sc0);
    sc0.dt = set_dt(c->mats, g.dcell, g.dtscale);
    CKF(cudaMemcpyAsync(s.sc, &sc0, sizeof sc0, cudaMemcpyHostToDevice, c->stream));
    if (g.shape == 3) {
      CKF(cudaMemsetAsync(s.cmg, 0, sizeof(double) * nc, c->stream));
      CKF(cudaMemsetAsync(s.cpx, 0, sizeof(double) * 3 * nc, c->stream));
    }
    // calcEnergy before the loop (MPM3D.f90:42)
    c->ops->reduce(&c->st, g, 1, c->red_blocks, c->stream);
    if (g.tlmpm) {
      // GridMassInitial (MPM3D.f90:162): cells of the initial positions kept
      // for the run, the grid mass mapped once
      CKF(cudaMemsetAsync(s.pk, 0, sizeof(double) * 9 * np, c->stream));
      CKF(cudaMemcpyAsync(s.vol0, s.vol, sizeof(double) * np, cudaMemcpyDeviceToDevice, c->stream));
      c->ops->tl_initial(&c->st, g, c->stream);
      CKF(cudaMemsetAsync(s.seg, 0, sizeof(int) * ((size_t)c->nkeys + 1), c->stream));
      c->ops->fixed_locate(&c->st, g, 1, c->stream);
      if ((r = sort_pairs(c))) goto fail;
      c->ops->p2g_mass(&c->st, g, 0, 0, c->stream);
    }
    CKF(cudaStreamSynchronize(c->stream));
    CKF(cudaGetLastError());
#undef UPB
#undef CKF
  }
  *out = c;
  return MPM_OK;
fail:
  g_lib_error = c->err;
  free_ctx(c);
  return r;
}

void mpm_destroy(mpm_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  free_ctx(c);
}

int mpm_step_phase(mpm_ctx* c, int phase) {
  if (!c) return set_err(nullptr, MPM_ERR_ARG, "ctx is NULL");
  if (c->batch) return set_err(c, MPM_ERR_UNSUPPORTED, "the mixed form runs whole steps only");
  ProfScope ps(c);
  const Geometry& g = c->g;
  const StepOps* o = c->ops;
  void* st = &c->st;
  cudaStream_t s = c->stream;
  int r = MPM_OK;
  switch (phase) {
    case MPM_PHASE_BEGIN_STEP: o->begin_step(st, g, s); break;
    case MPM_PHASE_GRID_MOMENTUM_INITIAL:
      if (g.tlmpm) {  // TLGridMomentumInitial: momentum with the cells of the initial positions
        cudaError_t e = cudaMemsetAsync(c->st.seg, 0, sizeof(int) * ((size_t)c->nkeys + 1), s);
        if (e != cudaSuccess) return cuda_err(c, e, "memset seg");
        o->fixed_locate(st, g, 1, s);
        if ((r = sort_pairs(c))) return r;
        o->tl_momentum(st, g, 0, s);
        break;
      }
      if ((r = build_pairs(c))) return r;
      o->p2g_mass(st, g, 0, 0, s);
      break;
    case MPM_PHASE_APPLY_BOUNDARY: o->apply_bc(st, g, s); break;
    case MPM_PHASE_PARTICLE_STRESS_UPDATE:
      o->node_velocity(st, g, s);
      if (g.tlmpm) o->tl_stress(st, g, s);
      else if ((r = stress_pass(c))) return r;
      break;
    case MPM_PHASE_GRID_MOMENTUM_UPDATE:
      o->force_prep(st, g, s);
      if (g.tlmpm) o->tl_force(st, g, 0, s);
      else o->p2g_force(st, g, 0, s);
      break;
    case MPM_PHASE_INTEGRATE_MOMENTUM: o->integrate(st, g, s); break;
    case MPM_PHASE_PARTICLE_POSITION_UPDATE:
      o->node_velocity(st, g, s);
      o->position(st, g, s);
      break;
    case MPM_PHASE_GRID_MOMENTUM_MUSL: o->p2g_momentum(st, g, 0, s); break;
    case MPM_PHASE_CALC_ENERGY: o->reduce(st, g, 1, c->red_blocks, s); break;
    case MPM_PHASE_UPDATE_DT: o->reduce(st, g, 2, c->red_blocks, s); break;
    case MPM_PHASE_DR_DAMPING: o->dr_damping(st, g, s); break;
    case MPM_PHASE_SMOOTH_STRESS:
      if ((r = smooth_pass(c))) return r;
      break;
    case MPM_PHASE_CONTACT:
      if (g.contact && g.contact_type == 1) o->contact(st, g, s);
      break;
    default: return set_err(c, MPM_ERR_ARG, "unknown phase %d", phase);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_err(c, e, "kernel launch");
  return r;
}

int mpm_step(mpm_ctx* c) {
  if (!c) return set_err(nullptr, MPM_ERR_ARG, "ctx is NULL");
  // one step replayed from the context's one-step CUDA graph
  if (c->batch) return batch_status(c, mpm_batch_run(c->batch, 1, 1));
  return mpm_run(c, 1, 1);
}

static int ensure_graph(mpm_ctx* c, int nsteps) {
  if (c->graph_exec && c->graph_steps == nsteps && c->graph_prof == c->prof.on) return MPM_OK;
  if (c->graph_exec) {
    cudaGraphExecDestroy(c->graph_exec);
    c->graph_exec = nullptr;
  }
  cudaGraph_t graph;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  c->prof.capturing = true;
  int r = MPM_OK;
  for (int i = 0; i < nsteps && r == MPM_OK; ++i) r = enqueue_step(c);
  c->prof.capturing = false;
  cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
  if (r) return r;
  if (e != cudaSuccess) return cuda_err(c, e, "end capture");
  e = cudaGraphInstantiate(&c->graph_exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_err(c, e, "graph instantiate");
  c->graph_steps = nsteps;
  c->graph_prof = c->prof.on;
  return MPM_OK;
}

int mpm_run(mpm_ctx* c, int nsteps, int use_graph) {
  if (!c) return set_err(nullptr, MPM_ERR_ARG, "ctx is NULL");
  if (nsteps <= 0) return MPM_OK;
  if (c->batch) return batch_status(c, mpm_batch_run(c->batch, nsteps, use_graph));
  ProfScope ps(c);
  if (!use_graph) {
    for (int i = 0; i < nsteps; ++i) {
      int r = enqueue_step(c);
      if (r) return r;
    }
    return MPM_OK;
  }
  // a graph of one step, launched nsteps times (profiling records only the
  // event nodes of the captured step, so profiled runs use a graph of all
  // steps instead)
  int gsteps = c->prof.on ? nsteps : 1;
  if (c->prof.on) {
    // re-capture so that the event records of this run are the live ones
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    c->graph_exec = nullptr;
    c->prof.nrec = 0;
    c->prof.next = 0;
  }
  int r = ensure_graph(c, gsteps);
  if (r) return r;
  for (int i = 0; i < nsteps / gsteps; ++i) CK(cudaGraphLaunch(c->graph_exec, c->stream));
  return MPM_OK;
}

int mpm_sync(mpm_ctx* c) {
  if (!c) return set_err(nullptr, MPM_ERR_ARG, "ctx is NULL");
  if (c->batch) return batch_status(c, mpm_batch_sync(c->batch));
  CK(cudaStreamSynchronize(c->stream));
  unsigned status = 0;
  CK(cudaMemcpy(&status, &c->st.sc->status, sizeof status, cudaMemcpyDeviceToHost));
  if (status & (ST_NONFINITE)) return set_err(c, MPM_ERR_NONFINITE, "non-finite particle state");
  if (status & ST_BAD_EOS) return set_err(c, MPM_ERR_ARG, "a material without equation of state called one");
  return MPM_OK;
}

int mpm_get_scalars(mpm_ctx* c, double* o) {
  if (!c || !o) return set_err(c, MPM_ERR_ARG, "bad argument");
  if (c->batch) return batch_status(c, mpm_batch_scene_scalars(c->batch, c->batch_scene, o));
  CK(cudaStreamSynchronize(c->stream));
  DevScalars sc;
  CK(cudaMemcpy(&sc, c->st.sc, sizeof sc, cudaMemcpyDeviceToHost));
  memset(o, 0, sizeof(double) * MPM_NSCALARS);
  o[0] = sc.istep; o[1] = sc.time; o[2] = sc.dt; o[3] = sc.ke; o[4] = sc.ie;
  o[5] = sc.mom[0]; o[6] = sc.mom[1]; o[7] = sc.mom[2]; o[8] = sc.ke_prev;
  o[9] = c->g.nn; o[10] = (double)c->g.np; o[11] = c->g.cutoff; o[12] = c->g.dcell;
  o[13] = (double)sc.active_nodes; o[14] = sc.status;
  return MPM_OK;
}

int64_t mpm_nb_particle(const mpm_ctx* c) { return c ? c->g.np : -1; }
int64_t mpm_nb_gridnode(const mpm_ctx* c) { return c ? c->g.nn : -1; }
int64_t mpm_nb_cell(const mpm_ctx* c) { return c ? c->g.ncell : -1; }
int mpm_nb_component(const mpm_ctx* c) { return c ? (c->batch ? 1 : c->g.ncomp) : -1; }

int mpm_contact_force(mpm_ctx* c, double f[3]) {
  if (!c || !f) return set_err(c, MPM_ERR_ARG, "bad argument");
  if (c->batch || !c->g.contact) {
    f[0] = f[1] = f[2] = 0.0;
    return MPM_OK;
  }
  DevScalars sc;
  CK(cudaMemcpyAsync(&sc, c->st.sc, sizeof sc, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < 3; ++k) f[k] = sc.cont_for[k];
  return MPM_OK;
}

int64_t mpm_device_bytes(const mpm_ctx* c) { return c ? (c->batch ? mpm_batch_device_bytes(c->batch) : c->bytes) : -1; }

static int field_ptr(mpm_ctx* c, int field, void** ptr, size_t* elem, long long* count) {
  DevState<double, double>& s = c->st;
  const long long np = c->g.np, nn = c->g.nn, nc = c->g.ncell;
  const size_t B = c->ops->bulk_size;
  *elem = 8;
  *count = np * mpm_field_components(field);
  switch (field) {
    case MPM_P_XP: *ptr = s.xp; break;
    case MPM_P_XX: *ptr = s.xx; break;
    case MPM_P_VXP: *ptr = s.vxp; break;
    case MPM_P_FXP: *ptr = s.fxp; break;
    case MPM_P_MASS: *ptr = s.mass; break;
    case MPM_P_IE: *ptr = s.ie; break;
    case MPM_P_XN: *ptr = s.xn; *elem = B; break;
    case MPM_P_XXN: *ptr = s.xxn; *elem = B; break;
    case MPM_P_VOL: *ptr = s.vol; *elem = B; break;
    case MPM_P_SIG_Y: *ptr = s.sig_y; *elem = B; break;
    case MPM_P_SM: *ptr = s.sm; *elem = B; break;
    case MPM_P_SEQV: *ptr = s.seqv; *elem = B; break;
    case MPM_P_SD: *ptr = s.sd; *elem = B; break;
    case MPM_P_FP:
      if (!c->g.uvfp) return set_err(c, MPM_ERR_ARG, "deformation gradient is not tracked (no UVFp)");
      *ptr = s.fp; *elem = B; break;
    case MPM_P_EPEFF: *ptr = s.epeff; *elem = B; break;
    case MPM_P_CELSIUS: *ptr = s.celsius; *elem = B; break;
    case MPM_P_DMG: *ptr = s.dmg; *elem = B; break;
    case MPM_P_LT: *ptr = s.lt; *elem = B; break;
    case MPM_P_CP: *ptr = s.cp; *elem = B; break;
    case MPM_P_Q: *ptr = s.q; *elem = B; break;
    case MPM_P_FAILURE: *ptr = s.failure; *elem = 1; break;
    case MPM_P_ICELL: *ptr = s.icell; *elem = 4; break;
    case MPM_P_CENTERICELL: *ptr = s.centericell; *elem = 4; break;
    case MPM_P_INODE: *ptr = s.inode; *elem = 4; break;
    case MPM_P_SPRE: *ptr = s.spre; break;  // null without 'smoo': reads as zeros
    case MPM_P_PK: *ptr = s.pk; break;      // null without 'TLmp': reads as zeros
    case MPM_P_VOL0:
      if (!s.vol0) return set_err(c, MPM_ERR_ARG, "initial volume is kept by TLMPM contexts only");
      *ptr = s.vol0; break;
    case MPM_G_MG: *ptr = s.mg; *count = c->g.nnt; break;  // every grid component, component-major
    case MPM_G_PX: *ptr = s.px; *count = 3 * c->g.nnt; break;
    case MPM_G_FX: *ptr = s.fx; *count = 3 * c->g.nnt; break;
    case MPM_C_MG:
      if (!s.cmg) return set_err(c, MPM_ERR_ARG, "no auxiliary grid (not SGMP)");
      *ptr = s.cmg; *count = nc; break;
    case MPM_C_PX:
      if (!s.cpx) return set_err(c, MPM_ERR_ARG, "no auxiliary grid (not SGMP)");
      *ptr = s.cpx; *count = 3 * nc; break;
    default: return set_err(c, MPM_ERR_ARG, "field %d is not available", field);
  }
  return MPM_OK;
}

int mpm_download(mpm_ctx* c, int field, double* out) {
  if (!c || !out) return set_err(c, MPM_ERR_ARG, "bad argument");
  if (c->batch) return batch_status(c, mpm_batch_scene_download(c->batch, c->batch_scene, field, out));
  void* p = nullptr;
  size_t elem = 0;
  long long n = 0;
  int r = field_ptr(c, field, &p, &elem, &n);
  if (r) return r;
  CK(cudaStreamSynchronize(c->stream));
  if (!p) {  // a field the deck does not switch on (Spre without 'smoo'): zero, as in the reference
    memset(out, 0, sizeof(double) * (size_t)n);
    return MPM_OK;
  }
  if (elem == 8) {
    mpm::prefault_host(out, (size_t)n * 8);
    CK(cudaMemcpy(out, p, (size_t)n * 8, cudaMemcpyDeviceToHost));
    return MPM_OK;
  }
  std::vector<unsigned char> tmp((size_t)n * elem);
  CK(cudaMemcpy(tmp.data(), p, tmp.size(), cudaMemcpyDeviceToHost));
  for (long long i = 0; i < n; ++i) {
    if (elem == 4 && (field == MPM_P_ICELL || field == MPM_P_CENTERICELL || field == MPM_P_INODE))
      out[i] = ((const int*)tmp.data())[i];
    else if (elem == 4)
      out[i] = ((const float*)tmp.data())[i];
    else
      out[i] = tmp[i];
  }
  return MPM_OK;
}

void* mpm_host_alloc(int64_t bytes) {
  if (bytes <= 0) {
    set_err(nullptr, MPM_ERR_ARG, "page-locked allocation of %lld bytes", (long long)bytes);
    return nullptr;
  }
  void* p = nullptr;
  cudaError_t e = cudaHostAlloc(&p, (size_t)bytes, cudaHostAllocPortable);
  if (e != cudaSuccess) {
    set_err(nullptr, MPM_ERR_OOM, "page-locked allocation of %lld bytes: %s", (long long)bytes, cudaGetErrorString(e));
    return nullptr;
  }
  return p;
}

void mpm_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

int mpm_host_register(void* p, int64_t bytes) {
  if (!p || bytes <= 0) return set_err(nullptr, MPM_ERR_ARG, "bad argument");
  cudaError_t e = cudaHostRegister(p, (size_t)bytes, cudaHostRegisterPortable);
  if (e != cudaSuccess) return set_err(nullptr, MPM_ERR_CUDA, "host register: %s", cudaGetErrorString(e));
  return MPM_OK;
}

int mpm_host_unregister(void* p) {
  if (!p) return set_err(nullptr, MPM_ERR_ARG, "bad argument");
  cudaError_t e = cudaHostUnregister(p);
  if (e != cudaSuccess) return set_err(nullptr, MPM_ERR_CUDA, "host unregister: %s", cudaGetErrorString(e));
  return MPM_OK;
}

int mpm_deck_pin(mpm_deck* d, int on) {
  if (!d) return set_err(nullptr, MPM_ERR_ARG, "deck is NULL");
  const int64_t np = d->nb_particle;
  double* a[4] = {d->mass, d->xp, d->vxp, d->fxp};
  const int64_t n[4] = {np, 3 * np, 3 * np, 3 * np};
  for (int k = 0; k < 4; ++k) {
    if (!a[k] || n[k] <= 0) continue;
    const int r = on ? mpm_host_register(a[k], n[k] * 8) : mpm_host_unregister(a[k]);
    if (r && on) {  // leave nothing half locked
      for (int u = 0; u < k; ++u)
        if (a[u] && n[u] > 0) cudaHostUnregister(a[u]);
      return r;
    }
    if (r) return r;
  }
  return MPM_OK;
}

int mpm_upload(mpm_ctx* c, int field, const double* in) {
  if (!c || !in) return set_err(c, MPM_ERR_ARG, "bad argument");
  if (c->batch) return set_err(c, MPM_ERR_UNSUPPORTED, "the mixed form takes its state from the deck only");
  if (field >= MPM_G_MG || field == MPM_P_ICELL || field == MPM_P_CENTERICELL || field == MPM_P_INODE ||
      field == MPM_P_FAILURE || field == MPM_P_SPRE)
    return set_err(c, MPM_ERR_ARG, "field %d cannot be uploaded", field);
  void* p = nullptr;
  size_t elem = 0;
  long long n = 0;
  int r = field_ptr(c, field, &p, &elem, &n);
  if (r) return r;
  if (!p) return set_err(c, MPM_ERR_ARG, "field %d is not kept by this context", field);
  CK(cudaStreamSynchronize(c->stream));
  if (elem == 8) {
    CK(cudaMemcpy(p, in, (size_t)n * 8, cudaMemcpyHostToDevice));
  } else {
    std::vector<float> tmp((size_t)n);
    for (long long i = 0; i < n; ++i) tmp[i] = (float)in[i];
    CK(cudaMemcpy(p, tmp.data(), (size_t)n * 4, cudaMemcpyHostToDevice));
  }
  if (c->graph_exec) {
    cudaGraphExecDestroy(c->graph_exec);
    c->graph_exec = nullptr;
  }
  return MPM_OK;
}

int mpm_time_steps(mpm_ctx* c, int nsteps, int use_graph, double* ms) {
  if (!c || !ms) return set_err(c, MPM_ERR_ARG, "bad argument");
  if (c->batch) return batch_status(c, mpm_batch_time_steps(c->batch, nsteps, use_graph, ms));
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaEventRecord(a, c->stream));
  int r = mpm_run(c, nsteps, use_graph);
  CK(cudaEventRecord(b, c->stream));
  CK(cudaEventSynchronize(b));
  float f = 0;
  cudaEventElapsedTime(&f, a, b);
  *ms = f;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (r) return r;
  if (c->prof.on) harvest_profile(c);
  return MPM_OK;
}

int mpm_profile_enable(mpm_ctx* c, int on) {
  if (!c) return set_err(nullptr, MPM_ERR_ARG, "ctx is NULL");
  if (c->batch) return batch_status(c, mpm_batch_profile_enable(c->batch, on));
  if (c->prof.on) harvest_profile(c);
  prof_reset(&c->prof);
  c->prof.on = on != 0;
  return MPM_OK;
}

int mpm_kernel_count(const mpm_ctx*) { return K_COUNT; }

int mpm_kernel_stats(mpm_ctx* c, int k, char* name, int namelen, int64_t* launches, double* total_ms) {
  if (!c || k < 0 || k >= K_COUNT) return set_err(c, MPM_ERR_ARG, "bad kernel index");
  if (c->batch) return batch_status(c, mpm_batch_kernel_stats(c->batch, k, name, namelen, launches, total_ms));
  harvest_profile(c);
  if (name && namelen > 0) snprintf(name, (size_t)namelen, "%s", kKernelNames[k]);
  if (launches) *launches = c->prof.n[k];
  if (total_ms) *total_ms = c->prof.ms[k];
  return MPM_OK;
}

// persistent particle fields of a snapshot (the grid and per-step data are
// recomputed by every step)
static const int kSnapFields[] = {MPM_P_XP,  MPM_P_XX,      MPM_P_VXP, MPM_P_FXP, MPM_P_XN,    MPM_P_XXN,
                                  MPM_P_VOL, MPM_P_SIG_Y,   MPM_P_SM,  MPM_P_SEQV, MPM_P_SD,   MPM_P_FP,
                                  MPM_P_EPEFF, MPM_P_CELSIUS, MPM_P_DMG, MPM_P_LT, MPM_P_IE,   MPM_P_MASS,
                                  MPM_P_CP,  MPM_P_Q,       MPM_P_FAILURE, MPM_P_PK};
static const char kSnapMagic[8] = {'M', 'P', 'M', '3', 'D', 'S', 'N', '1'};

struct SnapHeader {
  char magic[8];
  int32_t precision, nfields;
  int64_t np, nn, ncell;
  int32_t scalars_bytes, uvfp;
  uint64_t deck_hash;  // geometry, materials and particle masses of the context's deck
};

// FNV-1a over the set-up a snapshot belongs to
static uint64_t fnv1a(uint64_t h, const void* p, size_t n) {
  const unsigned char* b = (const unsigned char*)p;
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

static int deck_hash(mpm_ctx* c, uint64_t* out) {
  uint64_t h = 1469598103934665603ull;
  h = fnv1a(h, &c->g, sizeof c->g);
  h = fnv1a(h, c->mats.data(), sizeof(DevMaterial) * c->mats.size());
  std::vector<double> m((size_t)c->g.np);
  if (c->batch) {  // the masses in the deck's particle order
    if (int r = batch_status(c, mpm_batch_scene_download(c->batch, c->batch_scene, MPM_P_MASS, m.data()))) return r;
  } else {
    CK(cudaMemcpy(m.data(), c->st.mass, sizeof(double) * m.size(), cudaMemcpyDeviceToHost));
  }
  *out = fnv1a(h, m.data(), sizeof(double) * m.size());
  return MPM_OK;
}

// Mixed form: the header (nfields 0) is followed by the byte count and the
// scene's restart image from the batched engine (its persistent particle
// arrays in the engine's storage order and its step state).
static int snapshot_save_mixed(mpm_ctx* c, const char* path) {
  SnapHeader h;
  memset(&h, 0, sizeof h);
  memcpy(h.magic, kSnapMagic, 8);
  h.precision = c->precision;
  h.np = c->g.np;
  h.nn = c->g.nn;
  h.ncell = c->g.ncell;
  h.uvfp = c->g.uvfp;
  if (int r = deck_hash(c, &h.deck_hash)) return r;
  std::vector<unsigned char> img;
  try {
    if (int r = batch_status(c, mpm::mpm_batch_scene_snapshot(c->batch, c->batch_scene, img))) return r;
  } catch (const std::bad_alloc&) {
    return set_err(c, MPM_ERR_OOM, "no host memory for the restart image");
  }
  h.scalars_bytes = 0;
  FILE* f = fopen(path, "wb");
  if (!f) return set_err(c, MPM_ERR_IO, "cannot write %s", path);
  const int64_t n = (int64_t)img.size();
  bool ok = fwrite(&h, sizeof h, 1, f) == 1 && fwrite(&n, sizeof n, 1, f) == 1 &&
            fwrite(img.data(), 1, img.size(), f) == img.size();
  ok = (fclose(f) == 0) && ok;
  if (!ok) return set_err(c, MPM_ERR_IO, "writing %s failed", path);
  return MPM_OK;
}

static int snapshot_load_mixed(mpm_ctx* c, const char* path) {
  uint64_t mine = 0;
  if (int r = deck_hash(c, &mine)) return r;
  FILE* f = fopen(path, "rb");
  if (!f) return set_err(c, MPM_ERR_IO, "cannot read %s", path);
  SnapHeader h;
  int64_t n = 0;
  int r = MPM_OK;
  std::vector<unsigned char> img;
  // the image size this context expects; negative when the context has no
  // committed scene, so no file size can match it
  const long long want = mpm::mpm_batch_scene_restart_bytes(c->batch, c->batch_scene);
  if (want < 0) {
    fclose(f);
    return set_err(c, MPM_ERR_STATE, "the context holds no restartable scene");
  }
  if (fread(&h, sizeof h, 1, f) != 1 || memcmp(h.magic, kSnapMagic, 8) != 0) {
    r = set_err(c, MPM_ERR_IO, "%s is not a snapshot", path);
  } else if (h.precision != c->precision || h.np != c->g.np || h.nn != c->g.nn || h.ncell != c->g.ncell ||
             h.uvfp != c->g.uvfp || h.nfields != 0 || h.deck_hash != mine) {
    r = set_err(c, MPM_ERR_STATE, "snapshot of another deck or precision");
  } else if (fread(&n, sizeof n, 1, f) != 1) {
    r = set_err(c, MPM_ERR_IO, "truncated snapshot");
  } else if (n != want) {
    r = set_err(c, MPM_ERR_STATE, "snapshot image of %lld bytes does not fit this context", (long long)n);
  } else {
    try {
      img.resize((size_t)n);
    } catch (const std::bad_alloc&) {
      r = set_err(c, MPM_ERR_OOM, "no host memory for the restart image");
    }
    if (!r && fread(img.data(), 1, img.size(), f) != img.size()) r = set_err(c, MPM_ERR_IO, "truncated snapshot");
  }
  fclose(f);
  if (r) return r;
  return batch_status(c, mpm::mpm_batch_scene_restore(c->batch, c->batch_scene, img.data(), img.size()));
}

int mpm_snapshot_save(mpm_ctx* c, const char* path) {
  if (!c || !path) return set_err(c, MPM_ERR_ARG, "bad argument");
  if (c->batch) return snapshot_save_mixed(c, path);
  CK(cudaStreamSynchronize(c->stream));
  FILE* f = fopen(path, "wb");
  if (!f) return set_err(c, MPM_ERR_IO, "cannot write %s", path);
  SnapHeader h;
  memset(&h, 0, sizeof h);
  memcpy(h.magic, kSnapMagic, 8);
  h.precision = c->precision;
  h.nfields = (int)(sizeof kSnapFields / sizeof kSnapFields[0]);
  h.np = c->g.np;
  h.nn = c->g.nn;
  h.ncell = c->g.ncell;
  h.scalars_bytes = (int)sizeof(DevScalars);
  h.uvfp = c->g.uvfp;
  if (int r = deck_hash(c, &h.deck_hash)) {
    fclose(f);
    return r;
  }
  bool ok = fwrite(&h, sizeof h, 1, f) == 1;
  DevScalars sc;
  cudaError_t e = cudaMemcpy(&sc, c->st.sc, sizeof sc, cudaMemcpyDeviceToHost);
  ok = ok && e == cudaSuccess && fwrite(&sc, sizeof sc, 1, f) == 1;
  std::vector<unsigned char> buf;
  for (int k = 0; ok && k < h.nfields; ++k) {
    const int fld = kSnapFields[k];
    if ((fld == MPM_P_FP && !c->g.uvfp) || (fld == MPM_P_PK && !c->g.tlmpm)) continue;
    void* p = nullptr;
    size_t elem = 0;
    long long n = 0;
    if (field_ptr(c, fld, &p, &elem, &n)) {
      ok = false;
      break;
    }
    buf.resize((size_t)n * elem);
    e = cudaMemcpy(buf.data(), p, buf.size(), cudaMemcpyDeviceToHost);
    int32_t tag[2] = {fld, (int32_t)elem};
    ok = e == cudaSuccess && fwrite(tag, sizeof tag, 1, f) == 1 && fwrite(buf.data(), 1, buf.size(), f) == buf.size();
  }
  ok = (fclose(f) == 0) && ok;
  if (!ok) return set_err(c, MPM_ERR_IO, "writing %s failed", path);
  return MPM_OK;
}

int mpm_snapshot_load(mpm_ctx* c, const char* path) {
  if (!c || !path) return set_err(c, MPM_ERR_ARG, "bad argument");
  if (c->batch) return snapshot_load_mixed(c, path);
  FILE* f = fopen(path, "rb");
  if (!f) return set_err(c, MPM_ERR_IO, "cannot read %s", path);
  SnapHeader h;
  DevScalars sc;
  uint64_t mine = 0;
  int r = deck_hash(c, &mine);
  if (r) {
    fclose(f);
    return r;
  }
  if (fread(&h, sizeof h, 1, f) != 1 || memcmp(h.magic, kSnapMagic, 8) != 0) {
    r = set_err(c, MPM_ERR_IO, "%s is not a snapshot", path);
  } else if (h.precision != c->precision || h.np != c->g.np || h.nn != c->g.nn || h.ncell != c->g.ncell ||
             h.scalars_bytes != (int)sizeof(DevScalars) || h.uvfp != c->g.uvfp || h.deck_hash != mine) {
    r = set_err(c, MPM_ERR_STATE, "snapshot of another deck or precision");
  } else if (fread(&sc, sizeof sc, 1, f) != 1) {
    r = set_err(c, MPM_ERR_IO, "truncated snapshot");
  }
  std::vector<unsigned char> buf;
  for (int k = 0; r == MPM_OK && k < h.nfields; ++k) {
    const int fld = kSnapFields[k];
    if ((fld == MPM_P_FP && !c->g.uvfp) || (fld == MPM_P_PK && !c->g.tlmpm)) continue;
    void* p = nullptr;
    size_t elem = 0;
    long long n = 0;
    int32_t tag[2];
    if (field_ptr(c, fld, &p, &elem, &n) || fread(tag, sizeof tag, 1, f) != 1 || tag[0] != fld ||
        tag[1] != (int32_t)elem) {
      r = set_err(c, MPM_ERR_STATE, "snapshot field %d does not match this context", fld);
      break;
    }
    buf.resize((size_t)n * elem);
    if (fread(buf.data(), 1, buf.size(), f) != buf.size()) {
      r = set_err(c, MPM_ERR_IO, "truncated snapshot");
      break;
    }
    cudaError_t e = cudaMemcpy(p, buf.data(), buf.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) r = cuda_err(c, e, "snapshot upload");
  }
  fclose(f);
  if (r) return r;
  CK(cudaMemcpy(c->st.sc, &sc, sizeof sc, cudaMemcpyHostToDevice));
  return MPM_OK;
}

int mpm_gather_async(mpm_ctx* c, int n, const int64_t* particle, const int* field, const int* component) {
  if (!c || n < 0 || n > MPM_GATHER_MAX || (n > 0 && (!particle || !field || !component)))
    return set_err(c, MPM_ERR_ARG, "bad gather request");
  if (c->batch) return batch_status(c, mpm_batch_scene_gather_async(c->batch, c->batch_scene, n, particle, field, component));
  for (int k = 0; k < n; ++k) {
    const int nc = mpm_field_components(field[k]);
    if (field[k] < MPM_P_XP || field[k] > MPM_P_INODE || nc == 0 || component[k] < 0 || component[k] >= nc ||
        particle[k] < 0 || particle[k] >= c->g.np)
      return set_err(c, MPM_ERR_ARG, "gather item %d: particle %lld field %d component %d", k,
                     (long long)particle[k], field[k], component[k]);
    if (field[k] == MPM_P_FP && !c->g.uvfp) return set_err(c, MPM_ERR_ARG, "deformation gradient is not tracked");
    if (field[k] == MPM_P_VOL0) return set_err(c, MPM_ERR_ARG, "field %d is not available", field[k]);
  }
  if (!c->g_items_h) {
    CK(cudaMallocHost((void**)&c->g_items_h, sizeof(GatherItem) * MPM_GATHER_MAX));
    CK(cudaMallocHost((void**)&c->g_out_h, sizeof(double) * MPM_GATHER_MAX));
    CK(cudaMalloc((void**)&c->g_items_d, sizeof(GatherItem) * MPM_GATHER_MAX));
    CK(cudaMalloc((void**)&c->g_out_d, sizeof(double) * MPM_GATHER_MAX));
    CK(cudaEventCreateWithFlags(&c->g_done, cudaEventDisableTiming));
  }
  CK(cudaEventSynchronize(c->g_done));  // the previous gather has released the staging buffers
  for (int k = 0; k < n; ++k) c->g_items_h[k] = GatherItem{(long long)particle[k], field[k], component[k]};
  c->g_n = n;
  if (n > 0) {
    CK(cudaMemcpyAsync(c->g_items_d, c->g_items_h, sizeof(GatherItem) * n, cudaMemcpyHostToDevice, c->stream));
    k_gather<<<(n + 127) / 128, 128, 0, c->stream>>>(c->st, c->g.np, c->g_items_d, n, c->g_out_d);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(c->g_out_h, c->g_out_d, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  }
  CK(cudaEventRecord(c->g_done, c->stream));
  return MPM_OK;
}

int mpm_gather_wait(mpm_ctx* c, double* out) {
  if (!c || !out) return set_err(c, MPM_ERR_ARG, "bad argument");
  if (c->batch) return batch_status(c, mpm_batch_scene_gather_wait(c->batch, out));
  if (!c->g_done) return set_err(c, MPM_ERR_STATE, "no gather in flight");
  CK(cudaEventSynchronize(c->g_done));
  memcpy(out, c->g_out_h, sizeof(double) * (size_t)c->g_n);
  return MPM_OK;
}

int mpm_gather(mpm_ctx* c, int n, const int64_t* particle, const int* field, const int* component, double* out) {
  int r = mpm_gather_async(c, n, particle, field, component);
  return r ? r : mpm_gather_wait(c, out);
}

int mpm_algorithmic_bytes(mpm_ctx* c, double* bytes) {
  if (!c || !bytes) return set_err(c, MPM_ERR_ARG, "bad argument");
  double sc[MPM_NSCALARS];
  int r = mpm_get_scalars(c, sc);
  if (r) return r;
  const double Bw = c->batch ? 4.0 : (double)c->ops->bulk_size;
  // per particle: read {Xp, VXp, mass, VOL, SM, SD, q, ie, cp},
  // write {Xp, VXp, VOL, SM, SD, q, ie, seqv}
  double per_p = (24 + 24 + 8 + 8) + Bw * (1 + 1 + 6 + 1 + 1) + (24 + 24 + 8) + Bw * (1 + 1 + 6 + 1 + 1);
  bool jc = false, dp = false, neo = false, loads = false;
  for (auto& m : c->mats) {
    if (m.mat_type >= 4 && m.mat_type <= 7) jc = true;
    if (m.mat_type == 10) dp = true;
    if (m.mat_type == 11) neo = true;
  }
  if (c->g.qload || (c->flags & MPM_F_QUASILOAD)) loads = true;
  if (jc) per_p += 2 * 3 * Bw;
  if (dp) per_p += 2 * Bw;
  if (neo) per_p += 2 * 9 * Bw;
  if (loads) per_p += 24;
  double per_node = 112 + (c->g.musl ? 48 : 0);
  *bytes = per_p * (double)c->g.np + per_node * sc[13];
  return MPM_OK;
}

}  // extern "C"
