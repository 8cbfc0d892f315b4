// mpm_noalloc.cu -- energy / momentum / max-velocity reduction that allocates
// no device memory.
//
// Who needs it: hosts that own all device memory themselves and may not call
// cudaMalloc from inside a solver call -- a Fortran code that hands the
// library device arrays it manages (CUDA Fortran or OpenACC data regions), a
// host running under a fixed memory pool or budget, or a pipeline that must
// not trigger an allocation (and the device synchronisation it can imply) in
// the middle of its time loop. The caller passes device pointers for the
// inputs and the output; the block partial sums live in a file-scope
// __device__ array of fixed size instead of memory the library allocates.
//
// The arithmetic is that of the FP64 forms' calcEnergy reduction (block tree
// of 256 threads, min(1024, ceil(np/256)) blocks, block partials combined by
// the last block in the same fixed order, both compiled without multiply-add
// contraction), so both give the same bits for the same inputs. (The mixed
// form reduces per scene in its own order.)
#include <cuda_runtime.h>

#include <mutex>

#include "mpm3d_gpu.h"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 1024;
constexpr int kVals = 6;  // KE, IE, momentum x / y / z, max |velocity component|
// 6 x 1024 partial sums (48 KiB) + the block-arrival counter, rounded to 64 KiB
constexpr size_t kScratchBytes = 64 * 1024;
constexpr size_t kCounterOffset = sizeof(double) * kVals * kMaxBlocks;

// Shared by every call on a device and kept until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

__global__ void k_energy_noalloc(const double* __restrict__ vxp, const double* __restrict__ mass,
                                 const double* __restrict__ ie, long long np, unsigned char* scratch,
                                 double* out) {
  __shared__ double sh[kVals][kThreads];
  __shared__ bool last;
  double* part = reinterpret_cast<double*>(scratch);
  unsigned* count = reinterpret_cast<unsigned*>(scratch + kCounterOffset);
  double acc[kVals] = {0, 0, 0, 0, 0, 0};
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < np;
       p += (long long)gridDim.x * blockDim.x) {
    double v0 = vxp[p], v1 = vxp[np + p], v2 = vxp[2 * np + p];
    double m = mass[p];
    double vv = v0 * v0 + v1 * v1 + v2 * v2;
    acc[0] = acc[0] + vv * m * 0.5;
    acc[1] = acc[1] + ie[p];
    acc[2] = acc[2] + m * v0;
    acc[3] = acc[3] + m * v1;
    acc[4] = acc[4] + m * v2;
    double a = fabs(v0);
    if (fabs(v1) > a) a = fabs(v1);
    if (fabs(v2) > a) a = fabs(v2);
    if (acc[5] < a) acc[5] = a;
  }
  for (int i = 0; i < kVals; ++i) sh[i][threadIdx.x] = acc[i];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      for (int i = 0; i < 5; ++i) sh[i][threadIdx.x] = sh[i][threadIdx.x] + sh[i][threadIdx.x + w];
      if (sh[5][threadIdx.x + w] > sh[5][threadIdx.x]) sh[5][threadIdx.x] = sh[5][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int i = 0; i < kVals; ++i) part[(long long)i * gridDim.x + blockIdx.x] = sh[i][0];
    __threadfence();
    unsigned done = atomicAdd(count, 1u);
    last = (done == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double tot[kVals] = {0, 0, 0, 0, 0, 0};
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
    for (int i = 0; i < 5; ++i) tot[i] = tot[i] + part[(long long)i * gridDim.x + b];
    double mv = part[5LL * gridDim.x + b];
    if (tot[5] < mv) tot[5] = mv;
  }
  for (int i = 0; i < kVals; ++i) sh[i][threadIdx.x] = tot[i];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      for (int i = 0; i < 5; ++i) sh[i][threadIdx.x] = sh[i][threadIdx.x] + sh[i][threadIdx.x + w];
      if (sh[5][threadIdx.x + w] > sh[5][threadIdx.x]) sh[5][threadIdx.x] = sh[5][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  for (int i = 0; i < kVals; ++i) out[i] = sh[i][0];
  *count = 0;
}

// Device address of the scratch array for the current device, looked up once
// per device (the host-side symbol is not a device address).
int scratch_for_current_device(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MPM_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return MPM_ERR_CUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return MPM_OK;
}

}  // namespace

extern "C" int mpm_energy_reduce_noalloc(const double* vxp, const double* mass, const double* ie,
                                         int64_t np, double* out6, void* stream) {
  if (!vxp || !mass || !ie || !out6) return MPM_ERR_ARG;
  if (np <= 0 || np > MPM_NOALLOC_MAX_PARTICLES) return MPM_ERR_ARG;
  void* scratch = nullptr;
  int st = scratch_for_current_device(&scratch);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  // the arrival counter must start at zero
  if (cudaMemsetAsync((unsigned char*)scratch + kCounterOffset, 0, sizeof(unsigned), s) != cudaSuccess)
    return MPM_ERR_CUDA;
  long long blocks = (np + kThreads - 1) / kThreads;
  if (blocks > kMaxBlocks) blocks = kMaxBlocks;
  k_energy_noalloc<<<(unsigned)blocks, kThreads, 0, s>>>(vxp, mass, ie, (long long)np,
                                                         (unsigned char*)scratch, out6);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_ERR_CUDA;
}
