// mpm_sort.cuh -- the batched engine's per-step counting sort of particles by
// sort key, and the tile scans it uses.
//
// The particles arrive in the last step's key order and move less than a
// cell per step (the CFL bound), so a key's particles are nearly contiguous
// already and a key holds a handful of particles (about 8 at 8 particles
// per cell). The sort is a counting sort: per-key counts (taken by kb_keys),
// an inclusive scan of the counts into segment ends, placement of every
// particle into its key's segment through a per-key fill counter (one
// atomic per key and warp), then the order inside each segment restored to
// ascending particle index -- the stable order -- by one thread per short
// segment and one block per long one. The result is the permutation a
// stable radix sort by key would give, whatever order the placement atomics
// ran in, so the step stays deterministic.
#pragma once

#include <climits>

namespace mpm {
namespace bm {

// ------------------------------------------------------------------ scans
// Inclusive scans in tiles of kScanTile items: per-tile totals, an exclusive
// scan of the totals by one block, then each tile scanned with its carry. A
// source policy S gives the value type (S::T), the operation (S::Op), the
// item count, the load of item g and the store of its inclusive prefix; a
// block reads its whole tile before it stores into it and touches no other
// tile, so in-place scans are safe.
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr long long kScanTile = (long long)kScanThreads * kScanItems;

inline long long scan_tiles(long long n) { return (n + kScanTile - 1) / kScanTile; }

struct ScanSum {
  template <class T>
  __device__ __forceinline__ static T id() { return (T)0; }
  template <class T>
  __device__ __forceinline__ static T op(T a, T b) { return a + b; }
};
struct ScanMax {
  template <class T>
  __device__ __forceinline__ static T id() { return (T)INT_MIN; }
  template <class T>
  __device__ __forceinline__ static T op(T a, T b) { return a > b ? a : b; }
};

// Block-wide scan of one value per thread: thr[t] receives the inclusive
// prefix of threads 0..t; returns the exclusive prefix of this thread. Every
// thread of the block calls it; blockDim.x is a multiple of 32, at most 1024.
template <class T, class Op>
__device__ __forceinline__ T block_scan(T v, T* thr, T* wsum) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v = Op::op(u, v);
  }
  if (lane == 31) wsum[warp] = v;
  __syncthreads();
  if (warp == 0) {
    T w = lane < nw ? wsum[lane] : Op::template id<T>();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T u = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w = Op::op(u, w);
    }
    if (lane < nw) wsum[lane] = w;
  }
  __syncthreads();
  if (warp > 0) v = Op::op(wsum[warp - 1], v);
  thr[threadIdx.x] = v;
  __syncthreads();
  const T ex = threadIdx.x ? thr[threadIdx.x - 1] : Op::template id<T>();
  __syncthreads();  // thr and wsum are reused by the next call
  return ex;
}

// tile t into shared memory (coalesced); each thread then owns kScanItems
// consecutive items
template <class S>
__device__ __forceinline__ void load_tile(const S& src, long long t, typename S::T* tile) {
  const long long base = t * kScanTile;
  for (int e = threadIdx.x; e < kScanTile; e += blockDim.x) {
    const long long g = base + e;
    tile[e] = g < src.n ? src.load(g) : S::Op::template id<typename S::T>();
  }
  __syncthreads();
}

template <class S>
__global__ void __launch_bounds__(kScanThreads) ks_tile_total(S src, typename S::T* tiles) {
  using T = typename S::T;
  using Op = typename S::Op;
  __shared__ T tile[kScanTile];
  __shared__ T thr[kScanThreads], wsum[32];
  load_tile(src, blockIdx.x, tile);
  T v = Op::template id<T>();
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) v = Op::op(v, tile[threadIdx.x * kScanItems + k]);
  block_scan<T, Op>(v, thr, wsum);
  if (threadIdx.x == 0) tiles[blockIdx.x] = thr[kScanThreads - 1];
}

// exclusive scan of the nt tile totals in place, by one block of
// kScanThreads threads
template <class T, class Op>
__global__ void __launch_bounds__(kScanThreads) ks_tile_prefix(T* tiles, long long nt) {
  __shared__ T thr[kScanThreads], wsum[32];
  T carry = Op::template id<T>();
  for (long long b0 = 0; b0 < nt; b0 += kScanThreads) {
    const long long t = b0 + threadIdx.x;
    const T v = t < nt ? tiles[t] : Op::template id<T>();
    const T ex = block_scan<T, Op>(v, thr, wsum);
    const T total = thr[kScanThreads - 1];  // thr is not written again before the barrier below
    if (t < nt) tiles[t] = Op::op(carry, ex);
    carry = Op::op(carry, total);
    __syncthreads();
  }
}

// FUSED: tiles hold the tile totals themselves (no ks_tile_prefix launch):
// every block reduces the totals of the tiles before it (for up to
// kFusedTiles tiles, a few loads per thread)
constexpr long long kFusedTiles = 4096;
template <class S, bool FUSED>
__global__ void __launch_bounds__(kScanThreads) ks_tile_scan(S src, const typename S::T* tiles) {
  using T = typename S::T;
  using Op = typename S::Op;
  __shared__ T tile[kScanTile];
  __shared__ T thr[kScanThreads], wsum[32];
  T carry;
  if (FUSED) {
    T v = Op::template id<T>();
    for (long long t = threadIdx.x; t < blockIdx.x; t += blockDim.x) v = Op::op(v, tiles[t]);
    block_scan<T, Op>(v, thr, wsum);
    carry = thr[kScanThreads - 1];  // (thr is rewritten only after the next scan's first barrier)
  } else {
    carry = tiles[blockIdx.x];
  }
  load_tile(src, blockIdx.x, tile);
  T r[kScanItems];
  T v = Op::template id<T>();
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v = Op::op(v, tile[threadIdx.x * kScanItems + k]);
    r[k] = v;
  }
  const T pre = Op::op(carry, block_scan<T, Op>(v, thr, wsum));
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) tile[threadIdx.x * kScanItems + k] = Op::op(pre, r[k]);
  __syncthreads();
  const long long base = (long long)blockIdx.x * kScanTile;
  for (int e = threadIdx.x; e < kScanTile; e += blockDim.x) {
    const long long g = base + e;
    if (g < src.n) src.store(g, tile[e], e ? tile[e - 1] : carry);
  }
}

// an int array scanned into another (or itself); store(g, v, prev) receives
// the inclusive prefixes of items g and g - 1 (sources that also derive
// something from each item's own value use prev)
template <class O>
struct IntScan {
  using T = int;
  using Op = O;
  const int* in;
  int* out;
  long long n;
  __device__ __forceinline__ int load(long long g) const { return in[g]; }
  __device__ __forceinline__ void store(long long g, int v, int) const { out[g] = v; }
};

// the per-key counts scanned in place into segment ends, the keys' fill
// counters zeroed on the way (the placement's slots start at zero)
struct SegScan {
  using T = int;
  using Op = ScanSum;
  int* seg;
  int* fill;
  long long n;
  __device__ __forceinline__ int load(long long g) const { return seg[g]; }
  __device__ __forceinline__ void store(long long g, int v, int) const {
    seg[g] = v;
    fill[g] = 0;
  }
};

// ---------------------------------------------------------- counting sort
constexpr int kRegSeg = 32;         // segments up to this length are ordered by one thread
constexpr int kSegThreads = 256;    // threads of the long-segment blocks
constexpr int kSmemSeg = 8192;      // long segments up to this length are ordered in shared memory

// perm[seg start + slot] = i for every particle i, the slot taken from the
// key's fill counter (one atomic per key and warp; lanes of a warp with the
// same key take consecutive slots in lane order)
__global__ void ks_place(const unsigned* key, const int* seg, int* fill, int* perm, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned k = i < n ? key[i] : 0xffffffffu;
  const unsigned grp = __match_any_sync(0xffffffffu, k);
  if (i >= n) return;
  const int lane = threadIdx.x & 31, leader = __ffs(grp) - 1;
  const int rank = __popc(grp & ((1u << lane) - 1u));
  int base = 0;
  if (lane == leader) base = atomicAdd(&fill[k], __popc(grp));
  base = __shfl_sync(grp, base, leader);
  const int start = k == 0 ? 0 : seg[k - 1];
  perm[start + base + rank] = (int)i;
}

// Ascending order of perm inside each key's segment: segments of up to
// kRegSeg particles by one thread (insertion sort, skipped when already in
// order -- the common case), longer ones listed in big for ks_long_segments.
__global__ void ks_segments(const int* seg, long long nk, int* perm, int* big, int* nbig) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk) return;
  const int a = k == 0 ? 0 : seg[k - 1], e = seg[k];
  const int n = e - a;
  if (n <= 1) return;
  if (n > kRegSeg) {
    big[atomicAdd(nbig, 1)] = (int)k;
    return;
  }
  int* p = perm + a;
  bool sorted = true;
  int prev = p[0];
  for (int j = 1; j < n; ++j) {
    const int c = p[j];
    sorted = sorted && prev < c;
    prev = c;
  }
  if (sorted) return;
  int v[kRegSeg];
  for (int j = 0; j < n; ++j) {
    const int c = p[j];
    int m = j;
    while (m > 0 && v[m - 1] > c) {
      v[m] = v[m - 1];
      --m;
    }
    v[m] = c;
  }
  for (int j = 0; j < n; ++j) p[j] = v[j];
}

// ascending sort of d[0, n) (distinct values) by one block: a bitonic
// network over the next power of two whose every comparator puts the smaller
// value first (the first merge step of each stage compares mirrored
// partners), so the virtual elements past n (taken as +infinity) never move
// and are never touched
__device__ __forceinline__ void block_bitonic(int* d, int n) {
  int N = 1;
  while (N < n) N <<= 1;
  for (int k = 2; k <= N; k <<= 1) {
    for (int s = k >> 1; s > 0; s >>= 1) {
      for (int t = threadIdx.x; t < (N >> 1); t += blockDim.x) {
        int i, j;
        if (s == (k >> 1)) {  // mirrored partner within the block of k
          const int blk = t / s, o = t - blk * s;
          i = blk * k + o;
          j = blk * k + k - 1 - o;
        } else {
          i = (t / s) * 2 * s + (t % s);
          j = i + s;
        }
        if (j < n) {
          const int x = d[i], y = d[j];
          if (x > y) {
            d[i] = y;
            d[j] = x;
          }
        }
      }
      __syncthreads();
    }
  }
}

// the long segments: one block per segment (grid-stride over the list), in
// shared memory up to kSmemSeg particles, in place in global memory beyond
__global__ void __launch_bounds__(kSegThreads) ks_long_segments(const int* seg, int* perm, const int* big,
                                                                const int* nbig) {
  __shared__ int sm[kSmemSeg];
  const int nb = *nbig;
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    const int k = big[b];
    const int a = k == 0 ? 0 : seg[k - 1], n = seg[k] - a;
    int* p = perm + a;
    if (n <= kSmemSeg) {
      for (int j = threadIdx.x; j < n; j += blockDim.x) sm[j] = p[j];
      __syncthreads();
      block_bitonic(sm, n);
      for (int j = threadIdx.x; j < n; j += blockDim.x) p[j] = sm[j];
    } else {
      block_bitonic(p, n);
    }
    __syncthreads();
  }
}

}  // namespace bm
}  // namespace mpm
