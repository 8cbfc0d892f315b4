// mpm_batch_kernels.cuh -- kernels of the batched mixed-precision step (see
// mpm_batch.cuh for the layout). FP32 particle math, FP64 grid accumulation.
#pragma once

#include "mpm_batch.cuh"
#include "mpm_kernels.cuh"

namespace mpm {
namespace bm {

__device__ __forceinline__ long long btid() { return (long long)blockIdx.x * blockDim.x + threadIdx.x; }

__device__ __forceinline__ bool scene_live(const BState& b, int s) { return b.sst[s].active != 0; }

// local node (jx, jy, jz) of a global node index
// n / d for 0 <= n < 2^32 by the multiplier m of d (Scene::m*; 0: d = 1),
// a 64-bit high multiply instead of an integer division
__device__ __forceinline__ int div_by(long long n, unsigned long long m) {
  return m ? (int)__umul64hi((unsigned long long)n, m) : (int)n;
}

__device__ __forceinline__ void node_xyz(const Scene& sc, long long ln, int& jx, int& jy, int& jz) {
  jz = div_by(ln, sc.mNGxy);
  int rem = (int)(ln - (long long)jz * sc.NGxy);
  jy = div_by(rem, sc.mNGx);
  jx = rem - jy * sc.NGx;
}

// -------------------------------------------------------------- 1-D shapes
// Offsets are node index minus particle cell index (t) or the particle's
// position relative to the node in cells (r); derivatives are per cell.
__device__ __forceinline__ void lin1(int t, float off, float& w, float& d) {
  w = t ? off : 1.f - off;
  d = t ? 1.f : -1.f;
}
__device__ __forceinline__ void gimp1(float r, float& w, float& d) { gimp_1d<float>(r, w, d); }
// the same values as gimp1, every branch evaluated and the result selected:
// a warp's particles sit in different pieces of the shape, and the branches
// of gimp1 would run one after another
__device__ __forceinline__ void gimp1_select(float r, float& w, float& d) {
  const float a = r < 0.f ? -r : r, sg = copysignf(1.f, r);
  const float w1 = (7.f - 16.f * a * a) * 0.125f, d1 = -(4.f * r);
  const float w2 = 1.f - a, d2 = -sg;
  const float t = (5.f - 4.f * a) * 0.25f;
  const float w3 = t * t, d3 = 2.f * r - sg * 2.5f;
  w = a < 0.25f ? w1 : (a < 0.75f ? w2 : (a < 1.25f ? w3 : 0.f));
  d = a < 0.25f ? d1 : (a < 0.75f ? d2 : (a < 1.25f ? d3 : 0.f));
}
__device__ __forceinline__ void bsp1(int t, float off, float& w, float& d) {
  // NShape_Bspline pieces (Grid.f90:927-962) with r = off * 0.2 + 0.4
  float r = off * 0.2f + 0.4f;
  if (t < 0) {
    float a = 3.f - 5.f * r;
    w = 0.5f * a * a;
    d = (5.f * r - 3.f) * 5.f * 0.2f;
  } else if (t == 0) {
    w = -25.f * r * r + 25.f * r - 5.5f;
    d = (-50.f * r + 25.f) * 0.2f;
  } else {
    float a = 5.f * r - 2.f;
    w = 0.5f * a * a;
    d = (5.f * r - 2.f) * 5.f * 0.2f;
  }
}


// ------------------------------------------------------------- begin step
__global__ void kb_begin(BState b, const int* target) {
  int s = (int)btid();
  if (s >= b.nscene) return;
  SceneState& t = b.sst[s];
  t.active = t.istep < target[s] ? 1 : 0;
  if (!t.active) return;
  t.istep = t.istep + 1;
  if (t.istep == target[s]) atomicAdd(&b.ctl->finished, 1);  // the scene's last step
  t.time = t.time + t.dt;
  t.ftime = (float)t.time;
  t.ie = 0.0;
  t.active_nodes = 0;
  for (int k = 0; k < 4; ++k) t.qmax[k] = 0u;
}

// ---------------------------------------------- FP64 <-> FP32 off the FP64 pipe
// GB300 runs FP64 arithmetic and every conversion to or from a 64-bit type
// on a narrow pipe (1/64 of the FP32 rate); the mixed-precision kernels
// convert between FP64 storage and FP32 arithmetic with integer operations.
// Magnitudes below the FP32 normal range give 0 (sign kept), above it (and
// NaN) infinity; positions, velocities and masses lie far inside it.

// FP32 value of x truncated toward zero (its leading 24 bits)
__device__ __forceinline__ float f32_trunc(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
  const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned mag = e <= 0 ? 0u : (e >= 255 ? 0x7f800000u : ((unsigned)e << 23) | mant);
  return __uint_as_float((hi & 0x80000000u) | mag);
}

// FP32 rounding of x, to nearest even (the value of (float)x)
__device__ __forceinline__ float f32_rn(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
  const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
  // round bit: mantissa bit 28 of the low word; sticky: bits 0..27 (ties to
  // even on the kept last bit); a carry out of the mantissa steps the exponent
  const unsigned inc = ((lo >> 28) & 1u) & (((lo & 0x0fffffffu) != 0u) | (mant & 1u));
  unsigned mag = (((unsigned)e << 23) | mant) + inc;
  mag = e <= 0 ? 0u : (e >= 255 || mag >= 0x7f800000u ? 0x7f800000u : mag);
  return __uint_as_float((hi & 0x80000000u) | mag);
}

// exact FP64 value of an FP32 value (normal or zero)
__device__ __forceinline__ double f64_of(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned hi = (u & 0x80000000u) | (e ? ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3) : 0u);
  const unsigned lo = e ? u << 29 : 0u;
  return __hiloint2double((int)hi, (int)lo);
}

// x as hi + lo: hi its leading 24 bits, lo the remaining 29 rounded to FP32
// (one 32-bit integer conversion), so hi + lo = x to 2^-47 relative
__device__ __forceinline__ void f32_split(double x, float& hi, float& lo) {
  hi = f32_trunc(x);
  const unsigned w = (unsigned)__double2hiint(x), l = (unsigned)__double2loint(x);
  const int eb = (int)((w >> 20) & 0x7ffu);
  // lo = (l mod 2^29) * 2^(e - 52), e = eb - 1023: FP32 biased exponent eb - 948
  const float r = __uint2float_rn(l & 0x1fffffffu) * __uint_as_float(eb > 948 ? (unsigned)(eb - 948) << 23 : 0u);
  lo = (w & 0x80000000u) ? -r : r;
}

// cell of a position (InWhichCell, Grid.f90:123-155) and the offset in it, in
// cells (FP32); false off the grid. Every transfer and gather takes a
// particle's cell and shape-function offsets from this one routine (through
// the per-step data the permutation writes).
__device__ __forceinline__ bool cell_of(const Scene& sc, const double x[3], int cc[3], float off[3]) {
  bool in = true;
  for (int a = 0; a < 3; ++a) {
    if (x[a] < sc.span0[a] || x[a] > sc.span1[a]) in = false;
    double u = (x[a] - sc.span0[a]) * sc.idcell;
    cc[a] = (int)u;
    off[a] = (float)(u - (double)cc[a]);
  }
  return in && cc[0] < sc.NCx && cc[1] < sc.NCy && cc[2] < sc.NCz;
}

// cell_of for the linear, GIMP and B-spline scenes without FP64
// instructions: x - span0 and its product with 1 / dcell carried as FP32
// hi + lo pairs (to about 2^-46), so the offset is exact to far below its
// FP32 rounding. The cell can differ from cell_of's only for a position
// within about 1e-12 cells of a face (or of the grid's edge), where the
// shape functions of the two cells agree.
__device__ __forceinline__ bool cell_of_df(const Scene& sc, const double x[3], int cc[3], float off[3]) {
  bool in = true;
  const int nc[3] = {sc.NCx, sc.NCy, sc.NCz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float xh, xl;
    f32_split(x[a], xh, xl);
    // d = x - span0: TwoSum of the leading parts, the trailing parts added
    const float s = xh - sc.fspan0[a];
    const float bb = s - xh;
    const float err = (xh - (s - bb)) + (-sc.fspan0[a] - bb);
    const float t = err + (xl - sc.fspan0_lo[a]);
    const float dh = s + t, dl = t - (dh - s);
    // u = d * idcell (the lo * lo term is below the pair's precision)
    const float uh = dh * sc.fidcell;
    const float ul = fmaf(dh, sc.fidcell, -uh) + fmaf(dh, sc.fidcell_lo, dl * sc.fidcell);
    float c = floorf(uh);
    float f = (uh - c) + ul;  // uh - c is exact
    if (f < 0.f) {
      c -= 1.f;
      f += 1.f;
    } else if (f >= 1.f) {
      c += 1.f;
      f -= 1.f;
    }
    in = in && c >= 0.f && c < (float)nc[a];
    cc[a] = in ? (int)c : 0;
    off[a] = f;
  }
  return in;
}

// SGMP dual (cell-centre) cell of a position, CenterInWhichCell
// (Grid.f90:157-190): the flat index of the per-direction truncations, valid
// when it lies in 0..CNC-1. Like the reference, a position within half a cell
// of the upper grid faces yields a per-direction index past the last dual
// cell, and the flat index then continues into the next row / layer.
__device__ __forceinline__ long long dual_cell(const Scene& sc, const double x[3]) {
  long long d = 0;
  int dc[3];
  for (int a = 0; a < 3; ++a) dc[a] = (int)((x[a] - sc.span0[a]) * sc.idcell - 0.5);
  d = ((long long)dc[2] * sc.CNCy + dc[1]) * sc.CNCx + dc[0];
  return (d >= 0 && d < sc.CNC) ? d : -1;
}

// (xh + xl) - (sh + sl) as a pair dh + dl: TwoSum of the leading parts, the
// trailing parts added
__device__ __forceinline__ void df_diff(float xh, float xl, float sh, float sl, float& dh, float& dl) {
  const float s = xh - sh;
  const float bb = s - xh;
  const float err = (xh - (s - bb)) + (-sh - bb);
  const float t = err + (xl - sl);
  dh = s + t;
  dl = t - (dh - s);
}

// The SGMP decisions of a position -- its cell and offsets (cell_of), its
// nearest node (the cell's upper one from half a cell on) and its dual cell
// (dual_cell) -- in FP32 double-float arithmetic: x - span0 and x - span1
// as pairs, the coordinate in cells to about 2^-45. Returns false, leaving
// the decisions to the FP64 routines, for a position outside the grid or
// within 2^-40 (relative) of a grid face, a cell face or a half cell, where
// the roundings of the FP64 arithmetic could decide otherwise; every
// decision it returns is the FP64 one. (The nearest node and the dual cell
// are discontinuous at the half cell, so they must be the FP64 ones.)
__device__ __forceinline__ bool sg_locate_df(const Scene& sc, const double x[3], int cc[3], float off[3], int nd[3],
                                             long long& dual) {
  const int nc[3] = {sc.NCx, sc.NCy, sc.NCz};
  int dc[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float xh, xl, dh, dl, eh, el;
    f32_split(x[a], xh, xl);
    df_diff(xh, xl, sc.fspan0[a], sc.fspan0_lo[a], dh, dl);
    df_diff(xh, xl, sc.fspan1[a], sc.fspan1_lo[a], eh, el);
    const float gtol = 0x1p-40f * fabsf(xh);
    if (!(dh > gtol && eh < -gtol)) return false;  // outside or at a grid face
    const float uh = dh * sc.fidcell;
    const float ul = fmaf(dh, sc.fidcell, -uh) + fmaf(dh, sc.fidcell_lo, dl * sc.fidcell);
    const float cf = floorf(uh), fh = uh - cf;  // (exact)
    // distances to the cell's faces and its half (a rounded sum keeps the
    // sign of the exact one)
    const float r0 = fh + ul, r1 = (fh - 1.f) + ul, rh = (fh - 0.5f) + ul;
    const float tol = 0x1p-40f * fmaxf(1.f, uh);
    if (!(r0 > tol && r1 < -tol && fabsf(rh) > tol)) return false;
    const int c = (int)cf;
    if (c >= nc[a]) return false;
    cc[a] = c;
    off[a] = r0;
    nd[a] = c + (rh > 0.f);
    dc[a] = max(nd[a] - 1, 0);  // trunc(u - 1/2): 0 below half a cell
  }
  const long long d = ((long long)dc[2] * sc.CNCy + dc[1]) * sc.CNCx + dc[0];
  dual = (d >= 0 && d < sc.CNC) ? d : -1;
  return true;
}

// ------------------------------------------------------------------ keys
// Sort key of a particle: its scene's key base plus its cell (linear,
// B-spline), its nearest node (GIMP) or its dual cell (SGMP); the scene's
// last key collects the particles outside the grid. Sorting keeps the
// particles of a key contiguous, which the transfers rely on for locality
// (and the SGMP centre gathers for their particle ranges). A GIMP particle
// reaches the nodes within 1.25 cells of it (the cpGIMP quarter rule of
// FindInflNode), i.e. at most one node either side of its nearest node in
// each direction: binned by nearest node, a key's particles reach a 3 x 3 x
// 3 box of nodes instead of the 4 x 4 x 4 box of a cell's particles.
__global__ void kb_keys(BState b) {
  const long long i = btid();
  if (i == 0) *b.nbig = 0;  // long-segment count of this step's sort
  unsigned key = 0xffffffffu;
  if (i < b.NP) {
    const long long NP = b.NP;
    const Scene& sc = b.scenes[b.scene[i]];
    double x[3] = {b.x[i], b.x[NP + i], b.x[2 * NP + i]};
    long long c = -1;
    if (sc.shape == 3) {
      int cc[3], nd[3];
      float off[3];
      if (!sg_locate_df(sc, x, cc, off, nd, c)) c = dual_cell(sc, x);
    } else {
      // The coordinate in cells is formed in FP32 from the positions
      // truncated to FP32 by integer operations (GB300's FP64 pipe is
      // narrow), so it can put a particle within a few FP32 roundings of
      // the coordinate (about 1e-7 of it) on the other side of a face. The
      // sort only groups particles: the transfers take every particle's cell
      // and offsets from the permutation's exact routine (cell_of), so a
      // particle that this rounding puts on the other side of a cell face
      // (or of the grid's edge) is still transferred exactly, in a segment
      // of its own.
      int cc[3];
      float u[3];
      bool in = true;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        u[a] = (f32_trunc(x[a]) - sc.fspan0[a]) * sc.fidcell;
        in = in && u[a] >= 0.f;
        cc[a] = (int)u[a];
      }
      if (in && cc[0] < sc.NCx && cc[1] < sc.NCy && cc[2] < sc.NCz) {
        if (sc.shape == 1) {  // nearest node: the cell's lower node, or the upper one from half a cell on
#pragma unroll
          for (int a = 0; a < 3; ++a) cc[a] += u[a] - (float)cc[a] >= 0.5f;
          c = ((long long)cc[2] * sc.NGy + cc[1]) * sc.NGx + cc[0];
        } else {
          c = ((long long)cc[2] * sc.NCy + cc[1]) * sc.NCx + cc[0];
        }
      }
    }
    key = (unsigned)(sc.k0 + (c >= 0 ? c : sc.nk - 1));
    b.key[i] = key;
  }
  // per-key counts: the particles arrive sorted by the last step's keys, so
  // a warp's lanes mostly share a few keys -- one atomic per key and warp
  const unsigned grp = __match_any_sync(0xffffffffu, key);
  if (key != 0xffffffffu && (threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(&b.seg[key], __popc(grp));
}

// ---------------------------------------------------- permutation + derived
// dst[i] = src[perm[i]] for every persistent particle field, then the per-step
// derived data of the particle at its new position (ParticleInitial,
// update_step.f90:408-453, in FP32 form).
// returns the particle's scene; mass and velocity for the transfer bounds
__device__ __forceinline__ int permute_one(const BState& src, BState& dst, long long i, double& m_out,
                                           double (&v_out)[3]) {
  // every value is loaded before the first store: the stores could alias the
  // loads as far as the compiler knows, so interleaving them would serialise
  // one memory round trip per field
  const long long NP = src.NP;
  const long long j = src.perm[i];
  const int s = src.scene[j];
  const Scene& sc = src.scenes[s];
  // (the external forces move only in scenes that have some: elsewhere
  // they are zero and nothing reads them)
  double x[3], v[3], f[3] = {0.0, 0.0, 0.0};
  for (int a = 0; a < 3; ++a) {
    x[a] = src.x[a * NP + j];
    v[a] = src.v[a * NP + j];
    if (sc.has_fxp) f[a] = src.fxp[a * NP + j];
  }
  const double mass = src.mass[j], ie = src.ie[j];
  const float vol = src.vol[j], evol = src.evol[j], sig_y = src.sig_y[j], sm = src.sm[j], seqv = src.seqv[j];
  float sd[6];
  for (int a = 0; a < 6; ++a) sd[a] = src.sd[a * NP + j];
  const float epeff = src.epeff[j], celsius = src.celsius[j], dmg = src.dmg[j], lt = src.lt[j], cp = src.cp[j],
              q = src.q[j];
  const uint8_t failure = src.failure[j];
  const uint16_t body = src.body[j];
  const int orig = src.orig[j];
  if (src.any_uvfp) {
    float fp[18];
    for (int a = 0; a < 18; ++a) fp[a] = src.fp[a * NP + j];
    for (int a = 0; a < 18; ++a) dst.fp[a * NP + i] = fp[a];
  }
  for (int a = 0; a < 3; ++a) {
    dst.x[a * NP + i] = x[a];
    dst.v[a * NP + i] = v[a];
    if (sc.has_fxp) dst.fxp[a * NP + i] = f[a];
  }
  dst.mass[i] = mass;
  dst.ie[i] = ie;
  dst.vol[i] = vol;
  dst.evol[i] = evol;
  dst.sig_y[i] = sig_y;
  dst.sm[i] = sm;
  dst.seqv[i] = seqv;
  for (int a = 0; a < 6; ++a) dst.sd[a * NP + i] = sd[a];
  dst.epeff[i] = epeff;
  dst.celsius[i] = celsius;
  dst.dmg[i] = dmg;
  dst.lt[i] = lt;
  dst.cp[i] = cp;
  dst.q[i] = q;
  dst.failure[i] = failure;
  dst.body[i] = body;
  dst.scene[i] = (uint16_t)s;
  dst.orig[i] = orig;
  // derived
  int cc[3];
  float off[3];
  int nd[3];
  long long dualc = -1;
  bool in;
  if (sc.shape != 3) {
    in = cell_of_df(sc, x, cc, off);
  } else if (sg_locate_df(sc, x, cc, off, nd, dualc)) {
    in = true;
  } else {
    in = cell_of(sc, x, cc, off);
    for (int a = 0; a < 3; ++a) {
      const double u = (x[a] - sc.span0[a]) * sc.idcell;  // (as in cell_of)
      nd[a] = cc[a] + (u - (double)cc[a] >= 0.5);
    }
    dualc = dual_cell(sc, x);
  }
  for (int a = 0; a < 3; ++a) dst.off[a * NP + i] = off[a];
  dst.cell[i] = in ? (cc[2] * sc.NCy + cc[1]) * sc.NCx + cc[0] : -1;
  if (sc.shape == 3) {
    // dual (cell-centre) grid: CenterInWhichCell (as the sort keys) and the
    // nearest node with the particle's coordinates about it, both decided
    // as in FP64 (sg_locate_df or the FP64 routines above: the node must
    // stay the one above the dual cell, deciding on the FP32 offset would
    // move particles within 3e-8 of the half onto the other node);
    // XXN = 2 off - 2 (upper node) or 2 off in FP32
    dst.dual[i] = (int)dualc;
    bool nin = nd[0] >= 0 && nd[0] < sc.NGx && nd[1] >= 0 && nd[1] < sc.NGy && nd[2] >= 0 && nd[2] < sc.NGz;
    int ln = nin ? (nd[2] * sc.NGy + nd[1]) * sc.NGx + nd[0] : -1;
    dst.inode[i] = ln;
    int bd = ln >= 0 ? src.bd[sc.n0 + ln] : 0;
    for (int a = 0; a < 3; ++a) {
      float xxn = off[a] * 2.f - (nd[a] > cc[a] ? 2.f : 0.f);
      if ((bd >> (2 * a)) & 3) xxn = xxn > 0.f ? 1.f : (xxn < 0.f ? -1.f : 0.f);
      dst.xxn[a * NP + i] = xxn;
      dst.xn[a * NP + i] = off[a] * 2.f - 1.f;
    }
  }
  m_out = mass;
  for (int a = 0; a < 3; ++a) v_out[a] = v[a];
  return s;
}

// ------------------------------------------- deterministic P2G scatter
// Particle -> node transfers of linear, GIMP and B-spline scenes, and the
// particle -> centre-node transfers of SGMP scenes, are scatters: each cell's
// (dual cell's) particles add their FP32 contributions to the nodes they
// influence. Contributions are quantised to 64-bit fixed point with a
// per-scene, per-quantity power-of-two scale and summed with integer adds, so
// a node's sum is exact and independent of the order of the adds (and of
// which other scenes share the batch). The scale comes from a per-step bound
// B on any single contribution's magnitude (a max over the scene's particles,
// also order-independent): a node sums at most np contributions, np * B <
// 2^E, and contributions are scaled by 2^(61 - E), so no sum can reach 2^62.
// The rounding of a contribution to the fixed-point grid (np * B * 2^-61)
// is far below its FP32 rounding.
// The bounds are taken by the kernels that run before each transfer
// (permutation, force staging, position update).

// per-scene bound slots (SceneState::qmax, float bits, reset every step)
enum QSlot { Q_MASS = 0, Q_MOM = 1, Q_FORCE = 2, Q_MOM_MUSL = 3 };

// Max of non-negative values v[k] over the block into sst[s].qmax[slot[k]],
// per scene s (s < 0: no value). Every thread of the block must call it.
// Warps whose lanes all belong to one scene combine through shared memory,
// so a block usually issues one atomic per slot: a per-warp atomic on the
// same address from every warp of a large scene would serialise in L2.
template <int NS>
__device__ __forceinline__ void block_scene_max(BState& b, int s, const int (&slot)[NS], const float (&v)[NS]) {
  __shared__ int ws[32];
  __shared__ unsigned wv[32][NS];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  const unsigned grp = __match_any_sync(0xffffffffu, s);
  unsigned mx[NS];
  for (int k = 0; k < NS; ++k) mx[k] = __reduce_max_sync(grp, __float_as_uint(v[k]));
  const bool uniform = grp == 0xffffffffu;
  if (!uniform && s >= 0 && lane == __ffs(grp) - 1)
    for (int k = 0; k < NS; ++k) atomicMax(&b.sst[s].qmax[slot[k]], mx[k]);
  if (lane == 0) {
    ws[warp] = uniform ? s : -1;
    for (int k = 0; k < NS; ++k) wv[warp][k] = mx[k];
  }
  __syncthreads();
  if (warp == 0) {
    const int s2 = lane < nw ? ws[lane] : -1;
    const unsigned g2 = __match_any_sync(0xffffffffu, s2);
    for (int k = 0; k < NS; ++k) {
      const unsigned m2 = __reduce_max_sync(g2, lane < nw ? wv[lane][k] : 0u);
      if (s2 >= 0 && lane == __ffs(g2) - 1) atomicMax(&b.sst[s2].qmax[slot[k]], m2);
    }
  }
}

// Fixed-point shift sh of a scene's channel: contributions are rounded to
// integers after scaling by 2^sh, sh = 61 - E with np * bound < 2^E, so no
// sum of a scene's contributions overflows, and at most 47 - Eb with
// bound < 2^Eb, so that one flushed sum (at most 32 contributions) stays
// below 2^53 for quant (this limit binds below 16384 particles only);
// clamped to the FP32 exponent range, 0 when the bound is 0 and every
// contribution is 0.
__device__ __forceinline__ int q_shift(const Scene& sc, unsigned bound_bits) {
  const float bound = __uint_as_float(bound_bits);
  if (!(bound > 0.f)) return 0;
  int E, Eb;
  frexpf(sc.fnp * bound, &E);  // np < 2^31: the product is exact up to one rounding, covered by E + 1
  frexpf(bound, &Eb);
  return max(-126, min(127, min(61 - E, 47 - Eb)));
}
__device__ __forceinline__ float q_scale(int sh) { return __int_as_float((sh + 127) << 23); }
// f = c * 2^sh rounded to the nearest 64-bit integer (ties to even) for
// |f| <= 2^53, without the FP64 pipe (GB300 converts float to int64 there,
// at a small fraction of the 32-bit conversion rate). f splits exactly into
// h * 2^31 + r: the FP32 sum f + 1.5 * 2^54 lies in the binade whose ulp is
// 2^31, so it is 1.5 * 2^54 + h * 2^31 with h = f / 2^31 rounded to
// nearest, and h is the difference of the two bit patterns; the remainder
// r = f - h * 2^31 has |r| <= 2^30 and is exact (a multiple of f's ulp no
// larger than f), so one 32-bit conversion rounds it. h * 2^31 is an
// integer, so the result equals __float2ll_rn(f).
__device__ __forceinline__ long long quant(float c, float scale) {
  constexpr float M = 0x1.8p54f;
  const float f = c * scale;
  const float t = f + M;
  const int h = __float_as_int(t) - __float_as_int(M);
  const int r = __float2int_rn(f - (t - M));
  return (long long)h * 2147483648LL + r;
}
__device__ __forceinline__ double q_unit(int sh) { return __longlong_as_double((long long)(1023 - sh) << 52); }  // 2^-sh

// influence nodes of a particle along one direction: node = cell + t0 + k
// for k < the returned count (at most 3), weight w[k] and derivative d[k]
// (per cell) -- NShape / the cpGIMP quarter rule of FindInflNode with
// NShape_GIMP / NShape_Bspline. Fixed-size arrays with constant indices (the
// gathers unroll their node loops) stay in registers.
__device__ __forceinline__ int dim_nodes(int shape, float off, int& t0, float w[3], float d[3]) {
  if (shape == 0) {
    t0 = 0;
    lin1(0, off, w[0], d[0]);
    lin1(1, off, w[1], d[1]);
    w[2] = d[2] = 0.f;
    return 2;
  }
  if (shape == 2) {
    t0 = -1;
#pragma unroll
    for (int k = 0; k < 3; ++k) bsp1(k - 1, off, w[k], d[k]);
    return 3;
  }
  t0 = off < 0.25f ? -1 : 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) gimp1((float)(-(t0 + k)) + off, w[k], d[k]);
  return 2 + (off < 0.25f) + (off > 0.75f);
}

// permutation kernel; it also takes the mass and momentum bounds of the
// step's first particle -> node transfer
__global__ void kb_permute(BState src, BState dst) {
  const long long i = btid();
  int s = -1;
  float bm = 0.f, bv = 0.f;
  if (i < src.NP) {
    double m, v[3];
    s = permute_one(src, dst, i, m, v);
    // FP32 mass and velocity for the first transfer (the conversions run
    // once per particle here, not in every transfer lane)
    const float m32 = f32_rn(m), v32[3] = {f32_rn(v[0]), f32_rn(v[1]), f32_rn(v[2])};
    dst.m32[i] = m32;
    for (int a = 0; a < 3; ++a) dst.v32[a * dst.NP + i] = v32[a];
    if (scene_live(dst, s)) {
      bm = m32;
      bv = bm * fmaxf(fabsf(v32[0]), fmaxf(fabsf(v32[1]), fabsf(v32[2]))) * 1.0001f;
    } else {
      s = -1;
    }
  }
  block_scene_max<2>(dst, s, {Q_MASS, Q_MOM}, {bm, bv});
}

// Corner k of the dual cell (dx, dy, dz) as a scene cell (its centre node),
// with the reference's flat arithmetic (CenterCellNode, Grid.f90:380-418:
// first corner plus the corner's flat offset; corners at or past the last
// cell are dropped, and a direction with a single cell -- one dual cell --
// spills into the next row); -1 if dropped.
__device__ __forceinline__ long long sg_corner_cell(const Scene& sc, int dx, int dy, int dz, int k) {
  const long long c1 = ((long long)dz * sc.NCy + dy) * sc.NCx + dx;
  const long long cid = c1 + kCorner[k][0] + (long long)kCorner[k][1] * sc.NCx + (long long)kCorner[k][2] * sc.NCxy;
  return cid < (long long)sc.NCxy * sc.NCz ? cid : -1;
}

// -------------------------------------------- particle-parallel scatter
// Linear, GIMP and B-spline scenes scatter in tasks of 32 consecutive
// particles of one scene (task t of a scene: its sorted particles 32 t ..
// 32 t + 31). The lanes of a task that share a sort key (the key's cell, or
// for GIMP its nearest node) form a segment, and every segment's particles
// reach the same box of node offsets (2^3 linear, 3^3 GIMP / B-spline). The
// shapes are tensor products, N = Wx Wy Wz, so a slot's contribution splits
// into an x factor and a (y, z) factor per channel, e.g. for the force
//   f_x = Dx (-s_xx Wy Wz) + Wx (b_x Wy Wz - s_xy Dy Wz - s_xz Wy Dz).
// Two phases through the warp's shared workspace:
//   1. lane = particle: its x factors (W, and D for the force) per x offset
//      and its (y, z) factors per channel, one column per lane;
//   2. lane = box slot: the walk along the task's particles in storage order
//      (FP32 sums of x factor times (y, z) factor, every channel at once),
//      flushed at every segment end -- quantised and added to the node's
//      64-bit accumulators with one integer atomic per channel.
// The task boundaries are fixed by the scene's own sorted order (32 t from
// the scene's first particle), so a scene's sums are the same alone or in a
// batch. Phase 2's walk and its segment ends are the same for every lane
// (the segment mask comes from a warp vote), so the warp never diverges
// there.
template <int MODE>
struct PartShape {
  static constexpr int NV = MODE == 0 ? 4 : 3;          // channels
  static constexpr int NX = MODE == 2 ? 6 : 3;          // x-factor rows (W, and D, per x offset)
  static constexpr int NK = MODE == 2 ? 2 : 1;          // (y, z) factors per channel and (ty, tz)
  static constexpr int ROWS = NX + 9 * NV * NK;         // workspace rows (one column per lane)
  static constexpr int STRIDE = 33;                     // row stride: conflict-free in both phases
  static constexpr int WARPS = MODE == 2 ? 4 : 8;       // warps (tasks) per block (static shared memory)
};

// 1-D weight w[t] and derivative d[t] (per unit length) of node offset t
// from the key's base (linear: 0..1 from the cell; B-spline: -1..1 from the
// cell; GIMP: -1..1 from the nearest node)
template <int SH>
__device__ __forceinline__ void part_tab(float off, float idc, float (&w)[3], float (&d)[3]) {
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    if (SH == 0) {
      if (t < 2) lin1(t, off, w[t], d[t]);
      else w[t] = d[t] = 0.f;
    } else if (SH == 2) {
      bsp1(t - 1, off, w[t], d[t]);
    } else {
      gimp1_select(off - (float)(t - 1 + (off >= 0.5f)), w[t], d[t]);  // node = nearest - 1 + t
    }
    d[t] *= idc;
  }
}

template <int MODE, int SH>
__device__ __forceinline__ void part_scatter_task(BState& b, const Scene& sc, long long i0, int cnt, float sA,
                                                  float sB, float* ws) {
  using PS = PartShape<MODE>;
  constexpr int NV = PS::NV, NX = PS::NX, NK = PS::NK, ST = PS::STRIDE;
  constexpr int nt = SH == 0 ? 2 : 3, tlo = SH == 0 ? 0 : -1, NS = nt * nt * nt;
  const int lane = threadIdx.x & 31;
  const long long NP = b.NP, i = i0 + lane;
  const int cl = lane < cnt ? b.cell[i] : -1;
  int c[3] = {0, 0, 0};
  float off[3] = {0.f, 0.f, 0.f};
  int key = -1;
  if (cl >= 0) {
    c[2] = div_by(cl, sc.mNCxy);
    const int rem = cl - c[2] * sc.NCxy;
    c[1] = div_by(rem, sc.mNCx);
    c[0] = rem - c[1] * sc.NCx;
#pragma unroll
    for (int a = 0; a < 3; ++a) off[a] = b.off[a * NP + i];
    if (SH == 1) {
#pragma unroll
      for (int a = 0; a < 3; ++a) c[a] += off[a] >= 0.5f;
      key = (c[2] * sc.NGy + c[1]) * sc.NGx + c[0];
    } else {
      key = cl;
    }
  }
  // segment ends: the last lane of every run of equal keys
  const int knext = __shfl_down_sync(0xffffffffu, key, 1);
  const unsigned lasts = __ballot_sync(0xffffffffu, key >= 0 && (lane == 31 || knext != key));
  if (lasts == 0u) return;  // (uniform) nothing of this task on the grid
  // the segment's first box node (scene-local flat index) and whether the
  // whole box lies inside the grid
  const int nbase = ((c[2] + tlo) * sc.NGy + (c[1] + tlo)) * sc.NGx + (c[0] + tlo);
  const bool inner = c[0] + tlo >= 0 && c[0] + tlo + nt <= sc.NGx && c[1] + tlo >= 0 && c[1] + tlo + nt <= sc.NGy &&
                     c[2] + tlo >= 0 && c[2] + tlo + nt <= sc.NGz;
  // phase 1: the particle's factors (zero for a lane without a key)
  {
    constexpr int NQ = MODE == 2 ? 9 : 4;
    float pv[NQ];
    float w[3][3], d[3][3];
#pragma unroll
    for (int q = 0; q < NQ; ++q) pv[q] = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int t = 0; t < 3; ++t) w[a][t] = d[a][t] = 0.f;
    if (key >= 0) {
      if (MODE == 2) {
#pragma unroll
        for (int q = 0; q < 9; ++q) pv[q] = b.fs[q * NP + i];
      } else {
        pv[0] = b.m32[i];
#pragma unroll
        for (int a = 0; a < 3; ++a) pv[1 + a] = b.v32[a * NP + i];
      }
      const float idc = sc.fidcell;
#pragma unroll
      for (int a = 0; a < 3; ++a) part_tab<SH>(off[a], idc, w[a], d[a]);
    }
    float* col = ws + lane;
#pragma unroll
    for (int t = 0; t < nt; ++t) {
      col[t * ST] = w[0][t];
      if (MODE == 2) col[(3 + t) * ST] = d[0][t];
    }
#pragma unroll
    for (int tz = 0; tz < nt; ++tz)
#pragma unroll
      for (int ty = 0; ty < nt; ++ty) {
        const int yz = tz * nt + ty;
        const float A = w[1][ty] * w[2][tz];
        if (MODE == 2) {
          const float B = d[1][ty] * w[2][tz], C = w[1][ty] * d[2][tz];
          // per channel: o0 (times D) and o1 (times W)
          col[(NX + 0 * 9 + yz) * ST] = -pv[0] * A;
          col[(NX + 1 * 9 + yz) * ST] = pv[6] * A - pv[3] * B - pv[5] * C;
          col[(NX + 2 * 9 + yz) * ST] = -pv[3] * A;
          col[(NX + 3 * 9 + yz) * ST] = pv[7] * A - pv[1] * B - pv[4] * C;
          col[(NX + 4 * 9 + yz) * ST] = -pv[5] * A;
          col[(NX + 5 * 9 + yz) * ST] = pv[8] * A - pv[4] * B - pv[2] * C;
        } else {
          const float M = pv[0] * A;
          if (MODE == 0) col[(NX + yz) * ST] = M;
#pragma unroll
          for (int a = 0; a < 3; ++a) col[(NX + (MODE == 0 ? 1 + a : a) * 9 + yz) * ST] = M * pv[1 + a];
        }
      }
  }
  __syncwarp();
  // phase 2: lane = box slot (sx, sy, sz), the walk along the particles
  const int sz = lane / (nt * nt), sy = (lane / nt) % nt, sx = lane % nt;
  const int yz = lane < NS ? sz * nt + sy : 0;
  const int soff = (sz * sc.NGy + sy) * sc.NGx + sx;
  const float* xw = ws + (lane < NS ? sx : 0) * ST;
  const float* xd = ws + (lane < NS ? 3 + sx : 0) * ST;
  const float* fr = ws + (NX + yz) * ST;
  // segment by segment: the segment ends come from a warp vote, so the walk
  // and its flushes are the same for every lane
  unsigned rem = lasts;
  int j = 0;
  while (rem) {
    const int e = __ffs(rem) - 1;  // the segment's last lane
    rem &= rem - 1;
    float acc[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[v] = 0.f;
#pragma unroll 4
    for (; j <= e; ++j) {
      const float x = xw[j];
      if (MODE == 2) {
        const float dx = xd[j];
#pragma unroll
        for (int v = 0; v < 3; ++v) acc[v] += dx * fr[(2 * v) * 9 * ST + j] + x * fr[(2 * v + 1) * 9 * ST + j];
      } else {
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[v] += x * fr[v * 9 * ST + j];
      }
    }
    // flush the segment's sums into the nodes
    const int nb = __shfl_sync(0xffffffffu, nbase, e);
    bool ok = lane < NS;
    if (!__shfl_sync(0xffffffffu, (int)inner, e)) {  // (uniform) a box at the grid's edge
      const int jx = __shfl_sync(0xffffffffu, c[0], e) + tlo + sx, jy = __shfl_sync(0xffffffffu, c[1], e) + tlo + sy,
                jz = __shfl_sync(0xffffffffu, c[2], e) + tlo + sz;
      ok = ok && jx >= 0 && jx < sc.NGx && jy >= 0 && jy < sc.NGy && jz >= 0 && jz < sc.NGz;
    }
    if (ok) {
      const long long n = sc.n0 + nb + soff;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const long long q = quant(acc[v], MODE == 0 && v > 0 ? sB : sA);
        if (q) atomicAdd(&b.acc[v * b.NN + n], (unsigned long long)q);
      }
    }
  }
  __syncwarp();
}

// The SGMP form of a particle task: the key is the particle's dual cell,
// whose 8 corners are centre nodes with the SGNShape weights
// 0.125 (1 +- xi)(1 +- eta)(1 +- zeta). Phase 1 (lane = particle) writes the
// 8 corner weights -- times the mass for the momentum transfers -- and the
// transferred values; phase 2 (lane = corner and channel) walks the task's
// particles and flushes each segment's sums, quantised, into the centre
// nodes' 64-bit accumulators. Channels: mode 0 mass and momentum (CenterNode
// Mg, PXg), 1 momentum with the updated velocities, 2 external then internal
// force (Cfext, Cfint); a lane takes the corner lane / 4 (mode 0) or lane / 3
// (modes 1, 2: one channel, or three force channels g, g + 3, g + 6).
template <int MODE>
__device__ __forceinline__ void sg_part_task(BState& b, const Scene& sc, long long i0, int cnt, float sA, float sB,
                                             float* ws) {
  constexpr int ST = PartShape<MODE>::STRIDE;
  constexpr int CH0 = MODE == 2 ? CQ_FE : (MODE == 1 ? CQ_P : CQ_M);  // first accumulator channel
  const int lane = threadIdx.x & 31;
  const long long NP = b.NP, i = i0 + lane;
  const int d = lane < cnt ? b.dual[i] : -1;
  const int knext = __shfl_down_sync(0xffffffffu, d, 1);
  const unsigned lasts = __ballot_sync(0xffffffffu, d >= 0 && (lane == 31 || knext != d));
  if (lasts == 0u) return;  // (uniform) nothing of this task on the dual grid
  // phase 1: rows 0..7 the corner weights (times the mass for modes 0, 1),
  // then the values (velocity, or the 9 force inputs)
  {
    float* col = ws + lane;
    float xx[3] = {0.f, 0.f, 0.f}, m = 0.f;
    if (d >= 0) {
#pragma unroll
      for (int a = 0; a < 3; ++a) xx[a] = b.xxn[a * NP + i];
      if (MODE != 2) m = b.m32[i];
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      float w = 0.125f;
#pragma unroll
      for (int a = 0; a < 3; ++a) w *= kCorner[k][a] ? 1.f + xx[a] : 1.f - xx[a];
      col[k * ST] = d < 0 ? 0.f : (MODE == 2 ? w : w * m);
    }
    if (MODE == 2) {
#pragma unroll
      for (int c = 0; c < 9; ++c) col[(8 + c) * ST] = d < 0 ? 0.f : b.fs[(c < 3 ? 6 + c : c - 3) * NP + i];
    } else {
#pragma unroll
      for (int a = 0; a < 3; ++a) col[(8 + a) * ST] = d < 0 ? 0.f : b.v32[a * NP + i];
    }
  }
  __syncwarp();
  // phase 2
  constexpr int NPER = MODE == 0 ? 4 : 3;  // lanes per corner
  const int k = lane / NPER, g = lane - k * NPER;
  const bool active = k < 8;
  const float* wr = ws + (active ? k : 0) * ST;
  const float* vr = ws + (8 + (MODE == 0 ? (g > 0 ? g - 1 : 0) : g)) * ST;
  constexpr int NA = MODE == 2 ? 3 : 1;  // accumulators per lane
  unsigned rem = lasts;
  int j = 0;
  while (rem) {  // segment by segment (uniform: the segment ends come from a warp vote)
    const int e = __ffs(rem) - 1;
    rem &= rem - 1;
    float acc[NA];
#pragma unroll
    for (int a = 0; a < NA; ++a) acc[a] = 0.f;
#pragma unroll 4
    for (; j <= e; ++j) {
      const float w = wr[j];
      if (MODE == 2) {
#pragma unroll
        for (int a = 0; a < 3; ++a) acc[a] += w * vr[3 * a * ST + j];
      } else if (MODE == 0) {
        acc[0] += g == 0 ? w : w * vr[j];
      } else {
        acc[0] += w * vr[j];
      }
    }
    const int dj = __shfl_sync(0xffffffffu, d, e);  // flush into the centre nodes
    if (active) {
      const int dz = div_by(dj, sc.mCNCxy), rm = dj - dz * sc.CNCxy, dy = div_by(rm, sc.mCNCx), dx = rm - dy * sc.CNCx;
      const long long cid = sg_corner_cell(sc, dx, dy, dz, k);
      if (cid >= 0) {
#pragma unroll
        for (int a = 0; a < NA; ++a) {
          const int ch = MODE == 2 ? g + 3 * a : g;
          const long long q = quant(acc[a], MODE == 0 && ch != 0 ? sB : sA);
          if (q) atomicAdd(&b.cacc[(long long)(CH0 + ch) * b.NC + sc.c0 + cid], (unsigned long long)q);
        }
      }
    }
  }
  __syncwarp();
}

template <int MODE>
__global__ void __launch_bounds__(32 * PartShape<MODE>::WARPS, MODE == 2 ? 6 : 4) kb_part_scatter(BState b) {
  using PS = PartShape<MODE>;
  __shared__ float wsp[PS::WARPS][PS::ROWS * PS::STRIDE];
  const int warp = threadIdx.x >> 5;
  const int nt = b.task0[b.nscene];
  for (int t = blockIdx.x * PS::WARPS + warp; t < nt; t += gridDim.x * PS::WARPS) {
    // the scene of the task: the last scene whose first task is at or before t
    int lo = 0, hi = b.nscene - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (b.task0[mid] <= t) lo = mid;
      else hi = mid - 1;
    }
    const int s = lo;
    const Scene& sc = b.scenes[s];
    if (!scene_live(b, s) || (MODE == 1 && !sc.musl)) continue;
    const long long first = (long long)(t - b.task0[s]) * 32;
    const int cnt = (int)min(32LL, sc.np - first);
    const SceneState& st = b.sst[s];
    const float sA = q_scale(q_shift(sc, st.qmax[MODE == 0 ? Q_MASS : (MODE == 1 ? Q_MOM_MUSL : Q_FORCE)]));
    const float sB = MODE == 0 ? q_scale(q_shift(sc, st.qmax[Q_MOM])) : sA;
    float* ws = wsp[warp];
    switch (sc.shape) {
      case 0: part_scatter_task<MODE, 0>(b, sc, sc.p0 + first, cnt, sA, sB, ws); break;
      case 1: part_scatter_task<MODE, 1>(b, sc, sc.p0 + first, cnt, sA, sB, ws); break;
      case 2: part_scatter_task<MODE, 2>(b, sc, sc.p0 + first, cnt, sA, sB, ws); break;
      default: sg_part_task<MODE>(b, sc, sc.p0 + first, cnt, sA, sB, ws);
    }
  }
}

// Accumulated channels 0..nv-1 of node n in FP64 (the accumulators cleared
// for the next transfer). Returns false for an idle node: nothing
// accumulated and a node mass of +0, so every node field is still zero from
// the last time the node was written and nothing needs writing -- on sparse
// grids most nodes are idle. (A node that no particle reaches is never read
// by a particle, and one whose mass drops to zero is written once.) A
// massless node that received a force or a momentum (IntegrateMomentum
// integrates every node, so its momentum is F * DT) carries a mass of -0 as
// the mark that its fields are not zero, and the next transfer clears them.
__device__ __forceinline__ bool take_acc(BState& b, long long n, int nv, const double* unit, double* out) {
  unsigned long long q[4];
  unsigned long long any = 0ull;
  for (int v = 0; v < nv; ++v) {
    q[v] = b.acc[v * b.NN + n];
    any |= q[v];
  }
  if (any == 0ull && __double_as_longlong(b.mg[n]) == 0ll) return false;
  for (int v = 0; v < nv; ++v) {
    out[v] = (double)(long long)q[v] * unit[v];
    if (q[v]) b.acc[v * b.NN + n] = 0ull;
  }
  return true;
}

__device__ __forceinline__ void node_finish(BState& b, const Scene& sc, long long n, int bc, int vel) {
  const long long NN = b.NN;
  if (bc) {
    uint8_t f = b.fix[n];
    for (int a = 0; a < 3; ++a)
      if (f & (1 << a)) {
        b.px[a * NN + n] = 0.0;
        b.fx[a * NN + n] = 0.0;
      }
  }
  if (vel) {
    // node velocity for the FP32 particle gathers; nodes at or below the
    // cut-off mass contribute nothing, so they hold zero
    const double m = b.mg[n];
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (m > sc.cutoff) {
      const float m32 = (float)m;
      v.x = (float)b.px[n] / m32;
      v.y = (float)b.px[NN + n] / m32;
      v.z = (float)b.px[2 * NN + n] / m32;
    }
    b.nvel[n] = v;
  }
}

__global__ void kb_p2g_mass(BState b, int bc_usf, int vel_usf) {
  long long n = btid();
  bool act = false;
  int s = -1;
  if (n < b.NN) {
    s = b.node_scene[n];
    if (scene_live(b, s)) {
      const Scene& sc = b.scenes[s];
      const long long NN = b.NN;
      double M = 0, P0 = 0, P1 = 0, P2 = 0;
      bool live = true;
      int j[3];
      node_xyz(sc, n - sc.n0, j[0], j[1], j[2]);
      if (sc.shape == 3) {
        // centre nodes -> node (GridMomentumInitial of SGMP): 1/8 of the
        // adjacent cells' mass and momentum, cells at or below the cut-off
        // mass left out; the cells' fixed-point sums are added exactly
        const SceneState& st = b.sst[s];
        const int shm = q_shift(sc, st.qmax[Q_MASS]);
        const double um = q_unit(shm), up = q_unit(q_shift(sc, st.qmax[Q_MOM]));
        // cm = q * um > cutoff  <=>  q > floor(cutoff / um) (um a power of two)
        const double thr = ldexp(sc.cutoff, shm);
        const long long qcut = thr >= 9.0e18 ? LLONG_MAX : (long long)floor(thr);
        const unsigned long long* ca = b.cacc;
        const long long NC = b.NC;
        long long QM = 0, Q0 = 0, Q1 = 0, Q2 = 0;
        for (int cz = j[2] - 1; cz <= j[2]; ++cz) {
          if (cz < 0 || cz >= sc.NCz) continue;
          for (int cy = j[1] - 1; cy <= j[1]; ++cy) {
            if (cy < 0 || cy >= sc.NCy) continue;
            for (int cx = j[0] - 1; cx <= j[0]; ++cx) {
              if (cx < 0 || cx >= sc.NCx) continue;
              const long long c = sc.c0 + (cz * sc.NCy + cy) * sc.NCx + cx;
              const long long qm = (long long)ca[CQ_M * NC + c];
              if (qm <= qcut) continue;
              QM += qm;
              Q0 += (long long)ca[CQ_P * NC + c];
              Q1 += (long long)ca[(CQ_P + 1) * NC + c];
              Q2 += (long long)ca[(CQ_P + 2) * NC + c];
            }
          }
        }
        M = 0.125 * ((double)QM * um);
        P0 = 0.125 * ((double)Q0 * up);
        P1 = 0.125 * ((double)Q1 * up);
        P2 = 0.125 * ((double)Q2 * up);
      } else {
        const SceneState& st = b.sst[s];
        const double up = q_unit(q_shift(sc, st.qmax[Q_MOM]));
        const double unit[4] = {q_unit(q_shift(sc, st.qmax[Q_MASS])), up, up, up};
        double o[4];
        live = take_acc(b, n, 4, unit, o);
        M = o[0];
        P0 = o[1];
        P1 = o[2];
        P2 = o[3];
      }
      if (live) {
        b.mg[n] = M;
        b.px[n] = P0;
        b.px[NN + n] = P1;
        b.px[2 * NN + n] = P2;
        act = M > 0.0;
        node_finish(b, sc, n, bc_usf && sc.usf, vel_usf && sc.usf);
        if (!(M != 0.0) && sc.shape != 3) {
          // the node goes idle: clear the rest of its fields once (the idle
          // test of the later transfers skips it from now on)
          for (int a = 0; a < 3; ++a) b.fx[a * NN + n] = 0.0;
          b.nvel[n] = make_float4(0.f, 0.f, 0.f, 0.f);
          b.nacc[n] = make_float4(0.f, 0.f, 0.f, 0.f);
          // a momentum without mass (the mass contributions quantised to
          // zero, the momentum ones not) keeps the node marked (take_acc)
          if (b.px[n] != 0.0 || b.px[NN + n] != 0.0 || b.px[2 * NN + n] != 0.0) b.mg[n] = -0.0;
        }
      }
    }
  }
  // per-scene active-node count, combined per block (one atomic per scene
  // and block in the common case)
  __shared__ int ws[32];
  __shared__ unsigned wc[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  const unsigned grp = __match_any_sync(0xffffffffu, s);
  const unsigned actg = __ballot_sync(0xffffffffu, act) & grp;
  const bool uniform = grp == 0xffffffffu;
  if (!uniform && s >= 0 && actg && lane == __ffs(grp) - 1)
    atomicAdd(&b.sst[s].active_nodes, (unsigned long long)__popc(actg));
  if (lane == 0) {
    ws[warp] = uniform ? s : -1;
    wc[warp] = uniform ? (unsigned)__popc(actg) : 0u;
  }
  __syncthreads();
  if (warp == 0) {
    const int s2 = lane < nw ? ws[lane] : -1;
    const unsigned g2 = __match_any_sync(0xffffffffu, s2);
    const unsigned c2 = __reduce_add_sync(g2, lane < nw ? wc[lane] : 0u);
    if (s2 >= 0 && c2 && lane == __ffs(g2) - 1) atomicAdd(&b.sst[s2].active_nodes, (unsigned long long)c2);
  }
}

// -------------------------------------------------------------- stress
// ParticleStressUpdate + Constitution for one particle (FP32). The stress pass
// runs twice per step: before the force transfer for USF scenes (usf_pass 1)
// and after the position update for USL / MUSL scenes (usf_pass 0).
// MT != 0: the particles of material type MT (an instantiation for each of
// the common types, fewer registers); MT = 0: every other type
__host__ __device__ constexpr bool stress_specialised(int mat_type) {
  return mat_type == 1 || mat_type == 9 || mat_type == 10 || mat_type == 11;
}

// (the common types capped at 64 registers: four 256-thread blocks per SM)
__device__ __forceinline__ float force_stage(BState& b, const Scene& sc, const SceneState& st, long long i, float vol,
                                             float smq, const float (&sd)[6]);

// stages the particle's force input when its scene's USF pass has its final
// stress here (no Johnson-Cook tail after this kernel) and returns that
// contribution's bound; -1 otherwise. UV: the instantiation for scenes that
// update volumes by Fp (1) or not (0) -- without the Fp state's registers
// when not; uvf: the batch holds both kinds, so each launch takes its own.
template <int MT, int UV>
__device__ __forceinline__ float stress_one(BState& b, long long i, int usf_pass, int filter, int uvf) {
  using P = PMixed;
  using R = float;
  const int s = b.scene[i];
  if (!scene_live(b, s)) return -1.f;
  const Scene& sc = b.scenes[s];
  if (sc.usf != usf_pass || (uvf && sc.uvfp != UV)) return -1.f;
  const DevMaterialF& mt = b.fmats[b.bodies[b.body[i]].mat];
  // every particle goes through the instantiation of its own material type
  // (or the general one), whatever else shares the batch: the compiled FP32
  // arithmetic, and so the result, is the same alone or in a batch (filter
  // 0: the batch needs this instantiation only)
  if (filter && (MT ? mt.mat_type != MT : stress_specialised(mt.mat_type))) return -1.f;
  const long long NP = b.NP;
  const long long o = sc.p0 + b.orig[i];  // position in the reference processing order
  if (sc.has_jc) {
    b.setter[o] = -1;
    b.deferred[i] = 0;
  }
  R de[6] = {0, 0, 0, 0, 0, 0}, vort[3] = {0, 0, 0}, deFp[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  if (sc.shape == 3) {
    int d = b.dual[i];
    if (d < 0) return -1.f;
    int dz = div_by(d, sc.mCNCxy), rem = d - dz * sc.CNCxy, dy = div_by(rem, sc.mCNCx), dx = rem - dy * sc.CNCx;
    float xx[3] = {b.xxn[i], b.xxn[NP + i], b.xxn[2 * NP + i]};
    for (int k = 0; k < 8; ++k) {
      int oc[3] = {kCorner[k][0], kCorner[k][1], kCorner[k][2]};
      const long long cid = sg_corner_cell(sc, dx, dy, dz, k);
      if (cid < 0) continue;
      const long long c = sc.c0 + cid;
      float w = 0.125f;
      for (int a = 0; a < 3; ++a) w *= oc[a] ? 1.f + xx[a] : 1.f - xx[a];
      const long long NC = b.NC;
      for (int a = 0; a < 6; ++a) de[a] += b.co[a * NC + c] * w;
      for (int a = 0; a < 3; ++a) vort[a] += b.cw[a * NC + c] * w;
      for (int a = 0; a < 9; ++a) deFp[a / 3][a % 3] += w * b.cdefp[a * NC + c];
    }
  } else {
    const int cl = b.cell[i];
    if (cl < 0) return -1.f;
    int c[3];
    c[2] = div_by(cl, sc.mNCxy);
    int rem = cl - c[2] * sc.NCxy;
    c[1] = div_by(rem, sc.mNCx);
    c[0] = rem - c[1] * sc.NCx;
    float off[3] = {b.off[i], b.off[NP + i], b.off[2 * NP + i]};
    int t0[3], nt[3];
    float wd[3][3], dd[3][3];
    for (int a = 0; a < 3; ++a) nt[a] = dim_nodes(sc.shape, off[a], t0[a], wd[a], dd[a]);
    // velocity gradient L[a][k] = sum_n v_a(n) dN_n / dx_k; the shape is a
    // tensor product, so the node velocities are first summed along x with
    // the x weights and x derivatives, and each (y, z) row then adds its two
    // sums times the y-z factors: 6 multiply-adds per node instead of the 24
    // of forming de, vort and deFp node by node
    float L[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
    for (int az = 0; az < 3; ++az)
#pragma unroll
      for (int ay = 0; ay < 3; ++ay) {
        if (ay >= nt[1] || az >= nt[2]) continue;
        const int jy = c[1] + t0[1] + ay, jz = c[2] + t0[2] + az;
        if (jy < 0 || jy >= sc.NGy || jz < 0 || jz >= sc.NGz) continue;
        const long long row = sc.n0 + ((long long)jz * sc.NGy + jy) * sc.NGx;
        float S[3] = {0, 0, 0}, D[3] = {0, 0, 0};
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
          if (ax >= nt[0]) continue;
          const int jx = c[0] + t0[0] + ax;
          if (jx < 0 || jx >= sc.NGx) continue;
          const float4 v4 = b.nvel[row + jx];  // zero below the cut-off mass
          S[0] += wd[0][ax] * v4.x;
          S[1] += wd[0][ax] * v4.y;
          S[2] += wd[0][ax] * v4.z;
          D[0] += dd[0][ax] * v4.x;
          D[1] += dd[0][ax] * v4.y;
          D[2] += dd[0][ax] * v4.z;
        }
        const float fx = wd[1][ay] * wd[2][az], fy = dd[1][ay] * wd[2][az], fz = wd[1][ay] * dd[2][az];
        for (int a = 0; a < 3; ++a) {
          L[a][0] += D[a] * fx;
          L[a][1] += S[a] * fy;
          L[a][2] += S[a] * fz;
        }
      }
    const float idc = sc.fidcell;
    for (int a = 0; a < 3; ++a)
      for (int k = 0; k < 3; ++k) deFp[a][k] = L[a][k] * idc;
    de[0] = deFp[0][0];
    de[1] = deFp[1][1];
    de[2] = deFp[2][2];
    de[3] = deFp[2][1] + deFp[1][2];
    de[4] = deFp[0][2] + deFp[2][0];
    de[5] = deFp[1][0] + deFp[0][1];
    vort[0] = deFp[2][1] - deFp[1][2];
    vort[1] = deFp[0][2] - deFp[2][0];
    vort[2] = deFp[1][0] - deFp[0][1];
  }
  const SceneState& st = b.sst[s];
  const R DT = st.fdt;
  for (int a = 0; a < 6; ++a) de[a] *= DT;
  for (int a = 0; a < 3; ++a) vort[a] = vort[a] * DT / 2.f;
  for (int a = 0; a < 3; ++a)
    for (int k = 0; k < 3; ++k) deFp[a][k] *= DT;
  R Fpn[3][3], Fpn_lo[3][3];
  if (UV) {
    // Fp(n+1) = (I + dF) Fp(n), i.e. H += dF + dF H for H = Fp - I, with H
    // carried as a pair hi + lo of FP32 values: the increment in FP32 from
    // the rounded H, added to the pair without rounding error (TwoSum), so
    // that H keeps the precision of the increments instead of losing an
    // FP32 rounding of its whole size every step (a rotated body has |H|
    // far above its strain)
    R F0[3][3], L0[3][3];
    for (int a = 0; a < 9; ++a) {
      F0[a / 3][a % 3] = b.fp[a * NP + i];
      L0[a / 3][a % 3] = b.fp[(9 + a) * NP + i];
    }
    for (int a = 0; a < 3; ++a)
      for (int k = 0; k < 3; ++k) {
        const R inc = deFp[a][k] + (deFp[a][0] * F0[0][k] + deFp[a][1] * F0[1][k] + deFp[a][2] * F0[2][k]);
        const F2 t = two_sum(F0[a][k], inc);
        const F2 h = two_sum(t.hi, t.lo + L0[a][k]);
        Fpn[a][k] = h.hi;
        Fpn_lo[a][k] = h.lo;
        b.fp[(a * 3 + k) * NP + i] = h.hi;
        b.fp[(9 + a * 3 + k) * NP + i] = h.lo;
      }
  }
  PState<R> ps;
  ps.vol = b.vol[i];
  ps.epeff = b.epeff[i];
  ps.sig_y = b.sig_y[i];
  ps.seqv = b.seqv[i];
  ps.lt = b.lt[i];
  ps.celsius = b.celsius[i];
  ps.ie = (R)b.ie[i];
  ps.mass = b.m32[i];
  ps.dmg = b.dmg[i];
  ps.cp = b.cp[i];
  ps.sm = b.sm[i];
  ps.q = b.q[i];
  for (int a = 0; a < 6; ++a) ps.sd[a] = b.sd[a * NP + i];
  ps.failure = b.failure[i] != 0;
  ps.evol = b.evol[i];
  CResult<R> res;
  constitution<P, MT>(ps, mt, de, vort, deFp, Fpn, UV != 0, DT, st.time, sc.fdcell, sc.fbq1, sc.fbq2, res,
                      UV ? Fpn_lo : nullptr);
  if (res.negative_volume) atomicOr(&b.sst[s].status, (unsigned)ST_NEGATIVE_VOLUME);
  if (!res.eos_ok) atomicOr(&b.sst[s].status, (unsigned)ST_BAD_EOS);
  if (sc.has_jc) {
    if (res.dep_set) {
      b.setter[o] = (int)o;
      b.dep[o] = (double)res.depeff;
    }
    b.deferred[i] = res.defer ? (uint8_t)res.tail : 0;
    if (res.defer && res.tail == 7) {
      b.jc_aux[i] = res.vold;
      b.jc_aux[NP + i] = res.ieinc;
      b.jc_aux[2 * NP + i] = res.dvol;
      b.jc_aux[3 * NP + i] = res.smold;
      b.jc_aux[4 * NP + i] = res.vol_;
    }
  }
  b.vol[i] = ps.vol;
  b.evol[i] = ps.evol;
  b.sm[i] = ps.sm;
  b.seqv[i] = ps.seqv;
  for (int a = 0; a < 6; ++a) b.sd[a * NP + i] = ps.sd[a];
  b.sig_y[i] = ps.sig_y;
  b.epeff[i] = ps.epeff;
  b.ie[i] = (double)ps.ie;
  b.cp[i] = ps.cp;
  b.q[i] = ps.q;
  b.celsius[i] = ps.celsius;
  b.failure[i] = ps.failure ? 1 : 0;
  if (!isfinite(ps.sm) || !isfinite(ps.ie)) atomicOr(&b.sst[s].status, (unsigned)ST_NONFINITE);
  if (!sc.usf)
    for (int a = 0; a < 3; ++a) b.x[a * NP + i] = b.xx[a * NP + i];
  // GridMomentumUpdate follows a USF stress update directly: stage its
  // force input from the registers (the stress state is final unless a
  // Johnson-Cook tail still runs)
  if (!sc.usf || sc.has_jc) return -1.f;
  return force_stage(b, sc, st, i, ps.vol, ps.sm - ps.q, ps.sd);
}

// (Drucker-Prager runs best at 1536 threads per SM -- 40 registers, some
// spilled -- faster than at 1024 threads without spills; the other
// specialised models at 1024)
template <int MT, int UV>
__global__ void __launch_bounds__(512, MT == 10 ? 3 : (MT ? 2 : 1))
    kb_stress(BState b, int usf_pass, int filter, int uvf) {
  const long long i = btid();
  float bound = -1.f;
  if (i < b.NP) bound = stress_one<MT, UV>(b, i, usf_pass, filter, uvf);
  if (usf_pass) block_scene_max<1>(b, bound >= 0.f ? (int)b.scene[i] : -1, {Q_FORCE}, {fmaxf(bound, 0.f)});
}

// Johnson-Cook tails waiting for the depeff carried from the previous particle
// in the reference order (scene-local input order)
__global__ void kb_depeff_apply(BState b, int usf_pass) {
  using P = PMixed;
  using R = float;
  long long i = btid();
  if (i >= b.NP) return;
  const int s = b.scene[i];
  const Scene& sc = b.scenes[s];
  if (!sc.has_jc || !scene_live(b, s) || sc.usf != usf_pass) return;
  const int tail = b.deferred[i];
  if (tail == 0) return;
  const long long NP = b.NP;
  const long long o = sc.p0 + b.orig[i];
  int last = b.setter_scan[o];
  R D = (R)(last >= sc.p0 && last <= o ? b.dep[last] : b.sst[s].depeff_carry);
  const DevMaterial& mt = b.mats[b.bodies[b.body[i]].mat];
  if (tail == 4) {
    R den_ = (R)b.mass[i] / b.vol[i];
    b.celsius[i] = b.celsius[i] + b.seqv[i] * D / den_ / (R)mt.specheat;
    return;
  }
  Mm<R> m;
  m.epeff_ = b.epeff[i];
  m.sm = b.sm[i];
  m.bqf = b.q[i];
  m.iener = (R)b.ie[i];
  m.seqv = b.seqv[i];
  m.sd[0] = b.sd[i];
  m.sd[1] = b.sd[NP + i];
  m.sd[2] = b.sd[2 * NP + i];
  m.sd[3] = b.sd[4 * NP + i];
  m.sd[4] = b.sd[5 * NP + i];
  m.sd[5] = b.sd[3 * NP + i];
  m.vold = (R)b.jc_aux[i];
  m.ieinc = (R)b.jc_aux[NP + i];
  m.dvol = (R)b.jc_aux[2 * NP + i];
  m.smold = (R)b.jc_aux[3 * NP + i];
  m.vol_ = (R)b.jc_aux[4 * NP + i];
  m.DMG = b.dmg[i];
  m.oldDMG = m.DMG;
  bool failure = b.failure[i] != 0;
  R vol_store = m.vol_;
  jc7_tail<P>(m, mt, failure, D, vol_store);
  R den_ = (R)b.mass[i] / m.vol_;
  b.celsius[i] = b.celsius[i] + m.seqv * D / den_ / (R)mt.specheat;
  b.vol[i] = vol_store;
  b.sm[i] = m.sm;
  b.q[i] = m.bqf;
  b.ie[i] = (double)m.iener;
  b.epeff[i] = m.epeff_;
  b.sd[i] = m.sd[0];
  b.sd[NP + i] = m.sd[1];
  b.sd[2 * NP + i] = m.sd[2];
  b.sd[4 * NP + i] = m.sd[3];
  b.sd[5 * NP + i] = m.sd[4];
  b.sd[3 * NP + i] = m.sd[5];
  b.failure[i] = failure ? 1 : 0;
}

__global__ void kb_depeff_carry(BState b, int usf_pass) {
  int s = (int)btid();
  if (s >= b.nscene) return;
  const Scene& sc = b.scenes[s];
  if (!sc.has_jc || !scene_live(b, s) || sc.np == 0 || sc.usf != usf_pass) return;
  int last = b.setter_scan[sc.p0 + sc.np - 1];
  if (last >= sc.p0 && last < sc.p0 + sc.np) b.sst[s].depeff_carry = b.dep[last];
}

// ------------------------------------------------------------ force input
// external force (QuLo ramp, Damp, gravity; update_step.f90:889-903) and
// sigma * vol, staged per particle in FP32 for the force gather, from the
// particle's volume, SM - q and SD; returns the bound of one contribution
__device__ __forceinline__ float force_stage(BState& b, const Scene& sc, const SceneState& st, long long i, float vol,
                                             float smq, const float (&sd)[6]) {
  const long long NP = b.NP;
  // external force in FP32 (the staged force is FP32): load ramp, mass
  // damping, gravity
  float f[3];
  const float m = b.m32[i];
  if (sc.has_fxp) {
    const float ramp = (sc.qload && !(st.time >= sc.qload_time)) ? (float)(st.time / sc.qload_time) : 1.f;
    for (int a = 0; a < 3; ++a) f[a] = (float)b.fxp[a * NP + i] * ramp;
  } else {
    f[0] = f[1] = f[2] = 0.f;
  }
  if (sc.qdamp)
    for (int a = 0; a < 3; ++a) f[a] = f[a] - sc.fdamp * m * b.v32[a * NP + i];
  if (sc.gravity) {
    const DevBody& bd = b.bodies[b.body[i]];
    for (int a = 0; a < 3; ++a) f[a] = f[a] + m * bd.fgravp[a];
  }
  float fs[6];
  for (int a = 0; a < 3; ++a) fs[a] = (smq + sd[a]) * vol;
  for (int a = 3; a < 6; ++a) fs[a] = sd[a] * vol;
  for (int a = 0; a < 6; ++a) b.fs[a * NP + i] = fs[a];
  for (int a = 0; a < 3; ++a) b.fs[(6 + a) * NP + i] = f[a];
  // bound of one contribution: node force (|grad N| <= 1 / h per component,
  // N <= 1), or for SGMP one centre-node channel (N times a staged value)
  const float sig = fabsf(fs[0]) + fabsf(fs[1]) + fabsf(fs[2]) + 2.f * (fabsf(fs[3]) + fabsf(fs[4]) + fabsf(fs[5]));
  const float gscale = sc.shape == 3 ? 1.f : sc.fidcell;
  return (sig * gscale + fabsf(f[0]) + fabsf(f[1]) + fabsf(f[2])) * 1.0001f;
}

// the staging of the particles whose stress kernel did not stage them (scenes
// updating stresses after the position update, and Johnson-Cook scenes, whose
// tails run after the stress kernel)
__device__ __forceinline__ float force_prep_one(BState& b, long long i) {
  const int s = b.scene[i];
  if (!scene_live(b, s)) return -1.f;
  const Scene& sc = b.scenes[s];
  if (sc.usf && !sc.has_jc) return -1.f;
  const long long NP = b.NP;
  // (every value loaded before the first store, which could alias them)
  const float vol = b.vol[i];
  const float smq = b.sm[i] - b.q[i];
  float sd[6];
  for (int a = 0; a < 6; ++a) sd[a] = b.sd[a * NP + i];
  return force_stage(b, sc, b.sst[s], i, vol, smq, sd);
}

__global__ void kb_force_prep(BState b) {
  const long long i = btid();
  float bound = -1.f;
  if (i < b.NP) bound = force_prep_one(b, i);
  block_scene_max<1>(b, bound >= 0.f ? (int)b.scene[i] : -1, {Q_FORCE}, {fmaxf(bound, 0.f)});
}

// GridMomentumUpdate + IntegrateMomentum for one node
__device__ __forceinline__ void node_integrate(BState& b, const Scene& sc, long long n, const double f[3]) {
  const long long NN = b.NN;
  const SceneState& st = b.sst[b.node_scene[n]];
  const double dt = st.dt;
  for (int a = 0; a < 3; ++a) {
    b.fx[a * NN + n] = f[a];
    double p = b.px[a * NN + n];
    p = st.istep == 1 ? p + f[a] * dt * 0.5 : p + f[a] * dt;
    b.px[a * NN + n] = p;
  }
  node_finish(b, sc, n, 1, 1);
  const double m = b.mg[n];
  if (m == 0.0 && sc.shape != 3) b.mg[n] = -0.0;  // fields not zero at a massless node (take_acc)
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  if (m > sc.cutoff) {
    const float m32 = (float)m;
    acc.x = (float)b.fx[n] / m32;
    acc.y = (float)b.fx[NN + n] / m32;
    acc.z = (float)b.fx[2 * NN + n] / m32;
  }
  b.nacc[n] = acc;
}

__global__ void kb_p2g_force(BState b) {
  long long n = btid();
  if (n >= b.NN) return;
  const int s = b.node_scene[n];
  if (!scene_live(b, s)) return;
  const Scene& sc = b.scenes[s];
  int j[3];
  node_xyz(sc, n - sc.n0, j[0], j[1], j[2]);
  double F[3] = {0, 0, 0};
  if (sc.shape == 3) {
    // centre nodes -> node (GridMomentumUpdate of SGMP): 1/8 of the cells'
    // external force minus Cfint . dN, dN = +-1 / (4 Jacobi) per direction
    // by the node's side of the cell; the cells' fixed-point sums are
    // combined exactly, then scaled once
    const long long NC = b.NC;
    const unsigned long long* ca = b.cacc;
    long long E[3] = {0, 0, 0}, T[3] = {0, 0, 0};
    for (int cz = j[2] - 1; cz <= j[2]; ++cz) {
      if (cz < 0 || cz >= sc.NCz) continue;
      for (int cy = j[1] - 1; cy <= j[1]; ++cy) {
        if (cy < 0 || cy >= sc.NCy) continue;
        for (int cx = j[0] - 1; cx <= j[0]; ++cx) {
          if (cx < 0 || cx >= sc.NCx) continue;
          const long long c = sc.c0 + (cz * sc.NCy + cy) * sc.NCx + cx;
          long long I[6];
          for (int a = 0; a < 3; ++a) E[a] += (long long)ca[(CQ_FE + a) * NC + c];
          for (int a = 0; a < 6; ++a) I[a] = (long long)ca[(CQ_FI + a) * NC + c];
          // signed by the node's side: +dN at the upper corner of the cell
          const bool ux = j[0] != cx, uy = j[1] != cy, uz = j[2] != cz;
          const long long xx = ux ? I[0] : -I[0], xy_x = ux ? I[3] : -I[3], xz_x = ux ? I[5] : -I[5];
          const long long xy_y = uy ? I[3] : -I[3], yy = uy ? I[1] : -I[1], yz_y = uy ? I[4] : -I[4];
          const long long xz_z = uz ? I[5] : -I[5], yz_z = uz ? I[4] : -I[4], zz = uz ? I[2] : -I[2];
          T[0] += xx + xy_y + xz_z;
          T[1] += xy_x + yy + yz_z;
          T[2] += xz_x + yz_y + zz;
        }
      }
    }
    const double u = q_unit(q_shift(sc, b.sst[s].qmax[Q_FORCE]));
    for (int a = 0; a < 3; ++a) F[a] = (0.125 * (double)E[a] - sc.iJacobi4 * (double)T[a]) * u;
  } else {
    const double u = q_unit(q_shift(sc, b.sst[s].qmax[Q_FORCE]));
    const double unit[3] = {u, u, u};
    if (!take_acc(b, n, 3, unit, F)) return;  // idle node
  }
  node_integrate(b, sc, n, F);
}

// SGMP: strain rate / spin at the centre nodes from the 8 cell nodes
__global__ void kb_sg_centre_gradient(BState b, int usf_pass) {
  long long c = btid();
  if (c >= b.NC) return;
  int s = b.cscene[c];
  if (!scene_live(b, s)) return;
  const Scene& sc = b.scenes[s];
  if (sc.usf != usf_pass) return;
  const long long NC = b.NC;
  long long lc = c - sc.c0;
  int q[3];
  q[2] = div_by(lc, sc.mNCxy);
  int rem = (int)(lc - (long long)q[2] * sc.NCxy);
  q[1] = div_by(rem, sc.mNCx);
  q[0] = rem - q[1] * sc.NCx;
  float co[6] = {0, 0, 0, 0, 0, 0}, cw[3] = {0, 0, 0}, cf[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const float j4 = sc.fiJacobi4;
  for (int k = 0; k < 8; ++k) {
    long long n = sc.n0 + ((long long)(q[2] + kCorner[k][2]) * sc.NGy + q[1] + kCorner[k][1]) * sc.NGx + q[0] +
                  kCorner[k][0];
    const float4 v4 = b.nvel[n];  // zero below the cut-off mass
    const float v[3] = {v4.x, v4.y, v4.z};
    const float dx = kSN[0][k] * j4, dy = kSN[1][k] * j4, dz = kSN[2][k] * j4;
    co[0] += dx * v[0];
    co[1] += dy * v[1];
    co[2] += dz * v[2];
    co[3] += dz * v[1] + dy * v[2];
    co[4] += dz * v[0] + dx * v[2];
    co[5] += dy * v[0] + dx * v[1];
    cw[0] += dy * v[2] - dz * v[1];
    cw[1] += dz * v[0] - dx * v[2];
    cw[2] += dx * v[1] - dy * v[0];
    for (int a = 0; a < 3; ++a) {
      cf[a * 3 + 0] += dx * v[a];
      cf[a * 3 + 1] += dy * v[a];
      cf[a * 3 + 2] += dz * v[a];
    }
  }
  for (int a = 0; a < 6; ++a) b.co[a * NC + c] = co[a];
  for (int a = 0; a < 3; ++a) b.cw[a * NC + c] = cw[a];
  for (int a = 0; a < 9; ++a) b.cdefp[a * NC + c] = cf[a];
}

// SGMP: centre-node velocity / acceleration (BoundaryAuxiliaryNodeUpdate on
// the fixed / symmetric faces)
__global__ void kb_sg_centre_velocity(BState b) {
  long long c = btid();
  if (c >= b.NC) return;
  int s = b.cscene[c];
  if (!scene_live(b, s)) return;
  const Scene& sc = b.scenes[s];
  long long lc = c - sc.c0;
  int q[3];
  q[2] = div_by(lc, sc.mNCxy);
  int rem = (int)(lc - (long long)q[2] * sc.NCxy);
  q[1] = div_by(rem, sc.mNCx);
  q[0] = rem - q[1] * sc.NCx;
  const int NCd[3] = {sc.NCx, sc.NCy, sc.NCz};
  const long long NC = b.NC;
  bool boundary = false;
  for (int a = 0; a < 3; ++a)
    if (NCd[a] > 1 && ((q[a] == 0 && sc.fixs[2 * a] != 0) || (q[a] == NCd[a] - 1 && sc.fixs[2 * a + 1] != 0)))
      boundary = true;
  double cxx[3] = {0, 0, 0};
  if (boundary)
    for (int a = 0; a < 3; ++a)
      if (NCd[a] > 1) cxx[a] = q[a] == NCd[a] - 1 ? -1.0 : (q[a] == 0 ? 1.0 : 0.0);
  float v[3] = {0, 0, 0}, acc[3] = {0, 0, 0};
  for (int k = 0; k < 8; ++k) {
    long long n = sc.n0 + ((long long)(q[2] + kCorner[k][2]) * sc.NGy + q[1] + kCorner[k][1]) * sc.NGx + q[0] +
                  kCorner[k][0];
    float w = 0.125f;
    if (boundary)
      w = ((float)kSN[0][k] * (float)cxx[0] + 1.f) * ((float)kSN[1][k] * (float)cxx[1] + 1.f) *
          ((float)kSN[2][k] * (float)cxx[2] + 1.f) * 0.125f;
    const float4 vn = b.nvel[n], an = b.nacc[n];  // zero below the cut-off mass
    v[0] += w * vn.x;
    v[1] += w * vn.y;
    v[2] += w * vn.z;
    acc[0] += w * an.x;
    acc[1] += w * an.y;
    acc[2] += w * an.z;
  }
  for (int a = 0; a < 3; ++a) {
    b.cvx[a * NC + c] = v[a];
    b.cax[a * NC + c] = acc[a];
  }
  // the force sums are consumed (and so are the momentum sums when the
  // MUSL transfer refills them): cleared for the next scatter
  for (int a = sc.musl ? CQ_P : CQ_FE; a < CQ_N; ++a) b.cacc[a * NC + c] = 0ull;
}

// SGMP: clears the mass and momentum sums of the live scenes' centre nodes
// before the step's first transfer (they stay readable between steps)
__global__ void kb_sg_clear(BState b) {
  const long long c = btid();
  if (c >= b.NC) return;
  if (!scene_live(b, b.cscene[c])) return;
  for (int a = CQ_M; a < CQ_FE; ++a) b.cacc[a * b.NC + c] = 0ull;
}

// ---------------------------------------------------------- G2P position
__device__ __forceinline__ float position_one(BState& b, long long i) {
  const int s = b.scene[i];
  if (!scene_live(b, s)) return -1.f;
  const Scene& sc = b.scenes[s];
  const SceneState& st = b.sst[s];
  const long long NP = b.NP;
  // the particle's FP64 position and velocity, loaded before the node
  // gathers so that their latency overlaps the gathers'
  double x0[3], v0[3];
  for (int a = 0; a < 3; ++a) {
    x0[a] = b.x[a * NP + i];
    v0[a] = b.v[a * NP + i];
  }
  float v[3] = {0, 0, 0}, acc[3] = {0, 0, 0};
  if (sc.shape == 3) {
    int d = b.dual[i];
    if (d < 0) return -1.f;
    int dz = div_by(d, sc.mCNCxy), rem = d - dz * sc.CNCxy, dy = div_by(rem, sc.mCNCx), dx = rem - dy * sc.CNCx;
    int ln = b.inode[i];
    int bd = ln >= 0 ? b.bd[sc.n0 + ln] : 0;
    float xx[3];
    for (int a = 0; a < 3; ++a) {
      if ((bd >> (2 * a)) & 3) {  // AuxiliaryGridSHP
        float xn = b.xn[a * NP + i];
        xx[a] = xn < 0.f ? 1.f + 2.f * xn : 2.f * xn - 1.f;
      } else {
        xx[a] = b.xxn[a * NP + i];
      }
    }
    if (bd == 0)
      for (int a = 0; a < 3; ++a) xx[a] = b.xxn[a * NP + i];
    const long long NC = b.NC;
    for (int k = 0; k < 8; ++k) {
      int oc[3] = {kCorner[k][0], kCorner[k][1], kCorner[k][2]};
      const long long cid = sg_corner_cell(sc, dx, dy, dz, k);
      if (cid < 0) continue;
      const long long c = sc.c0 + cid;
      float w = 0.125f;
      for (int a = 0; a < 3; ++a) w *= oc[a] ? 1.f + xx[a] : 1.f - xx[a];
      for (int a = 0; a < 3; ++a) {
        v[a] += w * b.cvx[a * NC + c];
        acc[a] += w * b.cax[a * NC + c];
      }
    }
  } else {
    const int cl = b.cell[i];
    if (cl < 0) return -1.f;
    int c[3];
    c[2] = div_by(cl, sc.mNCxy);
    int rem = cl - c[2] * sc.NCxy;
    c[1] = div_by(rem, sc.mNCx);
    c[0] = rem - c[1] * sc.NCx;
    float off[3] = {b.off[i], b.off[NP + i], b.off[2 * NP + i]};
    int t0[3], nt[3];
    float wd[3][3], dd[3][3];
    for (int a = 0; a < 3; ++a) nt[a] = dim_nodes(sc.shape, off[a], t0[a], wd[a], dd[a]);
    // node rows along x: bounds and row index once per row, one multiply
    // per node for its weight (the shape is a tensor product)
#pragma unroll
    for (int az = 0; az < 3; ++az)
#pragma unroll
      for (int ay = 0; ay < 3; ++ay) {
        if (ay >= nt[1] || az >= nt[2]) continue;
        const int jy = c[1] + t0[1] + ay, jz = c[2] + t0[2] + az;
        if (jy < 0 || jy >= sc.NGy || jz < 0 || jz >= sc.NGz) continue;
        const long long row = sc.n0 + ((long long)jz * sc.NGy + jy) * sc.NGx;
        const float wyz = wd[1][ay] * wd[2][az];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
          if (ax >= nt[0]) continue;
          const int jx = c[0] + t0[0] + ax;
          if (jx < 0 || jx >= sc.NGx) continue;
          const float4 vn = b.nvel[row + jx], an = b.nacc[row + jx];  // zero below the cut-off mass
          const float w = wd[0][ax] * wyz;
          v[0] += w * vn.x;
          v[1] += w * vn.y;
          v[2] += w * vn.z;
          acc[0] += w * an.x;
          acc[1] += w * an.y;
          acc[2] += w * an.z;
        }
      }
  }
  // position and velocity integrated in FP64 (the FP32 interpolants
  // converted exactly by integer operations; the FP32 velocity copy
  // likewise)
  const double dt = st.dt;
  float pv[3];
  for (int a = 0; a < 3; ++a) {
    const double xx = x0[a] + f64_of(v[a]) * dt;
    b.xx[a * NP + i] = xx;
    const double vv = v0[a];
    const double vn = st.istep == 1 ? vv + f64_of(acc[a]) * dt * 0.5 : vv + f64_of(acc[a]) * dt;
    b.v[a * NP + i] = vn;
    pv[a] = f32_rn(vn);
    b.v32[a * NP + i] = pv[a];  // for GridMomentumMUSL's transfer
    if (sc.usf) b.x[a * NP + i] = xx;
  }
  if (!sc.musl) return -1.f;
  // bound of GridMomentumMUSL's contributions with the updated velocity
  const float m = b.m32[i];
  return m * fmaxf(fabsf(pv[0]), fmaxf(fabsf(pv[1]), fabsf(pv[2]))) * 1.0001f;
}

// (capped at 40 registers: six 256-thread blocks per SM hide the node
// gathers' latency better than fewer blocks with more registers; a pblock of
// 512 still launches)
__global__ void __launch_bounds__(512, 3) kb_position(BState b) {
  const long long i = btid();
  float bound = -1.f;
  if (i < b.NP) bound = position_one(b, i);
  block_scene_max<1>(b, bound >= 0.f ? (int)b.scene[i] : -1, {Q_MOM_MUSL}, {fmaxf(bound, 0.f)});
}

// GridMomentumMUSL: momentum re-map with the new particle velocities
__global__ void kb_p2g_momentum(BState b) {
  long long n = btid();
  if (n >= b.NN) return;
  const int s = b.node_scene[n];
  if (!scene_live(b, s)) return;
  const Scene& sc = b.scenes[s];
  if (!sc.musl) return;
  const long long NN = b.NN;
  int j[3];
  node_xyz(sc, n - sc.n0, j[0], j[1], j[2]);
  double P0 = 0, P1 = 0, P2 = 0;
  if (sc.shape == 3) {
    // centre nodes -> node (GridMomentumMUSL of SGMP), exact sums of the
    // cells' fixed-point momenta
    const long long NC = b.NC;
    const unsigned long long* ca = b.cacc;
    long long Q[3] = {0, 0, 0};
    for (int cz = j[2] - 1; cz <= j[2]; ++cz) {
      if (cz < 0 || cz >= sc.NCz) continue;
      for (int cy = j[1] - 1; cy <= j[1]; ++cy) {
        if (cy < 0 || cy >= sc.NCy) continue;
        for (int cx = j[0] - 1; cx <= j[0]; ++cx) {
          if (cx < 0 || cx >= sc.NCx) continue;
          const long long c = sc.c0 + (cz * sc.NCy + cy) * sc.NCx + cx;
          for (int a = 0; a < 3; ++a) Q[a] += (long long)ca[(CQ_P + a) * NC + c];
        }
      }
    }
    const double u = q_unit(q_shift(sc, b.sst[s].qmax[Q_MOM_MUSL]));
    P0 = 0.125 * ((double)Q[0] * u);
    P1 = 0.125 * ((double)Q[1] * u);
    P2 = 0.125 * ((double)Q[2] * u);
  } else {
    const double u = q_unit(q_shift(sc, b.sst[s].qmax[Q_MOM_MUSL]));
    const double unit[3] = {u, u, u};
    double o[3];
    if (!take_acc(b, n, 3, unit, o)) return;  // idle node
    P0 = o[0];
    P1 = o[1];
    P2 = o[2];
  }
  b.px[n] = P0;
  b.px[NN + n] = P1;
  b.px[2 * NN + n] = P2;
  if (sc.shape != 3 && b.mg[n] == 0.0 && (P0 != 0.0 || P1 != 0.0 || P2 != 0.0))
    b.mg[n] = -0.0;  // momentum at a massless node (take_acc)
  node_finish(b, sc, n, 1, !sc.usf);
}

// ------------------------------------------------------------ reductions
// calcEnergy + UpdateDT per scene: a block per chunk of kChunk particles of
// one scene (chunks are fixed relative to the scene start, so the sums of a
// scene do not depend on the other scenes of the batch), then a block per
// scene combining its chunks in order.
// the scene totals from its chunks' partial sums (FP64; fixed tree order)
// and, with mode & 2, UpdateDT; every thread of the block calls it
__device__ __forceinline__ void reduce_scene_finish(BState& b, int s, int mode, double (*sh)[256]) {
  const Scene& sc = b.scenes[s];
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (long long r = sc.r0 + threadIdx.x; r < sc.r0 + sc.nr; r += blockDim.x) {
    // (L2 loads: another SM wrote the partials, and this SM's L1 may hold
    // the last step's)
    for (int k = 0; k < 5; ++k) acc[k] += __ldcg(&b.red_part[k * b.NR + r]);
    acc[5] = fmax(acc[5], __ldcg(&b.red_part[5 * b.NR + r]));
  }
  for (int k = 0; k < 6; ++k) sh[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      for (int k = 0; k < 5; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
      sh[5][threadIdx.x] = fmax(sh[5][threadIdx.x], sh[5][threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  SceneState& st = b.sst[s];
  if (mode & 1) {
    st.ke_prev = st.ke;
    st.ke = sh[0][0];
    st.ie = sh[1][0];
    st.mom[0] = sh[2][0];
    st.mom[1] = sh[3][0];
    st.mom[2] = sh[4][0];
  }
  st.max_vp = sh[5][0];
  if (mode & 2) {
    double dt = (double)1e6f;
    for (int m = sc.mat0; m < sc.mat0 + sc.nmat; ++m) {
      const DevMaterial& mt = b.mats[m];
      if (mt.mat_type == 12) continue;
      double E = mt.young, nu = mt.poisson, ro = mt.density;
      double vv = sqrt(E * (1 - nu) / (1 + nu) / (1 - 2 * nu) / ro);
      vv = fmax(vv, mt.D);
      vv = fmax(vv, mt.wavespd);
      vv = vv + sh[5][0];
      dt = fmin(dt, sc.dcell / vv);
    }
    st.dt = dt * sc.dtscale;
    st.fdt = (float)st.dt;
  }
}

// calcEnergy / UpdateDT: one block per chunk of kChunk particles of a live
// scene sums the chunk in FP64 (the energy balance stays in FP64) and writes
// its partial sums; the scene's last chunk block to finish (a per-scene
// counter, reset by that block) forms the scene totals.
__global__ void __launch_bounds__(256) kb_reduce_chunks(BState b, int mode) {
  __shared__ double sh[6][256];
  __shared__ int last;
  const long long r = blockIdx.x;
  const int s = b.rscene[r];
  if (!scene_live(b, s)) return;  // (uniform: every block of the scene returns)
  const Scene& sc = b.scenes[s];
  const long long NP = b.NP;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  const long long p_begin = sc.p0 + (r - sc.r0) * kChunk;
  const long long p_end = min(p_begin + kChunk, sc.p0 + sc.np);
  for (long long i = p_begin + threadIdx.x; i < p_end; i += blockDim.x) {
    const double v0 = b.v[i], v1 = b.v[NP + i], v2 = b.v[2 * NP + i], m = b.mass[i];
    acc[0] += (v0 * v0 + v1 * v1 + v2 * v2) * m * 0.5;
    acc[1] += b.ie[i];
    acc[2] += m * v0;
    acc[3] += m * v1;
    acc[4] += m * v2;
    acc[5] = fmax(acc[5], fmax(fabs(v0), fmax(fabs(v1), fabs(v2))));
  }
  for (int k = 0; k < 6; ++k) sh[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      for (int k = 0; k < 5; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
      sh[5][threadIdx.x] = fmax(sh[5][threadIdx.x], sh[5][threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int k = 0; k < 6; ++k) b.red_part[k * b.NR + r] = sh[k][0];
    __threadfence();
    last = atomicAdd(&b.sst[s].red_done, 1u) == (unsigned)(sc.nr - 1);
  }
  __syncthreads();
  if (!last) return;
  if (threadIdx.x == 0) b.sst[s].red_done = 0u;
  reduce_scene_finish(b, s, mode, sh);
}

__global__ void kb_dr_damping(BState b) {
  long long i = btid();
  if (i >= b.NP) return;
  const int s = b.scene[i];
  const Scene& sc = b.scenes[s];
  if (!sc.drdamp || !scene_live(b, s)) return;
  const SceneState& st = b.sst[s];
  if (!(st.ke - st.ke_prev <= 0.0)) return;
  const long long NP = b.NP;
  b.v[i] = 0;
  b.v[NP + i] = 0;
  b.v[2 * NP + i] = 0;
}

__global__ void kb_dr_finish(BState b) {
  int s = (int)btid();
  if (s >= b.nscene) return;
  if (!b.scenes[s].drdamp || !scene_live(b, s)) return;
  SceneState& st = b.sst[s];
  if (st.ke - st.ke_prev <= 0.0) st.ke = 0;
}

// values of a few particles of one scene (by deck index) for the curve output
struct GatherItem {
  long long p;
  int field, comp;
};

// value of particle field `field` (component c) at storage position i
__device__ __forceinline__ double field_value(const BState& b, int field, long long c, long long i) {
  const long long NP = b.NP;
  double v = 0.0;
  switch (field) {
    case MPM_P_XP: v = b.x[c * NP + i]; break;
    case MPM_P_XX: v = b.x[c * NP + i]; break;  // XX equals Xp between steps
    case MPM_P_VXP: v = b.v[c * NP + i]; break;
    case MPM_P_FXP: v = b.scenes[b.scene[i]].has_fxp ? b.fxp[c * NP + i] : 0.0; break;
    case MPM_P_VOL: v = b.vol[i]; break;
    case MPM_P_SIG_Y: v = b.sig_y[i]; break;
    case MPM_P_SM: v = b.sm[i]; break;
    case MPM_P_SEQV: v = b.seqv[i]; break;
    case MPM_P_SD: v = b.sd[c * NP + i]; break;
    case MPM_P_FP: v = (double)b.fp[c * NP + i] + (double)b.fp[(9 + c) * NP + i]; break;
    case MPM_P_EPEFF: v = b.epeff[i]; break;
    case MPM_P_CELSIUS: v = b.celsius[i]; break;
    case MPM_P_DMG: v = b.dmg[i]; break;
    case MPM_P_LT: v = b.lt[i]; break;
    case MPM_P_IE: v = b.ie[i]; break;
    case MPM_P_MASS: v = b.mass[i]; break;
    case MPM_P_CP: v = b.cp[i]; break;
    case MPM_P_Q: v = b.q[i]; break;
    case MPM_P_FAILURE: v = b.failure[i] ? 1.0 : 0.0; break;
    default: v = 0.0; break;
  }
  return v;
}

__global__ void kb_gather(BState b, int scene, const GatherItem* it, int n, double* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const Scene& sc = b.scenes[scene];
  out[k] = field_value(b, it[k].field, it[k].comp, b.inv[sc.p0 + it[k].p]);
}

// one component of a particle field of a scene in deck order (downloads)
__global__ void kb_unpermute(BState b, int scene, int field, int ncomp, double* dst) {
  const Scene& sc = b.scenes[scene];
  const long long t = btid();
  if (t >= sc.np * ncomp) return;
  const int a = (int)(t / sc.np);
  const long long k = t - (long long)a * sc.np;
  dst[t] = field_value(b, field, a, b.inv[sc.p0 + k]);  // component-major, input order
}

// ----------------------------------------------------- stress smoothing
// SmoothStressbyGrid (update_step.f90:1876-2055) for one scene, computed
// from the state after its last step when Spre is read (it feeds only the
// output): -SM * VOL and VOL mapped to the grid, Gpre = their ratio on the
// mapped nodes, Spre interpolated back. Shapes as in the reference: GIMP and
// B-spline at the current position against the step's cell, linear ones at
// the step's offsets, SGMP ones at the step's XXN through the centre nodes
// (nodes above the cut-off mass on the way back). Contributions are FP32,
// quantised per particle and node and summed exactly (64-bit fixed point,
// scales from the scene's largest |SM * VOL| and VOL), so Spre does not
// depend on the other scenes of the batch.

// bounds: bnd[0] = max |SM * VOL|, bnd[1] = max VOL (float bits)
__global__ void kb_smooth_bound(BState b, int scene, unsigned* bnd) {
  const Scene& sc = b.scenes[scene];
  const long long k = btid();
  if (k >= sc.np) return;
  const long long i = sc.p0 + k;
  atomicMax(&bnd[0], __float_as_uint(fabsf(b.sm[i] * b.vol[i]) * 1.0001f));
  atomicMax(&bnd[1], __float_as_uint(fabsf(b.vol[i]) * 1.0001f));
}

// particles -> nodes (SGMP: centre nodes); acc = [2][nodes or cells of the scene]
__global__ void kb_smooth_p2g(BState b, int scene, const unsigned* bnd, unsigned long long* acc) {
  const Scene& sc = b.scenes[scene];
  const long long k = btid();
  if (k >= sc.np) return;
  const long long i = sc.p0 + k, NP = b.NP;
  const float sp = q_scale(q_shift(sc, bnd[0])), sv = q_scale(q_shift(sc, bnd[1]));
  const float pv = -b.sm[i] * b.vol[i], v = b.vol[i];
  if (sc.shape == 3) {
    const int d = b.dual[i];
    if (d < 0) return;
    const int dz = div_by(d, sc.mCNCxy), rem = d - dz * sc.CNCxy, dy = div_by(rem, sc.mCNCx), dx = rem - dy * sc.CNCx;
    const long long nc = sc.nc;
    for (int c = 0; c < 8; ++c) {
      const long long cid = sg_corner_cell(sc, dx, dy, dz, c);
      if (cid < 0) continue;
      float w = 0.125f;
      for (int a = 0; a < 3; ++a) w *= kCorner[c][a] ? 1.f + b.xxn[a * NP + i] : 1.f - b.xxn[a * NP + i];
      const long long qp = quant(w * pv, sp), qv = quant(w * v, sv);
      if (qp) atomicAdd(&acc[cid], (unsigned long long)qp);
      if (qv) atomicAdd(&acc[nc + cid], (unsigned long long)qv);
    }
    return;
  }
  const int cl = b.cell[i];
  if (cl < 0) return;
  int c[3];
  c[2] = div_by(cl, sc.mNCxy);
  c[1] = div_by(cl - c[2] * sc.NCxy, sc.mNCx);
  c[0] = cl - c[2] * sc.NCxy - c[1] * sc.NCx;
  float off[3];
  for (int a = 0; a < 3; ++a)
    off[a] = sc.shape == 0 ? b.off[a * NP + i] : (float)((b.x[a * NP + i] - sc.span0[a]) * sc.idcell - (double)c[a]);
  const int tlo = sc.shape == 0 ? 0 : -1, thi = sc.shape == 1 ? 2 : 1;
  float w1[3][4];
  for (int a = 0; a < 3; ++a)
    for (int t = tlo; t <= thi; ++t) {
      float w, dd;
      if (sc.shape == 0) lin1(t, off[a], w, dd);
      else if (sc.shape == 2) bsp1(t, off[a], w, dd);
      else gimp1((float)(-t) + off[a], w, dd);
      w1[a][t + 1] = w;
    }
  for (int tz = tlo; tz <= thi; ++tz)
    for (int ty = tlo; ty <= thi; ++ty)
      for (int tx = tlo; tx <= thi; ++tx) {
        const float w = w1[0][tx + 1] * w1[1][ty + 1] * w1[2][tz + 1];
        const int jx = c[0] + tx, jy = c[1] + ty, jz = c[2] + tz;
        if (w == 0.f || jx < 0 || jx >= sc.NGx || jy < 0 || jy >= sc.NGy || jz < 0 || jz >= sc.NGz) continue;
        const long long n = ((long long)jz * sc.NGy + jy) * sc.NGx + jx;
        const long long qp = quant(w * pv, sp), qv = quant(w * v, sv);
        if (qp) atomicAdd(&acc[n], (unsigned long long)qp);
        if (qv) atomicAdd(&acc[sc.nn + n], (unsigned long long)qv);
      }
}

// Gpre per node of the scene: the ratio of the sums where volume arrived
// (SGMP: of 1/8 of every adjacent cell's sums; every node counts as mapped,
// 0/0 where none arrived)
__global__ void kb_smooth_node(BState b, int scene, const unsigned* bnd, const unsigned long long* acc, double* gpre) {
  const Scene& sc = b.scenes[scene];
  const long long ln = btid();
  if (ln >= sc.nn) return;
  const double up = q_unit(q_shift(sc, bnd[0])), uv = q_unit(q_shift(sc, bnd[1]));
  if (sc.shape == 3) {
    int j[3];
    node_xyz(sc, ln, j[0], j[1], j[2]);
    long long qp = 0, qv = 0;
    for (int cz = j[2] - 1; cz <= j[2]; ++cz) {
      if (cz < 0 || cz >= sc.NCz) continue;
      for (int cy = j[1] - 1; cy <= j[1]; ++cy) {
        if (cy < 0 || cy >= sc.NCy) continue;
        for (int cx = j[0] - 1; cx <= j[0]; ++cx) {
          if (cx < 0 || cx >= sc.NCx) continue;
          const long long c = ((long long)cz * sc.NCy + cy) * sc.NCx + cx;
          qp += (long long)acc[c];
          qv += (long long)acc[sc.nc + c];
        }
      }
    }
    gpre[ln] = (0.125 * ((double)qp * up)) / (0.125 * ((double)qv * uv));
    return;
  }
  const long long qv = (long long)acc[sc.nn + ln];
  gpre[ln] = qv != 0 ? ((double)(long long)acc[ln] * up) / ((double)qv * uv) : 0.0;
}

// SGMP: nodes above the cut-off mass -> centre nodes
__global__ void kb_smooth_back(BState b, int scene, const double* gpre, double* cgpre) {
  const Scene& sc = b.scenes[scene];
  const long long c = btid();
  if (c >= sc.nc) return;
  const int cz = div_by(c, sc.mNCxy), rem = (int)(c - (long long)cz * sc.NCxy), cy = div_by(rem, sc.mNCx), cx = rem - cy * sc.NCx;
  double g = 0.0;
  for (int k = 0; k < 8; ++k) {
    const long long ln = ((long long)(cz + kCorner[k][2]) * sc.NGy + cy + kCorner[k][1]) * sc.NGx + cx + kCorner[k][0];
    if (b.mg[sc.n0 + ln] > sc.cutoff) g = g + 0.125 * gpre[ln];
  }
  cgpre[c] = g;
}

// (centre) nodes -> particles: Spre in the scene's input order
__global__ void kb_smooth_g2p(BState b, int scene, const double* gpre, const double* cgpre, double* spre) {
  const Scene& sc = b.scenes[scene];
  const long long k = btid();
  if (k >= sc.np) return;
  const long long i = sc.p0 + k, NP = b.NP;
  double s = 0.0;
  if (sc.shape == 3) {
    const int d = b.dual[i];
    if (d >= 0) {
      const int dz = div_by(d, sc.mCNCxy), rem = d - dz * sc.CNCxy, dy = div_by(rem, sc.mCNCx), dx = rem - dy * sc.CNCx;
      for (int c = 0; c < 8; ++c) {
        const long long cid = sg_corner_cell(sc, dx, dy, dz, c);
        if (cid < 0) continue;
        float w = 0.125f;
        for (int a = 0; a < 3; ++a) w *= kCorner[c][a] ? 1.f + b.xxn[a * NP + i] : 1.f - b.xxn[a * NP + i];
        s = s + (double)w * cgpre[cid];
      }
    }
  } else if (b.cell[i] >= 0) {
    const int cl = b.cell[i];
    int c[3];
    c[2] = div_by(cl, sc.mNCxy);
    c[1] = div_by(cl - c[2] * sc.NCxy, sc.mNCx);
    c[0] = cl - c[2] * sc.NCxy - c[1] * sc.NCx;
    float off[3];
    for (int a = 0; a < 3; ++a)
      off[a] = sc.shape == 0 ? b.off[a * NP + i] : (float)((b.x[a * NP + i] - sc.span0[a]) * sc.idcell - (double)c[a]);
    const int tlo = sc.shape == 0 ? 0 : -1, thi = sc.shape == 1 ? 2 : 1;
    float w1[3][4];
    for (int a = 0; a < 3; ++a)
      for (int t = tlo; t <= thi; ++t) {
        float w, dd;
        if (sc.shape == 0) lin1(t, off[a], w, dd);
        else if (sc.shape == 2) bsp1(t, off[a], w, dd);
        else gimp1((float)(-t) + off[a], w, dd);
        w1[a][t + 1] = w;
      }
    for (int tz = tlo; tz <= thi; ++tz)
      for (int ty = tlo; ty <= thi; ++ty)
        for (int tx = tlo; tx <= thi; ++tx) {
          const float w = w1[0][tx + 1] * w1[1][ty + 1] * w1[2][tz + 1];
          const int jx = c[0] + tx, jy = c[1] + ty, jz = c[2] + tz;
          if (w == 0.f || jx < 0 || jx >= sc.NGx || jy < 0 || jy >= sc.NGy || jz < 0 || jz >= sc.NGz) continue;
          s = s + (double)w * gpre[((long long)jz * sc.NGy + jy) * sc.NGx + jx];
        }
  }
  spre[b.orig[i]] = s;
}

// SGMP centre-node mass (comp -1) or momentum component of a scene from
// its fixed-point sums (downloads; the momentum of the last transfer, MUSL
// or not)
__global__ void kb_centre_field(BState b, int scene, int comp, double* dst) {
  const Scene& sc = b.scenes[scene];
  const long long k = btid();
  if (k >= sc.nc) return;
  const SceneState& st = b.sst[scene];
  const int q = comp < 0 ? Q_MASS : (sc.musl ? Q_MOM_MUSL : Q_MOM);
  const int ch = comp < 0 ? CQ_M : CQ_P + comp;
  dst[k] = (double)(long long)b.cacc[(long long)ch * b.NC + sc.c0 + k] * q_unit(q_shift(sc, st.qmax[q]));
}

}  // namespace bm
}  // namespace mpm
