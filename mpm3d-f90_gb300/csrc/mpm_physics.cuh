// mpm_physics.cuh -- per-particle device math of the explicit step:
// shape functions (Grid.f90) and the constitutive / EOS update
// (Constitution.f90), templated on the arithmetic form.
//
// FP64 forms reproduce the reference's operation order and REAL(4) roundings
// one expression at a time (the translation units that instantiate them are
// compiled with --fmad=false). The mixed form evaluates the same formulas in
// FP32.
#pragma once

#include <math.h>
#include <stdint.h>

#include "mpm_gpu_internal.cuh"
#include "mpm_math.h"

namespace mpm {

// Arithmetic forms.
struct PStrict {
  using R = double;  // shape functions, velocity gradient, constitutive update
  using B = double;  // stored particle state
  static constexpr int kLibm = 0;  // project libm (bit-identical to the oracle)
  static constexpr bool kExact = true;
};
struct PNative {
  using R = double;
  using B = double;
  static constexpr int kLibm = 1;  // CUDA libm
  static constexpr bool kExact = true;
};
struct PMixed {
  using R = float;
  using B = float;
  static constexpr int kLibm = 2;  // CUDA single-precision libm
  static constexpr bool kExact = false;
};

template <class P>
__device__ __forceinline__ typename P::R m_log(typename P::R x) {
  if constexpr (P::kLibm == 0) return mpm_log(x);
  else if constexpr (P::kLibm == 1) return log(x);
  else return logf(x);
}
template <class P>
__device__ __forceinline__ typename P::R m_exp(typename P::R x) {
  if constexpr (P::kLibm == 0) return mpm_exp(x);
  else if constexpr (P::kLibm == 1) return exp(x);
  else return expf(x);
}
template <class P>
__device__ __forceinline__ typename P::R m_pow(typename P::R x, typename P::R y) {
  if constexpr (P::kLibm == 0) return mpm_pow(x, y);
  else if constexpr (P::kLibm == 1) return pow(x, y);
  else return powf(x, y);
}

// Value of a default-REAL (FP32) literal or variable of the reference, in R.
template <class R>
__device__ __forceinline__ R f32(float v) { return (R)v; }

// ---------------------------------------------------------------- geometry

__device__ __forceinline__ double node_coord(const Geometry& g, int node0, int d) {
  // Grid.f90:300-302: Xg = (i - 1)*DCell + Span(1), node0 = flat id - 1
  int iz = node0 / g.NGxy;
  int rem = node0 - iz * g.NGxy;
  int iy = rem / g.NGx;
  int ix = rem - iy * g.NGx;
  int i = d == 0 ? ix : (d == 1 ? iy : iz);
  return (double)i * g.dcell + g.span0[d];
}

// InWhichCell, Grid.f90:123-155 (1-based id, -1 outside)
__device__ __forceinline__ int in_which_cell(const Geometry& g, const double x[3]) {
  for (int d = 0; d < 3; ++d)
    if (x[d] < g.span0[d] || x[d] > g.span1[d]) return -1;
  int ix = (int)((x[0] - g.span0[0]) / g.dcell) + 1;
  int iy = (int)((x[1] - g.span0[1]) / g.dcell) + 1;
  int iz = (int)((x[2] - g.span0[2]) / g.dcell) + 1;
  long long c = (long long)(iz - 1) * g.NCxy + (long long)(iy - 1) * g.NCx + ix;
  if (c > g.ncell || c <= 0) return -1;
  return (int)c;
}

// CenterInWhichCell, Grid.f90:157-190
__device__ __forceinline__ int center_in_which_cell(const Geometry& g, const double x[3]) {
  const double h2 = g.dcell / 2.0;
  int ix = (int)((x[0] - g.span0[0] - h2) / g.dcell) + 1;
  int iy = (int)((x[1] - g.span0[1] - h2) / g.dcell) + 1;
  int iz = (int)((x[2] - g.span0[2] - h2) / g.dcell) + 1;
  long long c = (long long)(iz - 1) * g.CNCxy + (long long)(iy - 1) * g.CNCx + ix;
  if (c > g.CNC || c <= 0) return -1;
  return (int)c;
}

// Corner order of a hexahedral cell (Grid.f90:117-119, 372-379).
__constant__ const signed char kSN[3][8] = {{-1, 1, 1, -1, -1, 1, 1, -1},
                                            {-1, -1, 1, 1, -1, -1, 1, 1},
                                            {-1, -1, -1, -1, 1, 1, 1, 1}};
__constant__ const unsigned char kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                                  {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

// cpGIMP influence-node layout: for each of the 27 cell-quarter cases
// (case = qz*9 + qy*3 + qx, q = 0: r < 0.25, 1: middle, 2: r > 0.75) the node
// count and, per slot, the node offset from the cell's first corner packed as
// (dx+1) + 4(dy+1) + 16(dz+1). Slot order is that of FindInflNode
// (Grid.f90:602-849); the same table drives every particle pass.
struct GimpCase {
  unsigned char n;
  unsigned char off[27];
};
__constant__ const GimpCase kGimp[27] = {
    {27, {21, 22, 26, 25, 37, 38, 42, 41, 5, 6, 10, 9, 1, 2, 17, 18, 33, 34, 20, 24, 36, 40, 4, 8, 0, 16, 32}},
    {18, {21, 22, 26, 25, 37, 38, 42, 41, 5, 6, 10, 9, 1, 2, 17, 18, 33, 34}},
    {27, {21, 22, 26, 25, 37, 38, 42, 41, 5, 6, 10, 9, 1, 2, 17, 18, 33, 34, 23, 27, 39, 43, 7, 11, 3, 19, 35}},
    {18, {21, 22, 26, 25, 37, 38, 42, 41, 5, 6, 10, 9, 4, 8, 20, 24, 36, 40}},
    {12, {21, 22, 26, 25, 37, 38, 42, 41, 5, 6, 10, 9}},
    {18, {21, 22, 26, 25, 37, 38, 42, 41, 5, 6, 10, 9, 7, 11, 23, 27, 39, 43}},
    {27, {21, 22, 26, 25, 37, 38, 42, 41, 5, 6, 10, 9, 14, 13, 30, 29, 46, 45, 20, 24, 36, 40, 4, 8, 12, 28, 44}},
    {18, {21, 22, 26, 25, 37, 38, 42, 41, 5, 6, 10, 9, 14, 13, 30, 29, 46, 45}},
    {27, {21, 22, 26, 25, 37, 38, 42, 41, 5, 6, 10, 9, 14, 13, 30, 29, 46, 45, 23, 27, 39, 43, 7, 11, 15, 31, 47}},
    {18, {21, 22, 26, 25, 37, 38, 42, 41, 17, 18, 33, 34, 20, 24, 36, 40, 16, 32}},
    {12, {21, 22, 26, 25, 37, 38, 42, 41, 17, 18, 33, 34}},
    {18, {21, 22, 26, 25, 37, 38, 42, 41, 17, 18, 33, 34, 23, 27, 39, 43, 19, 35}},
    {12, {21, 22, 26, 25, 37, 38, 42, 41, 20, 24, 36, 40}},
    {8, {21, 22, 26, 25, 37, 38, 42, 41}},
    {12, {21, 22, 26, 25, 37, 38, 42, 41, 23, 27, 39, 43}},
    {18, {21, 22, 26, 25, 37, 38, 42, 41, 30, 29, 46, 45, 20, 24, 36, 40, 28, 44}},
    {12, {21, 22, 26, 25, 37, 38, 42, 41, 30, 29, 46, 45}},
    {18, {21, 22, 26, 25, 37, 38, 42, 41, 30, 29, 46, 45, 23, 27, 39, 43, 31, 47}},
    {27, {21, 22, 26, 25, 37, 38, 42, 41, 53, 54, 58, 57, 49, 50, 17, 18, 33, 34, 20, 24, 36, 40, 52, 56, 48, 16, 32}},
    {18, {21, 22, 26, 25, 37, 38, 42, 41, 53, 54, 58, 57, 49, 50, 17, 18, 33, 34}},
    {27, {21, 22, 26, 25, 37, 38, 42, 41, 53, 54, 58, 57, 49, 50, 17, 18, 33, 34, 23, 27, 39, 43, 55, 59, 51, 19, 35}},
    {18, {21, 22, 26, 25, 37, 38, 42, 41, 53, 54, 58, 57, 52, 56, 20, 24, 36, 40}},
    {12, {21, 22, 26, 25, 37, 38, 42, 41, 53, 54, 58, 57}},
    {18, {21, 22, 26, 25, 37, 38, 42, 41, 53, 54, 58, 57, 55, 59, 23, 27, 39, 43}},
    {27, {21, 22, 26, 25, 37, 38, 42, 41, 53, 54, 58, 57, 62, 61, 30, 29, 46, 45, 20, 24, 36, 40, 52, 56, 60, 28, 44}},
    {18, {21, 22, 26, 25, 37, 38, 42, 41, 53, 54, 58, 57, 62, 61, 30, 29, 46, 45}},
    {27, {21, 22, 26, 25, 37, 38, 42, 41, 53, 54, 58, 57, 62, 61, 30, 29, 46, 45, 23, 27, 39, 43, 55, 59, 63, 31, 47}},
};

// Quadratic B-spline: 27 slots in BFindInflNode order (Grid.f90:852-895);
// per slot the 1-D piece used in x, y, z (0 lower node, 1 own, 2 upper),
// which is also the node offset + 1 (NShape_Bspline, Grid.f90:932-1048).
__constant__ const unsigned char kBsp[27][3] = {
    {1, 1, 1}, {2, 1, 1}, {2, 2, 1}, {1, 2, 1}, {1, 1, 2}, {2, 1, 2}, {2, 2, 2}, {1, 2, 2}, {1, 1, 0},
    {2, 1, 0}, {2, 2, 0}, {1, 2, 0}, {1, 0, 0}, {2, 0, 0}, {1, 0, 1}, {2, 0, 1}, {1, 0, 2}, {2, 0, 2},
    {0, 1, 1}, {0, 2, 1}, {0, 1, 2}, {0, 2, 2}, {0, 1, 0}, {0, 2, 0}, {0, 0, 0}, {0, 0, 1}, {0, 0, 2}};

// Flat node id (0-based) of the corner-1 node of a 1-based cell id.
__device__ __forceinline__ int cell_node1(const Geometry& g, int icell) {
  int c = icell - 1;
  int iz = c / g.NCxy;
  int rem = c - iz * g.NCxy;
  int iy = rem / g.NCx;
  int ix = rem - iy * g.NCx;
  return iz * g.NGxy + iy * g.NGx + ix;
}

// ------------------------------------------------------------- materials

// MaterialModel module state for one particle (Constitution.f90:24-74).
template <class R>
struct Mm {
  R vold, vol_, vol0_, dvol, den0_, den_, mu, rv, specen, iener, ieinc;
  R dden;  // den_ - den0_
  R dinc[6], sig[6], sd[6], sold[6], sm, smold, bqf, seqv, epeff_, sig_y_, depeff, ratio;
  R G2, K3, PlaMod, lamda, miu2, young_, poisson_, yield0_, tmprt, cp, DMG, oldDMG, bfac;
  R Fp[3][3];
  R H[3][3];     // Fp - I as stored per particle (the mixed form works from it)
  R Hlo[3][3];   // mixed form: the remainder of Fp - I beyond H (Fp - I = H + Hlo)
  bool has_hlo;  // Hlo is set
  bool dep_set;  // this particle assigned the module variable depeff
};

// ---------------------------------------- compensated FP32 arithmetic
// Error-free transformations for the mixed form where the FP64 reference
// cancels: TwoSum (Knuth) gives s + e = a + b exactly; TwoProduct (one fused
// multiply-add) gives p + e = a * b exactly. An FFAcc sums terms as an
// unevaluated pair hi + lo.
struct F2 {
  float hi, lo;
};
__device__ __forceinline__ F2 two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ F2 two_prod(float a, float b) {
  const float p = a * b;
  return {p, fmaf(a, b, -p)};
}
struct FFAcc {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x) {
    const F2 t = two_sum(hi, x);
    hi = t.hi;
    lo += t.lo;
  }
  __device__ __forceinline__ void add_prod(float a, float b) {
    const F2 p = two_prod(a, b);
    add(p.hi);
    lo += p.lo;
  }
  __device__ __forceinline__ float value() const { return hi + lo; }
};

// B - I (xx, yy, zz, xy, yz, xz) and J - 1 of F = I + H for H carried as
// Hh + Hl: B - I = H + H^T + H H^T and J - 1 = tr H + I2(H) + det H, the
// leading terms summed in compensated FP32 and the first-order terms of Hl
// added to the remainder. A rotation makes H + H^T cancel against H H^T and
// tr H against I2(H): a body turned by 0.3 rad at strains of 1e-4 would lose
// three more digits there than FP32 holds.
__device__ __forceinline__ void bmi_jm1_compensated(const float (*Hh)[3], const float (*Hl)[3], float B[6],
                                                    float& jm1) {
  const int bi[6] = {0, 1, 2, 0, 1, 0}, bj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int e = 0; e < 6; ++e) {
    const int i = bi[e], j = bj[e];
    FFAcc a;
    a.add(Hh[i][j]);
    a.add(Hh[j][i]);
    a.lo += Hl[i][j] + Hl[j][i];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      a.add_prod(Hh[i][k], Hh[j][k]);
      a.lo += Hh[i][k] * Hl[j][k] + Hl[i][k] * Hh[j][k];
    }
    B[e] = a.value();
  }
  FFAcc t;
  t.add(Hh[0][0]);
  t.add(Hh[1][1]);
  t.add(Hh[2][2]);
  t.lo += Hl[0][0] + Hl[1][1] + Hl[2][2];
  const int pi[3] = {0, 1, 0}, pj[3] = {1, 2, 2};
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    const int i = pi[e], j = pj[e];
    t.add_prod(Hh[i][i], Hh[j][j]);
    t.add_prod(-Hh[i][j], Hh[j][i]);
    t.lo += Hh[i][i] * Hl[j][j] + Hl[i][i] * Hh[j][j] - Hh[i][j] * Hl[j][i] - Hl[i][j] * Hh[j][i];
  }
  // det H and its first-order change cof(H) : Hl
  const float c00 = Hh[1][1] * Hh[2][2] - Hh[1][2] * Hh[2][1], c01 = Hh[1][2] * Hh[2][0] - Hh[1][0] * Hh[2][2],
              c02 = Hh[1][0] * Hh[2][1] - Hh[1][1] * Hh[2][0];
  const float c10 = Hh[0][2] * Hh[2][1] - Hh[0][1] * Hh[2][2], c11 = Hh[0][0] * Hh[2][2] - Hh[0][2] * Hh[2][0],
              c12 = Hh[0][1] * Hh[2][0] - Hh[0][0] * Hh[2][1];
  const float c20 = Hh[0][1] * Hh[1][2] - Hh[0][2] * Hh[1][1], c21 = Hh[0][2] * Hh[1][0] - Hh[0][0] * Hh[1][2],
              c22 = Hh[0][0] * Hh[1][1] - Hh[0][1] * Hh[1][0];
  t.add(Hh[0][0] * c00 + Hh[0][1] * c01 + Hh[0][2] * c02);
  t.lo += c00 * Hl[0][0] + c01 * Hl[0][1] + c02 * Hl[0][2] + c10 * Hl[1][0] + c11 * Hl[1][1] + c12 * Hl[1][2] +
          c20 * Hl[2][0] + c21 * Hl[2][1] + c22 * Hl[2][2];
  jm1 = t.value();
}

template <class P>
__device__ __forceinline__ typename P::R equivalent_stress(const Mm<typename P::R>& m) {
  using R = typename P::R;
  const R* sd = m.sd;
  R J2 = (R)0.5 * (sd[0] * sd[0] + sd[1] * sd[1] + sd[2] * sd[2]) + sd[3] * sd[3] + sd[4] * sd[4] +
         sd[5] * sd[5];
  J2 = J2 * (R)3.0;
  return (R)(float)sqrt(J2);  // default-REAL function result
}

template <class R>
__device__ __forceinline__ void sigrot(Mm<R>& m, const R vort[3]) {
  R* sig = m.sig;
  R q1 = (R)2.0 * sig[5] * vort[2];
  R q2 = (R)2.0 * sig[4] * vort[1];
  R q3 = (R)2.0 * sig[3] * vort[0];
  R rot[6];
  rot[0] = -q1 + q2;
  rot[1] = q1 - q3;
  rot[2] = -q2 + q3;
  rot[3] = vort[0] * (sig[1] - sig[2]) + vort[2] * sig[4] - vort[1] * sig[5];
  rot[4] = vort[1] * (sig[2] - sig[0]) + vort[0] * sig[5] - vort[2] * sig[3];
  rot[5] = vort[2] * (sig[0] - sig[1]) + vort[1] * sig[3] - vort[0] * sig[4];
#pragma unroll
  for (int i = 0; i < 6; ++i) sig[i] = sig[i] + rot[i];
  m.sm = (sig[0] + sig[1] + sig[2]) / (R)3.0;
  m.sd[0] = sig[0] - m.sm;
  m.sd[1] = sig[1] - m.sm;
  m.sd[2] = sig[2] - m.sm;
  m.sd[3] = sig[3];
  m.sd[4] = sig[4];
  m.sd[5] = sig[5];
}

template <class R>
__device__ __forceinline__ void elastic_devi(Mm<R>& m) {
  const R* d = m.dinc;
  R dem = (d[0] + d[1] + d[2]) / (R)3.0;
  R G = (R)0.5 * m.G2;
  m.sd[0] = m.sd[0] + m.G2 * (d[0] - dem);
  m.sd[1] = m.sd[1] + m.G2 * (d[1] - dem);
  m.sd[2] = m.sd[2] + m.G2 * (d[2] - dem);
  m.sd[3] = m.sd[3] + G * d[3];
  m.sd[4] = m.sd[4] + G * d[4];
  m.sd[5] = m.sd[5] + G * d[5];
}

template <class R>
__device__ __forceinline__ void elastic_p(Mm<R>& m) {
  const R* d = m.dinc;
  R dem = (d[0] + d[1] + d[2]) / (R)3.0;
  m.sm = m.sm + m.K3 * dem;
}

template <class R>
__device__ __forceinline__ void bulkq(Mm<R>& m, R DT, R dcell, R bq1, R bq2) {
  const R* d = m.dinc;
  R dd = (d[0] + d[1] + d[2]) / DT;
  if (!(dd < (R)0.0)) dd = (R)0.0;
  m.bqf = m.den_ * dcell * dcell * bq1 * dd * dd - bq2 * m.den_ * dcell * m.cp * dd;
}

template <class R>
__device__ __forceinline__ void lieupd(Mm<R>& m, R DT, R dcell, R bq1, R bq2) {
  const R* d = m.dinc;
  if (m.sm < (R)0) bulkq(m, DT, dcell, bq1, bq2);
  m.ieinc = m.ieinc - (R)2.0 * m.bqf * (d[0] + d[1] + d[2]);
  R vavg = (R)(float)(m.vol_ + m.vold);
  m.iener = m.iener + (R)0.25 * m.ieinc * vavg;
}

template <class R>
__device__ __forceinline__ void hieupd(Mm<R>& m, bool failure) {
  const R* d = m.dinc;
  if (failure) {
    m.ieinc = m.dvol * (m.smold - (R)2.0 * m.bqf);
  } else {
    R vavg = (R)(float)(m.vol_ + m.vold);
    R e = d[0] * (m.sold[0] + m.sd[0]) + d[1] * (m.sold[1] + m.sd[1]) + d[2] * (m.sold[2] + m.sd[2]) +
          d[3] * (m.sold[3] + m.sd[3]) + d[4] * (m.sold[4] + m.sd[4]) + d[5] * (m.sold[5] + m.sd[5]);
    m.ieinc = (R)0.25 * e * vavg + m.dvol * (m.smold - (R)2.0 * m.bqf);
  }
  m.iener = m.iener + m.ieinc;
  m.specen = m.iener / m.vol0_;
}

template <class R>
__device__ __forceinline__ R sig_work(const Mm<R>& m) {
  const R* s = m.sig;
  const R* d = m.dinc;
  return s[0] * d[0] + s[1] * d[1] + s[2] * d[2] + s[3] * d[3] + s[4] * d[4] + s[5] * d[5];
}

template <class R>
__device__ __forceinline__ R add_stress_work(const Mm<R>& m, R acc) {
  const R* s = m.sd;
  const R* d = m.dinc;
  acc = acc + (s[0] + m.sm) * d[0];
  acc = acc + (s[1] + m.sm) * d[1];
  acc = acc + (s[2] + m.sm) * d[2];
  acc = acc + s[3] * d[3];
  acc = acc + s[4] * d[4];
  acc = acc + s[5] * d[5];
  return acc;
}

template <class R>
__device__ __forceinline__ void scale_sd(Mm<R>& m, R r) {
#pragma unroll
  for (int i = 0; i < 6; ++i) m.sd[i] = m.sd[i] * r;
}

template <class R>
__device__ __forceinline__ R det3(const R F[3][3]) {
  return F[0][0] * F[1][1] * F[2][2] - F[0][0] * F[1][2] * F[2][1] - F[1][0] * F[0][1] * F[2][2] +
         F[1][0] * F[0][2] * F[2][1] + F[2][0] * F[0][1] * F[1][2] - F[2][0] * F[0][2] * F[1][1];
}

// plastic return shared by M3DM4 / M3DM5 / M3DM8 (Johnson-Cook family)
template <class P, class Mat>
__device__ __forceinline__ void jc_return(Mm<typename P::R>& m, const Mat& mt, typename P::R DT,
                                          int variant, bool* failure) {
  using R = typename P::R;
  const R e4 = f32<R>(0.0001f);
  const R Bjc = (R)mt.B_jc, njc = (R)mt.n_jc, Cjc = (R)mt.C_jc, mjc = (R)mt.m_jc, epso = (R)mt.epso;
  m.epeff_ = m.epeff_ + e4;
  m.PlaMod = Bjc * njc * m_pow<P>(m.epeff_, njc - (R)1);
  m.epeff_ = m.epeff_ - e4;
  elastic_devi(m);
  m.seqv = equivalent_stress<P>(m);
  if (m.seqv > m.sig_y_) {
    m.depeff = (m.seqv - m.sig_y_) / ((R)1.5 * m.G2 + m.PlaMod);
    m.dep_set = true;
    m.epeff_ = m.epeff_ + m.depeff;
    R tstar = 0;
    if (variant != 5) {
      tstar = (m.tmprt - (R)mt.roomt) / ((R)mt.melt - (R)mt.roomt);
      if (variant == 8) {
        if (tstar > (R)1.0) {
          tstar = (R)1.0;
          *failure = true;
        } else if (tstar < (R)0.0) {
          tstar = (R)0.0;
        }
      }
    }
    R srate = m.depeff / epso / DT;
    if (srate < f32<R>(0.001f)) srate = f32<R>(0.001f);
    if (variant == 5)
      m.sig_y_ = ((R)m.yield0_ + Bjc * m_pow<P>(m.epeff_, njc)) * ((R)1 + Cjc * m_log<P>(srate));
    else
      m.sig_y_ = ((R)m.yield0_ + Bjc * m_pow<P>(m.epeff_, njc)) * ((R)1 + Cjc * m_log<P>(srate)) *
                 ((R)1 - m_pow<P>(tstar, mjc));
    if (m.sig_y_ > m.seqv) {
      m.epeff_ = m.epeff_ - m.depeff;
      m.depeff = (R)0.0;
    } else {
      m.ratio = m.sig_y_ / m.seqv;
      scale_sd(m, m.ratio);
      m.seqv = m.seqv * m.ratio;
    }
  }
}

template <class R>
__device__ __forceinline__ void m3dm7(Mm<R>& m, R DT) {
  const R* d = m.dinc;
#pragma unroll
  for (int i = 0; i < 6; ++i) m.sd[i] = (R)0.0;
  R tri = (R)0.0 * (d[0] / DT + d[1] / DT + d[2] / DT);  // 1/3*(...) with integer 1/3
  m.sd[0] = m.miu2 * (d[0] / DT - tri);
  m.sd[1] = m.miu2 * (d[1] / DT - tri);
  m.sd[2] = m.miu2 * (d[2] / DT - tri);
  m.sd[3] = (R)0.5 * m.miu2 * d[3] / DT;
  m.sd[4] = (R)0.5 * m.miu2 * d[4] / DT;
  m.sd[5] = (R)0.5 * m.miu2 * d[5] / DT;
}

template <class P, class Mat>
__device__ __forceinline__ void m3dm9(Mm<typename P::R>& m, const Mat& mt) {
  using R = typename P::R;
  const R sqrt3f = (R)sqrtf(3.0f);
  const R third_f = (R)(1.0f / 3.0f);
  const R twoninth_f = (R)(2.0f / 9.0f);
  const R sqrt2f = (R)sqrtf(2.0f);
  R Gmod = m.young_ / ((R)2 * ((R)1 + m.poisson_));
  R Kmod = m.young_ / ((R)3 * ((R)1 - (R)2 * m.poisson_));
  R qfai = (R)mt.q_fai, kfai = (R)mt.k_fai, qpsi = (R)mt.q_psi, tenf;
  m.ieinc = sig_work(m);
  if (qfai == (R)0.0) {
    tenf = (R)0.0;
  } else {
    R tenf_max = kfai / qfai;
    tenf = (R)mt.ten_f < tenf_max ? (R)mt.ten_f : tenf_max;
  }
  elastic_devi(m);
  elastic_p(m);
  const R* sd = m.sd;
  R J2 = (R)0.5 * (sd[0] * sd[0] + sd[1] * sd[1] + sd[2] * sd[2]) + sd[3] * sd[3] + sd[4] * sd[4] +
         sd[5] * sd[5];
  R Tau = sqrt(J2);
  m.seqv = Tau * sqrt3f;
  R dpFi = Tau + qfai * m.sm - kfai;
  R dpsig = m.sm - tenf;
  bool shear = false;
  if (dpsig < (R)0.0) {
    shear = dpFi > (R)0.0;
  } else {
    R alphap = sqrt((R)1 + qfai * qfai) - qfai;
    R Taup = kfai - qfai * tenf;
    R dp_hfai = Tau - Taup - alphap * dpsig;
    if (dp_hfai > (R)0.0) {
      shear = true;
    } else {
      R dlamd = (m.sm - tenf) / Kmod;
      m.sm = tenf;
      m.depeff = dlamd * third_f * sqrt2f;
      m.dep_set = true;
      m.epeff_ = m.epeff_ + m.depeff;
    }
  }
  if (shear) {
    R dlamd = dpFi / (Gmod + Kmod * qfai * qpsi);
    m.sm = m.sm - Kmod * qpsi * dlamd;
    R newTau = kfai - qfai * m.sm;
    m.ratio = newTau / Tau;
    scale_sd(m, m.ratio);
    m.seqv = m.seqv * m.ratio;
    m.depeff = dlamd * sqrt(third_f + twoninth_f * (qpsi * qpsi));
    m.dep_set = true;
    m.epeff_ = m.epeff_ + m.depeff;
  }
  m.ieinc = add_stress_work(m, m.ieinc);
}

template <class P>
__device__ __forceinline__ void m3dm10(Mm<typename P::R>& m) {
  using R = typename P::R;
  const R (*F)[3] = m.Fp;
  R G = (R)0.5 * m.G2;
  R B[6];
  R iJ, lj;
  if constexpr (P::kExact) {
    R J = det3(m.Fp);
    B[0] = F[0][0] * F[0][0] + F[0][1] * F[0][1] + F[0][2] * F[0][2] - (R)1.0;
    B[1] = F[1][0] * F[1][0] + F[1][1] * F[1][1] + F[1][2] * F[1][2] - (R)1.0;
    B[2] = F[2][0] * F[2][0] + F[2][1] * F[2][1] + F[2][2] * F[2][2] - (R)1.0;
    B[3] = F[0][0] * F[1][0] + F[0][1] * F[1][1] + F[0][2] * F[1][2];
    B[4] = F[1][0] * F[2][0] + F[1][1] * F[2][1] + F[1][2] * F[2][2];
    B[5] = F[0][0] * F[2][0] + F[0][1] * F[2][1] + F[0][2] * F[2][2];
    iJ = (R)1.0 / J;
    lj = m_log<P>(J);
  } else {
    // the same quantities from H = F - I without cancellation, which FP32
    // needs for nearly incompressible materials (J - 1 and B - I ~ 1e-6):
    // B - I = H + H^T + H H^T;  J - 1 = tr H + I2(H) + det H;  ln J = log1p(J - 1)
    const R (*H)[3] = m.H;
    auto hh = [&](int i, int j) { return H[i][0] * H[j][0] + H[i][1] * H[j][1] + H[i][2] * H[j][2]; };
    if (m.has_hlo) {  // H carried as H + Hlo (the batched engine's UpdateVbyFp state)
      R jm1;
      bmi_jm1_compensated(m.H, m.Hlo, B, jm1);
      iJ = (R)1.0 / ((R)1.0 + jm1);
      lj = log1pf(jm1);
    } else {
    B[0] = (R)2 * H[0][0] + hh(0, 0);
    B[1] = (R)2 * H[1][1] + hh(1, 1);
    B[2] = (R)2 * H[2][2] + hh(2, 2);
    B[3] = H[0][1] + H[1][0] + hh(0, 1);
    B[4] = H[1][2] + H[2][1] + hh(1, 2);
    B[5] = H[0][2] + H[2][0] + hh(0, 2);
    R i2 = H[0][0] * H[1][1] + H[1][1] * H[2][2] + H[0][0] * H[2][2] - H[0][1] * H[1][0] - H[1][2] * H[2][1] -
           H[0][2] * H[2][0];
    R jm1 = (H[0][0] + H[1][1] + H[2][2]) + i2 + det3(H);
    iJ = (R)1.0 / ((R)1.0 + jm1);
    lj = log1pf(jm1);
    }
  }
  m.ieinc = sig_work(m);
  R* sig = m.sig;
  sig[0] = iJ * (G * B[0] + m.lamda * lj * (R)1.0);
  sig[1] = iJ * (G * B[1] + m.lamda * lj * (R)1.0);
  sig[2] = iJ * (G * B[2] + m.lamda * lj * (R)1.0);
  sig[3] = iJ * G * B[4];
  sig[4] = iJ * G * B[5];
  sig[5] = iJ * G * B[3];
  m.sm = (sig[0] + sig[1] + sig[2]) / (R)3.0;
  m.sd[0] = sig[0] - m.sm;
  m.sd[1] = sig[1] - m.sm;
  m.sd[2] = sig[2] - m.sm;
  m.sd[3] = sig[3];
  m.sd[4] = sig[4];
  m.sd[5] = sig[5];
  m.seqv = equivalent_stress<P>(m);
  m.ieinc = add_stress_work(m, m.ieinc);
}

// seleos + eos1..4 (Constitution.f90:1333-1541). Returns false for a material
// without an EOS.
template <class P, class Mat>
__device__ __forceinline__ bool seleos(Mm<typename P::R>& m, const Mat& mt, bool failure,
                                       typename P::R DT, typename P::R dcell, typename P::R bq1,
                                       typename P::R bq2) {
  using R = typename P::R;
  switch (mt.eos_type) {
    case 1: {
      // A, B, pnew and the coefficients are default REALs
      float c0 = (float)mt.cEos[0], c1 = (float)mt.cEos[1], c2 = (float)mt.cEos[2], c3 = (float)mt.cEos[3];
      float c4 = (float)mt.cEos[4], c5 = (float)mt.cEos[5], c6 = (float)mt.cEos[6];
      R mu = m.mu;
      float A = (float)((R)c0 + mu * ((R)c1 + mu * ((R)c2 + mu * (R)c3)));
      float B = (float)((R)c4 + mu * ((R)c5 + mu * (R)c6));
      hieupd(m, failure);
      float pnew = (float)(((R)A + (R)B * m.specen) / ((R)1 + (R)B * m.dvol / m.vol0_));
      if (failure && pnew < 0.0f) pnew = 0.0f;
      m.ieinc = m.ieinc - m.dvol * (R)pnew;
      m.iener = m.iener - m.dvol * (R)pnew;
      m.sm = -(R)pnew;
      return true;
    }
    case 2: {
      float c1 = (float)mt.cEos[0], c2 = (float)mt.cEos[1], c3 = (float)mt.cEos[2], c4 = (float)mt.cEos[3];
      float c5 = (float)mt.cEos[4];
      R mu = m.mu;
      float A, B;
      if (mu > (R)0) {
        R t = ((R)c1 * mu + (R)c2 * (mu * mu) + (R)c3 * (mu * mu * mu)) *
              ((R)1 - (R)c4 * mu * (R)0.5 / m.den_);
        A = (float)t;
        B = c5;
      } else {
        A = (float)((R)c1 * mu);
        B = 0.0f;
      }
      if (m.sm < (R)0) bulkq(m, DT, dcell, bq1, bq2);
      hieupd(m, failure);
      float pnew = (float)(((R)A + (R)B * m.specen) / ((R)1 + (R)B * m.dvol / m.vol0_));
      if (failure && pnew < 0.0f) pnew = 0.0f;
      m.ieinc = m.ieinc - m.dvol * (R)pnew;
      m.iener = m.iener - m.dvol * (R)pnew;
      m.sm = -(R)pnew;
      return true;
    }
    case 3: {
      R c1 = (R)mt.cEos[0], c2 = (R)mt.cEos[1], r1 = (R)mt.cEos[2], r2 = (R)mt.cEos[3], w1 = (R)mt.cEos[4];
      R r1v = r1 * m.rv;
      R r2v = r2 * m.rv;
      R wr1v = c1 * w1 / r1v;
      R wr2v = c2 * w1 / r2v;
      R wdr1v = c1 - wr1v;
      R wdr2v = c2 - wr2v;
      R er1v = m_exp<P>(-r1v);
      R er2v = m_exp<P>(-r2v);
      R A = wdr1v * er1v + wdr2v * er2v + m.bqf;
      R B = w1 / m.rv;
      hieupd(m, failure);
      A = A * m.bfac;
      B = B * m.bfac;
      R pnew = (A + B * m.specen) / ((R)1 + B * m.dvol / m.vol0_);
      if (failure && pnew < (R)0) pnew = (R)0.0;
      m.iener = m.iener - m.dvol * pnew;
      m.sm = -pnew;
      return true;
    }
    case 4: {
      R c0 = (R)mt.cEos[0];
      if (m.sm < (R)0) bulkq(m, DT, dcell, bq1, bq2);
      hieupd(m, failure);
      R pnew = c0 * c0 * m.dden;
      if (failure && pnew < (R)0) pnew = (R)0.0;
      m.iener = m.iener - m.dvol * pnew;
      m.sm = -pnew;
      return true;
    }
    default:
      return false;
  }
}

// Tail of the Johnson-Cook-with-failure branch (Constitution.f90:285-314) that
// reads the module variable depeff; D is that variable's value when this
// particle reaches it (its own increment, or the one left by the particle
// before it). Returns the new failure flag.
template <class R>
struct JcTail {
  R vold, ieinc, dvol, smold, vol_;
};

}  // namespace mpm
