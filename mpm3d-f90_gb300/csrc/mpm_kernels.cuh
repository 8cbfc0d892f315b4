// mpm_kernels.cuh -- kernels of the explicit MPM step, templated on the
// arithmetic form (mpm_physics.cuh). Included by one translation unit per
// form; mpm_gpu.cu sequences them (MPM3D.f90:69-118).
//
// Determinism: no kernel accumulates floating-point values with atomics.
//   * particle -> node transfers run one thread per node over that node's
//     slice of the node-sorted pair list, which holds the node's
//     (particle, slot) contributions in the reference order (particle index,
//     then slot), so every node sum is the reference's sequential sum;
//   * node -> particle transfers run one thread per particle over its slots
//     in the reference slot order;
//   * reductions use a fixed block tree and a fixed final order.
#pragma once

#include "mpm_physics.cuh"

namespace mpm {

template <class P>
using St = DevState<typename P::B, typename P::R>;

__device__ __forceinline__ long long gtid() { return (long long)blockIdx.x * blockDim.x + threadIdx.x; }

// ------------------------------------------------------------------ begin
// MPM3D.f90:72-74
static __global__ void k_begin_step(DevScalars* sc) {
  sc->istep = sc->istep + 1;
  sc->time = sc->time + sc->dt;
  sc->ie = 0.0;
  sc->active_nodes = 0;
}

// cpGIMP 1-D weight and its derivative in units of the cell (NShape_GIMP,
// Grid.f90:577-591): particle half-width h/4.
template <class R>
__device__ __forceinline__ void gimp_1d(R rr, R& sh, R& dn) {
  R a = rr < (R)0 ? -rr : rr;
  R sg = copysign((R)1.0, rr);
  if (a < (R)0.25) {
    sh = ((R)7 - (R)16 * a * a) * (R)0.125;
    dn = -((R)4 * rr);
  } else if (a < (R)0.75) {
    sh = (R)1 - a;
    dn = -sg;
  } else if (a < (R)1.25) {
    R t = ((R)5 - (R)4 * a) * (R)0.25;
    sh = t * t;
    dn = (R)2 * rr - sg * (R)2.5;
  } else {
    sh = (R)0.0;
    dn = (R)0.0;
  }
}

// Influence slots of particle p (node or, for SGMP, centre-node index per
// slot, -1 when invalid) and their shape functions, written to the shape
// cache; returns the number of slots used. x = the position the GIMP and
// B-spline weights are taken at, icell / xn = the particle's cell and its
// natural coordinates (linear), cc / xxn = its dual cell and coordinates
// (SGMP). ParticleInitial passes the state at the start of the step;
// SmoothStressbyGrid passes the current position with the step's cells.
template <class P>
__device__ __forceinline__ int slot_shapes(St<P>& s, const Geometry& g, long long p, const double x[3], int icell,
                                           const double xn[3], int cc, const double xxn[3], int slot_node[27]) {
  using R = typename P::R;
  const long long np = g.np;
  int nvalid = 0;
  if (g.shape == 3) {
    if (cc > 0) {
      int c = cc - 1;
      int cz = c / g.CNCxy, rem = c - cz * g.CNCxy, cy = rem / g.CNCx, cx = rem - cy * g.CNCx;
      int c1 = cz * g.NCxy + cy * g.NCx + cx;  // CenterCellNode(:,1), 0-based cell
      for (int k = 0; k < 8; ++k) {
        int cid = c1 + kCorner[k][0] + kCorner[k][1] * g.NCx + kCorner[k][2] * g.NCxy;
        bool ok = cid >= 0 && cid < g.ncell;
        slot_node[k] = ok ? cid : -1;
        R sx = (R)kSN[0][k] * (R)xxn[0] + (R)1.0;
        R sy = (R)kSN[1][k] * (R)xxn[1] + (R)1.0;
        R sz = (R)kSN[2][k] * (R)xxn[2] + (R)1.0;
        s.shp[k * np + p] = sx * sy * sz * (R)0.125;
      }
      nvalid = 8;
    }
  } else if (icell > 0) {
    const int n1 = cell_node1(g, icell);
    if (g.shape == 0) {  // linear hexahedron, NShape
      for (int k = 0; k < 8; ++k) {
        slot_node[k] = n1 + kCorner[k][0] + kCorner[k][1] * g.NGx + kCorner[k][2] * g.NGxy;
        R sx = (R)kSN[0][k] * (R)xn[0] + (R)1.0;
        R sy = (R)kSN[1][k] * (R)xn[1] + (R)1.0;
        R sz = (R)kSN[2][k] * (R)xn[2] + (R)1.0;
        const R j4 = (R)g.iJacobi4;
        s.shp[k * np + p] = sx * sy * sz * (R)0.125;
        s.dndx[k * np + p] = (R)kSN[0][k] * sy * sz * j4;
        s.dndy[k * np + p] = (R)kSN[1][k] * sx * sz * j4;
        s.dndz[k * np + p] = (R)kSN[2][k] * sx * sy * j4;
      }
      nvalid = 8;
    } else if (g.shape == 1) {  // cpGIMP
      int i1[3];
      {
        int iz = n1 / g.NGxy, rem = n1 - iz * g.NGxy, iy = rem / g.NGx;
        i1[0] = rem - iy * g.NGx;
        i1[1] = iy;
        i1[2] = iz;
      }
      double rel[3];
      for (int d = 0; d < 3; ++d) rel[d] = (x[d] - node_coord(g, n1, d)) * g.iDCell;
      int q[3];
      for (int d = 0; d < 3; ++d) q[d] = rel[d] < 0.25 ? 0 : (rel[d] > 0.75 ? 2 : 1);
      const GimpCase& gc = kGimp[q[2] * 9 + q[1] * 3 + q[0]];
      nvalid = gc.n;
      const R idc = (R)g.iDCell;
      // 1-D shape values for the four node offsets -1..2 of each direction
      // (NShape_GIMP, Grid.f90:577-591): every slot whose node is not a
      // wrapped flat index uses these, so each r is computed once
      R sh1[3][4], dn1[3][4];
      for (int d = 0; d < 3; ++d)
        for (int o = 0; o < 4; ++o) {
          R rr;
          if constexpr (P::kExact)
            rr = (x[d] - ((double)(i1[d] + o - 1) * g.dcell + g.span0[d])) * g.iDCell;
          else
            rr = (R)rel[d] - (R)(o - 1);
          gimp_1d<R>(rr, sh1[d][o], dn1[d][o]);
        }
      const int NGd[3] = {g.NGx, g.NGy, g.NGz};
      for (int k = 0; k < gc.n; ++k) {
        int off = gc.off[k];
        int od[3] = {(off & 3), ((off >> 2) & 3), (off >> 4)};  // offset + 1
        int nd = n1 + (od[0] - 1) + (od[1] - 1) * g.NGx + (od[2] - 1) * g.NGxy;  // flat arithmetic
        bool ok = nd >= 0 && nd < g.nn;
        slot_node[k] = ok ? nd : -1;
        if (!ok) continue;
        R sh[3], dn[3];
        bool wrapped = false;
        for (int d = 0; d < 2; ++d) {
          int id = i1[d] + od[d] - 1;
          if (id < 0 || id >= NGd[d]) wrapped = true;
        }
        if (!wrapped) {
          for (int d = 0; d < 3; ++d) {
            sh[d] = sh1[d][od[d]];
            dn[d] = dn1[d][od[d]];
          }
        } else {  // the +-1 / +-NGx offset crossed a grid row: the node lies elsewhere
          int iz = nd / g.NGxy, rem = nd - iz * g.NGxy, iy = rem / g.NGx, ix = rem - iy * g.NGx;
          for (int d = 0; d < 3; ++d) {
            R rr;
            if constexpr (P::kExact) {
              rr = (x[d] - node_coord(g, nd, d)) * g.iDCell;
            } else {
              int id = d == 0 ? ix : (d == 1 ? iy : iz);
              rr = (R)rel[d] - (R)(id - i1[d]);
            }
            gimp_1d<R>(rr, sh[d], dn[d]);
          }
        }
        s.shp[k * np + p] = sh[0] * sh[1] * sh[2];
        s.dndx[k * np + p] = dn[0] * sh[1] * sh[2] * idc;
        s.dndy[k * np + p] = sh[0] * dn[1] * sh[2] * idc;
        s.dndz[k * np + p] = sh[0] * sh[1] * dn[2] * idc;
      }
    } else {  // quadratic B-spline
      R sh[3][3], dn[3][3];
      const R c02 = f32<R>(0.2f), c04 = f32<R>(0.4f), idc = (R)g.iDCell;
      for (int d = 0; d < 3; ++d) {
        R r;
        if constexpr (P::kExact)
          r = (x[d] - node_coord(g, n1, d)) * g.iDCell * (double)0.2f + (double)0.4f;
        else
          r = (R)((x[d] - node_coord(g, n1, d)) * g.iDCell) * c02 + c04;
        R a = (R)3 - (R)5 * r;
        R b = (R)5 * r - (R)2;
        sh[0][d] = (R)0.5 * (a * a);
        sh[1][d] = -((R)25 * (r * r)) + (R)25 * r - (R)5.5;
        sh[2][d] = (R)0.5 * (b * b);
        dn[0][d] = ((R)5 * r - (R)3) * (R)5 * c02 * idc;
        dn[1][d] = (-((R)50 * r) + (R)25) * c02 * idc;
        dn[2][d] = ((R)5 * r - (R)2) * (R)5 * c02 * idc;
      }
      for (int k = 0; k < 27; ++k) {
        int a = kBsp[k][0], b = kBsp[k][1], c = kBsp[k][2];
        int nd = n1 + (a - 1) + (b - 1) * g.NGx + (c - 1) * g.NGxy;
        bool ok = nd >= 0 && nd < g.nn;
        slot_node[k] = ok ? nd : -1;
        s.shp[k * np + p] = sh[a][0] * sh[b][1] * sh[c][2];
        s.dndx[k * np + p] = dn[a][0] * sh[b][1] * sh[c][2];
        s.dndy[k * np + p] = sh[a][0] * dn[b][1] * sh[c][2];
        s.dndz[k * np + p] = sh[a][0] * sh[b][1] * dn[c][2];
      }
      nvalid = 27;
    }
  }
  return nvalid;
}

// pair keys of particle p's slots (node-sorted list; pair j = p*K + k keeps
// (particle, slot) order for the stable sort; invalid slots get the
// sentinel key nkeys) and the per-node pair counts; cbase = the first node
// of the particle's grid component
template <class P>
__device__ __forceinline__ void write_pairs(St<P>& s, const Geometry& g, long long p, int nvalid,
                                            const int slot_node[27], int nkeys, int cbase) {
  const long long np = g.np;
  const int K = g.K;
  for (int k = 0; k < K; ++k) {
    int nd = k < nvalid && slot_node[k] >= 0 ? cbase + slot_node[k] : -1;
    s.snode[k * np + p] = nd;
    long long j = p * K + k;
    s.key[j] = nd >= 0 ? (unsigned)nd : (unsigned)nkeys;
    s.val[j] = ((unsigned)p << 5) | (unsigned)k;
    if (nd >= 0) atomicAdd(&s.seg[nd], 1);  // per-node pair count (integer, deterministic)
  }
}

// ----------------------------------------------------------------- locate
// ParticleInitial (update_step.f90:408-453) plus the shape functions of the
// step (NShape / FindInflNode+NShape_GIMP / BFindInflNode+NShape_Bspline /
// SGNShape), cached per (slot, particle), and the pair keys of the
// node-sorted list. Pair j = p*K + k keeps (particle, slot) order for the
// stable sort; invalid slots get the sentinel key nkeys.
template <class P>
__global__ void k_locate(St<P> s, Geometry g, int nkeys) {
  using B = typename P::B;
  const long long p = gtid();
  if (p >= g.np) return;
  const long long np = g.np;
  double x[3] = {s.xp[p], s.xp[np + p], s.xp[2 * np + p]};
  int icell = in_which_cell(g, x);
  s.icell[p] = icell;
  double xn[3] = {0, 0, 0};
  if (icell > 0) {
    int n1 = cell_node1(g, icell);
    for (int d = 0; d < 3; ++d) {
      double cxg = node_coord(g, n1, d) + g.dcell / 2.0;  // Cxg, Grid.f90:380
      xn[d] = (x[d] - cxg) * g.iJacobi;
      s.xn[d * np + p] = (B)xn[d];
    }
  } else {
    atomicOr(&s.sc->status, (unsigned)ST_OUT_OF_GRID);
  }
  int cc = 0;
  double xxn[3] = {0, 0, 0};
  if (g.shape == 3) {  // SGMP: the dual (cell-centre) grid
    cc = center_in_which_cell(g, x);
    s.centericell[p] = cc;
    int ix = (int)((x[0] - g.span0[0]) / g.dcell + 0.5) + 1;
    int iy = (int)((x[1] - g.span0[1]) / g.dcell + 0.5) + 1;
    int iz = (int)((x[2] - g.span0[2]) / g.dcell + 0.5) + 1;
    long long inode = (long long)(iz - 1) * g.NGxy + (long long)(iy - 1) * g.NGx + ix;
    s.inode[p] = (int)inode;
    if (inode >= 1 && inode <= g.nn) {
      int bd = s.bd[inode - 1];
      for (int d = 0; d < 3; ++d) {
        double xg = node_coord(g, (int)inode - 1, d);
        xxn[d] = (x[d] - xg) * g.iJacobi;
        int bt = (bd >> (2 * d)) & 3;
        if (bt != 0) {
          if (xxn[d] > 0) xxn[d] = 1;
          else if (xxn[d] < 0) xxn[d] = -1;
        }
        s.xxn[d * np + p] = (B)xxn[d];
      }
    } else {
      for (int d = 0; d < 3; ++d) xxn[d] = (double)s.xxn[d * np + p];
    }
  }
  int slot_node[27];
  const int nvalid = slot_shapes<P>(s, g, p, x, icell, xn, cc, xxn, slot_node);
  write_pairs<P>(s, g, p, nvalid, slot_node, nkeys, g.shape == 3 ? 0 : s.bodies[s.body[p]].comp * g.nn);
}

__device__ __forceinline__ void decode_pair(unsigned v, long long np, long long* p, long long* idx) {
  long long pp = (long long)(v >> 5);
  int k = (int)(v & 31u);
  *p = pp;
  *idx = (long long)k * np + pp;
}

// ----------------------------------------------------- node-level helpers
__device__ __forceinline__ void node_bc(const uint8_t fix, double* px, double* fx, long long n, long long nn) {
  for (int c = 0; c < 3; ++c)
    if (fix & (1 << c)) {
      px[(long long)c * nn + n] = 0.0;
      fx[(long long)c * nn + n] = 0.0;
    }
}

__device__ __forceinline__ void node_vel(const double* mg, const double* px, double* vg, long long n, long long nn,
                                         double cutoff) {
  double m = mg[n];
  if (m > cutoff)
    for (int c = 0; c < 3; ++c) vg[(long long)c * nn + n] = px[(long long)c * nn + n] / m;
}

// count of nodes with mass (for the algorithmic-bytes figure)
__device__ __forceinline__ void count_active(bool active, unsigned long long* out) {
  unsigned b = __ballot_sync(0xffffffffu, active);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(out, (unsigned long long)__popc(b));
}

// --------------------------------------------------- P2G: mass, momentum
// GridMomentumInitial (update_step.f90:288-406), non-SGMP.
template <class P>
__global__ void k_p2g_mass(St<P> s, Geometry g, int bc, int vel) {
  const long long n = gtid();
  const long long nn = g.nnt;  // every grid component
  bool act = false;
  if (n < nn) {
    const long long np = g.np;
    double m = 0.0, px = 0.0, py = 0.0, pz = 0.0;
    const int j0 = n == 0 ? 0 : s.seg[n - 1], j1 = s.seg[n];
    for (int j = j0; j < j1; ++j) {
      long long p, idx;
      decode_pair(s.val_sorted[j], np, &p, &idx);
      double shm = (double)s.shp[idx] * s.mass[p];
      m = m + shm;
      px = px + s.vxp[p] * shm;
      py = py + s.vxp[np + p] * shm;
      pz = pz + s.vxp[2 * np + p] * shm;
    }
    s.mg[n] = m;
    s.px[n] = px;
    s.px[nn + n] = py;
    s.px[2LL * nn + n] = pz;
    act = m > 0.0;
    if (bc) node_bc(s.fix[n % g.nn], s.px, s.fx, n, nn);
    if (vel) node_vel(s.mg, s.px, s.vg, n, nn, g.cutoff);
  }
  count_active(act, &s.sc->active_nodes);
}

// seg holds per-node counts after k_locate; turn them into exclusive ends
// in place by the host-side scan (inclusive), see mpm_gpu.cu.

template <class P>
__global__ void k_node_velocity(St<P> s, Geometry g) {
  const long long n = gtid();
  if (n >= g.nnt) return;
  node_vel(s.mg, s.px, s.vg, n, g.nnt, g.cutoff);
}

template <class P>
__global__ void k_apply_bc(St<P> s, Geometry g) {
  const long long n = gtid();
  if (n >= g.nnt) return;
  node_bc(s.fix[n % g.nn], s.px, s.fx, n, g.nnt);
}

// ---------------------------------------------------------- stress update
// Constitution (Constitution.f90:79-368) for one particle. Returns the
// "depeff assigned" flag through m.dep_set; *deferred is set for the
// Johnson-Cook particles whose tail must wait for the depeff carried from the
// particle processed before them.
template <class P, class Mat>
__device__ __forceinline__ void jc7_tail(Mm<typename P::R>& m, const Mat& mt, bool& failure,
                                         typename P::R D, typename P::R& vol_out) {
  using R = typename P::R;
  const R epf = (R)mt.epf;
  if (m.epeff_ > epf) {
    m.epeff_ = epf + f32<R>(0.0000001f);
    m.DMG = (R)1.0;
    failure = true;
  } else {
    m.DMG = m.oldDMG + D / epf;
    if (m.DMG >= (R)1.0) m.DMG = (R)1.0;
    R r = ((R)1 - m.DMG) / ((R)1 - m.oldDMG);
    scale_sd(m, r);
    R dd = m.DMG - (R)1.0;
    if ((dd < (R)0 ? -dd : dd) < f32<R>(1e-5f)) failure = true;
  }
  if (failure && m.sm < (R)0) {
    m.sm = (R)0.0;
    m.bqf = (R)0.0;
    vol_out = m.vold;
  }
  if (failure) {
    for (int i = 0; i < 6; ++i) m.sd[i] = (R)0.0;
    m.iener = m.iener - m.ieinc + m.dvol * (m.smold + m.sm - (R)2 * m.bqf);
  }
}

// Particle state read and written by one Constitution call
// (Constitution.f90:79-368); sd in storage order xx, yy, zz, xy, yz, xz.
template <class R>
struct PState {
  R vol, epeff, sig_y, seqv, lt, celsius, ie, mass, dmg, cp, sm, q;
  R sd[6];
  R evol;  // mixed form only: volumetric strain V / V0 - 1, carried per particle
  bool failure;
};

// What the caller must do after the call: the Johnson-Cook tail (tail 4 / 7)
// deferred to the depeff carried from the previous particle, the value this
// particle assigned to depeff, and health flags.
template <class R>
struct CResult {
  int tail;
  bool defer, dep_set, eos_ok, negative_volume;
  R depeff, vold, ieinc, dvol, smold, vol_;
};

// Constitution (Constitution.f90:79-368) for one particle: volume update,
// material constants, the material model of the particle's material and the
// write-back of Constitution.f90:351-366. MT != 0 compiles the model of
// material type MT only (the caller guarantees mt.mat_type == MT).
template <class P, int MT = 0, class Mat>
__device__ __forceinline__ void constitution(PState<typename P::R>& ps, const Mat& mt,
                                             const typename P::R de[6], const typename P::R vort[3],
                                             const typename P::R deFp[3][3], const typename P::R Fpn[3][3],
                                             bool uvfp, typename P::R DT, double time, typename P::R dcell,
                                             typename P::R bq1, typename P::R bq2,
                                             CResult<typename P::R>& res,
                                             const typename P::R (*Fpn_lo)[3] = nullptr) {
  using R = typename P::R;
  Mm<R> m;
  m.dep_set = false;
  m.has_hlo = Fpn_lo != nullptr;
  m.depeff = (R)0;
  m.bfac = (R)0;
  for (int i = 0; i < 6; ++i) m.dinc[i] = de[i];
  m.vold = ps.vol;
  R dJ = (R)0;  // mixed form: volume ratio of the step minus one, without cancellation
  if (uvfp) {
    R dF[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        dF[i][j] = deFp[i][j];
        m.Fp[i][j] = Fpn[i][j];
        m.H[i][j] = Fpn[i][j];
        m.Hlo[i][j] = Fpn_lo ? Fpn_lo[i][j] : (R)0;
      }
    for (int i = 0; i < 3; ++i) {
      dF[i][i] = dF[i][i] + (R)1.0;
      m.Fp[i][i] = m.Fp[i][i] + (R)1.0;
    }
    m.vol_ = m.vold * det3(dF);
    if constexpr (!P::kExact) {
      const R(*A)[3] = deFp;  // det(I + A) - 1 = tr A + I2(A) + det A
      dJ = (A[0][0] + A[1][1] + A[2][2]) +
           (A[0][0] * A[1][1] + A[1][1] * A[2][2] + A[0][0] * A[2][2] - A[0][1] * A[1][0] - A[1][2] * A[2][1] -
            A[0][2] * A[2][0]) +
           det3(A);
    }
  } else {
    m.vol_ = m.vold * ((R)1 + de[0] + de[1] + de[2]);
    dJ = de[0] + de[1] + de[2];
    // without UpdateVbyFp the reference's module variable Fp is never set
    // (zero from program start)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        m.Fp[i][j] = (R)0;
        m.H[i][j] = i == j ? (R)-1 : (R)0;
      }
  }
  R vol_store = m.vol_;
  res.negative_volume = m.vol_ < (R)0;
  m.dvol = (R)0.5 * (m.vol_ - m.vold);
  m.epeff_ = ps.epeff;
  m.sig_y_ = ps.sig_y;
  m.seqv = ps.seqv;
  const R ltim = ps.lt;
  m.tmprt = ps.celsius;
  m.iener = ps.ie;
  const R mp_ = ps.mass;
  bool failure = ps.failure;
  const bool was_failed = failure;
  m.miu2 = (R)2 * (R)mt.miu;
  m.young_ = (R)mt.young;
  m.poisson_ = (R)mt.poisson;
  m.yield0_ = (R)mt.yield0;
  const R tangmod_ = (R)mt.tangmod;
  m.den0_ = (R)mt.density;
  m.vol0_ = mp_ / m.den0_;
  m.den_ = mp_ / m.vol_;
  m.mu = m.den_ / m.den0_ - (R)1;
  m.rv = m.vol_ / m.vol0_;
  m.dden = m.den_ - m.den0_;
  if constexpr (!P::kExact) {
    // FP32 volumes cannot resolve V / V0 - 1 of nearly incompressible
    // states (1e-6 and below): carry the volumetric strain e = V / V0 - 1
    // itself and derive the volume, its increment, mu and the density
    // change from it
    const R e0 = ps.evol;
    const R e1 = e0 + ((R)1 + e0) * dJ;
    ps.evol = e1;
    m.vol_ = m.vol0_ * ((R)1 + e1);
    vol_store = m.vol_;
    res.negative_volume = m.vol_ < (R)0;
    m.dvol = (R)0.5 * m.vol0_ * (e1 - e0);
    m.den_ = mp_ / m.vol_;
    m.mu = -e1 / ((R)1 + e1);
    m.rv = (R)1 + e1;
    m.dden = m.den0_ * m.mu;
  }
  m.specen = m.iener / m.vol0_;
  m.DMG = ps.dmg;
  m.oldDMG = m.DMG;
  if constexpr (P::kExact)
    m.young_ = m.young_ * ((R)1.0 - m.DMG + (R)2.220446049250313e-16);
  else
    m.young_ = m.young_ * ((R)1.0 - m.DMG);
  m.G2 = m.young_ / ((R)1 + m.poisson_);
  m.K3 = m.young_ / ((R)1 - (R)2 * m.poisson_);
  m.lamda = (m.young_ * m.poisson_) / (((R)1 + m.poisson_) * ((R)1 - (R)2 * m.poisson_));
  m.PlaMod = m.young_ * tangmod_ / (m.young_ - tangmod_);
  m.cp = ps.cp;
  m.sm = ps.sm;
  m.smold = m.sm;
  // sd(1..6) = SDxx, SDyy, SDzz, SDyz, SDxz, SDxy (Constitution.f90:184-189)
  m.sd[0] = ps.sd[0];
  m.sd[1] = ps.sd[1];
  m.sd[2] = ps.sd[2];
  m.sd[3] = ps.sd[4];
  m.sd[4] = ps.sd[5];
  m.sd[5] = ps.sd[3];
  m.sig[0] = m.sd[0] + m.sm;
  m.sig[1] = m.sd[1] + m.sm;
  m.sig[2] = m.sd[2] + m.sm;
  m.sig[3] = m.sd[3];
  m.sig[4] = m.sd[4];
  m.sig[5] = m.sd[5];
  for (int i = 0; i < 6; ++i) m.sold[i] = m.sd[i];
  m.bqf = (R)0.0;
  bool eos_ok = true;
  bool defer = false;  // Johnson-Cook tail needs the carried depeff
  int tail = 0;        // 4: celsius update only, 7: failure + damage tail
  switch (MT ? MT : mt.mat_type) {
    case 1:
      sigrot(m, vort);
      m.ieinc = sig_work(m);
      elastic_devi(m);
      elastic_p(m);
      m.seqv = equivalent_stress<P>(m);
      m.ieinc = add_stress_work(m, m.ieinc);
      lieupd(m, DT, dcell, bq1, bq2);
      break;
    case 2:
      sigrot(m, vort);
      m.ieinc = sig_work(m);
      elastic_devi(m);
      m.seqv = equivalent_stress<P>(m);
      if (m.seqv > m.yield0_) {
        m.depeff = (m.seqv - m.sig_y_) / ((R)1.5 * m.G2);
        m.dep_set = true;
        m.epeff_ = m.epeff_ + m.depeff;
        m.ratio = m.yield0_ / m.seqv;
        scale_sd(m, m.ratio);
        m.seqv = m.seqv * m.ratio;
      }
      elastic_p(m);
      m.ieinc = add_stress_work(m, m.ieinc);
      lieupd(m, DT, dcell, bq1, bq2);
      break;
    case 3:
      sigrot(m, vort);
      m.ieinc = sig_work(m);
      elastic_devi(m);
      m.seqv = equivalent_stress<P>(m);
      if (m.seqv > m.sig_y_) {
        m.depeff = (m.seqv - m.sig_y_) / ((R)1.5 * m.G2 + m.PlaMod);
        m.dep_set = true;
        m.epeff_ = m.epeff_ + m.depeff;
        m.sig_y_ = m.sig_y_ + m.PlaMod * m.depeff;
        m.ratio = m.sig_y_ / m.seqv;
        scale_sd(m, m.ratio);
        m.seqv = m.seqv * m.ratio;
      }
      elastic_p(m);
      m.ieinc = add_stress_work(m, m.ieinc);
      lieupd(m, DT, dcell, bq1, bq2);
      break;
    case 4: {
      sigrot(m, vort);
      m.ieinc = sig_work(m);
      jc_return<P>(m, mt, DT, 4, &failure);
      elastic_p(m);
      m.ieinc = add_stress_work(m, m.ieinc);
      const R* d = m.dinc;
      if (m.sm < (R)0) bulkq(m, DT, dcell, bq1, bq2);
      m.ieinc = m.ieinc - (R)2.0 * m.bqf * (d[0] + d[1] + d[2]);
      lieupd(m, DT, dcell, bq1, bq2);
      tail = 4;
      defer = !m.dep_set;
      break;
    }
    case 5:
      sigrot(m, vort);
      jc_return<P>(m, mt, DT, 5, &failure);
      eos_ok = seleos<P>(m, mt, failure, DT, dcell, bq1, bq2);
      break;
    case 6:
      sigrot(m, vort);
      if (!was_failed) {
        jc_return<P>(m, mt, DT, 5, &failure);
        eos_ok = seleos<P>(m, mt, failure, DT, dcell, bq1, bq2);
        if (m.epeff_ > (R)mt.epf) {
          m.epeff_ = (R)mt.epf + f32<R>(0.0000001f);
          failure = true;
        }
        if (failure && m.sm < (R)0) {
          m.sm = (R)0.0;
          m.bqf = (R)0.0;
          vol_store = m.vold;
        }
        if (failure) {
          for (int i = 0; i < 6; ++i) m.sd[i] = (R)0.0;
          m.iener = m.iener - m.ieinc + m.dvol * (m.smold + m.sm - (R)2 * m.bqf);
        }
      } else {
        m3dm7(m, DT);
        eos_ok = seleos<P>(m, mt, failure, DT, dcell, bq1, bq2);
      }
      break;
    case 7:
      sigrot(m, vort);
      if (!was_failed) {
        jc_return<P>(m, mt, DT, 8, &failure);
        eos_ok = seleos<P>(m, mt, failure, DT, dcell, bq1, bq2);
        tail = 7;
        defer = !m.dep_set;
      } else {
        m3dm7(m, DT);
        eos_ok = seleos<P>(m, mt, failure, DT, dcell, bq1, bq2);
      }
      break;
    case 8:
      m.bfac = time > (double)ltim ? (R)1.0 : (R)0.0;  // M3DM6
      eos_ok = seleos<P>(m, mt, failure, DT, dcell, bq1, bq2);
      break;
    case 9:
      m3dm7(m, DT);
      eos_ok = seleos<P>(m, mt, failure, DT, dcell, bq1, bq2);
      break;
    case 10:
      sigrot(m, vort);
      m3dm9<P>(m, mt);
      lieupd(m, DT, dcell, bq1, bq2);
      break;
    case 11:
      m3dm10<P>(m);
      lieupd(m, DT, dcell, bq1, bq2);
      break;
    default:
      eos_ok = false;
  }
  res.eos_ok = eos_ok;
  if (tail != 0 && !defer) {
    // this particle assigned depeff itself: finish now with its own value
    if (tail == 7) jc7_tail<P>(m, mt, failure, m.depeff, vol_store);
    R den_ = m.den_;
    ps.celsius = ps.celsius + m.seqv * m.depeff / den_ / (R)mt.specheat;
  }
  res.tail = tail;
  res.defer = defer;
  res.dep_set = m.dep_set;
  res.depeff = m.depeff;
  res.vold = m.vold;
  res.ieinc = m.ieinc;
  res.dvol = m.dvol;
  res.smold = m.smold;
  res.vol_ = m.vol_;
  ps.vol = vol_store;
  ps.sm = m.sm;
  ps.seqv = m.seqv;
  ps.sd[0] = m.sd[0];
  ps.sd[1] = m.sd[1];
  ps.sd[2] = m.sd[2];
  ps.sd[4] = m.sd[3];
  ps.sd[5] = m.sd[4];
  ps.sd[3] = m.sd[5];
  ps.sig_y = m.sig_y_;
  ps.epeff = m.epeff_;
  ps.ie = m.iener;
  ps.cp = m.cp;
  ps.q = m.bqf;
  ps.failure = failure;
}

template <class P>
__global__ void k_stress(St<P> s, Geometry g) {
  using R = typename P::R;
  using B = typename P::B;
  const long long p = gtid();
  if (p >= g.np) return;
  const long long np = g.np;
  const long long nn = g.nnt;  // node arrays of every grid component
  if (g.has_jc) {
    s.setter[p] = -1;
    s.deferred[p] = 0;
  }
  R de[6] = {0, 0, 0, 0, 0, 0}, vort[3] = {0, 0, 0}, deFp[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  if (g.shape == 3) {
    if (s.centericell[p] < 0) return;
    const long long nc = g.ncell;
    for (int k = 0; k < 8; ++k) {
      int c = s.snode[k * np + p];
      if (c < 0) continue;
      R sk = s.shp[k * np + p];
      for (int i = 0; i < 6; ++i) de[i] = de[i] + (R)s.co[i * nc + c] * sk;
      for (int i = 0; i < 3; ++i) vort[i] = vort[i] + (R)s.cw[i * nc + c] * sk;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) deFp[i][j] = deFp[i][j] + sk * (R)s.cdefp[(i * 3 + j) * nc + c];
    }
  } else {
    if (s.icell[p] < 0) return;
    for (int k = 0; k < g.K; ++k) {
      int n = s.snode[k * np + p];
      if (n < 0) continue;
      if (!(s.mg[n] > g.cutoff)) continue;
      R v[3] = {(R)s.vg[n], (R)s.vg[nn + n], (R)s.vg[2LL * nn + n]};
      const long long idx = k * np + p;
      R dx = s.dndx[idx], dy = s.dndy[idx], dz = s.dndz[idx];
      de[0] = de[0] + dx * v[0];
      de[1] = de[1] + dy * v[1];
      de[2] = de[2] + dz * v[2];
      de[3] = de[3] + (dy * v[2] + dz * v[1]);
      de[4] = de[4] + (dz * v[0] + dx * v[2]);
      de[5] = de[5] + (dx * v[1] + dy * v[0]);
      vort[0] = vort[0] + (dy * v[2] - dz * v[1]);
      vort[1] = vort[1] + (dz * v[0] - dx * v[2]);
      vort[2] = vort[2] + (dx * v[1] - dy * v[0]);
      for (int i = 0; i < 3; ++i) {
        deFp[i][0] = deFp[i][0] + dx * v[i];
        deFp[i][1] = deFp[i][1] + dy * v[i];
        deFp[i][2] = deFp[i][2] + dz * v[i];
      }
    }
  }
  const DevScalars& sc = *s.sc;
  const R DT = (R)sc.dt;
  for (int i = 0; i < 6; ++i) de[i] = de[i] * DT;
  for (int i = 0; i < 3; ++i) vort[i] = vort[i] * DT / (R)2.0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) deFp[i][j] = deFp[i][j] * DT;
  R Fpn[3][3];
  if (g.uvfp) {
    R F0[3][3];
    for (int i = 0; i < 9; ++i) F0[i / 3][i % 3] = (R)s.fp[i * np + p];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        Fpn[i][j] = F0[i][j] + deFp[i][j] + deFp[i][0] * F0[0][j] + deFp[i][1] * F0[1][j] + deFp[i][2] * F0[2][j];
        s.fp[(i * 3 + j) * np + p] = (B)Fpn[i][j];
      }
  }

  // ---- Constitution
  PState<R> ps;
  ps.vol = (R)s.vol[p];
  ps.epeff = (R)s.epeff[p];
  ps.sig_y = (R)s.sig_y[p];
  ps.seqv = (R)s.seqv[p];
  ps.lt = (R)s.lt[p];
  ps.celsius = (R)s.celsius[p];
  ps.ie = (R)s.ie[p];
  ps.mass = (R)s.mass[p];
  ps.dmg = (R)s.dmg[p];
  ps.cp = (R)s.cp[p];
  ps.sm = (R)s.sm[p];
  ps.q = (R)s.q[p];
  for (int i = 0; i < 6; ++i) ps.sd[i] = (R)s.sd[i * np + p];
  ps.failure = s.failure[p] != 0;
  ps.evol = (R)0;
  const DevMaterial& mt = s.mats[s.bodies[s.body[p]].mat];
  CResult<R> res;
  constitution<P>(ps, mt, de, vort, deFp, Fpn, g.uvfp != 0, DT, s.sc->time, (R)g.dcell, (R)g.bq1, (R)g.bq2, res);
  if (res.negative_volume) atomicOr(&s.sc->status, (unsigned)ST_NEGATIVE_VOLUME);
  if (!res.eos_ok) atomicOr(&s.sc->status, (unsigned)ST_BAD_EOS);
  if (res.defer && res.tail == 7) {
    // park the values the tail needs (Constitution.f90:285-314)
    s.jc_aux[p] = (double)res.vold;
    s.jc_aux[np + p] = (double)res.ieinc;
    s.jc_aux[2 * np + p] = (double)res.dvol;
    s.jc_aux[3 * np + p] = (double)res.smold;
    s.jc_aux[4 * np + p] = (double)res.vol_;
  }
  if (g.has_jc) {
    s.setter[p] = res.dep_set ? (int)p : -1;
    if (res.dep_set) s.dep[p] = (double)res.depeff;
    s.deferred[p] = res.defer ? (uint8_t)res.tail : 0;
  }
  s.vol[p] = (B)ps.vol;
  s.sm[p] = (B)ps.sm;
  s.seqv[p] = (B)ps.seqv;
  for (int i = 0; i < 6; ++i) s.sd[i * np + p] = (B)ps.sd[i];
  s.sig_y[p] = (B)ps.sig_y;
  s.epeff[p] = (B)ps.epeff;
  s.ie[p] = (double)ps.ie;
  s.cp[p] = (B)ps.cp;
  s.q[p] = (B)ps.q;
  s.celsius[p] = (B)ps.celsius;
  s.failure[p] = ps.failure ? 1 : 0;
  if (!isfinite((double)ps.sm) || !isfinite((double)ps.ie)) atomicOr(&s.sc->status, (unsigned)ST_NONFINITE);
  if (!g.usf) {
    s.xp[p] = s.xx[p];
    s.xp[np + p] = s.xx[np + p];
    s.xp[2 * np + p] = s.xx[2 * np + p];
  }
}

// Deferred Johnson-Cook tails: D is the depeff of the last particle before p
// (in processing order) that assigned it, or the value carried from the
// previous stress update.
template <class P>
__global__ void k_depeff_apply(St<P> s, Geometry g) {
  using R = typename P::R;
  using B = typename P::B;
  const long long p = gtid();
  if (p >= g.np) return;
  const int tail = s.deferred[p];
  if (tail == 0) return;
  const long long np = g.np;
  int last = s.setter_scan[p];
  R D = (R)(last >= 0 ? s.dep[last] : s.sc->depeff_carry);
  const DevMaterial& mt = s.mats[s.bodies[s.body[p]].mat];
  if (tail == 4) {
    R den_ = (R)s.mass[p] / (R)s.vol[p];
    s.celsius[p] = (B)((R)s.celsius[p] + (R)s.seqv[p] * D / den_ / (R)mt.specheat);
    return;
  }
  Mm<R> m;
  m.epeff_ = (R)s.epeff[p];
  m.sm = (R)s.sm[p];
  m.bqf = (R)s.q[p];
  m.iener = (R)s.ie[p];
  m.seqv = (R)s.seqv[p];
  m.sd[0] = (R)s.sd[p];
  m.sd[1] = (R)s.sd[np + p];
  m.sd[2] = (R)s.sd[2 * np + p];
  m.sd[3] = (R)s.sd[4 * np + p];
  m.sd[4] = (R)s.sd[5 * np + p];
  m.sd[5] = (R)s.sd[3 * np + p];
  m.vold = (R)s.jc_aux[p];
  m.ieinc = (R)s.jc_aux[np + p];
  m.dvol = (R)s.jc_aux[2 * np + p];
  m.smold = (R)s.jc_aux[3 * np + p];
  m.vol_ = (R)s.jc_aux[4 * np + p];
  m.DMG = (R)s.dmg[p];
  m.oldDMG = m.DMG;
  bool failure = s.failure[p] != 0;
  R vol_store = m.vol_;
  jc7_tail<P>(m, mt, failure, D, vol_store);
  R den_ = (R)s.mass[p] / m.vol_;
  s.celsius[p] = (B)((R)s.celsius[p] + m.seqv * D / den_ / (R)mt.specheat);
  s.vol[p] = (B)vol_store;
  s.sm[p] = (B)m.sm;
  s.q[p] = (B)m.bqf;
  s.ie[p] = (double)m.iener;
  s.epeff[p] = (B)m.epeff_;
  s.sd[p] = (B)m.sd[0];
  s.sd[np + p] = (B)m.sd[1];
  s.sd[2 * np + p] = (B)m.sd[2];
  s.sd[4 * np + p] = (B)m.sd[3];
  s.sd[5 * np + p] = (B)m.sd[4];
  s.sd[3 * np + p] = (B)m.sd[5];
  s.failure[p] = failure ? 1 : 0;
}

template <class P>
__global__ void k_depeff_carry(St<P> s, Geometry g) {
  int last = s.setter_scan[g.np - 1];
  if (last >= 0) s.sc->depeff_carry = s.dep[last];
}

// ----------------------------------------------------------- force input
// Per-particle external force (update_step.f90:889-903) and the diagonal
// stresses SM - q + SDii, prepared once per particle for the force transfer.
template <class P>
__global__ void k_force_prep(St<P> s, Geometry g) {
  using R = typename P::R;
  const long long p = gtid();
  if (p >= g.np) return;
  const long long np = g.np;
  const DevScalars& sc = *s.sc;
  double fx[3];
  for (int c = 0; c < 3; ++c) {
    double f = s.fxp[c * np + p];
    if (g.qload && !(sc.time >= g.qload_time)) f = f / g.qload_time * sc.time;
    fx[c] = f;
  }
  if (g.qdamp)
    for (int c = 0; c < 3; ++c) fx[c] = fx[c] - g.damp_factor * s.mass[p] * s.vxp[c * np + p];
  if (g.gravity) {
    const DevBody& bd = s.bodies[s.body[p]];
    for (int c = 0; c < 3; ++c) fx[c] = fx[c] + s.mass[p] * bd.gravp[c];
  }
  for (int c = 0; c < 3; ++c) s.fext[c * np + p] = fx[c];
  R smq = (R)s.sm[p] - (R)s.q[p];
  for (int c = 0; c < 3; ++c) s.sdiag[c * np + p] = (double)(smq + (R)s.sd[c * np + p]);
}

// ------------------------------------------------- P2G force (+integrate)
// GridMomentumUpdate (update_step.f90:831-1013) for one node, then, when
// integ != 0, IntegrateMomentum (1194-1239) and the node velocity.
template <class P>
__device__ __forceinline__ void node_integrate(St<P>& s, const Geometry& g, long long n, double fxn[3]) {
  const long long nn = g.nnt;
  const DevScalars& sc = *s.sc;
  const double dt = sc.dt;
  for (int c = 0; c < 3; ++c) {
    double pxc = s.px[(long long)c * nn + n];
    if (sc.istep == 1)
      pxc = pxc + fxn[c] * dt * 0.5;
    else
      pxc = pxc + fxn[c] * dt;
    s.px[(long long)c * nn + n] = pxc;
  }
  node_bc(s.fix[n % g.nn], s.px, s.fx, n, nn);
  node_vel(s.mg, s.px, s.vg, n, nn, g.cutoff);
}

template <class P>
__global__ void k_p2g_force(St<P> s, Geometry g, int integ) {
  using R = typename P::R;
  const long long n = gtid();
  const long long nn = g.nnt;  // every grid component
  if (n >= nn) return;
  const long long np = g.np;
  double f0 = 0.0, f1 = 0.0, f2 = 0.0;
  double nd0 = 0.0, nd1 = 0.0, nd2 = 0.0;  // contact normal: mass gradient (update_step.f90:977-982)
  const int j0 = n == 0 ? 0 : s.seg[n - 1], j1 = s.seg[n];
  for (int j = j0; j < j1; ++j) {
    long long p, idx;
    decode_pair(s.val_sorted[j], np, &p, &idx);
    R sk = s.shp[idx], dx = s.dndx[idx], dy = s.dndy[idx], dz = s.dndz[idx];
    if (g.contact) {
      const double mp = s.mass[p];
      nd0 = nd0 + (double)dx * mp;
      nd1 = nd1 + (double)dy * mp;
      nd2 = nd2 + (double)dz * mp;
    }
    R sxx = (R)s.sdiag[p], syy = (R)s.sdiag[np + p], szz = (R)s.sdiag[2 * np + p];
    R sxy = (R)s.sd[3 * np + p], syz = (R)s.sd[4 * np + p], sxz = (R)s.sd[5 * np + p];
    R vol = (R)s.vol[p];
    R fi0 = -(sxx * dx + sxy * dy + sxz * dz) * vol;
    R fi1 = -(sxy * dx + syy * dy + syz * dz) * vol;
    R fi2 = -(sxz * dx + syz * dy + szz * dz) * vol;
    if constexpr (P::kExact) {
      f0 = f0 + fi0 + s.fext[p] * sk;
      f1 = f1 + fi1 + s.fext[np + p] * sk;
      f2 = f2 + fi2 + s.fext[2 * np + p] * sk;
    } else {
      f0 = f0 + (double)(fi0 + (R)s.fext[p] * sk);
      f1 = f1 + (double)(fi1 + (R)s.fext[np + p] * sk);
      f2 = f2 + (double)(fi2 + (R)s.fext[2 * np + p] * sk);
    }
  }
  s.fx[n] = f0;
  s.fx[nn + n] = f1;
  s.fx[2LL * nn + n] = f2;
  if (g.contact) {
    s.ndir[n] = nd0;
    s.ndir[nn + n] = nd1;
    s.ndir[2LL * nn + n] = nd2;
  }
  if (integ) {
    double fxn[3] = {f0, f1, f2};
    node_integrate<P>(s, g, n, fxn);
  }
}

template <class P>
__global__ void k_integrate(St<P> s, Geometry g) {
  const long long n = gtid();
  if (n >= g.nnt) return;
  const long long nn = g.nnt;
  double fxn[3] = {s.fx[n], s.fx[nn + n], s.fx[2LL * nn + n]};
  node_integrate<P>(s, g, n, fxn);
}

// ---------------------------------------------------------------- contact
// Lagr_NodContact (update_step.f90:1241-1376), Bardenhagen's method between
// grid components 1 and 2, after IntegrateMomentum: per node, the contact
// normal from the components' mass gradients (normbody 0: their
// difference, 1: component 1's, 2: minus component 2's), unitised; where
// both components have mass above the cut-off and approach along the normal
// (crit > epsilon), the normal contact force crit / ((Mg1 + Mg2) DT) -- with
// friction, the full sticking force limited to fricfa |normal force|
// tangentially -- is taken from component 1 and given to component 2, in
// force and momentum, on the node's free directions. The node velocities of
// both components are refreshed for the position update; the force per node
// is kept for the total.
template <class P>
__global__ void k_contact(St<P> s, Geometry g) {
  const long long n = gtid();
  const long long nn = g.nn, nt = g.nnt;
  if (n >= nn) return;
  const double eps = 2.220446049250313e-16;  // epsilon(1d0)
  const long long n2 = nn + n;               // the node in component 2
  double nx = 0.0, ny = 0.0, nz = 0.0;
  if (g.normbody == 0) {
    nx = s.ndir[n] - s.ndir[n2];
    ny = s.ndir[nt + n] - s.ndir[nt + n2];
    nz = s.ndir[2 * nt + n] - s.ndir[2 * nt + n2];
  } else if (g.normbody == 1) {
    nx = s.ndir[n];
    ny = s.ndir[nt + n];
    nz = s.ndir[2 * nt + n];
  } else {
    nx = -s.ndir[n2];
    ny = -s.ndir[nt + n2];
    nz = -s.ndir[2 * nt + n2];
  }
  double tt = sqrt(nx * nx + ny * ny + nz * nz);
  if (tt > eps) {
    nx = nx / tt;
    ny = ny / tt;
    nz = nz / tt;
  }
  const double nd[3] = {nx, ny, nz};
  const double m1 = s.mg[n], m2 = s.mg[n2];
  double p1[3], p2[3], cforce[3] = {0.0, 0.0, 0.0};
  for (int c = 0; c < 3; ++c) {
    p1[c] = s.px[c * nt + n];
    p2[c] = s.px[c * nt + n2];
  }
  double crit = 0.0;
  if (m1 > g.cutoff && m2 > g.cutoff)
    crit = (p1[0] * m2 - p2[0] * m1) * nx + (p1[1] * m2 - p2[1] * m1) * ny + (p1[2] * m2 - p2[2] * m1) * nz;
  if (crit > eps) {
    const double dt = s.sc->dt;
    tt = (m1 + m2) * dt;
    const double nomforce = crit / tt;
    if (g.fricfa > eps) {
      double fstick[3];
      for (int c = 0; c < 3; ++c) cforce[c] = (p1[c] * m2 - p2[c] * m1) / tt;
      for (int c = 0; c < 3; ++c) fstick[c] = cforce[c] - nomforce * nd[c];
      const double val_fstick = sqrt(fstick[0] * fstick[0] + fstick[1] * fstick[1] + fstick[2] * fstick[2]);
      const double val_fslip = g.fricfa * fabs(nomforce);
      if (val_fslip < val_fstick)
        for (int c = 0; c < 3; ++c) cforce[c] = nomforce * nd[c] + val_fslip * (fstick[c] / val_fstick);
    } else {
      for (int c = 0; c < 3; ++c) cforce[c] = nomforce * nd[c];
    }
    const uint8_t fix = s.fix[n];
    for (int c = 0; c < 3; ++c) {
      if (fix & (1 << c)) continue;
      s.fx[c * nt + n] = s.fx[c * nt + n] - cforce[c];
      s.fx[c * nt + n2] = s.fx[c * nt + n2] + cforce[c];
      s.px[c * nt + n] = p1[c] - cforce[c] * dt;
      s.px[c * nt + n2] = p2[c] + cforce[c] * dt;
    }
    node_vel(s.mg, s.px, s.vg, n, nt, g.cutoff);
    node_vel(s.mg, s.px, s.vg, n2, nt, g.cutoff);
  }
  for (int c = 0; c < 3; ++c) s.cforce[c * nn + n] = cforce[c];
}

// the total contact force (tot_cont_for): one block, fixed summation tree
template <class P>
__global__ void k_contact_sum(St<P> s, Geometry g) {
  __shared__ double part[3][kBlock];
  const int t = threadIdx.x;
  const long long nn = g.nn;
  double a[3] = {0.0, 0.0, 0.0};
  for (long long n = t; n < nn; n += kBlock)
    for (int c = 0; c < 3; ++c) a[c] = a[c] + s.cforce[c * nn + n];
  for (int c = 0; c < 3; ++c) part[c][t] = a[c];
  __syncthreads();
  for (int w = kBlock / 2; w > 0; w >>= 1) {
    if (t < w)
      for (int c = 0; c < 3; ++c) part[c][t] = part[c][t] + part[c][t + w];
    __syncthreads();
  }
  if (t == 0)
    for (int c = 0; c < 3; ++c) s.sc->cont_for[c] = part[c][0];
}

// ------------------------------------------------------ position update
// ParticlePositionUpdate (update_step.f90:1378-1526), non-SGMP and SGMP.
template <class P>
__global__ void k_position(St<P> s, Geometry g) {
  using R = typename P::R;
  const long long p = gtid();
  if (p >= g.np) return;
  const long long np = g.np;
  const long long nn = g.nnt;  // node arrays of every grid component
  const DevScalars& sc = *s.sc;
  double vx[3] = {0, 0, 0}, ax[3] = {0, 0, 0};
  if (g.shape == 3) {
    if (s.centericell[p] < 0) return;
    const long long nc = g.ncell;
    int inode = s.inode[p];
    int bd = s.bd[inode - 1];
    R w[8];
    if (bd == 0) {
      for (int k = 0; k < 8; ++k) w[k] = s.shp[k * np + p];
    } else {  // AuxiliaryGridSHP, Grid.f90:193-220
      R xinb[3];
      for (int d = 0; d < 3; ++d) {
        R xnd = (R)s.xn[d * np + p];
        if ((bd >> (2 * d)) & 3)
          xinb[d] = xnd < (R)0 ? (R)1 + (R)2 * xnd : (R)2 * xnd - (R)1;
        else
          xinb[d] = (R)s.xxn[d * np + p];
      }
      for (int k = 0; k < 8; ++k) {
        R sx = (R)kSN[0][k] * xinb[0] + (R)1.0;
        R sy = (R)kSN[1][k] * xinb[1] + (R)1.0;
        R sz = (R)kSN[2][k] * xinb[2] + (R)1.0;
        w[k] = sx * sy * sz * (R)0.125;
      }
    }
    for (int k = 0; k < 8; ++k) {
      int c = s.snode[k * np + p];
      if (c < 0) continue;
      double sk = (double)w[k];
      for (int d = 0; d < 3; ++d) {
        vx[d] = vx[d] + sk * s.cvx[d * nc + c];
        ax[d] = ax[d] + sk * s.cax[d * nc + c];
      }
    }
  } else {
    if (s.icell[p] < 0) return;
    if constexpr (P::kExact) {
      for (int k = 0; k < g.K; ++k) {
        int n = s.snode[k * np + p];
        if (n < 0) continue;
        double m = s.mg[n];
        if (!(m > g.cutoff)) continue;
        double sk = s.shp[k * np + p];
        for (int d = 0; d < 3; ++d) {
          vx[d] = vx[d] + sk * s.vg[(long long)d * nn + n];
          ax[d] = ax[d] + sk * s.fx[(long long)d * nn + n] / m;
        }
      }
    } else {
      // mixed form: FP32 interpolation of the node velocity / acceleration
      float v32[3] = {0, 0, 0}, a32[3] = {0, 0, 0};
      for (int k = 0; k < g.K; ++k) {
        int n = s.snode[k * np + p];
        if (n < 0) continue;
        double m = s.mg[n];
        if (!(m > g.cutoff)) continue;
        float sk = (float)s.shp[k * np + p];
        float im = (float)(1.0 / m);
        for (int d = 0; d < 3; ++d) {
          v32[d] = v32[d] + sk * (float)s.vg[(long long)d * nn + n];
          a32[d] = a32[d] + sk * (float)s.fx[(long long)d * nn + n] * im;
        }
      }
      for (int d = 0; d < 3; ++d) {
        vx[d] = v32[d];
        ax[d] = a32[d];
      }
    }
  }
  const double dt = sc.dt;
  for (int d = 0; d < 3; ++d) {
    double xx = s.xp[d * np + p] + vx[d] * dt;
    s.xx[d * np + p] = xx;
    double v = s.vxp[d * np + p];
    if (sc.istep == 1)
      v = v + ax[d] * dt * 0.5;
    else
      v = v + ax[d] * dt;
    s.vxp[d * np + p] = v;
    if (g.usf) s.xp[d * np + p] = xx;
  }
}

// ------------------------------------------------------ MUSL momentum
// GridMomentumMUSL (update_step.f90:1668-1793), non-SGMP.
template <class P>
__global__ void k_p2g_momentum(St<P> s, Geometry g, int vel) {
  const long long n = gtid();
  const long long nn = g.nnt;  // every grid component
  if (n >= nn) return;
  const long long np = g.np;
  double px = 0.0, py = 0.0, pz = 0.0;
  const int j0 = n == 0 ? 0 : s.seg[n - 1], j1 = s.seg[n];
  for (int j = j0; j < j1; ++j) {
    long long p, idx;
    decode_pair(s.val_sorted[j], np, &p, &idx);
    double shm = (double)s.shp[idx] * s.mass[p];
    px = px + s.vxp[p] * shm;
    py = py + s.vxp[np + p] * shm;
    pz = pz + s.vxp[2 * np + p] * shm;
  }
  s.px[n] = px;
  s.px[nn + n] = py;
  s.px[2LL * nn + n] = pz;
  node_bc(s.fix[n % g.nn], s.px, s.fx, n, nn);
  if (vel) node_vel(s.mg, s.px, s.vg, n, nn, g.cutoff);
}

// ================================================================ SGMP
// Particle -> centre-node (cell) transfers walk the cell-keyed pair list;
// centre-node -> node transfers visit a node's (up to 8) adjacent cells in
// ascending cell order, which is the order of the reference's cell loops.

template <class F>
__device__ __forceinline__ void for_adjacent_cells(const Geometry& g, long long n, F f) {
  int jz = (int)(n / g.NGxy);
  int rem = (int)(n - (long long)jz * g.NGxy);
  int jy = rem / g.NGx;
  int jx = rem - jy * g.NGx;
  for (int cz = jz - 1; cz <= jz; ++cz) {
    if (cz < 0 || cz >= g.NCz) continue;
    for (int cy = jy - 1; cy <= jy; ++cy) {
      if (cy < 0 || cy >= g.NCy) continue;
      for (int cx = jx - 1; cx <= jx; ++cx) {
        if (cx < 0 || cx >= g.NCx) continue;
        int c = cz * g.NCxy + cy * g.NCx + cx;
        int ox = jx - cx, oy = jy - cy, oz = jz - cz;  // node's corner in the cell
        int corner = oz * 4 + (oy ? (ox ? 2 : 3) : (ox ? 1 : 0));
        f(c, corner);
      }
    }
  }
}

// GridMomentumInitial, SGMP branch: particles -> cells
template <class P>
__global__ void k_sg_cell_mass(St<P> s, Geometry g) {
  const long long c = gtid();
  const int nc = g.ncell;
  if (c >= nc) return;
  const long long np = g.np;
  double m = 0.0, px = 0.0, py = 0.0, pz = 0.0;
  const int j0 = c == 0 ? 0 : s.seg[c - 1], j1 = s.seg[c];
  for (int j = j0; j < j1; ++j) {
    long long p, idx;
    decode_pair(s.val_sorted[j], np, &p, &idx);
    double shm = (double)s.shp[idx] * s.mass[p];
    m = m + shm;
    px = px + s.vxp[p] * shm;
    py = py + s.vxp[np + p] * shm;
    pz = pz + s.vxp[2 * np + p] * shm;
  }
  s.cmg[c] = m;
  s.cpx[c] = px;
  s.cpx[nc + c] = py;
  s.cpx[2LL * nc + c] = pz;
}

// ... cells -> nodes (mass and momentum, only cells above the cut-off)
template <class P>
__global__ void k_sg_node_mass(St<P> s, Geometry g, int bc, int vel) {
  const long long n = gtid();
  const int nn = g.nn;
  bool act = false;
  if (n < nn) {
    const long long nc = g.ncell;
    double m = 0.0, px = 0.0, py = 0.0, pz = 0.0;
    for_adjacent_cells(g, n, [&](int c, int) {
      double cm = s.cmg[c];
      if (!(cm > g.cutoff)) return;
      m = m + 0.125 * cm;
      px = px + 0.125 * s.cpx[c];
      py = py + 0.125 * s.cpx[nc + c];
      pz = pz + 0.125 * s.cpx[2 * nc + c];
    });
    s.mg[n] = m;
    s.px[n] = px;
    s.px[nn + n] = py;
    s.px[2LL * nn + n] = pz;
    act = m > 0.0;
    if (bc) node_bc(s.fix[n], s.px, s.fx, (int)n, nn);
    if (vel) node_vel(s.mg, s.px, s.vg, (int)n, nn, g.cutoff);
  }
  count_active(act, &s.sc->active_nodes);
}

// ParticleStressUpdate, SGMP branch: centre-node strain rate and spin from
// the 8 nodes of each cell (CNShape derivatives at the cell centre)
template <class P>
__global__ void k_sg_cell_gradient(St<P> s, Geometry g) {
  const long long c = gtid();
  const int nc = g.ncell;
  if (c >= nc) return;
  const int nn = g.nn;
  double co[6] = {0, 0, 0, 0, 0, 0}, cw[3] = {0, 0, 0}, cf[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const int n1 = cell_node1(g, (int)c + 1);
  for (int j = 0; j < 8; ++j) {
    int n = n1 + kCorner[j][0] + kCorner[j][1] * g.NGx + kCorner[j][2] * g.NGxy;
    if (!(s.mg[n] > g.cutoff)) continue;
    double v[3] = {s.vg[n], s.vg[nn + n], s.vg[2LL * nn + n]};
    // CNShape(2): sx = sy = sz = 1 at the centre
    double dx = (double)kSN[0][j] * 1.0 * 1.0 * g.iJacobi4;
    double dy = (double)kSN[1][j] * 1.0 * 1.0 * g.iJacobi4;
    double dz = (double)kSN[2][j] * 1.0 * 1.0 * g.iJacobi4;
    co[0] = co[0] + dx * v[0];
    co[1] = co[1] + dy * v[1];
    co[2] = co[2] + dz * v[2];
    co[3] = co[3] + dz * v[1] + dy * v[2];
    co[4] = co[4] + dz * v[0] + dx * v[2];
    co[5] = co[5] + dy * v[0] + dx * v[1];
    cw[0] = cw[0] + dy * v[2] - dz * v[1];
    cw[1] = cw[1] + dz * v[0] - dx * v[2];
    cw[2] = cw[2] + dx * v[1] - dy * v[0];
    for (int i = 0; i < 3; ++i) {
      cf[i * 3 + 0] = cf[i * 3 + 0] + dx * v[i];
      cf[i * 3 + 1] = cf[i * 3 + 1] + dy * v[i];
      cf[i * 3 + 2] = cf[i * 3 + 2] + dz * v[i];
    }
  }
  for (int i = 0; i < 6; ++i) s.co[(long long)i * nc + c] = co[i];
  for (int i = 0; i < 3; ++i) s.cw[(long long)i * nc + c] = cw[i];
  for (int i = 0; i < 9; ++i) s.cdefp[(long long)i * nc + c] = cf[i];
}

// GridMomentumUpdate, SGMP branch: particles -> cells
template <class P>
__global__ void k_sg_cell_force(St<P> s, Geometry g) {
  using R = typename P::R;
  const long long c = gtid();
  const int nc = g.ncell;
  if (c >= nc) return;
  const long long np = g.np;
  double fe[3] = {0, 0, 0}, fi[6] = {0, 0, 0, 0, 0, 0};
  const int j0 = c == 0 ? 0 : s.seg[c - 1], j1 = s.seg[c];
  for (int j = j0; j < j1; ++j) {
    long long p, idx;
    decode_pair(s.val_sorted[j], np, &p, &idx);
    double sk = (double)s.shp[idx];
    double vol = (double)s.vol[p];
    for (int d = 0; d < 3; ++d) fe[d] = fe[d] + s.fext[d * np + p] * sk;
    fi[0] = fi[0] + sk * s.sdiag[p] * vol;
    fi[1] = fi[1] + sk * s.sdiag[np + p] * vol;
    fi[2] = fi[2] + sk * s.sdiag[2 * np + p] * vol;
    fi[3] = fi[3] + sk * (double)s.sd[3 * np + p] * vol;
    fi[4] = fi[4] + sk * (double)s.sd[4 * np + p] * vol;
    fi[5] = fi[5] + sk * (double)s.sd[5 * np + p] * vol;
  }
  for (int d = 0; d < 3; ++d) s.cfext[(long long)d * nc + c] = fe[d];
  for (int d = 0; d < 6; ++d) s.cfint[(long long)d * nc + c] = fi[d];
}

// ... cells -> nodes (every cell, no cut-off), then optionally integrate
template <class P>
__global__ void k_sg_node_force(St<P> s, Geometry g, int integ) {
  const long long n = gtid();
  const int nn = g.nn;
  if (n >= nn) return;
  const long long nc = g.ncell;
  double f[3] = {0.0, 0.0, 0.0};
  for_adjacent_cells(g, n, [&](int c, int j) {
    double dx = (double)kSN[0][j] * 1.0 * 1.0 * g.iJacobi4;
    double dy = (double)kSN[1][j] * 1.0 * 1.0 * g.iJacobi4;
    double dz = (double)kSN[2][j] * 1.0 * 1.0 * g.iJacobi4;
    const double* ci = s.cfint;
    double c0 = ci[c], c1 = ci[nc + c], c2 = ci[2 * nc + c], c3 = ci[3 * nc + c], c4 = ci[4 * nc + c],
           c5 = ci[5 * nc + c];
    double fi0 = -(c0 * dx + c3 * dy + c5 * dz);
    double fi1 = -(c3 * dx + c1 * dy + c4 * dz);
    double fi2 = -(c5 * dx + c4 * dy + c2 * dz);
    f[0] = f[0] + 0.125 * s.cfext[c] + fi0;
    f[1] = f[1] + 0.125 * s.cfext[nc + c] + fi1;
    f[2] = f[2] + 0.125 * s.cfext[2 * nc + c] + fi2;
  });
  s.fx[n] = f[0];
  s.fx[nn + n] = f[1];
  s.fx[2LL * nn + n] = f[2];
  if (integ) node_integrate<P>(s, g, n, f);
}

// ParticlePositionUpdate, SGMP branch: centre-node velocity / acceleration
// (and BoundaryAuxiliaryNodeUpdate, update_step.f90:1528-1666, for the
// cells on a fixed or symmetric face)
template <class P>
__global__ void k_sg_cell_velocity(St<P> s, Geometry g) {
  const long long c = gtid();
  const int nc = g.ncell;
  if (c >= nc) return;
  const int nn = g.nn;
  int cz = (int)(c / g.NCxy), rem = (int)(c - (long long)cz * g.NCxy), cy = rem / g.NCx, cx = rem - cy * g.NCx;
  int ci[3] = {cx, cy, cz}, NC[3] = {g.NCx, g.NCy, g.NCz};
  bool boundary = false;
  for (int d = 0; d < 3; ++d)
    if (NC[d] > 1 && ((ci[d] == 0 && g.fixs[2 * d] != 0) || (ci[d] == NC[d] - 1 && g.fixs[2 * d + 1] != 0)))
      boundary = true;
  double v[3] = {0, 0, 0}, a[3] = {0, 0, 0};
  const int n1 = cell_node1(g, (int)c + 1);
  if (!boundary) {
    for (int j = 0; j < 8; ++j) {
      int n = n1 + kCorner[j][0] + kCorner[j][1] * g.NGx + kCorner[j][2] * g.NGxy;
      double m = s.mg[n];
      if (!(m > g.cutoff)) continue;
      for (int d = 0; d < 3; ++d) {
        v[d] = v[d] + 0.125 * s.px[(long long)d * nn + n] / m;
        a[d] = a[d] + 0.125 * s.fx[(long long)d * nn + n] / m;
      }
    }
  } else {
    double cxx[3];
    for (int d = 0; d < 3; ++d) {
      cxx[d] = 0.0;
      if (NC[d] > 1) {
        if (ci[d] == 0) cxx[d] = 1.0;
        if (ci[d] == NC[d] - 1) cxx[d] = -1.0;
      }
    }
    for (int j = 0; j < 8; ++j) {
      int n = n1 + kCorner[j][0] + kCorner[j][1] * g.NGx + kCorner[j][2] * g.NGxy;
      double sx = (double)kSN[0][j] * cxx[0] + 1.0;
      double sy = (double)kSN[1][j] * cxx[1] + 1.0;
      double sz = (double)kSN[2][j] * cxx[2] + 1.0;
      double w = sx * sy * sz * 0.125;
      double m = s.mg[n];
      if (!(m > g.cutoff)) continue;
      for (int d = 0; d < 3; ++d) {
        v[d] = v[d] + w * s.px[(long long)d * nn + n] / m;
        a[d] = a[d] + w * s.fx[(long long)d * nn + n] / m;
      }
    }
  }
  for (int d = 0; d < 3; ++d) {
    s.cvx[(long long)d * nc + c] = v[d];
    s.cax[(long long)d * nc + c] = a[d];
  }
}

// GridMomentumMUSL, SGMP branch
template <class P>
__global__ void k_sg_cell_momentum(St<P> s, Geometry g) {
  const long long c = gtid();
  const int nc = g.ncell;
  if (c >= nc) return;
  const long long np = g.np;
  double px = 0.0, py = 0.0, pz = 0.0;
  const int j0 = c == 0 ? 0 : s.seg[c - 1], j1 = s.seg[c];
  for (int j = j0; j < j1; ++j) {
    long long p, idx;
    decode_pair(s.val_sorted[j], np, &p, &idx);
    double shm = (double)s.shp[idx] * s.mass[p];
    px = px + s.vxp[p] * shm;
    py = py + s.vxp[np + p] * shm;
    pz = pz + s.vxp[2 * np + p] * shm;
  }
  s.cpx[c] = px;
  s.cpx[nc + c] = py;
  s.cpx[2LL * nc + c] = pz;
}

template <class P>
__global__ void k_sg_node_momentum(St<P> s, Geometry g, int vel) {
  const long long n = gtid();
  const int nn = g.nn;
  if (n >= nn) return;
  const long long nc = g.ncell;
  double px = 0.0, py = 0.0, pz = 0.0;
  for_adjacent_cells(g, n, [&](int c, int) {
    px = px + 0.125 * s.cpx[c];
    py = py + 0.125 * s.cpx[nc + c];
    pz = pz + 0.125 * s.cpx[2 * nc + c];
  });
  s.px[n] = px;
  s.px[nn + n] = py;
  s.px[2LL * nn + n] = pz;
  node_bc(s.fix[n], s.px, s.fx, (int)n, nn);
  if (vel) node_vel(s.mg, s.px, s.vg, (int)n, nn, g.cutoff);
}

// ================================================================= TLMPM
// The total Lagrangian form (MPM3D.f90:161-244): the grid mass is mapped
// once from the initial positions (GridMassInitial), each particle keeps the
// cell of its initial position for the whole run (TLParticleInitial; shapes
// as k_fixed_locate), the deformation gradient grows by the velocity
// gradient, the stress is the neo-Hookean first Piola-Kirchhoff stress
// (TLConstitution, M3DM11) and the internal forces come from it on the
// initial volume (TLGridMomentumUpdate). Position update, MUSL re-map and
// contact are those of the updated form.

// TLParticleInitial (update_step.f90:127-172) at the initial positions;
// XN is not set there for non-SGMP shapes and keeps its initial value 0
template <class P>
__global__ void k_tl_initial(St<P> s, Geometry g) {
  using B = typename P::B;
  const long long p = gtid();
  if (p >= g.np) return;
  const long long np = g.np;
  const double x[3] = {s.xp[p], s.xp[np + p], s.xp[2 * np + p]};
  const int icell = in_which_cell(g, x);
  s.icell[p] = icell;
  for (int d = 0; d < 3; ++d) s.xn[d * np + p] = (B)0;
  if (g.shape != 3) return;
  s.centericell[p] = center_in_which_cell(g, x);
  const int ix = (int)((x[0] - g.span0[0]) / g.dcell + 0.5) + 1;
  const int iy = (int)((x[1] - g.span0[1]) / g.dcell + 0.5) + 1;
  const int iz = (int)((x[2] - g.span0[2]) / g.dcell + 0.5) + 1;
  const long long inode = (long long)(iz - 1) * g.NGxy + (long long)(iy - 1) * g.NGx + ix;
  s.inode[p] = (int)inode;
  if (inode < 1 || inode > g.nn || icell < 1) return;  // outside the grid
  const int bd = s.bd[inode - 1];
  const int n1 = cell_node1(g, icell);
  for (int d = 0; d < 3; ++d) {
    double xxn = (x[d] - node_coord(g, (int)inode - 1, d)) * g.iJacobi;
    if ((bd >> (2 * d)) & 3) xxn = xxn > 0 ? 1.0 : (xxn < 0 ? -1.0 : xxn);
    s.xxn[d * np + p] = (B)xxn;
    s.xn[d * np + p] = (B)((x[d] - (node_coord(g, n1, d) + g.dcell / 2.0)) * g.iJacobi);
  }
}

// TLGridMomentumInitial, SGMP: centre nodes -> nodes, momentum of the cells
// above the cut-off mass (the mass stays that of GridMassInitial)
template <class P>
__global__ void k_tl_sg_node_momentum(St<P> s, Geometry g, int vel) {
  const long long n = gtid();
  const int nn = g.nn;
  if (n >= nn) return;
  const long long nc = g.ncell;
  double px = 0.0, py = 0.0, pz = 0.0;
  for_adjacent_cells(g, n, [&](int c, int) {
    if (!(s.cmg[c] > g.cutoff)) return;
    px = px + 0.125 * s.cpx[c];
    py = py + 0.125 * s.cpx[nc + c];
    pz = pz + 0.125 * s.cpx[2 * nc + c];
  });
  s.px[n] = px;
  s.px[nn + n] = py;
  s.px[2LL * nn + n] = pz;
  node_bc(s.fix[n], s.px, s.fx, n, nn);
  if (vel) node_vel(s.mg, s.px, s.vg, n, nn, g.cutoff);
}

// TLParticleStressUpdate + TLConstitution / M3DM11 (update_step.f90:649-828,
// Constitution.f90:370-523, 782-882) for one particle. Like the reference,
// sig_y and epeff are written from the constitutive module's state, which
// the TL update never loads (0 in a TL run).
template <class P>
__global__ void k_tl_stress(St<P> s, Geometry g) {
  using R = typename P::R;
  using B = typename P::B;
  const long long p = gtid();
  if (p >= g.np) return;
  const long long np = g.np, nn = g.nnt;
  R deFp[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  if (g.shape == 3) {
    if (s.centericell[p] < 0) return;
    const long long nc = g.ncell;
    for (int k = 0; k < 8; ++k) {
      int c = s.snode[k * np + p];
      if (c < 0) continue;
      R sk = s.shp[k * np + p];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) deFp[i][j] = deFp[i][j] + sk * (R)s.cdefp[(i * 3 + j) * nc + c];
    }
  } else {
    if (s.icell[p] < 0) return;
    for (int k = 0; k < g.K; ++k) {
      int n = s.snode[k * np + p];
      if (n < 0) continue;
      if (!(s.mg[n] > g.cutoff)) continue;
      R v[3] = {(R)s.vg[n], (R)s.vg[nn + n], (R)s.vg[2LL * nn + n]};
      const long long idx = k * np + p;
      R dx = s.dndx[idx], dy = s.dndy[idx], dz = s.dndz[idx];
      for (int i = 0; i < 3; ++i) {
        deFp[i][0] = deFp[i][0] + dx * v[i];
        deFp[i][1] = deFp[i][1] + dy * v[i];
        deFp[i][2] = deFp[i][2] + dz * v[i];
      }
    }
  }
  const DevScalars& sc = *s.sc;
  const R DT = (R)sc.dt;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) deFp[i][j] = deFp[i][j] * DT;
  if (g.uvfp)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) s.fp[(i * 3 + j) * np + p] = (B)((R)s.fp[(i * 3 + j) * np + p] + deFp[i][j]);
  // ---- TLConstitution
  R ppk_old[9], ppk_new[9];
  for (int i = 0; i < 9; ++i) ppk_old[i] = (R)s.pk[i * np + p];
  const R vold = (R)s.vol[p];
  R F3[3][3];
  for (int i = 0; i < 9; ++i) F3[i / 3][i % 3] = (R)s.fp[i * np + p];
  for (int i = 0; i < 3; ++i) F3[i][i] = F3[i][i] + (R)1.0;
  const R detF = F3[0][0] * F3[1][1] * F3[2][2] - F3[0][0] * F3[1][2] * F3[2][1] -
                 F3[1][0] * F3[0][1] * F3[2][2] + F3[1][0] * F3[0][2] * F3[2][1] +
                 F3[2][0] * F3[0][1] * F3[1][2] - F3[2][0] * F3[0][2] * F3[1][1];
  const R vol = detF * (R)s.vol0[p];
  const DevMaterial& mt = s.mats[s.bodies[s.body[p]].mat];
  const R young = (R)mt.young * ((R)1.0 - (R)s.dmg[p] + (R)2.220446049250313e-16);
  const R nu = (R)mt.poisson;
  const R G2 = young / (1 + nu);
  const R lamda = (young * nu) / ((1 + nu) * (1 - 2 * nu));
  const R G = (R)0.5 * G2, J = detF;
  // F and its transposed inverse in the order 11 22 33 23 13 12 32 31 21
  const R F[9] = {F3[0][0], F3[1][1], F3[2][2], F3[1][2], F3[0][2], F3[0][1], F3[2][1], F3[2][0], F3[1][0]};
  R FIT[9];
  FIT[0] = (F[1] * F[2] - F[3] * F[6]) / J;
  FIT[1] = (F[0] * F[2] - F[4] * F[7]) / J;
  FIT[2] = (F[0] * F[1] - F[5] * F[8]) / J;
  FIT[3] = (F[5] * F[7] - F[0] * F[6]) / J;
  FIT[4] = (F[8] * F[6] - F[1] * F[7]) / J;
  FIT[5] = (F[3] * F[7] - F[2] * F[8]) / J;
  FIT[6] = (F[4] * F[8] - F[3] * F[0]) / J;
  FIT[7] = (F[3] * F[5] - F[4] * F[1]) / J;
  FIT[8] = (F[4] * F[6] - F[5] * F[2]) / J;
  const R lnJ = m_log<P>(J);
  for (int i = 0; i < 9; ++i) ppk_new[i] = G * (F[i] - FIT[i]) + lamda * lnJ * FIT[i];
  const R FT[9] = {F[0], F[1], F[2], F[6], F[7], F[8], F[3], F[4], F[5]};
  R sig[6];
  sig[0] = (ppk_new[0] * FT[0] + ppk_new[5] * FT[8] + ppk_new[4] * FT[7]) / J;
  sig[1] = (ppk_new[8] * FT[5] + ppk_new[1] * FT[1] + ppk_new[3] * FT[6]) / J;
  sig[2] = (ppk_new[7] * FT[4] + ppk_new[6] * FT[3] + ppk_new[2] * FT[2]) / J;
  sig[3] = (ppk_new[8] * FT[4] + ppk_new[1] * FT[3] + ppk_new[3] * FT[2]) / J;  // yz
  sig[4] = (ppk_new[0] * FT[4] + ppk_new[5] * FT[3] + ppk_new[4] * FT[2]) / J;  // xz
  sig[5] = (ppk_new[0] * FT[5] + ppk_new[5] * FT[1] + ppk_new[4] * FT[6]) / J;  // xy
  const R sm = (sig[0] + sig[1] + sig[2]) / (R)3.0;
  const R sd[6] = {sig[0] - sm, sig[1] - sm, sig[2] - sm, sig[3], sig[4], sig[5]};
  R J2 = (R)0.5 * (sd[0] * sd[0] + sd[1] * sd[1] + sd[2] * sd[2]) + sd[3] * sd[3] + sd[4] * sd[4] + sd[5] * sd[5];
  J2 = J2 * (R)3.0;
  const R seqv = (R)(float)sqrt(J2);  // EquivalentStress: a default-REAL result
  // increment of F in the same order as F
  const R dF[9] = {deFp[0][0], deFp[1][1], deFp[2][2], deFp[1][2], deFp[0][2], deFp[0][1], deFp[2][1], deFp[2][0],
                   deFp[1][0]};
  R ieinc = 0;
  for (int i = 0; i < 9; ++i) ieinc = ieinc + (R)0.5 * (ppk_old[i] + ppk_new[i]) * dF[i];
  const R iener = (R)s.ie[p] + ieinc * (R)0.5 * (vol + vold);
  for (int i = 0; i < 9; ++i) s.pk[i * np + p] = (double)ppk_new[i];
  s.vol[p] = (B)vol;
  s.sm[p] = (B)sm;
  s.seqv[p] = (B)seqv;
  s.sd[p] = (B)sd[0];
  s.sd[np + p] = (B)sd[1];
  s.sd[2 * np + p] = (B)sd[2];
  s.sd[3 * np + p] = (B)sd[5];  // xy
  s.sd[4 * np + p] = (B)sd[3];  // yz
  s.sd[5 * np + p] = (B)sd[4];  // xz
  s.sig_y[p] = (B)0;
  s.epeff[p] = (B)0;
  s.ie[p] = (double)iener;
  s.q[p] = (B)0;
  if (!g.usf)
    for (int d = 0; d < 3; ++d) s.xp[d * np + p] = s.xx[d * np + p];
}

// TLGridMomentumUpdate (update_step.f90:1015-1191): nodal force from the
// PK stress on the initial volume, then optionally IntegrateMomentum
template <class P>
__global__ void k_tl_p2g_force(St<P> s, Geometry g, int integ) {
  using R = typename P::R;
  const long long n = gtid();
  const long long nn = g.nnt;
  if (n >= nn) return;
  const long long np = g.np;
  double f0 = 0.0, f1 = 0.0, f2 = 0.0, nd0 = 0.0, nd1 = 0.0, nd2 = 0.0;
  const int j0 = n == 0 ? 0 : s.seg[n - 1], j1 = s.seg[n];
  for (int j = j0; j < j1; ++j) {
    long long p, idx;
    decode_pair(s.val_sorted[j], np, &p, &idx);
    const R sk = s.shp[idx], dx = s.dndx[idx], dy = s.dndy[idx], dz = s.dndz[idx];
    R K[9];
    for (int k = 0; k < 9; ++k) K[k] = (R)s.pk[k * np + p];  // xx yy zz yz xz xy zy zx yx
    const R vol = (R)s.vol0[p];
    const R fi0 = -(K[0] * dx + K[5] * dy + K[4] * dz) * vol;
    const R fi1 = -(K[8] * dx + K[1] * dy + K[3] * dz) * vol;
    const R fi2 = -(K[7] * dx + K[6] * dy + K[2] * dz) * vol;
    f0 = f0 + fi0 + s.fext[p] * sk;
    f1 = f1 + fi1 + s.fext[np + p] * sk;
    f2 = f2 + fi2 + s.fext[2 * np + p] * sk;
    if (g.contact) {
      const double mp = s.mass[p];
      nd0 = nd0 + (double)dx * mp;
      nd1 = nd1 + (double)dy * mp;
      nd2 = nd2 + (double)dz * mp;
    }
  }
  s.fx[n] = f0;
  s.fx[nn + n] = f1;
  s.fx[2LL * nn + n] = f2;
  if (g.contact) {
    s.ndir[n] = nd0;
    s.ndir[nn + n] = nd1;
    s.ndir[2LL * nn + n] = nd2;
  }
  if (integ) {
    double fxn[3] = {f0, f1, f2};
    node_integrate<P>(s, g, n, fxn);
  }
}

// ... SGMP: particles -> cells (external force, PK * VOL0)
template <class P>
__global__ void k_tl_sg_cell_force(St<P> s, Geometry g) {
  const long long c = gtid();
  const int nc = g.ncell;
  if (c >= nc) return;
  const long long np = g.np;
  double fe[3] = {0, 0, 0}, fk[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const int j0 = c == 0 ? 0 : s.seg[c - 1], j1 = s.seg[c];
  for (int j = j0; j < j1; ++j) {
    long long p, idx;
    decode_pair(s.val_sorted[j], np, &p, &idx);
    const double sk = (double)s.shp[idx], vol = (double)s.vol0[p];
    for (int d = 0; d < 3; ++d) fe[d] = fe[d] + s.fext[d * np + p] * sk;
    for (int k = 0; k < 9; ++k) fk[k] = fk[k] + sk * s.pk[k * np + p] * vol;
  }
  for (int d = 0; d < 3; ++d) s.cfext[(long long)d * nc + c] = fe[d];
  for (int k = 0; k < 9; ++k) s.cpk[(long long)k * nc + c] = fk[k];
}

// ... cells -> nodes (every cell), then optionally integrate
template <class P>
__global__ void k_tl_sg_node_force(St<P> s, Geometry g, int integ) {
  const long long n = gtid();
  const int nn = g.nn;
  if (n >= nn) return;
  const long long nc = g.ncell;
  double f[3] = {0.0, 0.0, 0.0};
  for_adjacent_cells(g, n, [&](int c, int j) {
    double dx = (double)kSN[0][j] * 1.0 * 1.0 * g.iJacobi4;
    double dy = (double)kSN[1][j] * 1.0 * 1.0 * g.iJacobi4;
    double dz = (double)kSN[2][j] * 1.0 * 1.0 * g.iJacobi4;
    double C[9];
    for (int k = 0; k < 9; ++k) C[k] = s.cpk[k * nc + c];
    double fi0 = -(C[0] * dx + C[5] * dy + C[4] * dz);
    double fi1 = -(C[8] * dx + C[1] * dy + C[3] * dz);
    double fi2 = -(C[7] * dx + C[6] * dy + C[2] * dz);
    f[0] = f[0] + 0.125 * s.cfext[c] + fi0;
    f[1] = f[1] + 0.125 * s.cfext[nc + c] + fi1;
    f[2] = f[2] + 0.125 * s.cfext[2 * nc + c] + fi2;
  });
  s.fx[n] = f[0];
  s.fx[nn + n] = f[1];
  s.fx[2LL * nn + n] = f[2];
  if (integ) node_integrate<P>(s, g, n, f);
}

// ====================================================== stress smoothing
// SmoothStressbyGrid (update_step.f90:1876-2055): the particles' pressure
// -SM mapped to the grid with volume weights, normalised by the mapped
// volume, and interpolated back into Spre. Runs after UpdateDT with the
// shapes of the step's cells: GIMP and B-spline weights at the current Xp
// against the cell found at the start of the step, linear ones at XN, SGMP
// ones at XXN (the reference recomputes them from those fields). The pair
// list is rebuilt for these shapes and every sum runs in the reference's
// order (ascending particle per node or centre node; ascending cell per node;
// slot order per particle).

// shapes and pair keys of every particle with the cells it holds (those of
// the start of the step for the smoothing, those of the start of the run for
// TLMPM): GIMP / B-spline weights at the current position, linear ones at
// XN, SGMP ones at XXN; with_comp: keys in the particle's grid component
template <class P>
__global__ void k_fixed_locate(St<P> s, Geometry g, int nkeys, int with_comp) {
  const long long p = gtid();
  if (p >= g.np) return;
  const long long np = g.np;
  const double x[3] = {s.xp[p], s.xp[np + p], s.xp[2 * np + p]};
  const int icell = s.icell[p];
  double xn[3] = {0, 0, 0}, xxn[3] = {0, 0, 0};
  for (int d = 0; d < 3; ++d) {
    xn[d] = (double)s.xn[d * np + p];
    if (g.shape == 3) xxn[d] = (double)s.xxn[d * np + p];
  }
  const int cc = g.shape == 3 ? s.centericell[p] : 0;
  int slot_node[27];
  const int nvalid = slot_shapes<P>(s, g, p, x, g.shape == 3 ? 0 : icell, xn, cc, xxn, slot_node);
  const int cbase = with_comp && g.shape != 3 ? s.bodies[s.body[p]].comp * g.nn : 0;  // smoothing: component 1
  write_pairs<P>(s, g, p, nvalid, slot_node, nkeys, cbase);
}

// pressure * volume and volume of one (node or centre node) slice of pairs,
// in particle order; returns false for an empty slice
template <class P>
__device__ __forceinline__ bool smooth_sums(const St<P>& s, const Geometry& g, int j0, int j1, double& gp, double& gv) {
  const long long np = g.np;
  gp = 0.0;
  gv = 0.0;
  for (int j = j0; j < j1; ++j) {
    long long p, idx;
    decode_pair(s.val_sorted[j], np, &p, &idx);
    const double shp = (double)s.shp[idx], sm = (double)s.sm[p];
    const double vol = g.tlmpm ? (double)s.vol0[p] : (double)s.vol[p];  // TLSmoothStressbyGrid: VOL0
    gp = gp + shp * (-1 * sm) * vol;
    gv = gv + shp * vol;
  }
  return j1 > j0;
}

// particles -> nodes, Gpre / GV_all on the mapped nodes
template <class P>
__global__ void k_smooth_node(St<P> s, Geometry g) {
  const long long n = gtid();
  if (n >= g.nn) return;
  double gp, gv;
  const bool mapped = smooth_sums<P>(s, g, n == 0 ? 0 : s.seg[n - 1], s.seg[n], gp, gv);
  s.gpre[n] = mapped ? gp / gv : gp;
}

// SGMP: particles -> centre nodes
template <class P>
__global__ void k_smooth_cell(St<P> s, Geometry g) {
  const long long c = gtid();
  if (c >= g.ncell) return;
  double gp, gv;
  smooth_sums<P>(s, g, c == 0 ? 0 : s.seg[c - 1], s.seg[c], gp, gv);
  s.cgpre[c] = gp;
  s.cgvall[c] = gv;
}

// SGMP: centre nodes -> nodes (1/8 of every adjacent cell; every node is
// mapped, 0/0 where no volume reached it)
template <class P>
__global__ void k_smooth_sg_node(St<P> s, Geometry g) {
  const long long n = gtid();
  if (n >= g.nn) return;
  double gp = 0.0, gv = 0.0;
  for_adjacent_cells(g, n, [&](int c, int) {
    gp = gp + 0.125 * s.cgpre[c];
    gv = gv + 0.125 * s.cgvall[c];
  });
  s.gpre[n] = gp / gv;
}

// SGMP: nodes above the cut-off mass -> centre nodes
template <class P>
__global__ void k_smooth_sg_back(St<P> s, Geometry g) {
  const long long c = gtid();
  if (c >= g.ncell) return;
  const int n1 = cell_node1(g, (int)c + 1);
  double cp = 0.0;
  for (int j = 0; j < 8; ++j) {
    const int n = n1 + kCorner[j][0] + kCorner[j][1] * g.NGx + kCorner[j][2] * g.NGxy;
    if (s.mg[n] > g.cutoff) cp = cp + 0.125 * s.gpre[n];
  }
  s.cgpre[c] = cp;
}

// (centre) nodes -> particles: Spre
template <class P>
__global__ void k_smooth_g2p(St<P> s, Geometry g) {
  const long long p = gtid();
  if (p >= g.np) return;
  const long long np = g.np;
  const double* src = g.shape == 3 ? s.cgpre : s.gpre;
  double sp = 0.0;
  for (int k = 0; k < g.K; ++k) {
    const int nd = s.snode[k * np + p];
    if (nd < 0) continue;
    sp = sp + (double)s.shp[k * np + p] * src[nd];
  }
  s.spre[p] = sp;
}

// ============================================================ reductions
// calcEnergy (Particle.f90:204-230) and UpdateDT (update_step.f90:1833-1874)
// in one pass: a fixed-shape block tree, then the last block to finish
// combines the block partials in block order and derives the next DT.
// kRedVals (mpm_gpu_internal.cuh): ke, ie, mom x/y/z, max |v| component

// mode bit 0: update the energies and momentum; bit 1: derive the next DT
template <class P>
__global__ void k_reduce(St<P> s, Geometry g, int mode) {
  __shared__ double sh[kRedVals][kBlock];
  __shared__ bool last;
  const long long np = g.np;
  double acc[kRedVals] = {0, 0, 0, 0, 0, 0};
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < np;
       p += (long long)gridDim.x * blockDim.x) {
    double v0 = s.vxp[p], v1 = s.vxp[np + p], v2 = s.vxp[2 * np + p];
    double m = s.mass[p];
    double vv = v0 * v0 + v1 * v1 + v2 * v2;
    acc[0] = acc[0] + vv * m * 0.5;
    acc[1] = acc[1] + s.ie[p];
    acc[2] = acc[2] + m * v0;
    acc[3] = acc[3] + m * v1;
    acc[4] = acc[4] + m * v2;
    double a = fabs(v0);
    if (fabs(v1) > a) a = fabs(v1);
    if (fabs(v2) > a) a = fabs(v2);
    if (acc[5] < a) acc[5] = a;
  }
  for (int i = 0; i < kRedVals; ++i) sh[i][threadIdx.x] = acc[i];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      for (int i = 0; i < 5; ++i) sh[i][threadIdx.x] = sh[i][threadIdx.x] + sh[i][threadIdx.x + w];
      if (sh[5][threadIdx.x + w] > sh[5][threadIdx.x]) sh[5][threadIdx.x] = sh[5][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int i = 0; i < kRedVals; ++i) s.red_part[(long long)i * gridDim.x + blockIdx.x] = sh[i][0];
    __threadfence();
    unsigned done = atomicAdd(s.red_count, 1u);
    last = (done == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the last block combines the block partials: thread t takes blocks t,
  // t + blockDim, ... in order, then the same fixed tree as above
  double tot[kRedVals] = {0, 0, 0, 0, 0, 0};
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
    for (int i = 0; i < 5; ++i) tot[i] = tot[i] + s.red_part[(long long)i * gridDim.x + b];
    double mv = s.red_part[5LL * gridDim.x + b];
    if (tot[5] < mv) tot[5] = mv;
  }
  for (int i = 0; i < kRedVals; ++i) sh[i][threadIdx.x] = tot[i];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      for (int i = 0; i < 5; ++i) sh[i][threadIdx.x] = sh[i][threadIdx.x] + sh[i][threadIdx.x + w];
      if (sh[5][threadIdx.x + w] > sh[5][threadIdx.x]) sh[5][threadIdx.x] = sh[5][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  for (int i = 0; i < kRedVals; ++i) tot[i] = sh[i][0];
  DevScalars* sc = s.sc;
  if (mode & 1) {
    sc->ke_prev = sc->ke;
    sc->ke = tot[0];
    sc->ie = tot[1];
    sc->mom[0] = tot[2];
    sc->mom[1] = tot[3];
    sc->mom[2] = tot[4];
  }
  sc->max_vp = tot[5];
  *s.red_count = 0;
  if (mode & 2) {
    double dt = (double)1e6f;
    for (int m = 0; m < g.nb_mat; ++m) {
      const DevMaterial& mt = s.mats[m];
      if (mt.mat_type == 12) continue;
      double E = mt.young, nu = mt.poisson, ro = mt.density;
      double vv = sqrt(E * (1 - nu) / (1 + nu) / (1 - 2 * nu) / ro);
      if (mt.D > vv) vv = mt.D;
      if (mt.wavespd > vv) vv = mt.wavespd;
      vv = vv + tot[5];
      double t = g.dcell / vv;
      if (t < dt) dt = t;
    }
    sc->dt = dt * g.dtscale;
  }
}

// dynamicRelaxationDamping (Particle.f90:172-202)
template <class P>
__global__ void k_dr_damping(St<P> s, Geometry g) {
  const long long p = gtid();
  const DevScalars* sc = s.sc;
  bool damp = sc->istep != 0 && (sc->ke - sc->ke_prev <= 0.0);
  if (!damp || p >= g.np) return;
  const long long np = g.np;
  s.vxp[p] = 0;
  s.vxp[np + p] = 0;
  s.vxp[2 * np + p] = 0;
}

static __global__ void k_dr_finish(DevScalars* sc) {
  if (sc->istep != 0 && (sc->ke - sc->ke_prev <= 0.0)) sc->ke = 0;
}

}  // namespace mpm
