/*
 * mpm_oracle.c -- sequential CPU restatement of the MPM3D-F90 explicit step
 * (test infrastructure; see mpm_oracle.h).
 *
 * Build with -O2 -ffp-contract=off: every a*b+c of the reference is a
 * rounded multiply followed by a rounded add. Expressions are written in the
 * reference's left-to-right evaluation order; REAL(4) literals and REAL(4)
 * variables of the reference appear as float constants / float casts.
 *
 * Scope: the updated-Lagrangian step (MPM3D.f90:68-160) with linear, GIMP,
 * B-spline and SGMP shape functions, USF / USL / MUSL, material types 1-11
 * and EOS 1-4, the stress smoothing of SmoothStressbyGrid, grid components
 * with the Lagrangian contact of Lagr_NodContact, and the total Lagrangian
 * form (TLMPM, neo-Hookean). SGMP with several grid components is not
 * restated; orc_create rejects decks that ask for it.
 */
#include "mpm_oracle.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mpm3d_gpu.h"
#include "mpm_math.h"

typedef struct opart {
  double XX[3], Xp[3], Xo[3], VXp[3], FXp[3], XXN[3], XN[3];
  int inode;
  double VOL, VOL0, sig_y, SM, Seqv;
  double SDxx, SDyy, SDzz, SDxy, SDyz, SDxz;
  double Fp[3][3];
  double epeff, celsius_t;
  int failure, icell, centericell;
  double DMG, LT, ie, mass, cp, q;
  double Spre; /* smoothed pressure (Particle.f90:40) */
  double PK[9]; /* first Piola-Kirchhoff stress of TLMPM: xx yy zz yz xz xy zy zx yx (Particle.f90:29) */
} opart;

typedef struct onode {
  double Xg[3];
  int fix[3];
  int bd_type[3];
} onode;

typedef struct ogrid {
  double Mg, PXg[3], FXg[3];
  double Gpre, GV_all; /* stress smoothing (Grid.f90:41-43) */
  int mapped;
} ogrid;

typedef struct ocellp {
  double Cmg, Cpxg[3], Cfint[6], Cfext[3], Cvx[3], Cax[3], Co[6], Cw[3], CdeFp[3][3];
  double CGpre, CGV_all; /* stress smoothing (Grid.f90:62-64) */
  double CPKint[9];      /* TLMPM internal-force sums (Grid.f90:61) */
} ocellp;

struct orc {
  /* ParticleData (Particle.f90:67-107) */
  int64_t np;
  opart* pt;
  int nb_body;
  mpm_body* body;
  int nb_mat;
  mpm_material* mat;
  int MUSL, USL, USF, GIMP, Bspline, SGMP, QuasiLoad, QuasiDamp, UpdateVbyFp, Gravity, DR_DAMPING, SmoothStress;
  int TLMPM; /* total Lagrangian form (MPM3D.f90:161-244) */
  /* grid components and contact (Particle.f90:69-92, Grid.f90:66-80): grid
   * component c (0-based) holds nodes c*nb_gridnode .. ; a body's particles
   * map to its component (comID) when contact is on, to component 0 otherwise */
  int nb_component, contact, contact_type, normbody;
  double fricfa, tot_cont_for[3];
  double (*ndir)[3]; /* CP_list%ndir per component node */
  int istep;
  double DT, QuasiLoadTime, DampFactor, CurrentTime, EndTime, DTScale;
  double EngInternal, EngKinetic, EngKinetic_prev, Momentum[3];
  /* GridData (Grid.f90:74-119) */
  double SpanX[2], SpanY[2], SpanZ[2], DCell, CutOff;
  int FixS[6];
  int nb_gridnode, nb_centernode;
  int NumCell, NumCellx, NumCelly, NumCellz, NumCellxy;
  int CenterNumCell, CenterNumCellx, CenterNumCelly, CenterNumCellz, CenterNumCellxy;
  int NGx, NGy, NGz, NGxy;
  onode* node;
  ogrid* grid;
  double (*Cxg)[3];
  ocellp* cellp;
  int (*CellsNode)[8];
  int (*CenterCellNode)[8];
  double iJacobi, iJacobi4, iDCell;
  /* GridData module scratch */
  int nb_InflNode, centernb_InflNode;
  int InflNode[27], CenterInflNode[8];
  double rpg[27][3];
  double SHP[27], DNDX[27], DNDY[27], DNDZ[27];
  double CDNDX[8], CDNDY[8], CDNDZ[8];
  /* MaterialModel module state (Constitution.f90:24-74): persists across
   * particles and steps exactly as the module variables do. */
  int mid, etype_, mtype_;
  double young_, poisson_, yield0_, tangmod_, den0_, den_, vold, vol_, vol0_, dvol;
  double dinc[6], deF[3][3], sm, smold, sd[6], Fp[3][3], sig[6], sold[6], dsm, bqf;
  double seqv, epeff_, sig_y_, depeff, ratio, G2, K3, PlaMod, lamda, miu2, specheat_, tmprt;
  double iener, specen, ieinc, mu, rv, bfac, cp, DMG, oldDMG;
  double bq1, bq2;
  int64_t active_nodes;
  double (*f_log)(double);
  double (*f_exp)(double);
  double (*f_pow)(double, double);
  char err[256];
};

static const int SNX[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
static const int SNY[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
static const int SNZ[8] = {-1, -1, -1, -1, 1, 1, 1, 1};

static double proj_log(double x) { return mpm_log(x); }
static double proj_exp(double x) { return mpm_exp(x); }
static double proj_pow(double x, double y) { return mpm_pow(x, y); }

static int oerr(orc* o, int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(o->err, sizeof o->err, fmt, ap);
  va_end(ap);
  return code;
}

/* ====================================================================
 * Grid.f90: cell location and shape functions
 * ==================================================================== */

/* InWhichCell, Grid.f90:123-155 */
static int in_which_cell(const orc* o, const double x[3]) {
  if (x[0] < o->SpanX[0] || x[0] > o->SpanX[1] || x[1] < o->SpanY[0] || x[1] > o->SpanY[1] ||
      x[2] < o->SpanZ[0] || x[2] > o->SpanZ[1])
    return -1;
  int ix = (int)((x[0] - o->SpanX[0]) / o->DCell) + 1;
  int iy = (int)((x[1] - o->SpanY[0]) / o->DCell) + 1;
  int iz = (int)((x[2] - o->SpanZ[0]) / o->DCell) + 1;
  int c = (iz - 1) * o->NumCellxy + (iy - 1) * o->NumCellx + ix;
  if (c > o->NumCell || c <= 0) c = -1;
  return c;
}

/* CenterInWhichCell, Grid.f90:157-190 (no span test) */
static int center_in_which_cell(const orc* o, const double x[3]) {
  double h2 = o->DCell / 2.0;
  int ix = (int)((x[0] - o->SpanX[0] - h2) / o->DCell) + 1;
  int iy = (int)((x[1] - o->SpanY[0] - h2) / o->DCell) + 1;
  int iz = (int)((x[2] - o->SpanZ[0] - h2) / o->DCell) + 1;
  int c = (iz - 1) * o->CenterNumCellxy + (iy - 1) * o->CenterNumCellx + ix;
  if (c > o->CenterNumCell || c <= 0) c = -1;
  return c;
}

/* SGNShape, Grid.f90:434-458 */
static void sg_nshape(orc* o, const double xxn[3]) {
  for (int i = 0; i < 8; ++i) {
    double sx = (double)SNX[i] * xxn[0] + 1.0;
    double sy = (double)SNY[i] * xxn[1] + 1.0;
    double sz = (double)SNZ[i] * xxn[2] + 1.0;
    o->SHP[i] = sx * sy * sz * 0.125;
  }
}

/* NShape, Grid.f90:461-501 (values do not depend on ider) */
static void nshape(orc* o, const double XN[3]) {
  for (int i = 0; i < 8; ++i) {
    double sx = (double)SNX[i] * XN[0] + 1.0;
    double sy = (double)SNY[i] * XN[1] + 1.0;
    double sz = (double)SNZ[i] * XN[2] + 1.0;
    o->SHP[i] = sx * sy * sz * 0.125;
    o->DNDX[i] = (double)SNX[i] * sy * sz * o->iJacobi4;
    o->DNDY[i] = (double)SNY[i] * sx * sz * o->iJacobi4;
    o->DNDZ[i] = (double)SNZ[i] * sx * sy * o->iJacobi4;
  }
}

/* CNShape(2), Grid.f90:503-544: derivatives at the cell centre */
static void cnshape(orc* o) {
  for (int i = 0; i < 8; ++i) {
    double sx = (double)SNX[i] * 0.0 + 1.0;
    double sy = (double)SNY[i] * 0.0 + 1.0;
    double sz = (double)SNZ[i] * 0.0 + 1.0;
    o->CDNDX[i] = (double)SNX[i] * sy * sz * o->iJacobi4;
    o->CDNDY[i] = (double)SNY[i] * sx * sz * o->iJacobi4;
    o->CDNDZ[i] = (double)SNZ[i] * sx * sy * o->iJacobi4;
  }
}

static int node_valid(const orc* o, int n) { return n <= o->nb_gridnode && n > 0; }

/* first node of body b's grid component (comID when contact is on) */
static int64_t comp_base(const orc* o, int b) {
  return o->contact ? (int64_t)(o->body[b].comID - 1) * o->nb_gridnode : 0;
}
static int64_t all_nodes(const orc* o) { return (int64_t)o->nb_gridnode * o->nb_component; }

/* NShape_GIMP, Grid.f90:546-599 */
static void nshape_gimp(orc* o) {
  for (int i = 0; i < o->nb_InflNode; ++i) {
    if (!node_valid(o, o->InflNode[i])) continue; /* SHP(i) keeps its old value */
    double sh[3], dn[3];
    for (int j = 0; j < 3; ++j) {
      double rr = o->rpg[i][j];
      double r = fabs(rr);
      double sg = copysign(1.0, rr); /* sign(1d0, rr) */
      if (r < 0.25) {
        sh[j] = (7 - 16 * r * r) * 0.125;
        dn[j] = -(4 * rr);
      } else if (r < 0.75) {
        sh[j] = 1 - r;
        dn[j] = -sg;
      } else if (r < 1.25) {
        double t = (5 - 4 * r) * 0.25;
        sh[j] = t * t;
        dn[j] = 2 * rr - sg * 2.5;
      } else {
        sh[j] = 0.0;
        dn[j] = 0.0;
      }
    }
    o->SHP[i] = sh[0] * sh[1] * sh[2];
    o->DNDX[i] = dn[0] * sh[1] * sh[2] * o->iDCell;
    o->DNDY[i] = sh[0] * dn[1] * sh[2] * o->iDCell;
    o->DNDZ[i] = sh[0] * sh[1] * dn[2] * o->iDCell;
  }
}

/* FindInflNode, Grid.f90:602-849. Influence nodes of a cpGIMP particle: the 8
 * cell corners plus the node layers on the side(s) of the cell quarter the
 * particle lies in. Node ids are 1-based flat ids; the +-1 / +-NGx / +-NGxy
 * offsets are applied to flat ids exactly as the reference does. */
static void find_infl_node(orc* o, const opart* p, int icell) {
  int* N = o->InflNode;
  for (int i = 0; i < 8; ++i) {
    N[i] = o->CellsNode[icell - 1][i];
    const double* xg = o->node[N[i] - 1].Xg;
    for (int j = 0; j < 3; ++j) o->rpg[i][j] = (p->Xp[j] - xg[j]) * o->iDCell;
  }
  const double rx = o->rpg[0][0], ry = o->rpg[0][1], rz = o->rpg[0][2];
  const int NGx = o->NGx, NGxy = o->NGxy;
  /* N[] below uses 0-based slots: slot k is the reference's InflNode(k+1) */
  if (rz < 0.25 || rz > 0.75) {
    if (rz < 0.25) {
      N[8] = N[0] - NGxy; N[9] = N[1] - NGxy; N[10] = N[2] - NGxy; N[11] = N[3] - NGxy;
    } else {
      N[8] = N[4] + NGxy; N[9] = N[5] + NGxy; N[10] = N[6] + NGxy; N[11] = N[7] + NGxy;
    }
    if (ry < 0.25) {
      N[12] = N[8] - NGx; N[13] = N[9] - NGx; N[14] = N[0] - NGx;
      N[15] = N[1] - NGx; N[16] = N[4] - NGx; N[17] = N[5] - NGx;
      if (rx < 0.25) {
        N[18] = N[0] - 1; N[19] = N[3] - 1; N[20] = N[4] - 1; N[21] = N[7] - 1; N[22] = N[8] - 1;
        N[23] = N[11] - 1; N[24] = N[12] - 1; N[25] = N[14] - 1; N[26] = N[16] - 1;
        o->nb_InflNode = 27;
      } else if (rx > 0.75) {
        N[18] = N[1] + 1; N[19] = N[2] + 1; N[20] = N[5] + 1; N[21] = N[6] + 1; N[22] = N[9] + 1;
        N[23] = N[10] + 1; N[24] = N[13] + 1; N[25] = N[15] + 1; N[26] = N[17] + 1;
        o->nb_InflNode = 27;
      } else {
        o->nb_InflNode = 18;
      }
    } else if (ry > 0.75) {
      N[12] = N[10] + NGx; N[13] = N[11] + NGx; N[14] = N[2] + NGx;
      N[15] = N[3] + NGx; N[16] = N[6] + NGx; N[17] = N[7] + NGx;
      if (rx < 0.25) {
        N[18] = N[0] - 1; N[19] = N[3] - 1; N[20] = N[4] - 1; N[21] = N[7] - 1; N[22] = N[8] - 1;
        N[23] = N[11] - 1; N[24] = N[13] - 1; N[25] = N[15] - 1; N[26] = N[17] - 1;
        o->nb_InflNode = 27;
      } else if (rx > 0.75) {
        N[18] = N[1] + 1; N[19] = N[2] + 1; N[20] = N[5] + 1; N[21] = N[6] + 1; N[22] = N[9] + 1;
        N[23] = N[10] + 1; N[24] = N[12] + 1; N[25] = N[14] + 1; N[26] = N[16] + 1;
        o->nb_InflNode = 27;
      } else {
        o->nb_InflNode = 18;
      }
    } else {
      if (rx < 0.25) {
        N[12] = N[8] - 1; N[13] = N[11] - 1; N[14] = N[0] - 1;
        N[15] = N[3] - 1; N[16] = N[4] - 1; N[17] = N[7] - 1;
        o->nb_InflNode = 18;
      } else if (rx > 0.75) {
        N[12] = N[9] + 1; N[13] = N[10] + 1; N[14] = N[1] + 1;
        N[15] = N[2] + 1; N[16] = N[5] + 1; N[17] = N[6] + 1;
        o->nb_InflNode = 18;
      } else {
        o->nb_InflNode = 12;
      }
    }
  } else {
    if (ry < 0.25) {
      N[8] = N[0] - NGx; N[9] = N[1] - NGx; N[10] = N[4] - NGx; N[11] = N[5] - NGx;
      if (rx < 0.25) {
        N[12] = N[0] - 1; N[13] = N[3] - 1; N[14] = N[4] - 1;
        N[15] = N[7] - 1; N[16] = N[8] - 1; N[17] = N[10] - 1;
        o->nb_InflNode = 18;
      } else if (rx > 0.75) {
        N[12] = N[1] + 1; N[13] = N[2] + 1; N[14] = N[5] + 1;
        N[15] = N[6] + 1; N[16] = N[9] + 1; N[17] = N[11] + 1;
        o->nb_InflNode = 18;
      } else {
        o->nb_InflNode = 12;
      }
    } else if (ry > 0.75) {
      N[8] = N[2] + NGx; N[9] = N[3] + NGx; N[10] = N[6] + NGx; N[11] = N[7] + NGx;
      if (rx < 0.25) {
        N[12] = N[0] - 1; N[13] = N[3] - 1; N[14] = N[4] - 1;
        N[15] = N[7] - 1; N[16] = N[9] - 1; N[17] = N[11] - 1;
        o->nb_InflNode = 18;
      } else if (rx > 0.75) {
        N[12] = N[1] + 1; N[13] = N[2] + 1; N[14] = N[5] + 1;
        N[15] = N[6] + 1; N[16] = N[8] + 1; N[17] = N[10] + 1;
        o->nb_InflNode = 18;
      } else {
        o->nb_InflNode = 12;
      }
    } else {
      if (rx < 0.25) {
        N[8] = N[0] - 1; N[9] = N[3] - 1; N[10] = N[4] - 1; N[11] = N[7] - 1;
        o->nb_InflNode = 12;
      } else if (rx > 0.75) {
        N[8] = N[1] + 1; N[9] = N[2] + 1; N[10] = N[5] + 1; N[11] = N[6] + 1;
        o->nb_InflNode = 12;
      } else {
        o->nb_InflNode = 8;
      }
    }
  }
  for (int i = 8; i < o->nb_InflNode; ++i) {
    for (int j = 0; j < 3; ++j) {
      double d = node_valid(o, N[i]) ? p->Xp[j] - o->node[N[i] - 1].Xg[j] : 100.0;
      o->rpg[i][j] = d * o->iDCell;
    }
  }
}

/* BFindInflNode, Grid.f90:852-895 */
static void bfind_infl_node(orc* o, int icell) {
  int* N = o->InflNode;
  for (int i = 0; i < 8; ++i) N[i] = o->CellsNode[icell - 1][i];
  const int NGx = o->NGx, NGxy = o->NGxy;
  N[8] = N[0] - NGxy; N[9] = N[1] - NGxy; N[10] = N[2] - NGxy; N[11] = N[3] - NGxy;
  N[12] = N[8] - NGx; N[13] = N[9] - NGx; N[14] = N[0] - NGx;
  N[15] = N[1] - NGx; N[16] = N[4] - NGx; N[17] = N[5] - NGx;
  N[18] = N[0] - 1; N[19] = N[3] - 1; N[20] = N[4] - 1; N[21] = N[7] - 1; N[22] = N[8] - 1;
  N[23] = N[11] - 1; N[24] = N[12] - 1; N[25] = N[14] - 1; N[26] = N[16] - 1;
  o->nb_InflNode = 27;
}

/* NShape_Bspline, Grid.f90:898-1049. Weights are products of the 1-D quadratic
 * B-spline pieces sh(1..3, dim); the REAL(4) literals 0.2 and 0.4 enter as
 * float constants. */
static void nshape_bspline(orc* o, const opart* p) {
  const double* xg = o->node[o->InflNode[0] - 1].Xg;
  const double c02 = (double)0.2f, c04 = (double)0.4f;
  double sh[3][3], dn[3][3];
  for (int d = 0; d < 3; ++d) {
    double r = (p->Xp[d] - xg[d]) * o->iDCell * c02 + c04;
    double a = 3 - 5 * r;
    double b = 5 * r - 2;
    sh[0][d] = 0.5 * (a * a);
    sh[1][d] = -(25 * (r * r)) + 25 * r - 5.5;
    sh[2][d] = 0.5 * (b * b);
    dn[0][d] = (5 * r - 3) * 5 * c02 * o->iDCell;
    dn[1][d] = (-(50 * r) + 25) * c02 * o->iDCell;
    dn[2][d] = (5 * r - 2) * 5 * c02 * o->iDCell;
  }
  /* slot -> (x piece, y piece, z piece), each 0:lower 1:own 2:upper */
  static const int PX[27] = {1, 2, 2, 1, 1, 2, 2, 1, 1, 2, 2, 1, 1, 2, 1, 2, 1, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  static const int PY[27] = {1, 1, 2, 2, 1, 1, 2, 2, 1, 1, 2, 2, 0, 0, 0, 0, 0, 0, 1, 2, 1, 2, 1, 2, 0, 0, 0};
  static const int PZ[27] = {1, 1, 1, 1, 2, 2, 2, 2, 0, 0, 0, 0, 0, 0, 1, 1, 2, 2, 1, 1, 2, 2, 0, 0, 0, 1, 2};
  for (int k = 0; k < 27; ++k) {
    int a = PX[k], b = PY[k], c = PZ[k];
    o->SHP[k] = sh[a][0] * sh[b][1] * sh[c][2];
    o->DNDX[k] = dn[a][0] * sh[b][1] * sh[c][2];
    o->DNDY[k] = sh[a][0] * dn[b][1] * sh[c][2];
    o->DNDZ[k] = sh[a][0] * sh[b][1] * dn[c][2];
  }
}

/* shape functions of particle p in its cell (the GIMP / B-spline / linear
 * selection repeated in every particle loop of update_step.f90) */
static void particle_shape(orc* o, const opart* p, int icell) {
  for (int i = 0; i < 8; ++i) o->InflNode[i] = o->CellsNode[icell - 1][i];
  if (o->GIMP) {
    find_infl_node(o, p, icell);
    nshape_gimp(o);
  } else if (o->Bspline) {
    bfind_infl_node(o, icell);
    nshape_bspline(o, p);
  } else {
    o->nb_InflNode = 8;
    nshape(o, p->XN);
  }
}

/* AuxiliaryGridSHP, Grid.f90:193-220 */
static void aux_grid_shp(const double XN[3], const double XXN[3], const int pt[3], double out[3]) {
  for (int i = 0; i < 3; ++i) {
    if (pt[i] != 0)
      out[i] = XN[i] < 0 ? 1 + 2 * XN[i] : 2 * XN[i] - 1;
    else
      out[i] = XXN[i];
  }
}

/* ====================================================================
 * Set-up: Initial (DataIn.f90:1211-1267), SetGridData (Grid.f90:222-418),
 * SetDT (DataIn.f90:1269-1297)
 * ==================================================================== */

static int set_grid_data(orc* o) {
  double spx = o->SpanX[1] - o->SpanX[0];
  double spy = o->SpanY[1] - o->SpanY[0];
  double spz = o->SpanZ[1] - o->SpanZ[0];
  if (o->DCell == 0) return oerr(o, MPM_ERR_ARG, "DCell must be defined");
  if (spx <= 0 || spy <= 0 || spz <= 0) return oerr(o, MPM_ERR_ARG, "spans must be defined");
  o->NumCellx = (int)(spx / o->DCell + 0.5);
  o->NumCelly = (int)(spy / o->DCell + 0.5);
  o->NumCellz = (int)(spz / o->DCell + 0.5);
  o->CenterNumCellx = o->NumCellx - 1;
  o->CenterNumCelly = o->NumCelly - 1;
  o->CenterNumCellz = o->NumCellz - 1;
  if (o->CenterNumCellx == 0) o->CenterNumCellx = 1;
  if (o->CenterNumCelly == 0) o->CenterNumCelly = 1;
  if (o->CenterNumCellz == 0) o->CenterNumCellz = 1;
  o->SpanX[1] = o->SpanX[0] + o->NumCellx * o->DCell;
  o->SpanY[1] = o->SpanY[0] + o->NumCelly * o->DCell;
  o->SpanZ[1] = o->SpanZ[0] + o->NumCellz * o->DCell;
  o->NumCellxy = o->NumCellx * o->NumCelly;
  o->CenterNumCellxy = o->CenterNumCellx * o->CenterNumCelly;
  o->NumCell = o->NumCellxy * o->NumCellz;
  o->CenterNumCell = o->CenterNumCellxy * o->CenterNumCellz;
  o->nb_centernode = o->NumCell;
  o->NGx = o->NumCellx + 1;
  o->NGy = o->NumCelly + 1;
  o->NGz = o->NumCellz + 1;
  o->NGxy = o->NGx * o->NGy;
  o->nb_gridnode = o->NGxy * o->NGz;

  o->node = (onode*)calloc((size_t)o->nb_gridnode, sizeof(onode));
  o->grid = (ogrid*)calloc((size_t)o->nb_gridnode * (size_t)o->nb_component, sizeof(ogrid));
  if (o->contact) {
    o->ndir = (double(*)[3])calloc((size_t)o->nb_gridnode * (size_t)o->nb_component, sizeof(double[3]));
    if (!o->ndir) return oerr(o, MPM_ERR_OOM, "out of memory");
  }
  o->Cxg = (double(*)[3])calloc((size_t)o->NumCell, sizeof(double[3]));
  o->CellsNode = (int(*)[8])calloc((size_t)o->NumCell, sizeof(int[8]));
  if (!o->node || !o->grid || !o->Cxg || !o->CellsNode) return oerr(o, MPM_ERR_OOM, "out of memory");
  if (o->SGMP) {
    o->cellp = (ocellp*)calloc((size_t)o->NumCell, sizeof(ocellp));
    o->CenterCellNode = (int(*)[8])calloc((size_t)o->CenterNumCell, sizeof(int[8]));
    if (!o->cellp || !o->CenterCellNode) return oerr(o, MPM_ERR_OOM, "out of memory");
  }
  const int* F = o->FixS;
  const int NGx = o->NGx, NGy = o->NGy, NGz = o->NGz;
  for (int iz = 1; iz <= NGz; ++iz)
    for (int iy = 1; iy <= NGy; ++iy)
      for (int ix = 1; ix <= NGx; ++ix) {
        int i = (iz - 1) * o->NGxy + (iy - 1) * NGx + ix;
        onode* nd = &o->node[i - 1];
        nd->Xg[0] = (ix - 1) * o->DCell + o->SpanX[0];
        nd->Xg[1] = (iy - 1) * o->DCell + o->SpanY[0];
        nd->Xg[2] = (iz - 1) * o->DCell + o->SpanZ[0];
        if (ix == 1 && F[0] != 0) nd->bd_type[0] = 1;
        if (ix == NGx && F[1] != 0) nd->bd_type[0] = 2;
        if (iy == 1 && F[2] != 0) nd->bd_type[1] = 1;
        if (iy == NGy && F[3] != 0) nd->bd_type[1] = 2;
        if (iz == 1 && F[4] != 0) nd->bd_type[2] = 1;
        if (iz == NGz && F[5] != 0) nd->bd_type[2] = 2;
        if (o->SGMP) {
          if (ix == 2 && F[0] != 0) nd->bd_type[0] = 1;
          if (ix == NGx - 1 && F[1] != 0) nd->bd_type[0] = 2;
          if (iy == 2 && F[2] != 0) nd->bd_type[1] = 1;
          if (iy == NGy - 1 && F[3] != 0) nd->bd_type[1] = 2;
          if (iz == 2 && F[4] != 0) nd->bd_type[2] = 1;
          if (iz == NGz - 1 && F[5] != 0) nd->bd_type[2] = 2;
        }
        int lox = (ix == 1 || ix == 2), hix = (ix == NGx || ix == NGx - 1);
        int loy = (iy == 1 || iy == 2), hiy = (iy == NGy || iy == NGy - 1);
        int loz = (iz == 1 || iz == 2), hiz = (iz == NGz || iz == NGz - 1);
        if (o->Bspline || o->GIMP || o->SGMP) {
          if ((lox && F[0] == 1) || (hix && F[1] == 1) || (loy && F[2] == 1) || (hiy && F[3] == 1) ||
              (loz && F[4] == 1) || (hiz && F[5] == 1))
            nd->fix[0] = nd->fix[1] = nd->fix[2] = 1;
          if ((lox && F[0] == 2) || (hix && F[1] == 2)) nd->fix[0] = 1;
          if ((loy && F[2] == 2) || (hiy && F[3] == 2)) nd->fix[1] = 1;
          if ((loz && F[4] == 2) || (hiz && F[5] == 2)) nd->fix[2] = 1;
        }
        if ((ix == 1 && F[0] == 1) || (ix == NGx && F[1] == 1) || (iy == 1 && F[2] == 1) ||
            (iy == NGy && F[3] == 1) || (iz == 1 && F[4] == 1) || (iz == NGz && F[5] == 1))
          nd->fix[0] = nd->fix[1] = nd->fix[2] = 1;
        if ((ix == 1 && F[0] == 2) || (ix == NGx && F[1] == 2)) nd->fix[0] = 1;
        if ((iy == 1 && F[2] == 2) || (iy == NGy && F[3] == 2)) nd->fix[1] = 1;
        if ((iz == 1 && F[4] == 2) || (iz == NGz && F[5] == 2)) nd->fix[2] = 1;
      }
  for (int iz = 1; iz <= o->NumCellz; ++iz)
    for (int iy = 1; iy <= o->NumCelly; ++iy)
      for (int ix = 1; ix <= o->NumCellx; ++ix) {
        int i = (iz - 1) * o->NumCellxy + (iy - 1) * o->NumCellx + ix;
        int n1 = (iz - 1) * o->NGxy + (iy - 1) * NGx + ix;
        int n5 = n1 + o->NGxy;
        int* c = o->CellsNode[i - 1];
        c[0] = n1; c[1] = n1 + 1; c[2] = n1 + 1 + NGx; c[3] = n1 + NGx;
        c[4] = n5; c[5] = n5 + 1; c[6] = n5 + 1 + NGx; c[7] = n5 + NGx;
        for (int d = 0; d < 3; ++d) o->Cxg[i - 1][d] = o->node[n1 - 1].Xg[d] + o->DCell / 2.0;
      }
  if (o->SGMP) {
    for (int iz = 1; iz <= o->CenterNumCellz; ++iz)
      for (int iy = 1; iy <= o->CenterNumCelly; ++iy)
        for (int ix = 1; ix <= o->CenterNumCellx; ++ix) {
          int i = (iz - 1) * o->CenterNumCellxy + (iy - 1) * o->CenterNumCellx + ix;
          int c1 = (iz - 1) * o->NumCellxy + (iy - 1) * o->NumCellx + ix;
          int c5 = c1 + o->NumCellxy;
          int* c = o->CenterCellNode[i - 1];
          c[0] = c1; c[1] = c1 + 1; c[2] = c1 + 1 + o->NumCellx; c[3] = c1 + o->NumCellx;
          c[4] = c5; c[5] = c5 + 1; c[6] = c5 + 1 + o->NumCellx; c[7] = c5 + o->NumCellx;
        }
  }
  o->iJacobi = 2.0 / o->DCell;
  o->iJacobi4 = o->iJacobi * 0.125;
  o->iDCell = 1.0 / o->DCell;
  return MPM_OK;
}

static void initial(orc* o, const mpm_deck* d) {
  for (int b = 0; b < o->nb_body; ++b) {
    const mpm_body* bd = &o->body[b];
    for (int64_t i = bd->par_begin; i < bd->par_end; ++i) {
      opart* pt = &o->pt[i];
      mpm_material* m = &o->mat[bd->mat - 1];
      int mtype = m->mat_type;
      if (mtype == 12) continue;
      pt->VOL = pt->mass / m->density;
      pt->VOL0 = pt->VOL;
      pt->sig_y = m->yield0;
      pt->ie = m->cEos[9] * pt->VOL;
      if (mtype == 1 || mtype == 11) {
        double E = m->young, nu = m->poisson, ro = m->density;
        pt->cp = sqrt(E * (1 - nu) / (1 + nu) / (1 - 2 * nu) / ro);
      }
      if (mtype == 9) {
        pt->cp = m->wavespd;
        m->cEos[0] = m->wavespd;
      }
      pt->LT = (double)10e6f;
      for (int j = 0; j < d->n_deto; ++j) {
        double dx = pt->Xp[0] - d->deto[j][0];
        double dy = pt->Xp[1] - d->deto[j][1];
        double dz = pt->Xp[2] - d->deto[j][2];
        float temp = (float)(sqrt(dx * dx + dy * dy + dz * dz) / m->D);
        if ((double)temp < pt->LT) pt->LT = (double)temp;
      }
    }
  }
}

static void set_dt(orc* o) {
  o->DT = (double)1.0e6f;
  for (int m = 0; m < o->nb_mat; ++m) {
    const mpm_material* mt = &o->mat[m];
    if (mt->mat_type == 12) continue;
    double E = mt->young, nu = mt->poisson, ro = mt->density;
    double cp = sqrt(E * (1 - nu) / (1 + nu) / (1 - 2 * nu) / ro);
    if (mt->D > cp) cp = mt->D;
    if (mt->wavespd > cp) cp = mt->wavespd;
    double t = o->DCell / cp;
    if (t < o->DT) o->DT = t;
  }
  o->DT = o->DT * o->DTScale;
}

/* ====================================================================
 * Particle.f90: energies and dynamic-relaxation damping
 * ==================================================================== */

/* calcEnergy, Particle.f90:204-230 */
static void calc_energy(orc* o) {
  o->EngKinetic_prev = o->EngKinetic;
  o->EngKinetic = 0.0;
  o->EngInternal = 0.0;
  o->Momentum[0] = o->Momentum[1] = o->Momentum[2] = 0.0;
  for (int64_t p = 0; p < o->np; ++p) {
    const opart* pt = &o->pt[p];
    double mp = pt->mass;
    double vv = pt->VXp[0] * pt->VXp[0] + pt->VXp[1] * pt->VXp[1] + pt->VXp[2] * pt->VXp[2];
    double dke = vv * mp * 0.5;
    o->EngKinetic = o->EngKinetic + dke;
    o->EngInternal = o->EngInternal + pt->ie;
    for (int c = 0; c < 3; ++c) o->Momentum[c] = o->Momentum[c] + mp * pt->VXp[c];
  }
}

/* dynamicRelaxationDamping, Particle.f90:172-202 */
static void dr_damping(orc* o) {
  if (o->istep == 0) {
    o->EngKinetic_prev = 0;
    return;
  }
  double dke = o->EngKinetic - o->EngKinetic_prev;
  if (dke <= 0.0) {
    for (int64_t p = 0; p < o->np; ++p) o->pt[p].VXp[0] = o->pt[p].VXp[1] = o->pt[p].VXp[2] = 0;
    o->EngKinetic = 0;
  }
}

/* ====================================================================
 * Constitution.f90: MaterialModel
 * ==================================================================== */

/* EquivalentStress, Constitution.f90:679-699: a default-REAL function */
static double equivalent_stress(const orc* o) {
  const double* sd = o->sd;
  double J2 = 0.5 * (sd[0] * sd[0] + sd[1] * sd[1] + sd[2] * sd[2]) + sd[3] * sd[3] + sd[4] * sd[4] +
              sd[5] * sd[5];
  J2 = J2 * 3.0;
  return (double)(float)sqrt(J2);
}

/* sigrot, Constitution.f90:527-575 (Jaumann rotation) */
static void sigrot(orc* o, const double vort[3]) {
  double* sig = o->sig;
  double q1 = 2.0 * sig[5] * vort[2];
  double q2 = 2.0 * sig[4] * vort[1];
  double q3 = 2.0 * sig[3] * vort[0];
  double rot[6];
  rot[0] = -q1 + q2;
  rot[1] = q1 - q3;
  rot[2] = -q2 + q3;
  rot[3] = vort[0] * (sig[1] - sig[2]) + vort[2] * sig[4] - vort[1] * sig[5];
  rot[4] = vort[1] * (sig[2] - sig[0]) + vort[0] * sig[5] - vort[2] * sig[3];
  rot[5] = vort[2] * (sig[0] - sig[1]) + vort[1] * sig[3] - vort[0] * sig[4];
  for (int i = 0; i < 6; ++i) sig[i] = sig[i] + rot[i];
  o->sm = (sig[0] + sig[1] + sig[2]) / 3.0;
  o->sd[0] = sig[0] - o->sm;
  o->sd[1] = sig[1] - o->sm;
  o->sd[2] = sig[2] - o->sm;
  o->sd[3] = sig[3];
  o->sd[4] = sig[4];
  o->sd[5] = sig[5];
}

/* elastic_devi, Constitution.f90:578-604 */
static void elastic_devi(orc* o) {
  const double* di = o->dinc;
  double dem = (di[0] + di[1] + di[2]) / 3.0;
  double G = 0.5 * o->G2;
  o->sd[0] = o->sd[0] + o->G2 * (di[0] - dem);
  o->sd[1] = o->sd[1] + o->G2 * (di[1] - dem);
  o->sd[2] = o->sd[2] + o->G2 * (di[2] - dem);
  o->sd[3] = o->sd[3] + G * di[3];
  o->sd[4] = o->sd[4] + G * di[4];
  o->sd[5] = o->sd[5] + G * di[5];
}

/* elastic_p, Constitution.f90:607-624 */
static void elastic_p(orc* o) {
  const double* di = o->dinc;
  double dem = (di[0] + di[1] + di[2]) / 3.0;
  o->dsm = o->K3 * dem;
  o->sm = o->sm + o->dsm;
}

/* bulkq, Constitution.f90:1543-1563 */
static void bulkq(orc* o) {
  const double* di = o->dinc;
  double dd = (di[0] + di[1] + di[2]) / o->DT;
  if (!(dd < 0.0)) dd = 0.0;
  o->bqf = o->den_ * o->DCell * o->DCell * o->bq1 * dd * dd - o->bq2 * o->den_ * o->DCell * o->cp * dd;
}

/* lieupd, Constitution.f90:627-646 (vavg is a default REAL) */
static void lieupd(orc* o) {
  const double* di = o->dinc;
  if (o->sm < 0) bulkq(o);
  o->ieinc = o->ieinc - 2.0 * o->bqf * (di[0] + di[1] + di[2]);
  float vavg = (float)(o->vol_ + o->vold);
  o->iener = o->iener + 0.25 * o->ieinc * (double)vavg;
}

/* hieupd, Constitution.f90:649-676 */
static void hieupd(orc* o, int failure) {
  const double* di = o->dinc;
  if (failure) {
    o->ieinc = o->dvol * (o->smold - 2.0 * o->bqf);
  } else {
    float vavg = (float)(o->vol_ + o->vold);
    double e = di[0] * (o->sold[0] + o->sd[0]) + di[1] * (o->sold[1] + o->sd[1]) +
               di[2] * (o->sold[2] + o->sd[2]) + di[3] * (o->sold[3] + o->sd[3]) +
               di[4] * (o->sold[4] + o->sd[4]) + di[5] * (o->sold[5] + o->sd[5]);
    o->ieinc = 0.25 * e * (double)vavg + o->dvol * (o->smold - 2.0 * o->bqf);
  }
  o->iener = o->iener + o->ieinc;
  o->specen = o->iener / o->vol0_;
}

static double sig_dot_dinc(const orc* o) {
  const double* s = o->sig;
  const double* d = o->dinc;
  return s[0] * d[0] + s[1] * d[1] + s[2] * d[2] + s[3] * d[3] + s[4] * d[4] + s[5] * d[5];
}

/* ieinc + (sd+sm).dinc evaluated left to right from ieinc */
static double add_stress_work(const orc* o, double acc) {
  const double* s = o->sd;
  const double* d = o->dinc;
  acc = acc + (s[0] + o->sm) * d[0];
  acc = acc + (s[1] + o->sm) * d[1];
  acc = acc + (s[2] + o->sm) * d[2];
  acc = acc + s[3] * d[3];
  acc = acc + s[4] * d[4];
  acc = acc + s[5] * d[5];
  return acc;
}

static void scale_sd(orc* o, double r) {
  for (int i = 0; i < 6; ++i) o->sd[i] = o->sd[i] * r;
}

/* M3DM1 elastic, Constitution.f90:702-724 */
static void m3dm1(orc* o) {
  o->ieinc = sig_dot_dinc(o);
  elastic_devi(o);
  elastic_p(o);
  o->seqv = equivalent_stress(o);
  o->ieinc = add_stress_work(o, o->ieinc);
}

/* M3DM2 elastic-perfectly plastic, Constitution.f90:885-923 */
static void m3dm2(orc* o) {
  o->ieinc = sig_dot_dinc(o);
  elastic_devi(o);
  o->seqv = equivalent_stress(o);
  if (o->seqv > o->yield0_) {
    o->depeff = (o->seqv - o->sig_y_) / (1.5 * o->G2);
    o->epeff_ = o->epeff_ + o->depeff;
    o->ratio = o->yield0_ / o->seqv;
    scale_sd(o, o->ratio);
    o->seqv = o->seqv * o->ratio;
  }
  elastic_p(o);
  o->ieinc = add_stress_work(o, o->ieinc);
}

/* M3DM3 isotropic hardening, Constitution.f90:926-966 */
static void m3dm3(orc* o) {
  o->ieinc = sig_dot_dinc(o);
  elastic_devi(o);
  o->seqv = equivalent_stress(o);
  if (o->seqv > o->sig_y_) {
    o->depeff = (o->seqv - o->sig_y_) / (1.5 * o->G2 + o->PlaMod);
    o->epeff_ = o->epeff_ + o->depeff;
    o->sig_y_ = o->sig_y_ + o->PlaMod * o->depeff;
    o->ratio = o->sig_y_ / o->seqv;
    scale_sd(o, o->ratio);
    o->seqv = o->seqv * o->ratio;
  }
  elastic_p(o);
  o->ieinc = add_stress_work(o, o->ieinc);
}

/* Johnson-Cook hardening modulus at epeff + 1e-4 (REAL literal) */
static void jc_plamod(orc* o, const mpm_material* m) {
  const double e4 = (double)0.0001f;
  o->epeff_ = o->epeff_ + e4;
  o->PlaMod = m->B_jc * m->n_jc * o->f_pow(o->epeff_, m->n_jc - 1);
  o->epeff_ = o->epeff_ - e4;
}

/* M3DM4 Johnson-Cook, Constitution.f90:969-1040 */
static void m3dm4(orc* o, const mpm_material* m) {
  o->ieinc = sig_dot_dinc(o);
  jc_plamod(o, m);
  elastic_devi(o);
  o->seqv = equivalent_stress(o);
  if (o->seqv > o->sig_y_) {
    o->depeff = (o->seqv - o->sig_y_) / (1.5 * o->G2 + o->PlaMod);
    o->epeff_ = o->epeff_ + o->depeff;
    double tstar = (o->tmprt - m->roomt) / (m->melt - m->roomt);
    double srate = o->depeff / m->epso / o->DT;
    if (srate < (double)0.001f) srate = (double)0.001f;
    o->sig_y_ = (o->yield0_ + m->B_jc * o->f_pow(o->epeff_, m->n_jc)) * (1 + m->C_jc * o->f_log(srate)) *
                (1 - o->f_pow(tstar, m->m_jc));
    if (o->sig_y_ > o->seqv) {
      o->epeff_ = o->epeff_ - o->depeff;
      o->depeff = 0.0;
    } else {
      o->ratio = o->sig_y_ / o->seqv;
      scale_sd(o, o->ratio);
      o->seqv = o->seqv * o->ratio;
    }
  }
  elastic_p(o);
  o->ieinc = add_stress_work(o, o->ieinc);
}

/* M3DM5 simplified Johnson-Cook, Constitution.f90:1043-1100 */
static void m3dm5(orc* o, const mpm_material* m) {
  jc_plamod(o, m);
  elastic_devi(o);
  o->seqv = equivalent_stress(o);
  if (o->seqv > o->sig_y_) {
    o->depeff = (o->seqv - o->sig_y_) / (1.5 * o->G2 + o->PlaMod);
    o->epeff_ = o->epeff_ + o->depeff;
    double srate = o->depeff / m->epso / o->DT;
    if (srate < (double)0.001f) srate = (double)0.001f;
    o->sig_y_ = (o->yield0_ + m->B_jc * o->f_pow(o->epeff_, m->n_jc)) * (1 + m->C_jc * o->f_log(srate));
    if (o->sig_y_ > o->seqv) {
      o->epeff_ = o->epeff_ - o->depeff;
      o->depeff = 0.0;
    } else {
      o->ratio = o->sig_y_ / o->seqv;
      scale_sd(o, o->ratio);
      o->seqv = o->seqv * o->ratio;
    }
  }
}

/* M3DM7 null material, Constitution.f90:1124-1142 (tri = 1/3*(...) with
 * integer 1/3 = 0) */
static void m3dm7(orc* o) {
  const double* d = o->dinc;
  const double DT = o->DT;
  for (int i = 0; i < 6; ++i) o->sd[i] = 0.0;
  double tri = 0.0 * (d[0] / DT + d[1] / DT + d[2] / DT);
  o->sd[0] = o->miu2 * (d[0] / DT - tri);
  o->sd[1] = o->miu2 * (d[1] / DT - tri);
  o->sd[2] = o->miu2 * (d[2] / DT - tri);
  o->sd[3] = 0.5 * o->miu2 * d[3] / DT;
  o->sd[4] = 0.5 * o->miu2 * d[4] / DT;
  o->sd[5] = 0.5 * o->miu2 * d[5] / DT;
}

/* M3DM8 Johnson-Cook with failure, Constitution.f90:1144-1212 */
static void m3dm8(orc* o, const mpm_material* m, int* failure) {
  jc_plamod(o, m);
  elastic_devi(o);
  o->seqv = equivalent_stress(o);
  if (o->seqv > o->sig_y_) {
    o->depeff = (o->seqv - o->sig_y_) / (1.5 * o->G2 + o->PlaMod);
    o->epeff_ = o->epeff_ + o->depeff;
    double tstar = (o->tmprt - m->roomt) / (m->melt - m->roomt);
    if (tstar > 1.0) {
      tstar = 1.0;
      *failure = 1;
    } else if (tstar < 0.0) {
      tstar = 0.0;
    }
    double srate = o->depeff / m->epso / o->DT;
    if (srate < (double)0.001f) srate = (double)0.001f;
    o->sig_y_ = (o->yield0_ + m->B_jc * o->f_pow(o->epeff_, m->n_jc)) * (1 + m->C_jc * o->f_log(srate)) *
                (1 - o->f_pow(tstar, m->m_jc));
    if (o->sig_y_ > o->seqv) {
      o->epeff_ = o->epeff_ - o->depeff;
      o->depeff = 0.0;
    } else {
      o->ratio = o->sig_y_ / o->seqv;
      scale_sd(o, o->ratio);
      o->seqv = o->seqv * o->ratio;
    }
  }
}

/* M3DM9 Drucker-Prager, Constitution.f90:1214-1330. sqrt(3.0), 1.0/3.0,
 * 2.0/9.0 and sqrt(2.0) are REAL constants. */
static void m3dm9(orc* o, const mpm_material* m) {
  const double sqrt3f = (double)sqrtf(3.0f);
  const double third_f = (double)(1.0f / 3.0f);
  const double twoninth_f = (double)(2.0f / 9.0f);
  const double sqrt2f = (double)sqrtf(2.0f);
  double Gmod = o->young_ / (2 * (1 + o->poisson_));
  double Kmod = o->young_ / (3 * (1 - 2 * o->poisson_));
  double qfai = m->q_fai, kfai = m->k_fai, qpsi = m->q_psi, tenf;
  o->ieinc = sig_dot_dinc(o);
  if (qfai == 0.0) {
    tenf = 0.0;
  } else {
    double tenf_max = kfai / qfai;
    tenf = m->ten_f < tenf_max ? m->ten_f : tenf_max;
  }
  elastic_devi(o);
  elastic_p(o);
  const double* sd = o->sd;
  double J2 = 0.5 * (sd[0] * sd[0] + sd[1] * sd[1] + sd[2] * sd[2]) + sd[3] * sd[3] + sd[4] * sd[4] +
              sd[5] * sd[5];
  double Tau = sqrt(J2);
  o->seqv = Tau * sqrt3f;
  double dpFi = Tau + qfai * o->sm - kfai;
  double dpsig = o->sm - tenf;
  if (dpsig < 0.0) {
    if (dpFi > 0.0) {
      double dlamd = dpFi / (Gmod + Kmod * qfai * qpsi);
      o->sm = o->sm - Kmod * qpsi * dlamd;
      double newTau = kfai - qfai * o->sm;
      o->ratio = newTau / Tau;
      scale_sd(o, o->ratio);
      o->seqv = o->seqv * o->ratio;
      o->depeff = dlamd * sqrt(third_f + twoninth_f * (qpsi * qpsi));
      o->epeff_ = o->epeff_ + o->depeff;
    }
  } else {
    double alphap = sqrt(1 + qfai * qfai) - qfai;
    double Taup = kfai - qfai * tenf;
    double dp_hfai = Tau - Taup - alphap * dpsig;
    if (dp_hfai > 0.0) {
      double dlamd = dpFi / (Gmod + Kmod * qfai * qpsi);
      o->sm = o->sm - Kmod * qpsi * dlamd;
      double newTau = kfai - qfai * o->sm;
      o->ratio = newTau / Tau;
      scale_sd(o, o->ratio);
      o->seqv = o->seqv * o->ratio;
      o->depeff = dlamd * sqrt(third_f + twoninth_f * (qpsi * qpsi));
      o->epeff_ = o->epeff_ + o->depeff;
    } else {
      double dlamd = (o->sm - tenf) / Kmod;
      o->sm = tenf;
      o->depeff = dlamd * third_f * sqrt2f;
      o->epeff_ = o->epeff_ + o->depeff;
    }
  }
  o->ieinc = add_stress_work(o, o->ieinc);
}

static double det3(const double F[3][3]) {
  return F[0][0] * F[1][1] * F[2][2] - F[0][0] * F[1][2] * F[2][1] - F[1][0] * F[0][1] * F[2][2] +
         F[1][0] * F[0][2] * F[2][1] + F[2][0] * F[0][1] * F[1][2] - F[2][0] * F[0][2] * F[1][1];
}

/* M3DM10 neo-Hookean, Constitution.f90:725-780 */
static void m3dm10(orc* o) {
  const double (*F)[3] = (const double (*)[3])o->Fp;
  double G = 0.5 * o->G2;
  double J = det3(o->Fp);
  double B[6];
  B[0] = F[0][0] * F[0][0] + F[0][1] * F[0][1] + F[0][2] * F[0][2] - 1.0;
  B[1] = F[1][0] * F[1][0] + F[1][1] * F[1][1] + F[1][2] * F[1][2] - 1.0;
  B[2] = F[2][0] * F[2][0] + F[2][1] * F[2][1] + F[2][2] * F[2][2] - 1.0;
  B[3] = F[0][0] * F[1][0] + F[0][1] * F[1][1] + F[0][2] * F[1][2];
  B[4] = F[1][0] * F[2][0] + F[1][1] * F[2][1] + F[1][2] * F[2][2];
  B[5] = F[0][0] * F[2][0] + F[0][1] * F[2][1] + F[0][2] * F[2][2];
  o->ieinc = sig_dot_dinc(o);
  double iJ = 1.0 / J;
  double lj = o->f_log(J);
  double* sig = o->sig;
  sig[0] = iJ * (G * B[0] + o->lamda * lj * 1.0);
  sig[1] = iJ * (G * B[1] + o->lamda * lj * 1.0);
  sig[2] = iJ * (G * B[2] + o->lamda * lj * 1.0);
  sig[3] = iJ * G * B[4];
  sig[4] = iJ * G * B[5];
  sig[5] = iJ * G * B[3];
  o->sm = (sig[0] + sig[1] + sig[2]) / 3.0;
  o->sd[0] = sig[0] - o->sm;
  o->sd[1] = sig[1] - o->sm;
  o->sd[2] = sig[2] - o->sm;
  o->sd[3] = sig[3];
  o->sd[4] = sig[4];
  o->sd[5] = sig[5];
  o->seqv = equivalent_stress(o);
  o->ieinc = add_stress_work(o, o->ieinc);
}

/* eos1 linear polynomial, Constitution.f90:1364-1405 (A, B, pnew, c0..c6 are
 * default REALs) */
static void eos1(orc* o, int failure) {
  const double* c = o->mat[o->mid - 1].cEos;
  float c0 = (float)c[0], c1 = (float)c[1], c2 = (float)c[2], c3 = (float)c[3];
  float c4 = (float)c[4], c5 = (float)c[5], c6 = (float)c[6];
  double mu = o->mu;
  float A = (float)((double)c0 + mu * ((double)c1 + mu * ((double)c2 + mu * (double)c3)));
  float B = (float)((double)c4 + mu * ((double)c5 + mu * (double)c6));
  hieupd(o, failure);
  float pnew = (float)(((double)A + (double)B * o->specen) / (1 + (double)B * o->dvol / o->vol0_));
  if (failure && pnew < 0) pnew = 0.0f;
  o->ieinc = o->ieinc - o->dvol * (double)pnew;
  o->iener = o->iener - o->dvol * (double)pnew;
  o->sm = -(double)pnew;
}

/* eos2 Mie-Gruneisen, Constitution.f90:1408-1455 */
static void eos2(orc* o, int failure) {
  const double* c = o->mat[o->mid - 1].cEos;
  float c1 = (float)c[0], c2 = (float)c[1], c3 = (float)c[2], c4 = (float)c[3], c5 = (float)c[4];
  double mu = o->mu;
  float A, B;
  if (mu > 0) {
    double t = ((double)c1 * mu + (double)c2 * (mu * mu) + (double)c3 * (mu * mu * mu)) *
               (1 - (double)c4 * mu * 0.5 / o->den_);
    A = (float)t;
    B = c5;
  } else {
    A = (float)((double)c1 * mu);
    B = 0.0f;
  }
  if (o->sm < 0) bulkq(o);
  hieupd(o, failure);
  float pnew = (float)(((double)A + (double)B * o->specen) / (1 + (double)B * o->dvol / o->vol0_));
  if (failure && pnew < 0) pnew = 0.0f;
  o->ieinc = o->ieinc - o->dvol * (double)pnew;
  o->iener = o->iener - o->dvol * (double)pnew;
  o->sm = -(double)pnew;
}

/* eos3 JWL, Constitution.f90:1458-1511 */
static void eos3(orc* o, int failure) {
  const double* c = o->mat[o->mid - 1].cEos;
  double c1 = c[0], c2 = c[1], r1 = c[2], r2 = c[3], w1 = c[4];
  double r1v = r1 * o->rv;
  double r2v = r2 * o->rv;
  double wr1v = c1 * w1 / r1v;
  double wr2v = c2 * w1 / r2v;
  double wdr1v = c1 - wr1v;
  double wdr2v = c2 - wr2v;
  double er1v = o->f_exp(-r1v);
  double er2v = o->f_exp(-r2v);
  double A = wdr1v * er1v + wdr2v * er2v + o->bqf;
  double B = w1 / o->rv;
  hieupd(o, failure);
  A = A * o->bfac;
  B = B * o->bfac;
  double pnew = (A + B * o->specen) / (1 + B * o->dvol / o->vol0_);
  if (failure && pnew < 0) pnew = 0.0;
  o->iener = o->iener - o->dvol * pnew;
  o->sm = -pnew;
}

/* eos4 weakly compressible, Constitution.f90:1513-1541 */
static void eos4(orc* o, int failure) {
  double c0 = o->mat[o->mid - 1].cEos[0];
  if (o->sm < 0) bulkq(o);
  hieupd(o, failure);
  double pnew = c0 * c0 * (o->den_ - o->den0_);
  if (failure && pnew < 0) pnew = 0.0;
  o->iener = o->iener - o->dvol * pnew;
  o->sm = -pnew;
}

/* seleos, Constitution.f90:1333-1361 */
static int seleos(orc* o, int failure) {
  switch (o->etype_) {
    case 1: eos1(o, failure); return MPM_OK;
    case 2: eos2(o, failure); return MPM_OK;
    case 3: eos3(o, failure); return MPM_OK;
    case 4: eos4(o, failure); return MPM_OK;
    default: return oerr(o, MPM_ERR_ARG, "material %d needs an EOS (seos)", o->mid);
  }
}

/* Constitution, Constitution.f90:79-368 */
static int constitution(orc* o, const double de[6], const double vort[3], int b, int64_t pidx,
                        const double deFp[3][3]) {
  opart* p = &o->pt[pidx];
  for (int i = 0; i < 6; ++i) o->dinc[i] = de[i];
  memcpy(o->deF, deFp, sizeof o->deF);
  o->vold = p->VOL;
  if (o->UpdateVbyFp) {
    memcpy(o->Fp, p->Fp, sizeof o->Fp);
    for (int i = 0; i < 3; ++i) {
      o->deF[i][i] = o->deF[i][i] + 1.0;
      o->Fp[i][i] = o->Fp[i][i] + 1.0;
    }
    double detF = det3(o->deF);
    p->VOL = o->vold * detF;
  } else {
    p->VOL = o->vold * (1 + de[0] + de[1] + de[2]);
  }
  o->vol_ = p->VOL;
  o->dvol = 0.5 * (o->vol_ - o->vold);
  o->mid = o->body[b].mat;
  const mpm_material* m = &o->mat[o->mid - 1];
  o->epeff_ = p->epeff;
  o->sig_y_ = p->sig_y;
  o->seqv = p->Seqv;
  double ltim = p->LT;
  o->tmprt = p->celsius_t;
  o->iener = p->ie;
  double mp_ = p->mass;
  int failure = p->failure;
  o->mtype_ = m->mat_type;
  o->etype_ = m->eos_type;
  o->miu2 = 2 * m->miu;
  o->young_ = m->young;
  o->poisson_ = m->poisson;
  o->yield0_ = m->yield0;
  o->tangmod_ = m->tangmod;
  o->den0_ = m->density;
  o->vol0_ = mp_ / o->den0_;
  o->den_ = mp_ / o->vol_;
  o->mu = o->den_ / o->den0_ - 1;
  o->rv = o->vol_ / o->vol0_;
  o->specen = o->iener / o->vol0_;
  o->DMG = p->DMG;
  o->oldDMG = o->DMG;
  o->young_ = o->young_ * (1.0 - o->DMG + 2.220446049250313e-16);
  o->G2 = o->young_ / (1 + o->poisson_);
  o->K3 = o->young_ / (1 - 2 * o->poisson_);
  o->lamda = (o->young_ * o->poisson_) / ((1 + o->poisson_) * (1 - 2 * o->poisson_));
  o->PlaMod = o->young_ * o->tangmod_ / (o->young_ - o->tangmod_);
  o->cp = p->cp;
  o->sm = p->SM;
  o->smold = p->SM;
  o->sd[0] = p->SDxx; o->sd[1] = p->SDyy; o->sd[2] = p->SDzz;
  o->sd[3] = p->SDyz; o->sd[4] = p->SDxz; o->sd[5] = p->SDxy;
  o->sig[0] = o->sd[0] + o->sm;
  o->sig[1] = o->sd[1] + o->sm;
  o->sig[2] = o->sd[2] + o->sm;
  o->sig[3] = o->sd[3];
  o->sig[4] = o->sd[4];
  o->sig[5] = o->sd[5];
  memcpy(o->sold, o->sd, sizeof o->sold);
  o->bqf = 0.0;
  const double epf_eps = (double)0.0000001f;
  int st = MPM_OK;
  switch (o->mtype_) {
    case 1:
      sigrot(o, vort); m3dm1(o); lieupd(o);
      break;
    case 2:
      sigrot(o, vort); m3dm2(o); lieupd(o);
      break;
    case 3:
      sigrot(o, vort); m3dm3(o); lieupd(o);
      break;
    case 4: {
      const double* di = o->dinc;
      sigrot(o, vort);
      m3dm4(o, m);
      if (o->sm < 0) bulkq(o);
      o->ieinc = o->ieinc - 2.0 * o->bqf * (di[0] + di[1] + di[2]);
      lieupd(o);
      o->specheat_ = m->specheat;
      p->celsius_t = p->celsius_t + o->seqv * o->depeff / o->den_ / o->specheat_;
      break;
    }
    case 5:
      sigrot(o, vort); m3dm5(o, m); st = seleos(o, failure);
      break;
    case 6:
      sigrot(o, vort);
      if (!p->failure) {
        m3dm5(o, m);
        st = seleos(o, failure);
        if (o->epeff_ > m->epf) {
          o->epeff_ = m->epf + epf_eps;
          failure = 1;
        }
        if (failure && o->sm < 0) {
          o->sm = 0.0; o->bqf = 0.0; p->VOL = o->vold;
        }
        if (failure) {
          for (int i = 0; i < 6; ++i) o->sd[i] = 0.0;
          o->iener = o->iener - o->ieinc + o->dvol * (o->smold + o->sm - 2 * o->bqf);
        }
        p->failure = failure;
      } else {
        m3dm7(o); st = seleos(o, failure);
      }
      break;
    case 7:
      sigrot(o, vort);
      if (!p->failure) {
        m3dm8(o, m, &failure);
        st = seleos(o, failure);
        if (o->epeff_ > m->epf) {
          o->epeff_ = m->epf + epf_eps;
          o->DMG = 1.0;
          failure = 1;
        } else {
          o->DMG = o->oldDMG + o->depeff / m->epf;
          if (o->DMG >= 1.0) o->DMG = 1.0;
          double r = (1 - o->DMG) / (1 - o->oldDMG);
          scale_sd(o, r);
          if (fabs(o->DMG - 1.0) < (double)1e-5f) failure = 1;
        }
        if (failure && o->sm < 0) {
          o->sm = 0.0; o->bqf = 0.0; p->VOL = o->vold;
        }
        if (failure) {
          for (int i = 0; i < 6; ++i) o->sd[i] = 0.0;
          o->iener = o->iener - o->ieinc + o->dvol * (o->smold + o->sm - 2 * o->bqf);
        }
        p->failure = failure;
        o->specheat_ = m->specheat;
        p->celsius_t = p->celsius_t + o->seqv * o->depeff / o->den_ / o->specheat_;
      } else {
        m3dm7(o); st = seleos(o, failure);
      }
      break;
    case 8:
      o->bfac = (o->CurrentTime > ltim) ? 1.0 : 0.0; /* M3DM6 */
      st = seleos(o, failure);
      break;
    case 9:
      m3dm7(o); st = seleos(o, failure);
      break;
    case 10:
      sigrot(o, vort); m3dm9(o, m); lieupd(o);
      break;
    case 11:
      m3dm10(o); lieupd(o);
      break;
    default:
      return oerr(o, MPM_ERR_UNSUPPORTED, "material type %d not implemented", o->mtype_);
  }
  if (st) return st;
  p->SM = o->sm;
  p->Seqv = o->seqv;
  p->SDxx = o->sd[0]; p->SDyy = o->sd[1]; p->SDzz = o->sd[2];
  p->SDyz = o->sd[3]; p->SDxz = o->sd[4]; p->SDxy = o->sd[5];
  p->sig_y = o->sig_y_;
  p->epeff = o->epeff_;
  p->ie = o->iener;
  p->cp = o->cp;
  p->q = o->bqf;
  return MPM_OK;
}

/* ====================================================================
 * update_step.f90: the step routines
 * ==================================================================== */

/* ParticleInitial, update_step.f90:408-453 */
static void particle_initial(orc* o) {
  for (int64_t ip = 0; ip < o->np; ++ip) {
    opart* p = &o->pt[ip];
    p->icell = in_which_cell(o, p->Xp);
    if (p->icell > 0) {
      for (int d = 0; d < 3; ++d) p->XN[d] = (p->Xp[d] - o->Cxg[p->icell - 1][d]) * o->iJacobi;
    }
    if (o->SGMP) {
      p->centericell = center_in_which_cell(o, p->Xp);
      int ix = (int)((p->Xp[0] - o->SpanX[0]) / o->DCell + 0.5) + 1;
      int iy = (int)((p->Xp[1] - o->SpanY[0]) / o->DCell + 0.5) + 1;
      int iz = (int)((p->Xp[2] - o->SpanZ[0]) / o->DCell + 0.5) + 1;
      p->inode = (iz - 1) * o->NGxy + (iy - 1) * o->NGx + ix;
      if (p->inode < 1 || p->inode > o->nb_gridnode) continue; /* outside the grid */
      const onode* nd = &o->node[p->inode - 1];
      for (int d = 0; d < 3; ++d) p->XXN[d] = (p->Xp[d] - nd->Xg[d]) * o->iJacobi;
      for (int d = 0; d < 3; ++d) {
        if (nd->bd_type[d] != 0) {
          if (p->XXN[d] > 0) p->XXN[d] = 1;
          else if (p->XXN[d] < 0) p->XXN[d] = -1;
        }
      }
    }
  }
}

static int center_valid(const orc* o, int c) { return c <= o->nb_centernode && c > 0; }

/* GridMomentumInitial, update_step.f90:288-406 */
static void grid_momentum_initial(orc* o) {
  for (int64_t n = 0; n < all_nodes(o); ++n) {
    o->grid[n].Mg = 0.0;
    o->grid[n].PXg[0] = o->grid[n].PXg[1] = o->grid[n].PXg[2] = 0.0;
  }
  particle_initial(o);
  if (o->SGMP) {
    for (int c = 0; c < o->NumCell; ++c) {
      o->cellp[c].Cmg = 0.0;
      o->cellp[c].Cpxg[0] = o->cellp[c].Cpxg[1] = o->cellp[c].Cpxg[2] = 0.0;
    }
  }
  for (int b = 0; b < o->nb_body; ++b) {
    const int64_t cb = comp_base(o, b);
    for (int64_t ip = o->body[b].par_begin; ip < o->body[b].par_end; ++ip) {
      opart* p = &o->pt[ip];
      if (o->SGMP) {
        if (p->centericell < 0) continue;
        double mp_ = p->mass;
        for (int n = 0; n < 8; ++n) o->CenterInflNode[n] = o->CenterCellNode[p->centericell - 1][n];
        sg_nshape(o, p->XXN);
        for (int n = 0; n < 8; ++n) {
          if (!center_valid(o, o->CenterInflNode[n])) continue;
          ocellp* cd = &o->cellp[o->CenterInflNode[n] - 1];
          double shm = o->SHP[n] * mp_;
          cd->Cmg = cd->Cmg + shm;
          for (int c = 0; c < 3; ++c) cd->Cpxg[c] = cd->Cpxg[c] + p->VXp[c] * shm;
        }
      } else {
        if (p->icell < 0) continue;
        double mp_ = p->mass;
        particle_shape(o, p, p->icell);
        for (int n = 0; n < o->nb_InflNode; ++n) {
          if (!node_valid(o, o->InflNode[n])) continue;
          ogrid* gd = &o->grid[cb + o->InflNode[n] - 1];
          double shm = o->SHP[n] * mp_;
          gd->Mg = gd->Mg + shm;
          for (int c = 0; c < 3; ++c) gd->PXg[c] = gd->PXg[c] + p->VXp[c] * shm;
        }
      }
    }
  }
  if (o->SGMP) {
    for (int i = 0; i < o->nb_centernode; ++i) {
      if (!(o->cellp[i].Cmg > o->CutOff)) continue;
      for (int j = 0; j < 8; ++j) {
        ogrid* gd = &o->grid[o->CellsNode[i][j] - 1];
        gd->Mg = gd->Mg + 0.125 * o->cellp[i].Cmg;
        for (int c = 0; c < 3; ++c) gd->PXg[c] = gd->PXg[c] + 0.125 * o->cellp[i].Cpxg[c];
      }
    }
  }
  int64_t act = 0;
  for (int64_t n = 0; n < all_nodes(o); ++n) act += o->grid[n].Mg > 0;
  o->active_nodes = act;
}

/* zero the momentum and force of fixed DOFs (ApplyBoundaryConditions,
 * update_step.f90:1795-1830; the same loop closes IntegrateMomentum and
 * GridMomentumMUSL) */
static void apply_bc(orc* o) {
  for (int64_t k = 0; k < all_nodes(o); ++k) {
    const int64_t n = k % o->nb_gridnode;
    for (int c = 0; c < 3; ++c) {
      if (o->node[n].fix[c]) {
        o->grid[k].PXg[c] = 0.0;
        o->grid[k].FXg[c] = 0.0;
      }
    }
  }
}

/* centre-node strain rate, spin and velocity gradient from the cell nodes
 * (the SGMP part of ParticleStressUpdate, update_step.f90:478-523, and of
 * TLParticleStressUpdate, 671-716) */
static void sg_cell_gradients(orc* o) {
  for (int i = 0; i < o->nb_centernode; ++i) {
    ocellp* cd = &o->cellp[i];
    memset(cd->Co, 0, sizeof cd->Co);
    memset(cd->Cw, 0, sizeof cd->Cw);
    memset(cd->CdeFp, 0, sizeof cd->CdeFp);
  }
  for (int i = 0; i < o->nb_centernode; ++i) {
    ocellp* cd = &o->cellp[i];
    cnshape(o);
    for (int j = 0; j < 8; ++j) {
      const ogrid* gd = &o->grid[o->CellsNode[i][j] - 1];
      if (!(gd->Mg > o->CutOff)) continue;
      double v[3];
      for (int c = 0; c < 3; ++c) v[c] = gd->PXg[c] / gd->Mg;
      double dx = o->CDNDX[j], dy = o->CDNDY[j], dz = o->CDNDZ[j];
      cd->Co[0] = cd->Co[0] + dx * v[0];
      cd->Co[1] = cd->Co[1] + dy * v[1];
      cd->Co[2] = cd->Co[2] + dz * v[2];
      cd->Co[3] = cd->Co[3] + dz * v[1] + dy * v[2];
      cd->Co[4] = cd->Co[4] + dz * v[0] + dx * v[2];
      cd->Co[5] = cd->Co[5] + dy * v[0] + dx * v[1];
      cd->Cw[0] = cd->Cw[0] + dy * v[2] - dz * v[1];
      cd->Cw[1] = cd->Cw[1] + dz * v[0] - dx * v[2];
      cd->Cw[2] = cd->Cw[2] + dx * v[1] - dy * v[0];
      for (int n = 0; n < 3; ++n) {
        cd->CdeFp[n][0] = cd->CdeFp[n][0] + dx * v[n];
        cd->CdeFp[n][1] = cd->CdeFp[n][1] + dy * v[n];
        cd->CdeFp[n][2] = cd->CdeFp[n][2] + dz * v[n];
      }
    }
  }
}

/* ParticleStressUpdate, update_step.f90:456-647 */
static int particle_stress_update(orc* o) {
  if (o->SGMP) sg_cell_gradients(o);
  for (int b = 0; b < o->nb_body; ++b) {
    const int64_t cb = comp_base(o, b);
    for (int64_t ip = o->body[b].par_begin; ip < o->body[b].par_end; ++ip) {
      opart* p = &o->pt[ip];
      double de[6] = {0, 0, 0, 0, 0, 0}, vort[3] = {0, 0, 0}, deFp[3][3];
      memset(deFp, 0, sizeof deFp);
      if (o->SGMP) {
        if (p->centericell < 0) continue;
        for (int n = 0; n < 8; ++n) o->CenterInflNode[n] = o->CenterCellNode[p->centericell - 1][n];
        sg_nshape(o, p->XXN);
        for (int n = 0; n < 8; ++n) {
          if (!center_valid(o, o->CenterInflNode[n])) continue;
          const ocellp* cd = &o->cellp[o->CenterInflNode[n] - 1];
          double s = o->SHP[n];
          for (int k = 0; k < 6; ++k) de[k] = de[k] + cd->Co[k] * s;
          for (int k = 0; k < 3; ++k) vort[k] = vort[k] + cd->Cw[k] * s;
          for (int i = 0; i < 3; ++i) {
            deFp[i][0] = deFp[i][0] + s * cd->CdeFp[i][0];
            deFp[i][1] = deFp[i][1] + s * cd->CdeFp[i][1];
            deFp[i][2] = deFp[i][2] + s * cd->CdeFp[i][2];
          }
        }
      } else {
        if (p->icell < 0) continue;
        particle_shape(o, p, p->icell);
        for (int n = 0; n < o->nb_InflNode; ++n) {
          if (!node_valid(o, o->InflNode[n])) continue;
          const ogrid* gd = &o->grid[cb + o->InflNode[n] - 1];
          if (!(gd->Mg > o->CutOff)) continue;
          double v[3];
          for (int c = 0; c < 3; ++c) v[c] = gd->PXg[c] / gd->Mg;
          double dx = o->DNDX[n], dy = o->DNDY[n], dz = o->DNDZ[n];
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
      for (int k = 0; k < 6; ++k) de[k] = de[k] * o->DT;
      for (int k = 0; k < 3; ++k) vort[k] = vort[k] * o->DT / 2.0;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) deFp[i][j] = deFp[i][j] * o->DT;
      if (o->UpdateVbyFp) {
        double F0[3][3];
        memcpy(F0, p->Fp, sizeof F0);
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j)
            p->Fp[i][j] = p->Fp[i][j] + deFp[i][j] + deFp[i][0] * F0[0][j] + deFp[i][1] * F0[1][j] +
                          deFp[i][2] * F0[2][j];
      }
      int st = constitution(o, de, vort, b, ip, (const double (*)[3])deFp);
      if (st) return st;
      if (!o->USF) memcpy(p->Xp, p->XX, sizeof p->Xp);
    }
  }
  return MPM_OK;
}

/* external force of a particle (update_step.f90:889-903) */
static void particle_fx(const orc* o, const opart* p, int b, double fx[3]) {
  for (int c = 0; c < 3; ++c) {
    if (o->QuasiLoad && !(o->CurrentTime >= o->QuasiLoadTime))
      fx[c] = p->FXp[c] / o->QuasiLoadTime * o->CurrentTime;
    else
      fx[c] = p->FXp[c];
  }
  if (o->QuasiDamp)
    for (int c = 0; c < 3; ++c) fx[c] = fx[c] - o->DampFactor * p->mass * p->VXp[c];
  if (o->Gravity)
    for (int c = 0; c < 3; ++c) fx[c] = fx[c] + p->mass * o->body[b].gravp[c];
}

/* GridMomentumUpdate, update_step.f90:831-1013 */
static void grid_momentum_update(orc* o) {
  if (o->SGMP) {
    for (int i = 0; i < o->nb_centernode; ++i) {
      memset(o->cellp[i].Cfint, 0, sizeof o->cellp[i].Cfint);
      memset(o->cellp[i].Cfext, 0, sizeof o->cellp[i].Cfext);
    }
  }
  for (int64_t n = 0; n < all_nodes(o); ++n) o->grid[n].FXg[0] = o->grid[n].FXg[1] = o->grid[n].FXg[2] = 0.0;
  if (o->contact) memset(o->ndir, 0, sizeof(double[3]) * (size_t)all_nodes(o));
  for (int b = 0; b < o->nb_body; ++b) {
    const int64_t cb = comp_base(o, b);
    for (int64_t ip = o->body[b].par_begin; ip < o->body[b].par_end; ++ip) {
      opart* p = &o->pt[ip];
      double fx[3];
      const double mp_ = p->mass;
      particle_fx(o, p, b, fx);
      double vol_ = p->VOL;
      double sxx = p->SM - p->q + p->SDxx;
      double syy = p->SM - p->q + p->SDyy;
      double szz = p->SM - p->q + p->SDzz;
      double sxy = p->SDxy, syz = p->SDyz, sxz = p->SDxz;
      if (o->SGMP) {
        if (p->centericell < 0) continue;
        for (int n = 0; n < 8; ++n) o->CenterInflNode[n] = o->CenterCellNode[p->centericell - 1][n];
        sg_nshape(o, p->XXN);
        for (int n = 0; n < 8; ++n) {
          if (!center_valid(o, o->CenterInflNode[n])) continue;
          ocellp* cd = &o->cellp[o->CenterInflNode[n] - 1];
          double s = o->SHP[n];
          for (int c = 0; c < 3; ++c) cd->Cfext[c] = cd->Cfext[c] + fx[c] * s;
          cd->Cfint[0] = cd->Cfint[0] + s * sxx * vol_;
          cd->Cfint[1] = cd->Cfint[1] + s * syy * vol_;
          cd->Cfint[2] = cd->Cfint[2] + s * szz * vol_;
          cd->Cfint[3] = cd->Cfint[3] + s * sxy * vol_;
          cd->Cfint[4] = cd->Cfint[4] + s * syz * vol_;
          cd->Cfint[5] = cd->Cfint[5] + s * sxz * vol_;
        }
      } else {
        if (p->icell < 0) continue;
        particle_shape(o, p, p->icell);
        for (int n = 0; n < o->nb_InflNode; ++n) {
          if (!node_valid(o, o->InflNode[n])) continue;
          ogrid* gd = &o->grid[cb + o->InflNode[n] - 1];
          double s = o->SHP[n], dx = o->DNDX[n], dy = o->DNDY[n], dz = o->DNDZ[n];
          double fi[3];
          fi[0] = -(sxx * dx + sxy * dy + sxz * dz) * vol_;
          fi[1] = -(sxy * dx + syy * dy + syz * dz) * vol_;
          fi[2] = -(sxz * dx + syz * dy + szz * dz) * vol_;
          for (int c = 0; c < 3; ++c) gd->FXg[c] = gd->FXg[c] + fi[c] + fx[c] * s;
          if (o->contact) { /* mass-gradient normal of the component's node (update_step.f90:977-982) */
            double* nd = o->ndir[cb + o->InflNode[n] - 1];
            nd[0] = nd[0] + dx * mp_;
            nd[1] = nd[1] + dy * mp_;
            nd[2] = nd[2] + dz * mp_;
          }
        }
      }
    }
  }
  if (o->SGMP) {
    cnshape(o);
    for (int i = 0; i < o->nb_centernode; ++i) {
      const ocellp* cd = &o->cellp[i];
      for (int j = 0; j < 8; ++j) {
        ogrid* gd = &o->grid[o->CellsNode[i][j] - 1];
        double dx = o->CDNDX[j], dy = o->CDNDY[j], dz = o->CDNDZ[j];
        double fi[3];
        fi[0] = -(cd->Cfint[0] * dx + cd->Cfint[3] * dy + cd->Cfint[5] * dz);
        fi[1] = -(cd->Cfint[3] * dx + cd->Cfint[1] * dy + cd->Cfint[4] * dz);
        fi[2] = -(cd->Cfint[5] * dx + cd->Cfint[4] * dy + cd->Cfint[2] * dz);
        for (int c = 0; c < 3; ++c) gd->FXg[c] = gd->FXg[c] + 0.125 * cd->Cfext[c] + fi[c];
      }
    }
  }
}

/* IntegrateMomentum, update_step.f90:1194-1239 */
static void integrate_momentum(orc* o) {
  for (int64_t k = 0; k < all_nodes(o); ++k) {
    const int64_t n = k % o->nb_gridnode;
    ogrid* gd = &o->grid[k];
    for (int c = 0; c < 3; ++c) {
      if (o->istep == 1)
        gd->PXg[c] = gd->PXg[c] + gd->FXg[c] * o->DT * 0.5;
      else
        gd->PXg[c] = gd->PXg[c] + gd->FXg[c] * o->DT;
    }
    for (int c = 0; c < 3; ++c) {
      if (o->node[n].fix[c]) {
        gd->PXg[c] = 0.0;
        gd->FXg[c] = 0.0;
      }
    }
  }
}

/* Lagr_NodContact, update_step.f90:1241-1376 (Bardenhagen's method between
 * grid components 1 and 2): per node, the contact normal from the two
 * components' mass gradients (normbody 0: their difference, 1: body a's,
 * 2: minus body b's), unitised; where both components have mass above the
 * cut-off and approach along the normal (crit > epsilon), the normal contact
 * force crit / ((Mg1 + Mg2) DT) -- with friction, the full sticking force
 * limited to fricfa |normal force| tangentially -- is taken from component 1
 * and given to component 2 in force and momentum, on the free directions of
 * the node; the forces add up to the plotted total contact force. */
static void lagr_contact(orc* o) {
  const double eps = 2.220446049250313e-16; /* epsilon(1d0) */
  const int64_t nn = o->nb_gridnode;
  o->tot_cont_for[0] = o->tot_cont_for[1] = o->tot_cont_for[2] = 0.0;
  for (int64_t n = 0; n < nn; ++n) {
    double* cp1 = o->ndir[n];
    double* cp2 = o->ndir[nn + n];
    ogrid* gd1 = &o->grid[n];
    ogrid* gd2 = &o->grid[nn + n];
    double nx = 0, ny = 0, nz = 0;
    if (o->normbody == 0) {
      nx = cp1[0] - cp2[0];
      ny = cp1[1] - cp2[1];
      nz = cp1[2] - cp2[2];
    }
    if (o->normbody == 1) {
      nx = cp1[0];
      ny = cp1[1];
      nz = cp1[2];
    }
    if (o->normbody == 2) {
      nx = -cp2[0];
      ny = -cp2[1];
      nz = -cp2[2];
    }
    double tt = sqrt(nx * nx + ny * ny + nz * nz);
    if (tt > eps) {
      nx = nx / tt;
      ny = ny / tt;
      nz = nz / tt;
    }
    cp1[0] = nx;
    cp1[1] = ny;
    cp1[2] = nz;
    cp2[0] = -cp1[0];
    cp2[1] = -cp1[1];
    cp2[2] = -cp1[2];
    double crit = 0.0;
    if (gd1->Mg > o->CutOff && gd2->Mg > o->CutOff)
      crit = (gd1->PXg[0] * gd2->Mg - gd2->PXg[0] * gd1->Mg) * nx + (gd1->PXg[1] * gd2->Mg - gd2->PXg[1] * gd1->Mg) * ny +
             (gd1->PXg[2] * gd2->Mg - gd2->PXg[2] * gd1->Mg) * nz;
    if (!(crit > eps)) continue;
    tt = (gd1->Mg + gd2->Mg) * o->DT;
    const double nomforce = crit / tt;
    double cforce[3];
    if (o->fricfa > eps) {
      double fstick[3];
      for (int c = 0; c < 3; ++c) cforce[c] = (gd1->PXg[c] * gd2->Mg - gd2->PXg[c] * gd1->Mg) / tt;
      for (int c = 0; c < 3; ++c) fstick[c] = cforce[c] - nomforce * cp1[c];
      const double val_fstick = sqrt(fstick[0] * fstick[0] + fstick[1] * fstick[1] + fstick[2] * fstick[2]);
      const double val_fslip = o->fricfa * fabs(nomforce);
      if (val_fslip < val_fstick)
        for (int c = 0; c < 3; ++c) cforce[c] = nomforce * cp1[c] + val_fslip * (fstick[c] / val_fstick);
    } else {
      for (int c = 0; c < 3; ++c) cforce[c] = nomforce * cp1[c];
    }
    for (int c = 0; c < 3; ++c) {
      if (o->node[n].fix[c]) continue;
      gd1->FXg[c] = gd1->FXg[c] - cforce[c];
      gd2->FXg[c] = gd2->FXg[c] + cforce[c];
      gd1->PXg[c] = gd1->PXg[c] - cforce[c] * o->DT;
      gd2->PXg[c] = gd2->PXg[c] + cforce[c] * o->DT;
    }
    for (int c = 0; c < 3; ++c) o->tot_cont_for[c] = o->tot_cont_for[c] + cforce[c];
  }
}

/* Cvx / Cax of one boundary auxiliary node (BoundaryAuxiliaryNodeUpdate,
 * update_step.f90:1528-1666) */
static void boundary_aux_cell(orc* o, int ix, int iy, int iz, const double cxx[3]) {
  int n = ix + (iy - 1) * o->NumCellx + (iz - 1) * o->NumCellxy;
  double vx[3] = {0, 0, 0}, ax[3] = {0, 0, 0};
  sg_nshape(o, cxx);
  for (int j = 0; j < 8; ++j) {
    const ogrid* gd = &o->grid[o->CellsNode[n - 1][j] - 1];
    if (!(gd->Mg > o->CutOff)) continue;
    for (int c = 0; c < 3; ++c) {
      vx[c] = vx[c] + o->SHP[j] * gd->PXg[c] / gd->Mg;
      ax[c] = ax[c] + o->SHP[j] * gd->FXg[c] / gd->Mg;
    }
  }
  memcpy(o->cellp[n - 1].Cvx, vx, sizeof vx);
  memcpy(o->cellp[n - 1].Cax, ax, sizeof ax);
}

static void boundary_aux_update(orc* o) {
  const int NX = o->NumCellx, NY = o->NumCelly, NZ = o->NumCellz;
  if (NX > 1) {
    for (int i = 1; i <= 2; ++i) {
      int ix;
      if (i == 1 && o->FixS[0] != 0) ix = 1;
      else if (i == 2 && o->FixS[1] != 0) ix = NX;
      else continue;
      for (int iz = 1; iz <= NZ; ++iz)
        for (int iy = 1; iy <= NY; ++iy) {
          double cxx[3] = {0, 0, 0};
          if (ix == 1) cxx[0] = 1;
          if (ix == NX) cxx[0] = -1;
          if (NY > 1) { if (iy == 1) cxx[1] = 1; if (iy == NY) cxx[1] = -1; }
          if (NZ > 1) { if (iz == 1) cxx[2] = 1; if (iz == NZ) cxx[2] = -1; }
          boundary_aux_cell(o, ix, iy, iz, cxx);
        }
    }
  }
  if (NY > 1) {
    for (int i = 1; i <= 2; ++i) {
      int iy;
      if (i == 1 && o->FixS[2] != 0) iy = 1;
      else if (i == 2 && o->FixS[3] != 0) iy = NY;
      else continue;
      for (int iz = 1; iz <= NZ; ++iz)
        for (int ix = 1; ix <= NX; ++ix) {
          double cxx[3] = {0, 0, 0};
          if (iy == 1) cxx[1] = 1;
          if (iy == NY) cxx[1] = -1;
          if (NX > 1) { if (ix == 1) cxx[0] = 1; if (ix == NX) cxx[0] = -1; }
          if (NZ > 1) { if (iz == 1) cxx[2] = 1; if (iz == NZ) cxx[2] = -1; }
          boundary_aux_cell(o, ix, iy, iz, cxx);
        }
    }
  }
  if (NZ > 1) {
    for (int i = 1; i <= 2; ++i) {
      int iz;
      if (i == 1 && o->FixS[4] != 0) iz = 1;
      else if (i == 2 && o->FixS[5] != 0) iz = NZ;
      else continue;
      for (int iy = 1; iy <= NY; ++iy)
        for (int ix = 1; ix <= NX; ++ix) {
          double cxx[3] = {0, 0, 0};
          if (iz == 1) cxx[2] = 1;
          if (iz == NZ) cxx[2] = -1;
          if (NX > 1) { if (ix == 1) cxx[0] = 1; if (ix == NX) cxx[0] = -1; }
          if (NY > 1) { if (iy == 1) cxx[1] = 1; if (iy == NY) cxx[1] = -1; }
          boundary_aux_cell(o, ix, iy, iz, cxx);
        }
    }
  }
}

/* ParticlePositionUpdate, update_step.f90:1378-1526 */
static void particle_position_update(orc* o) {
  if (o->SGMP) {
    for (int i = 0; i < o->nb_centernode; ++i) {
      ocellp* cd = &o->cellp[i];
      memset(cd->Cvx, 0, sizeof cd->Cvx);
      memset(cd->Cax, 0, sizeof cd->Cax);
      for (int j = 0; j < 8; ++j) {
        const ogrid* gd = &o->grid[o->CellsNode[i][j] - 1];
        if (!(gd->Mg > o->CutOff)) continue;
        for (int c = 0; c < 3; ++c) {
          cd->Cvx[c] = cd->Cvx[c] + 0.125 * gd->PXg[c] / gd->Mg;
          cd->Cax[c] = cd->Cax[c] + 0.125 * gd->FXg[c] / gd->Mg;
        }
      }
    }
    boundary_aux_update(o);
  }
  for (int b = 0; b < o->nb_body; ++b) {
    const int64_t cb = comp_base(o, b);
    for (int64_t ip = o->body[b].par_begin; ip < o->body[b].par_end; ++ip) {
      opart* p = &o->pt[ip];
      double xx[3], vx[3] = {0, 0, 0}, ax[3] = {0, 0, 0};
      if (o->SGMP) {
        memcpy(xx, p->Xp, sizeof xx);
        if (p->centericell < 0) continue;
        for (int n = 0; n < 8; ++n) o->CenterInflNode[n] = o->CenterCellNode[p->centericell - 1][n];
        const int* ptype = o->node[p->inode - 1].bd_type;
        int internal = ptype[0] == 0 && ptype[1] == 0 && ptype[2] == 0;
        if (internal) {
          sg_nshape(o, p->XXN);
        } else {
          double xinb[3];
          aux_grid_shp(p->XN, p->XXN, ptype, xinb);
          sg_nshape(o, xinb);
        }
        for (int n = 0; n < 8; ++n) {
          if (!center_valid(o, o->CenterInflNode[n])) continue;
          const ocellp* cd = &o->cellp[o->CenterInflNode[n] - 1];
          double s = o->SHP[n];
          for (int c = 0; c < 3; ++c) {
            vx[c] = vx[c] + s * cd->Cvx[c];
            ax[c] = ax[c] + s * cd->Cax[c];
          }
        }
      } else {
        if (p->icell < 0) continue;
        memcpy(xx, p->Xp, sizeof xx);
        particle_shape(o, p, p->icell);
        for (int n = 0; n < o->nb_InflNode; ++n) {
          if (!node_valid(o, o->InflNode[n])) continue;
          const ogrid* gd = &o->grid[cb + o->InflNode[n] - 1];
          if (!(gd->Mg > o->CutOff)) continue;
          double s = o->SHP[n];
          for (int c = 0; c < 3; ++c) {
            vx[c] = vx[c] + s * (gd->PXg[c] / gd->Mg);
            ax[c] = ax[c] + s * gd->FXg[c] / gd->Mg;
          }
        }
      }
      for (int c = 0; c < 3; ++c) p->XX[c] = xx[c] + vx[c] * o->DT;
      for (int c = 0; c < 3; ++c) {
        if (o->istep == 1)
          p->VXp[c] = p->VXp[c] + ax[c] * o->DT * 0.5;
        else
          p->VXp[c] = p->VXp[c] + ax[c] * o->DT;
      }
      if (o->USF) memcpy(p->Xp, p->XX, sizeof p->Xp);
    }
  }
}

/* GridMomentumMUSL, update_step.f90:1668-1793 */
static void grid_momentum_musl(orc* o) {
  for (int64_t n = 0; n < all_nodes(o); ++n) o->grid[n].PXg[0] = o->grid[n].PXg[1] = o->grid[n].PXg[2] = 0.0;
  if (o->SGMP)
    for (int i = 0; i < o->nb_centernode; ++i) memset(o->cellp[i].Cpxg, 0, sizeof o->cellp[i].Cpxg);
  for (int b = 0; b < o->nb_body; ++b) {
    const int64_t cb = comp_base(o, b);
    for (int64_t ip = o->body[b].par_begin; ip < o->body[b].par_end; ++ip) {
      opart* p = &o->pt[ip];
      if (o->SGMP) {
        if (p->centericell < 0) continue;
        double mp_ = p->mass;
        for (int n = 0; n < 8; ++n) o->CenterInflNode[n] = o->CenterCellNode[p->centericell - 1][n];
        sg_nshape(o, p->XXN);
        for (int n = 0; n < 8; ++n) {
          if (!center_valid(o, o->CenterInflNode[n])) continue;
          ocellp* cd = &o->cellp[o->CenterInflNode[n] - 1];
          double shm = o->SHP[n] * mp_;
          for (int c = 0; c < 3; ++c) cd->Cpxg[c] = cd->Cpxg[c] + p->VXp[c] * shm;
        }
      } else {
        if (p->icell < 0) continue;
        double mp_ = p->mass;
        particle_shape(o, p, p->icell);
        for (int n = 0; n < o->nb_InflNode; ++n) {
          if (!node_valid(o, o->InflNode[n])) continue;
          ogrid* gd = &o->grid[cb + o->InflNode[n] - 1];
          double shm = o->SHP[n] * mp_;
          for (int c = 0; c < 3; ++c) gd->PXg[c] = gd->PXg[c] + p->VXp[c] * shm;
        }
      }
    }
  }
  if (o->SGMP) {
    for (int i = 0; i < o->nb_centernode; ++i)
      for (int j = 0; j < 8; ++j) {
        ogrid* gd = &o->grid[o->CellsNode[i][j] - 1];
        for (int c = 0; c < 3; ++c) gd->PXg[c] = gd->PXg[c] + 0.125 * o->cellp[i].Cpxg[c];
      }
  }
  apply_bc(o);
}

/* ====================================================================
 * Total Lagrangian MPM (MPM3D.f90:161-244): the grid mass is mapped once,
 * cells are those of the initial positions for the whole run, the
 * deformation gradient grows by the velocity gradient, and the internal
 * forces come from the first Piola-Kirchhoff stress on the initial volume.
 * Shapes are evaluated as the reference does: GIMP and B-spline at the
 * current Xp against the initial cell, SGMP at the initial XXN, linear at
 * XN -- which TLParticleInitial does not set for linear shapes, so it keeps
 * its initial value (0 here: the cell centre).
 * ==================================================================== */

/* TLParticleInitial, update_step.f90:127-172 */
static void tl_particle_initial(orc* o) {
  for (int64_t ip = 0; ip < o->np; ++ip) {
    opart* p = &o->pt[ip];
    p->icell = in_which_cell(o, p->Xo);
    if (!o->SGMP) continue;
    p->centericell = center_in_which_cell(o, p->Xo);
    int ix = (int)((p->Xo[0] - o->SpanX[0]) / o->DCell + 0.5) + 1;
    int iy = (int)((p->Xo[1] - o->SpanY[0]) / o->DCell + 0.5) + 1;
    int iz = (int)((p->Xo[2] - o->SpanZ[0]) / o->DCell + 0.5) + 1;
    p->inode = (iz - 1) * o->NGxy + (iy - 1) * o->NGx + ix;
    if (p->inode < 1 || p->inode > o->nb_gridnode || p->icell < 1) continue; /* outside the grid */
    const onode* nd = &o->node[p->inode - 1];
    for (int d = 0; d < 3; ++d) p->XXN[d] = (p->Xo[d] - nd->Xg[d]) * o->iJacobi;
    for (int d = 0; d < 3; ++d) p->XN[d] = (p->Xo[d] - o->Cxg[p->icell - 1][d]) * o->iJacobi;
    for (int d = 0; d < 3; ++d)
      if (nd->bd_type[d] != 0) {
        if (p->XXN[d] > 0) p->XXN[d] = 1;
        else if (p->XXN[d] < 0) p->XXN[d] = -1;
      }
  }
}

/* GridMassInitial, update_step.f90:22-125 (once, before the time loop) */
static void grid_mass_initial(orc* o) {
  for (int64_t n = 0; n < all_nodes(o); ++n) o->grid[n].Mg = 0.0;
  tl_particle_initial(o);
  if (o->SGMP)
    for (int c = 0; c < o->NumCell; ++c) o->cellp[c].Cmg = 0.0;
  for (int b = 0; b < o->nb_body; ++b) {
    const int64_t cb = comp_base(o, b);
    for (int64_t ip = o->body[b].par_begin; ip < o->body[b].par_end; ++ip) {
      opart* p = &o->pt[ip];
      double mp_ = p->mass;
      if (o->SGMP) {
        if (p->centericell < 0) continue;
        for (int n = 0; n < 8; ++n) o->CenterInflNode[n] = o->CenterCellNode[p->centericell - 1][n];
        sg_nshape(o, p->XXN);
        for (int n = 0; n < 8; ++n) {
          if (!center_valid(o, o->CenterInflNode[n])) continue;
          ocellp* cd = &o->cellp[o->CenterInflNode[n] - 1];
          cd->Cmg = cd->Cmg + o->SHP[n] * mp_;
        }
      } else {
        if (p->icell < 0) continue;
        particle_shape(o, p, p->icell);
        for (int n = 0; n < o->nb_InflNode; ++n) {
          if (!node_valid(o, o->InflNode[n])) continue;
          ogrid* gd = &o->grid[cb + o->InflNode[n] - 1];
          gd->Mg = gd->Mg + o->SHP[n] * mp_;
        }
      }
    }
  }
  if (o->SGMP)
    for (int i = 0; i < o->nb_centernode; ++i) {
      if (!(o->cellp[i].Cmg > o->CutOff)) continue;
      for (int j = 0; j < 8; ++j) {
        ogrid* gd = &o->grid[o->CellsNode[i][j] - 1];
        gd->Mg = gd->Mg + 0.125 * o->cellp[i].Cmg;
      }
    }
  int64_t act = 0;
  for (int64_t n = 0; n < all_nodes(o); ++n) act += o->grid[n].Mg > 0;
  o->active_nodes = act;
}

/* TLGridMomentumInitial, update_step.f90:174-286 (momentum only) */
static void tl_grid_momentum_initial(orc* o) {
  for (int64_t n = 0; n < all_nodes(o); ++n) o->grid[n].PXg[0] = o->grid[n].PXg[1] = o->grid[n].PXg[2] = 0.0;
  if (o->SGMP)
    for (int c = 0; c < o->NumCell; ++c) o->cellp[c].Cpxg[0] = o->cellp[c].Cpxg[1] = o->cellp[c].Cpxg[2] = 0.0;
  for (int b = 0; b < o->nb_body; ++b) {
    const int64_t cb = comp_base(o, b);
    for (int64_t ip = o->body[b].par_begin; ip < o->body[b].par_end; ++ip) {
      opart* p = &o->pt[ip];
      double mp_ = p->mass;
      if (o->SGMP) {
        if (p->centericell < 0) continue;
        for (int n = 0; n < 8; ++n) o->CenterInflNode[n] = o->CenterCellNode[p->centericell - 1][n];
        sg_nshape(o, p->XXN);
        for (int n = 0; n < 8; ++n) {
          if (!center_valid(o, o->CenterInflNode[n])) continue;
          ocellp* cd = &o->cellp[o->CenterInflNode[n] - 1];
          double shm = o->SHP[n] * mp_;
          for (int c = 0; c < 3; ++c) cd->Cpxg[c] = cd->Cpxg[c] + p->VXp[c] * shm;
        }
      } else {
        if (p->icell < 0) continue;
        particle_shape(o, p, p->icell);
        for (int n = 0; n < o->nb_InflNode; ++n) {
          if (!node_valid(o, o->InflNode[n])) continue;
          ogrid* gd = &o->grid[cb + o->InflNode[n] - 1];
          double shm = o->SHP[n] * mp_;
          for (int c = 0; c < 3; ++c) gd->PXg[c] = gd->PXg[c] + p->VXp[c] * shm;
        }
      }
    }
  }
  if (o->SGMP)
    for (int i = 0; i < o->nb_centernode; ++i) {
      if (!(o->cellp[i].Cmg > o->CutOff)) continue;
      for (int j = 0; j < 8; ++j) {
        ogrid* gd = &o->grid[o->CellsNode[i][j] - 1];
        for (int c = 0; c < 3; ++c) gd->PXg[c] = gd->PXg[c] + 0.125 * o->cellp[i].Cpxg[c];
      }
    }
}

/* TLConstitution + M3DM11 (neo-Hookean), Constitution.f90:370-523, 782-882:
 * the first Piola-Kirchhoff stress from F = I + Fp, the Cauchy stress from
 * it, the volume det(F) VOL0, and the internal energy from the mid-step PK
 * stress on the increment of F. Like the reference, sig_y and epeff are
 * written from the constitutive module's state, which the TL update does
 * not load from the particle. */
static int tl_constitution(orc* o, int b, int64_t pidx, const double deFp[3][3]) {
  opart* p = &o->pt[pidx];
  double ppk_old[9], ppk_new[9];
  memcpy(ppk_old, p->PK, sizeof ppk_old);
  memcpy(o->deF, deFp, sizeof o->deF);
  o->vold = p->VOL;
  memcpy(o->Fp, p->Fp, sizeof o->Fp);
  for (int i = 0; i < 3; ++i) o->Fp[i][i] = o->Fp[i][i] + 1.0;
  double (*F3)[3] = o->Fp;
  const double detF = F3[0][0] * F3[1][1] * F3[2][2] - F3[0][0] * F3[1][2] * F3[2][1] -
                      F3[1][0] * F3[0][1] * F3[2][2] + F3[1][0] * F3[0][2] * F3[2][1] +
                      F3[2][0] * F3[0][1] * F3[1][2] - F3[2][0] * F3[0][2] * F3[1][1];
  p->VOL = detF * p->VOL0;
  o->vol_ = p->VOL;
  o->dvol = 0.5 * (o->vol_ - o->vold);
  o->mid = o->body[b].mat;
  const mpm_material* m = &o->mat[o->mid - 1];
  if (m->mat_type != 11) return oerr(o, MPM_ERR_UNSUPPORTED, "TLMPM supports the neo-Hookean material only");
  o->seqv = p->Seqv;
  o->mtype_ = m->mat_type;
  o->etype_ = m->eos_type;
  o->miu2 = 2 * m->miu;
  o->young_ = m->young;
  o->poisson_ = m->poisson;
  o->yield0_ = m->yield0;
  o->tangmod_ = m->tangmod;
  o->den0_ = m->density;
  o->DMG = p->DMG;
  o->oldDMG = o->DMG;
  o->young_ = o->young_ * (1.0 - o->DMG + 2.220446049250313e-16);
  o->G2 = o->young_ / (1 + o->poisson_);
  o->K3 = o->young_ / (1 - 2 * o->poisson_);
  o->lamda = (o->young_ * o->poisson_) / ((1 + o->poisson_) * (1 - 2 * o->poisson_));
  o->PlaMod = o->young_ * o->tangmod_ / (o->young_ - o->tangmod_);
  o->cp = p->cp;
  o->sm = p->SM;
  o->smold = p->SM;
  o->iener = p->ie;
  o->bqf = 0.0;
  /* M3DM11: F / transposed inverse in the order 11 22 33 23 13 12 32 31 21 */
  const double G = 0.5 * o->G2;
  const double J = detF;
  const double F[9] = {F3[0][0], F3[1][1], F3[2][2], F3[1][2], F3[0][2], F3[0][1], F3[2][1], F3[2][0], F3[1][0]};
  double FIT[9];
  FIT[0] = (F[1] * F[2] - F[3] * F[6]) / J;
  FIT[1] = (F[0] * F[2] - F[4] * F[7]) / J;
  FIT[2] = (F[0] * F[1] - F[5] * F[8]) / J;
  FIT[3] = (F[5] * F[7] - F[0] * F[6]) / J;
  FIT[4] = (F[8] * F[6] - F[1] * F[7]) / J;
  FIT[5] = (F[3] * F[7] - F[2] * F[8]) / J;
  FIT[6] = (F[4] * F[8] - F[3] * F[0]) / J;
  FIT[7] = (F[3] * F[5] - F[4] * F[1]) / J;
  FIT[8] = (F[4] * F[6] - F[5] * F[2]) / J;
  const double lnJ = o->f_log(J);
  for (int i = 0; i < 9; ++i) ppk_new[i] = G * (F[i] - FIT[i]) + o->lamda * lnJ * FIT[i];
  const double FT[9] = {F[0], F[1], F[2], F[6], F[7], F[8], F[3], F[4], F[5]};
  double* sig = o->sig;
  sig[0] = (ppk_new[0] * FT[0] + ppk_new[5] * FT[8] + ppk_new[4] * FT[7]) / J;
  sig[1] = (ppk_new[8] * FT[5] + ppk_new[1] * FT[1] + ppk_new[3] * FT[6]) / J;
  sig[2] = (ppk_new[7] * FT[4] + ppk_new[6] * FT[3] + ppk_new[2] * FT[2]) / J;
  sig[3] = (ppk_new[8] * FT[4] + ppk_new[1] * FT[3] + ppk_new[3] * FT[2]) / J;
  sig[4] = (ppk_new[0] * FT[4] + ppk_new[5] * FT[3] + ppk_new[4] * FT[2]) / J;
  sig[5] = (ppk_new[0] * FT[5] + ppk_new[5] * FT[1] + ppk_new[4] * FT[6]) / J;
  o->sm = (sig[0] + sig[1] + sig[2]) / 3.0;
  o->sd[0] = sig[0] - o->sm;
  o->sd[1] = sig[1] - o->sm;
  o->sd[2] = sig[2] - o->sm;
  o->sd[3] = sig[3];
  o->sd[4] = sig[4];
  o->sd[5] = sig[5];
  o->seqv = equivalent_stress(o);
  const double* dF = &o->deF[0][0];
  const double deltaFp[9] = {dF[0], dF[4], dF[8], dF[5], dF[2], dF[1], dF[7], dF[6], dF[3]};
  o->ieinc = 0.0;
  for (int i = 0; i < 9; ++i) o->ieinc = o->ieinc + 0.5 * (ppk_old[i] + ppk_new[i]) * deltaFp[i];
  o->iener = o->iener + o->ieinc * 0.5 * (o->vol_ + o->vold);
  memcpy(p->PK, ppk_new, sizeof p->PK);
  p->SM = o->sm;
  p->Seqv = o->seqv;
  p->SDxx = o->sd[0]; p->SDyy = o->sd[1]; p->SDzz = o->sd[2];
  p->SDyz = o->sd[3]; p->SDxz = o->sd[4]; p->SDxy = o->sd[5];
  p->sig_y = o->sig_y_;
  p->epeff = o->epeff_;
  p->ie = o->iener;
  p->cp = o->cp;
  p->q = o->bqf;
  return MPM_OK;
}

/* TLParticleStressUpdate, update_step.f90:649-828 (the strain-rate and spin
 * sums of the reference are not used by TLConstitution) */
static int tl_particle_stress_update(orc* o) {
  if (o->SGMP) sg_cell_gradients(o);
  for (int b = 0; b < o->nb_body; ++b) {
    const int64_t cb = comp_base(o, b);
    for (int64_t ip = o->body[b].par_begin; ip < o->body[b].par_end; ++ip) {
      opart* p = &o->pt[ip];
      double deFp[3][3];
      memset(deFp, 0, sizeof deFp);
      if (o->SGMP) {
        if (p->centericell < 0) continue;
        for (int n = 0; n < 8; ++n) o->CenterInflNode[n] = o->CenterCellNode[p->centericell - 1][n];
        sg_nshape(o, p->XXN);
        for (int n = 0; n < 8; ++n) {
          if (!center_valid(o, o->CenterInflNode[n])) continue;
          const ocellp* cd = &o->cellp[o->CenterInflNode[n] - 1];
          double s = o->SHP[n];
          for (int i = 0; i < 3; ++i) {
            deFp[i][0] = deFp[i][0] + s * cd->CdeFp[i][0];
            deFp[i][1] = deFp[i][1] + s * cd->CdeFp[i][1];
            deFp[i][2] = deFp[i][2] + s * cd->CdeFp[i][2];
          }
        }
      } else {
        if (p->icell < 0) continue;
        particle_shape(o, p, p->icell);
        for (int n = 0; n < o->nb_InflNode; ++n) {
          if (!node_valid(o, o->InflNode[n])) continue;
          const ogrid* gd = &o->grid[cb + o->InflNode[n] - 1];
          if (!(gd->Mg > o->CutOff)) continue;
          double v[3];
          for (int c = 0; c < 3; ++c) v[c] = gd->PXg[c] / gd->Mg;
          double dx = o->DNDX[n], dy = o->DNDY[n], dz = o->DNDZ[n];
          for (int i = 0; i < 3; ++i) {
            deFp[i][0] = deFp[i][0] + dx * v[i];
            deFp[i][1] = deFp[i][1] + dy * v[i];
            deFp[i][2] = deFp[i][2] + dz * v[i];
          }
        }
      }
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) deFp[i][j] = deFp[i][j] * o->DT;
      if (o->UpdateVbyFp)
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) p->Fp[i][j] = p->Fp[i][j] + deFp[i][j];
      int st = tl_constitution(o, b, ip, (const double (*)[3])deFp);
      if (st) return st;
      if (!o->USF) memcpy(p->Xp, p->XX, sizeof p->Xp);
    }
  }
  return MPM_OK;
}

/* TLGridMomentumUpdate, update_step.f90:1015-1191 */
static void tl_grid_momentum_update(orc* o) {
  if (o->SGMP)
    for (int i = 0; i < o->nb_centernode; ++i) {
      memset(o->cellp[i].CPKint, 0, sizeof o->cellp[i].CPKint);
      memset(o->cellp[i].Cfext, 0, sizeof o->cellp[i].Cfext);
    }
  for (int64_t n = 0; n < all_nodes(o); ++n) o->grid[n].FXg[0] = o->grid[n].FXg[1] = o->grid[n].FXg[2] = 0.0;
  if (o->contact) memset(o->ndir, 0, sizeof(double[3]) * (size_t)all_nodes(o));
  for (int b = 0; b < o->nb_body; ++b) {
    const int64_t cb = comp_base(o, b);
    for (int64_t ip = o->body[b].par_begin; ip < o->body[b].par_end; ++ip) {
      opart* p = &o->pt[ip];
      const double* K = p->PK; /* xx yy zz yz xz xy zy zx yx */
      const double vol_ = p->VOL0, mp_ = p->mass;
      double fx[3];
      particle_fx(o, p, b, fx);
      if (o->SGMP) {
        if (p->centericell < 0) continue;
        for (int n = 0; n < 8; ++n) o->CenterInflNode[n] = o->CenterCellNode[p->centericell - 1][n];
        sg_nshape(o, p->XXN);
        for (int n = 0; n < 8; ++n) {
          if (!center_valid(o, o->CenterInflNode[n])) continue;
          ocellp* cd = &o->cellp[o->CenterInflNode[n] - 1];
          double s = o->SHP[n];
          for (int c = 0; c < 3; ++c) cd->Cfext[c] = cd->Cfext[c] + fx[c] * s;
          for (int k = 0; k < 9; ++k) cd->CPKint[k] = cd->CPKint[k] + s * K[k] * vol_;
        }
      } else {
        if (p->icell < 0) continue;
        particle_shape(o, p, p->icell);
        for (int n = 0; n < o->nb_InflNode; ++n) {
          if (!node_valid(o, o->InflNode[n])) continue;
          ogrid* gd = &o->grid[cb + o->InflNode[n] - 1];
          double s = o->SHP[n], dx = o->DNDX[n], dy = o->DNDY[n], dz = o->DNDZ[n];
          double fi[3];
          fi[0] = -(K[0] * dx + K[5] * dy + K[4] * dz) * vol_;
          fi[1] = -(K[8] * dx + K[1] * dy + K[3] * dz) * vol_;
          fi[2] = -(K[7] * dx + K[6] * dy + K[2] * dz) * vol_;
          for (int c = 0; c < 3; ++c) gd->FXg[c] = gd->FXg[c] + fi[c] + fx[c] * s;
          if (o->contact) {
            double* nd = o->ndir[cb + o->InflNode[n] - 1];
            nd[0] = nd[0] + dx * mp_;
            nd[1] = nd[1] + dy * mp_;
            nd[2] = nd[2] + dz * mp_;
          }
        }
      }
    }
  }
  if (o->SGMP) {
    cnshape(o);
    for (int i = 0; i < o->nb_centernode; ++i) {
      const ocellp* cd = &o->cellp[i];
      const double* C = cd->CPKint;
      for (int j = 0; j < 8; ++j) {
        ogrid* gd = &o->grid[o->CellsNode[i][j] - 1];
        double dx = o->CDNDX[j], dy = o->CDNDY[j], dz = o->CDNDZ[j];
        double fi[3];
        fi[0] = -(C[0] * dx + C[5] * dy + C[4] * dz);
        fi[1] = -(C[8] * dx + C[1] * dy + C[3] * dz);
        fi[2] = -(C[7] * dx + C[6] * dy + C[2] * dz);
        for (int c = 0; c < 3; ++c) gd->FXg[c] = gd->FXg[c] + 0.125 * cd->Cfext[c] + fi[c];
      }
    }
  }
}

/* UpdateDT, update_step.f90:1833-1874 */
static void update_dt(orc* o) {
  double max_vp = 0;
  for (int b = 0; b < o->nb_body; ++b)
    for (int64_t ip = o->body[b].par_begin; ip < o->body[b].par_end; ++ip) {
      const double* v = o->pt[ip].VXp;
      double m = fabs(v[0]);
      if (fabs(v[1]) > m) m = fabs(v[1]);
      if (fabs(v[2]) > m) m = fabs(v[2]);
      if (max_vp < m) max_vp = m;
    }
  o->DT = (double)1e6f;
  for (int m = 0; m < o->nb_mat; ++m) {
    const mpm_material* mt = &o->mat[m];
    if (mt->mat_type == 12) continue;
    double E = mt->young, nu = mt->poisson, ro = mt->density;
    double vv = sqrt(E * (1 - nu) / (1 + nu) / (1 - 2 * nu) / ro);
    if (mt->D > vv) vv = mt->D;
    if (mt->wavespd > vv) vv = mt->wavespd;
    vv = vv + max_vp;
    double t = o->DCell / vv;
    if (t < o->DT) o->DT = t;
  }
  o->DT = o->DT * o->DTScale;
}

/* SmoothStressbyGrid, update_step.f90:1876-2055: the particles' pressure
 * -SM mapped to the grid with volume weights, normalised by the mapped
 * volume, and interpolated back (Spre). The shapes are those of the
 * step's cells: GIMP and B-spline weights use the current Xp against the
 * cell found at the start of the step, linear ones XN, SGMP ones XXN. With
 * SGMP the map goes through the centre nodes (every grid node counts as
 * mapped, so a node without volume gets 0/0) and back through nodes above
 * the cut-off mass. */
static void smooth_stress(orc* o) {
  for (int n = 0; n < o->nb_gridnode; ++n) {
    o->grid[n].Gpre = 0.0;
    o->grid[n].GV_all = 0.0;
    o->grid[n].mapped = 0;
  }
  if (o->SGMP)
    for (int c = 0; c < o->nb_centernode; ++c) {
      o->cellp[c].CGpre = 0.0;
      o->cellp[c].CGV_all = 0.0;
    }
  for (int b = 0; b < o->nb_body; ++b)
    for (int64_t ip = o->body[b].par_begin; ip < o->body[b].par_end; ++ip) {
      opart* p = &o->pt[ip];
      if (o->SGMP) {
        if (p->centericell < 0) continue;
        for (int n = 0; n < 8; ++n) o->CenterInflNode[n] = o->CenterCellNode[p->centericell - 1][n];
        sg_nshape(o, p->XXN);
        for (int n = 0; n < 8; ++n) {
          if (!center_valid(o, o->CenterInflNode[n])) continue;
          ocellp* cd = &o->cellp[o->CenterInflNode[n] - 1];
          double SHPn = o->SHP[n];
          const double v = o->TLMPM ? p->VOL0 : p->VOL; /* TLSmoothStressbyGrid: VOL0 */
          cd->CGpre = cd->CGpre + SHPn * (-1 * p->SM) * v;
          cd->CGV_all = cd->CGV_all + SHPn * v;
        }
      } else {
        if (p->icell < 0) continue;
        particle_shape(o, p, p->icell);
        for (int n = 0; n < o->nb_InflNode; ++n) {
          if (!node_valid(o, o->InflNode[n])) continue;
          ogrid* gd = &o->grid[o->InflNode[n] - 1];
          gd->mapped = 1;
          double SHPn = o->SHP[n];
          const double v = o->TLMPM ? p->VOL0 : p->VOL;
          gd->Gpre = gd->Gpre + SHPn * (-1 * p->SM) * v;
          gd->GV_all = gd->GV_all + SHPn * v;
        }
      }
    }
  if (o->SGMP)
    for (int i = 0; i < o->nb_centernode; ++i)
      for (int j = 0; j < 8; ++j) {
        ogrid* gd = &o->grid[o->CellsNode[i][j] - 1];
        gd->mapped = 1;
        gd->Gpre = gd->Gpre + 0.125 * o->cellp[i].CGpre;
        gd->GV_all = gd->GV_all + 0.125 * o->cellp[i].CGV_all;
      }
  for (int n = 0; n < o->nb_gridnode; ++n)
    if (o->grid[n].mapped) o->grid[n].Gpre = o->grid[n].Gpre / o->grid[n].GV_all;
  if (o->SGMP) {
    for (int i = 0; i < o->nb_centernode; ++i) o->cellp[i].CGpre = 0.0;
    for (int i = 0; i < o->nb_centernode; ++i)
      for (int j = 0; j < 8; ++j) {
        const ogrid* gd = &o->grid[o->CellsNode[i][j] - 1];
        if (gd->Mg > o->CutOff) o->cellp[i].CGpre = o->cellp[i].CGpre + 0.125 * gd->Gpre;
      }
  }
  for (int b = 0; b < o->nb_body; ++b)
    for (int64_t ip = o->body[b].par_begin; ip < o->body[b].par_end; ++ip) {
      opart* p = &o->pt[ip];
      p->Spre = 0;
      if (o->SGMP) {
        if (p->centericell < 0) continue;
        for (int n = 0; n < 8; ++n) o->CenterInflNode[n] = o->CenterCellNode[p->centericell - 1][n];
        sg_nshape(o, p->XXN);
        for (int n = 0; n < 8; ++n) {
          if (!center_valid(o, o->CenterInflNode[n])) continue;
          p->Spre = p->Spre + o->SHP[n] * o->cellp[o->CenterInflNode[n] - 1].CGpre;
        }
      } else {
        if (p->icell < 0) continue;
        particle_shape(o, p, p->icell);
        for (int n = 0; n < o->nb_InflNode; ++n) {
          if (!node_valid(o, o->InflNode[n])) continue;
          p->Spre = p->Spre + o->SHP[n] * o->grid[o->InflNode[n] - 1].Gpre;
        }
      }
    }
}

/* ====================================================================
 * driver
 * ==================================================================== */

int orc_phase(orc* o, int phase) {
  if (!o) return MPM_ERR_ARG;
  switch (phase) {
    case MPM_PHASE_BEGIN_STEP:
      o->istep = o->istep + 1;
      o->CurrentTime = o->CurrentTime + o->DT;
      o->EngInternal = 0.0;
      return MPM_OK;
    case MPM_PHASE_GRID_MOMENTUM_INITIAL:
      if (o->TLMPM) tl_grid_momentum_initial(o);
      else grid_momentum_initial(o);
      return MPM_OK;
    case MPM_PHASE_APPLY_BOUNDARY: apply_bc(o); return MPM_OK;
    case MPM_PHASE_PARTICLE_STRESS_UPDATE: return o->TLMPM ? tl_particle_stress_update(o) : particle_stress_update(o);
    case MPM_PHASE_GRID_MOMENTUM_UPDATE:
      if (o->TLMPM) tl_grid_momentum_update(o);
      else grid_momentum_update(o);
      return MPM_OK;
    case MPM_PHASE_INTEGRATE_MOMENTUM: integrate_momentum(o); return MPM_OK;
    case MPM_PHASE_PARTICLE_POSITION_UPDATE: particle_position_update(o); return MPM_OK;
    case MPM_PHASE_GRID_MOMENTUM_MUSL: grid_momentum_musl(o); return MPM_OK;
    case MPM_PHASE_CALC_ENERGY: calc_energy(o); return MPM_OK;
    case MPM_PHASE_UPDATE_DT: update_dt(o); return MPM_OK;
    case MPM_PHASE_DR_DAMPING: dr_damping(o); return MPM_OK;
    case MPM_PHASE_SMOOTH_STRESS: smooth_stress(o); return MPM_OK;
    case MPM_PHASE_CONTACT:
      if (o->contact && o->contact_type == 1) lagr_contact(o);
      return MPM_OK;
    default: return oerr(o, MPM_ERR_ARG, "unknown phase %d", phase);
  }
}

/* one pass of the time loop body, MPM3D.f90:69-118 */
int orc_step(orc* o) {
  int st;
  orc_phase(o, MPM_PHASE_BEGIN_STEP);
  if (o->TLMPM) tl_grid_momentum_initial(o); /* MPM3D.f90:168-244 */
  else grid_momentum_initial(o);
  if (o->USF) {
    apply_bc(o);
    if ((st = o->TLMPM ? tl_particle_stress_update(o) : particle_stress_update(o))) return st;
  }
  if (o->TLMPM) tl_grid_momentum_update(o);
  else grid_momentum_update(o);
  integrate_momentum(o);
  if (o->contact && o->contact_type == 1) lagr_contact(o);
  particle_position_update(o);
  if (o->MUSL) {
    grid_momentum_musl(o);
    apply_bc(o);
  }
  if (!o->USF) {
    if ((st = o->TLMPM ? tl_particle_stress_update(o) : particle_stress_update(o))) return st;
  }
  calc_energy(o);
  update_dt(o);
  if (o->SmoothStress) smooth_stress(o);
  if (o->DR_DAMPING) dr_damping(o);
  return MPM_OK;
}

int orc_run(orc* o, int nsteps) {
  for (int s = 0; s < nsteps; ++s) {
    int st = orc_step(o);
    if (st) return st;
  }
  return MPM_OK;
}

int orc_create(const mpm_deck* d, int libm_mode, orc** out) {
  if (!d || !out) return MPM_ERR_ARG;
  *out = NULL;
  orc* o = (orc*)calloc(1, sizeof(orc));
  if (!o) return MPM_ERR_OOM;
  *out = o;
  o->TLMPM = !!(d->flags & MPM_F_TLMPM);
  if (o->TLMPM)
    for (int m = 0; m < d->nb_mat; ++m)
      if (d->mats[m].mat_type != 11)
        return oerr(o, MPM_ERR_UNSUPPORTED, "TLMPM supports the neo-Hookean material only (TLConstitution)");
  o->nb_component = d->nb_component > 0 ? d->nb_component : 1;
  o->contact = !!(d->flags & MPM_F_CONTACT);
  o->contact_type = d->contact_type;
  o->normbody = d->normbody;
  o->fricfa = d->fricfa;
  if ((d->flags & MPM_F_SGMP) && o->nb_component > 1)
    return oerr(o, MPM_ERR_UNSUPPORTED, "SGMP with several grid components is outside the restated step");
  if (o->contact && o->contact_type == 1 && (o->nb_component < 2 || o->normbody < 0 || o->normbody > 2))
    return oerr(o, MPM_ERR_ARG, "contact needs two grid components and normbody 0, 1 or 2");
  for (int b = 0; b < d->nb_body; ++b)
    if (o->contact && (d->bodies[b].comID < 1 || d->bodies[b].comID > o->nb_component))
      return oerr(o, MPM_ERR_ARG, "body %d: component %d out of 1..%d", b + 1, d->bodies[b].comID, o->nb_component);
  if (libm_mode == ORC_LIBM_PROJECT) {
    o->f_log = proj_log; o->f_exp = proj_exp; o->f_pow = proj_pow;
  } else {
    o->f_log = log; o->f_exp = exp; o->f_pow = pow;
  }
  const int f = d->flags;
  o->MUSL = !!(f & MPM_F_MUSL); o->USL = !!(f & MPM_F_USL); o->USF = !!(f & MPM_F_USF);
  o->GIMP = !!(f & MPM_F_GIMP); o->Bspline = !!(f & MPM_F_BSPLINE); o->SGMP = !!(f & MPM_F_SGMP);
  o->QuasiLoad = !!(f & MPM_F_QUASILOAD); o->QuasiDamp = !!(f & MPM_F_QUASIDAMP);
  o->UpdateVbyFp = !!(f & MPM_F_UVFP); o->Gravity = !!(f & MPM_F_GRAVITY);
  o->DR_DAMPING = !!(f & MPM_F_DRDAMP);
  o->SmoothStress = !!(f & MPM_F_SMOOTH);
  o->QuasiLoadTime = d->quasi_load_time;
  o->DampFactor = d->damp_factor;
  o->EndTime = d->endtime;
  o->DTScale = d->dtscale;
  o->bq1 = d->bq1;
  o->bq2 = d->bq2;
  o->np = d->nb_particle;
  o->nb_body = d->nb_body;
  o->nb_mat = d->nb_mat;
  o->body = (mpm_body*)malloc(sizeof(mpm_body) * (size_t)(d->nb_body > 0 ? d->nb_body : 1));
  o->mat = (mpm_material*)malloc(sizeof(mpm_material) * (size_t)(d->nb_mat > 0 ? d->nb_mat : 1));
  o->pt = (opart*)calloc((size_t)o->np, sizeof(opart));
  if (!o->body || !o->mat || !o->pt) return oerr(o, MPM_ERR_OOM, "out of memory");
  memcpy(o->body, d->bodies, sizeof(mpm_body) * (size_t)d->nb_body);
  memcpy(o->mat, d->mats, sizeof(mpm_material) * (size_t)d->nb_mat);
  for (int b = 0; b < o->nb_body; ++b)
    if (o->body[b].mat < 1 || o->body[b].mat > o->nb_mat) return oerr(o, MPM_ERR_ARG, "body %d has no material", b + 1);
  const int64_t np = o->np;
  for (int64_t p = 0; p < np; ++p) {
    opart* pt = &o->pt[p];
    pt->celsius_t = (double)293.0f; /* InitParticle, Particle.f90:131 */
    pt->mass = d->mass[p];
    for (int c = 0; c < 3; ++c) {
      pt->Xp[c] = d->xp[c * np + p];
      pt->Xo[c] = pt->Xp[c];
      pt->VXp[c] = d->vxp[c * np + p];
      pt->FXp[c] = d->fxp[c * np + p];
    }
  }
  for (int a = 0; a < 2; ++a) {
    o->SpanX[a] = d->span[0][a];
    o->SpanY[a] = d->span[1][a];
    o->SpanZ[a] = d->span[2][a];
  }
  o->DCell = d->dcell;
  o->CutOff = d->cutoff;
  memcpy(o->FixS, d->fixs, sizeof o->FixS);
  o->nb_InflNode = 8;
  o->centernb_InflNode = 8;
  initial(o, d);
  int st = set_grid_data(o);
  if (st) return st;
  set_dt(o);
  calc_energy(o); /* MPM3D.f90:42 */
  if (o->TLMPM) grid_mass_initial(o); /* MPM3D.f90:162 */
  return MPM_OK;
}

void orc_destroy(orc* o) {
  if (!o) return;
  free(o->pt); free(o->body); free(o->mat); free(o->node); free(o->grid); free(o->ndir); free(o->Cxg);
  free(o->cellp); free(o->CellsNode); free(o->CenterCellNode);
  free(o);
}

const char* orc_error(const orc* o) { return o ? o->err : "null oracle"; }
int64_t orc_nb_particle(const orc* o) { return o ? o->np : -1; }
int64_t orc_nb_gridnode(const orc* o) { return o ? o->nb_gridnode : -1; }
int orc_nb_component(const orc* o) { return o ? o->nb_component : -1; }
int orc_contact_force(const orc* o, double f[3]) {
  if (!o || !f) return MPM_ERR_ARG;
  for (int c = 0; c < 3; ++c) f[c] = o->tot_cont_for[c];
  return MPM_OK;
}
int64_t orc_nb_cell(const orc* o) { return o ? o->NumCell : -1; }

int orc_get_scalars(orc* o, double* s) {
  if (!o || !s) return MPM_ERR_ARG;
  memset(s, 0, sizeof(double) * MPM_NSCALARS);
  s[0] = o->istep; s[1] = o->CurrentTime; s[2] = o->DT; s[3] = o->EngKinetic;
  s[4] = o->EngInternal; s[5] = o->Momentum[0]; s[6] = o->Momentum[1]; s[7] = o->Momentum[2];
  s[8] = o->EngKinetic_prev; s[9] = o->nb_gridnode; s[10] = (double)o->np; s[11] = o->CutOff;
  s[12] = o->DCell; s[13] = (double)o->active_nodes;
  return MPM_OK;
}

#define PFIELD3(member)                                                           \
  for (int64_t p = 0; p < np; ++p)                                                \
    for (int c = 0; c < 3; ++c) {                                                 \
      if (set) o->pt[p].member[c] = in[c * np + p]; else out[c * np + p] = o->pt[p].member[c]; \
    }
#define PFIELD1(expr)                                                              \
  for (int64_t p = 0; p < np; ++p) {                                               \
    if (set) o->pt[p].expr = in[p]; else out[p] = (double)o->pt[p].expr;           \
  }

static int field_io(orc* o, int field, double* out, const double* in, int set) {
  const int64_t np = o->np;
  switch (field) {
    case MPM_P_XP: PFIELD3(Xp); break;
    case MPM_P_XX: PFIELD3(XX); break;
    case MPM_P_VXP: PFIELD3(VXp); break;
    case MPM_P_FXP: PFIELD3(FXp); break;
    case MPM_P_XN: PFIELD3(XN); break;
    case MPM_P_XXN: PFIELD3(XXN); break;
    case MPM_P_VOL: PFIELD1(VOL); break;
    case MPM_P_VOL0: PFIELD1(VOL0); break;
    case MPM_P_SIG_Y: PFIELD1(sig_y); break;
    case MPM_P_SM: PFIELD1(SM); break;
    case MPM_P_SEQV: PFIELD1(Seqv); break;
    case MPM_P_EPEFF: PFIELD1(epeff); break;
    case MPM_P_CELSIUS: PFIELD1(celsius_t); break;
    case MPM_P_DMG: PFIELD1(DMG); break;
    case MPM_P_LT: PFIELD1(LT); break;
    case MPM_P_IE: PFIELD1(ie); break;
    case MPM_P_MASS: PFIELD1(mass); break;
    case MPM_P_CP: PFIELD1(cp); break;
    case MPM_P_Q: PFIELD1(q); break;
    case MPM_P_SPRE: PFIELD1(Spre); break;
    case MPM_P_PK:
      for (int64_t p = 0; p < np; ++p)
        for (int c = 0; c < 9; ++c) {
          if (set) o->pt[p].PK[c] = in[c * np + p];
          else out[c * np + p] = o->pt[p].PK[c];
        }
      break;
    case MPM_P_SD:
      for (int64_t p = 0; p < np; ++p) {
        opart* t = &o->pt[p];
        double* f[6] = {&t->SDxx, &t->SDyy, &t->SDzz, &t->SDxy, &t->SDyz, &t->SDxz};
        for (int c = 0; c < 6; ++c) {
          if (set) *f[c] = in[c * np + p]; else out[c * np + p] = *f[c];
        }
      }
      break;
    case MPM_P_FP:
      for (int64_t p = 0; p < np; ++p)
        for (int c = 0; c < 9; ++c) {
          if (set) o->pt[p].Fp[c / 3][c % 3] = in[c * np + p];
          else out[c * np + p] = o->pt[p].Fp[c / 3][c % 3];
        }
      break;
    case MPM_P_FAILURE:
      for (int64_t p = 0; p < np; ++p) {
        if (set) o->pt[p].failure = in[p] != 0; else out[p] = o->pt[p].failure;
      }
      break;
    case MPM_P_ICELL:
      if (set) return MPM_ERR_ARG;
      for (int64_t p = 0; p < np; ++p) out[p] = o->pt[p].icell;
      break;
    case MPM_P_CENTERICELL:
      if (set) return MPM_ERR_ARG;
      for (int64_t p = 0; p < np; ++p) out[p] = o->pt[p].centericell;
      break;
    case MPM_P_INODE:
      if (set) return MPM_ERR_ARG;
      for (int64_t p = 0; p < np; ++p) out[p] = o->pt[p].inode;
      break;
    case MPM_G_MG:
      if (set) return MPM_ERR_ARG;
      for (int64_t n = 0; n < all_nodes(o); ++n) out[n] = o->grid[n].Mg;
      break;
    case MPM_G_PX:
    case MPM_G_FX: {
      if (set) return MPM_ERR_ARG;
      const int64_t nn = all_nodes(o);
      for (int64_t n = 0; n < nn; ++n)
        for (int c = 0; c < 3; ++c)
          out[c * nn + n] = field == MPM_G_PX ? o->grid[n].PXg[c] : o->grid[n].FXg[c];
      break;
    }
    case MPM_C_MG:
      if (set || !o->cellp) return MPM_ERR_ARG;
      for (int n = 0; n < o->NumCell; ++n) out[n] = o->cellp[n].Cmg;
      break;
    case MPM_C_PX: {
      if (set || !o->cellp) return MPM_ERR_ARG;
      const int64_t nc = o->NumCell;
      for (int64_t n = 0; n < nc; ++n)
        for (int c = 0; c < 3; ++c) out[c * nc + n] = o->cellp[n].Cpxg[c];
      break;
    }
    default:
      return oerr(o, MPM_ERR_ARG, "unknown field %d", field);
  }
  return MPM_OK;
}

int orc_download(orc* o, int field, double* out) {
  if (!o || !out) return MPM_ERR_ARG;
  return field_io(o, field, out, NULL, 0);
}

int orc_upload(orc* o, int field, const double* in) {
  if (!o || !in) return MPM_ERR_ARG;
  return field_io(o, field, NULL, in, 1);
}
