// mpm_setup.cu -- derivation of a scene's set-up from a parsed deck, shared by
// the single-scene contexts and the batched runtime: Initial
// (DataIn.f90:1211-1267), SetGridData (Grid.f90:222-418) and SetDT
// (DataIn.f90:1269-1297).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "mpm_setup.h"

namespace mpm {

static int fail(SceneSetup& out, int code, const char* fmt, ...) {
  char buf[256];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  out.err = buf;
  return code;
}

int scene_setup(const mpm_deck* d, SceneSetup& out, bool particle_fields) {
  Geometry& g = out.g;
  std::vector<double>& host_vol = out.vol;
  std::vector<double>& sig_y = out.sig_y;
  std::vector<double>& ie = out.ie;
  std::vector<double>& cp = out.cp;
  std::vector<double>& lt = out.lt;
  std::vector<uint8_t>& fix = out.fix;
  std::vector<uint8_t>& bd = out.bd;
  memset(&g, 0, sizeof g);
  const long long np = d->nb_particle;
  // materials (Initial overrides cEos(1) of null materials with the wave speed)
  out.mats.resize(d->nb_mat);
  for (int m = 0; m < d->nb_mat; ++m) {
    const mpm_material& s = d->mats[m];
    DevMaterial& t = out.mats[m];
    memset(&t, 0, sizeof t);
    t.mat_type = s.mat_type;
    t.eos_type = s.eos_type;
    t.density = s.density; t.miu = s.miu; t.young = s.young; t.poisson = s.poisson;
    t.yield0 = s.yield0; t.tangmod = s.tangmod; t.roomt = s.roomt; t.melt = s.melt; t.specheat = s.specheat;
    t.B_jc = s.B_jc; t.n_jc = s.n_jc; t.C_jc = s.C_jc; t.m_jc = s.m_jc; t.epso = s.epso; t.epf = s.epf;
    t.D = s.D;
    for (int k = 0; k < 10; ++k) t.cEos[k] = s.cEos[k];
    t.wavespd = s.wavespd; t.q_fai = s.q_fai; t.k_fai = s.k_fai; t.q_psi = s.q_psi; t.ten_f = s.ten_f;
    if (t.mat_type < 1 || t.mat_type > 11) return fail(out, MPM_ERR_ARG, "material %d has no type", m + 1);
    bool needs_eos = t.mat_type == 5 || t.mat_type == 6 || t.mat_type == 7 || t.mat_type == 8 || t.mat_type == 9;
    if (needs_eos && (t.eos_type < 1 || t.eos_type > 4))
      return fail(out, MPM_ERR_ARG, "material %d (type %d) needs an equation of state", m + 1, t.mat_type);
    if (t.eos_type == 3 && t.mat_type != 8)
      return fail(out, MPM_ERR_UNSUPPORTED, "JWL EOS is only supported with the 'hiex' material");
  }
  for (int m = 0; m < d->nb_mat; ++m)
    if (out.mats[m].mat_type == 9) out.mats[m].cEos[0] = out.mats[m].wavespd;
  out.bodies.resize(d->nb_body);
  for (int b = 0; b < d->nb_body; ++b) {
    if (d->bodies[b].mat < 1 || d->bodies[b].mat > d->nb_mat)
      return fail(out, MPM_ERR_ARG, "body %d has no material", b + 1);
    out.bodies[b].mat = d->bodies[b].mat - 1;
    for (int k = 0; k < 3; ++k) {
      out.bodies[b].gravp[k] = d->bodies[b].gravp[k];
      out.bodies[b].fgravp[k] = (float)d->bodies[b].gravp[k];
    }
  }
  // Initial: per-particle volume, yield stress, internal energy, sound speed,
  // lighting time (sqrt(...)/D is a default-REAL temporary)
  if (particle_fields) {
    host_vol.assign(np, 0.0); sig_y.assign(np, 0.0); ie.assign(np, 0.0); cp.assign(np, 0.0);
    lt.assign(np, 0.0);
  }
  for (int b = 0; b < (particle_fields ? d->nb_body : 0); ++b) {
    const DevMaterial& m = out.mats[out.bodies[b].mat];
    if (m.mat_type == 12) continue;
    // the body's material constants (the same for each of its particles)
    double cp_b = 0.0;
    if (m.mat_type == 1 || m.mat_type == 11) {
      double E = m.young, nu = m.poisson, ro = m.density;
      cp_b = std::sqrt(E * (1 - nu) / (1 + nu) / (1 - 2 * nu) / ro);
    }
    if (m.mat_type == 9) cp_b = m.wavespd;
    const double e0 = d->mats[out.bodies[b].mat].cEos[9];
    for (long long p = d->bodies[b].par_begin; p < d->bodies[b].par_end; ++p) {
      double vol = d->mass[p] / m.density;
      host_vol[p] = vol;
      sig_y[p] = m.yield0;
      ie[p] = e0 * vol;
      cp[p] = cp_b;
      double ltv = (double)10e6f;
      for (int j = 0; j < d->n_deto; ++j) {
        double dx = d->xp[p] - d->deto[j][0];
        double dy = d->xp[np + p] - d->deto[j][1];
        double dz = d->xp[2 * np + p] - d->deto[j][2];
        float t = (float)(std::sqrt(dx * dx + dy * dy + dz * dz) / m.D);
        if ((double)t < ltv) ltv = (double)t;
      }
      lt[p] = ltv;
    }
  }
  // SetGridData
  const double h = d->dcell;
  if (h == 0) return fail(out, MPM_ERR_ARG, "DCell must be defined");
  double sp[3], s0[3];
  for (int a = 0; a < 3; ++a) {
    s0[a] = d->span[a][0];
    sp[a] = d->span[a][1] - d->span[a][0];
    if (sp[a] <= 0) return fail(out, MPM_ERR_ARG, "computational region must be defined");
  }
  int NC[3], CNC[3];
  for (int a = 0; a < 3; ++a) {
    NC[a] = (int)(sp[a] / h + 0.5);
    CNC[a] = NC[a] - 1 == 0 ? 1 : NC[a] - 1;
  }
  long long nn = (long long)(NC[0] + 1) * (NC[1] + 1) * (NC[2] + 1);
  long long ncell = (long long)NC[0] * NC[1] * NC[2];
  if (nn > 2000000000LL) return fail(out, MPM_ERR_UNSUPPORTED, "grid too large for 32-bit node ids");
  if (np >= (1LL << 27)) return fail(out, MPM_ERR_UNSUPPORTED, "more than 2^27 particles per context");
  g.np = np;
  g.NCx = NC[0]; g.NCy = NC[1]; g.NCz = NC[2]; g.NCxy = NC[0] * NC[1];
  g.CNCx = CNC[0]; g.CNCy = CNC[1]; g.CNCz = CNC[2]; g.CNCxy = CNC[0] * CNC[1]; g.CNC = g.CNCxy * CNC[2];
  g.ncell = (int)ncell;
  g.NGx = NC[0] + 1; g.NGy = NC[1] + 1; g.NGz = NC[2] + 1; g.NGxy = g.NGx * g.NGy;
  g.nn = (int)nn;
  for (int a = 0; a < 3; ++a) {
    g.span0[a] = s0[a];
    g.span1[a] = s0[a] + NC[a] * h;
  }
  g.dcell = h;
  g.cutoff = d->cutoff;
  g.iJacobi = 2.0 / h;
  g.iJacobi4 = g.iJacobi * 0.125;
  g.iDCell = 1.0 / h;
  const int f = d->flags;
  const bool gimp = f & MPM_F_GIMP, bsp = f & MPM_F_BSPLINE, sgmp = f & MPM_F_SGMP;
  g.shape = sgmp ? 3 : (gimp ? 1 : (bsp ? 2 : 0));
  g.K = (g.shape == 1 || g.shape == 2) ? 27 : 8;
  for (int k = 0; k < 6; ++k) g.fixs[k] = d->fixs[k];
  g.usf = !!(f & MPM_F_USF);
  g.usl = !!(f & MPM_F_USL);
  g.musl = !!(f & MPM_F_MUSL);
  g.uvfp = !!(f & MPM_F_UVFP);
  g.qload = !!(f & MPM_F_QUASILOAD);
  g.qdamp = !!(f & MPM_F_QUASIDAMP);
  g.gravity = !!(f & MPM_F_GRAVITY);
  g.qload_time = d->quasi_load_time;
  g.damp_factor = d->damp_factor;
  g.bq1 = d->bq1;
  g.bq2 = d->bq2;
  g.dtscale = d->dtscale;
  g.nb_mat = d->nb_mat;
  g.nb_body = d->nb_body;
  g.has_jc = 0;
  for (auto& m : out.mats)
    if (m.mat_type == 4 || m.mat_type == 7) g.has_jc = 1;
  // grid components and contact (Particle.f90:69-92, DataIn.f90:1348-1393)
  g.ncomp = d->nb_component > 0 ? d->nb_component : 1;
  g.nnt = (long long)g.ncomp * nn;
  if (g.nnt > 2000000000LL) return fail(out, MPM_ERR_UNSUPPORTED, "grid too large for 32-bit node ids");
  g.contact = !!(f & MPM_F_CONTACT);
  g.contact_type = d->contact_type;
  g.normbody = d->normbody;
  g.fricfa = d->fricfa;
  g.tlmpm = !!(f & MPM_F_TLMPM);
  if (g.tlmpm)
    for (const auto& m : out.mats)
      if (m.mat_type != 11) return fail(out, MPM_ERR_UNSUPPORTED, "TLMPM supports the neo-Hookean material only");
  if (sgmp && g.ncomp > 1)
    return fail(out, MPM_ERR_UNSUPPORTED, "SGMP with several grid components (the reference shares its centre grid)");
  if (g.contact && g.contact_type == 1 && (g.ncomp < 2 || g.normbody < 0 || g.normbody > 2))
    return fail(out, MPM_ERR_ARG, "contact needs two grid components and normbody 0, 1 or 2");
  for (int b = 0; b < d->nb_body; ++b) {
    const int com = d->bodies[b].comID;
    if (g.contact && (com < 1 || com > g.ncomp)) return fail(out, MPM_ERR_ARG, "body component out of range");
    out.bodies[b].comp = g.contact ? com - 1 : 0;
  }
  // fixities and SGMP boundary types (Grid.f90:291-359)
  fix.assign(nn, 0);
  bd.assign(nn, 0);
  const int* F = d->fixs;
  const int NGx = g.NGx, NGy = g.NGy, NGz = g.NGz;
  for (int iz = 1; iz <= NGz; ++iz)
    for (int iy = 1; iy <= NGy; ++iy)
      for (int ix = 1; ix <= NGx; ++ix) {
        long long i = (long long)(iz - 1) * g.NGxy + (long long)(iy - 1) * NGx + (ix - 1);
        int bt[3] = {0, 0, 0};
        int idx[3] = {ix, iy, iz}, NG[3] = {NGx, NGy, NGz};
        for (int a = 0; a < 3; ++a) {
          if (idx[a] == 1 && F[2 * a] != 0) bt[a] = 1;
          if (idx[a] == NG[a] && F[2 * a + 1] != 0) bt[a] = 2;
          if (sgmp) {
            if (idx[a] == 2 && F[2 * a] != 0) bt[a] = 1;
            if (idx[a] == NG[a] - 1 && F[2 * a + 1] != 0) bt[a] = 2;
          }
        }
        bd[i] = (uint8_t)(bt[0] | (bt[1] << 2) | (bt[2] << 4));
        uint8_t fx = 0;
        bool all = false;
        for (int a = 0; a < 3; ++a) {
          bool lo1 = idx[a] == 1, hi1 = idx[a] == NG[a];
          bool lo2 = lo1 || idx[a] == 2, hi2 = hi1 || idx[a] == NG[a] - 1;
          bool two = gimp || bsp || sgmp;  // a second node layer is fixed too
          bool lo = two ? lo2 : lo1, hi = two ? hi2 : hi1;
          if ((lo && F[2 * a] == 1) || (hi && F[2 * a + 1] == 1)) all = true;
          if ((lo && F[2 * a] == 2) || (hi && F[2 * a + 1] == 2)) fx |= (uint8_t)(1 << a);
        }
        if (all) fx = 7;
        fix[i] = fx;
      }
  return MPM_OK;
}

double set_dt(const std::vector<DevMaterial>& mats, double dcell, double dtscale) {
  double dt = (double)1.0e6f;
  for (const auto& m : mats) {
    if (m.mat_type == 12) continue;
    double E = m.young, nu = m.poisson, ro = m.density;
    double cp = std::sqrt(E * (1 - nu) / (1 + nu) / (1 - 2 * nu) / ro);
    if (m.D > cp) cp = m.D;
    if (m.wavespd > cp) cp = m.wavespd;
    double t = dcell / cp;
    if (t < dt) dt = t;
  }
  return dt * dtscale;
}


}  // namespace mpm
