/* mpm_output.c -- MPM3D-F90 result files (DataOut.f90, the output parts of
 * DataIn.f90:34-103 and MPM3D.f90:284-305) from host arrays. The layouts and
 * the Fortran edit descriptors are the reference's; the code is this
 * project's own. */
#include "mpm_output.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mpm3d_gpu.h"

/* result option names (DataOut.f90:30-34) */
static const char* const kOutName[19] = {"", "seqv", "epef", "mat ", "pres", "volu", "engk", "engi", "velx", "vely",
                                         "velz", "cels", "fail", "sspd", "damg", "stsx", "disx", "disy", "disz"};

enum { kMaxCurves = 15 + 2, kMaxAnim = 10 + 1 };

struct mpm_output {
  const mpm_deck* d;
  FILE *curv, *energy, *momentum, *contact, *tec, *pvd;
  char job[1024];
  int ncurves, curve_option[kMaxCurves];
  int64_t curve_point[kMaxCurves]; /* 0-based */
  int nanim, anim_option[kMaxAnim];
  long ncurve_rows, nanim_frames;
  int pv_step; /* next ParaView frame number (the reference's iplotstep) */
  double* xo;  /* initial positions (Xo), component-major */
};

/* ------------------------------------------------------ Fortran edits */
int mpm_format_e(char* buf, int bufsize, int w, int d, double x) {
  char digits[64], body[96];
  int neg = signbit(x) ? 1 : 0;
  double a = fabs(x);
  int e10 = 0;
  if (d < 1 || d > 30 || bufsize < w + 1) return -1;
  if (a == 0.0 || !isfinite(a)) {
    memset(digits, '0', (size_t)d);
    digits[d] = 0;
    if (!isfinite(a)) { /* gfortran writes Infinity / NaN right-justified */
      const char* t = isnan(x) ? "NaN" : (neg ? "-Infinity" : "Infinity");
      snprintf(buf, (size_t)bufsize, "%*s", w, t);
      return 0;
    }
  } else {
    char m[64];
    snprintf(m, sizeof m, "%.*e", d - 1, a); /* D.DDDDe+XX, correctly rounded */
    int k = 0;
    digits[k++] = m[0];
    for (const char* p = m + 2; *p && *p != 'e'; ++p) digits[k++] = *p;
    digits[k] = 0;
    e10 = atoi(strchr(m, 'e') + 1) + 1; /* 0.DDDD x 10^e10 */
  }
  if (e10 >= -99 && e10 <= 99)
    snprintf(body, sizeof body, "%s0.%sE%c%02d", neg ? "-" : "", digits, e10 < 0 ? '-' : '+', abs(e10));
  else
    snprintf(body, sizeof body, "%s0.%s%c%03d", neg ? "-" : "", digits, e10 < 0 ? '-' : '+', abs(e10));
  int len = (int)strlen(body);
  if (len > w) {
    memset(buf, '*', (size_t)w);
    buf[w] = 0;
    return 0;
  }
  snprintf(buf, (size_t)bufsize, "%*s", w, body);
  return 0;
}

static void put_e(FILE* f, int w, int d, double x) {
  char b[64];
  mpm_format_e(b, sizeof b, w, d, x);
  fputs(b, f);
}

/* Aw of a string: right-justified when shorter, leftmost w characters when longer */
static void put_a(FILE* f, int w, const char* s) {
  int len = (int)strlen(s);
  if (len >= w) {
    fwrite(s, 1, (size_t)w, f);
  } else {
    for (int i = 0; i < w - len; ++i) fputc(' ', f);
    fputs(s, f);
  }
}

/* --------------------------------------------------------------- open */
static FILE* open_w(const char* path) { return fopen(path, "w"); }

static void grid_file(const mpm_output* o, const char* path);

int mpm_output_open(const mpm_deck* d, const char* job, const char* plot_dir, mpm_output** out) {
  if (!out) return MPM_ERR_ARG;
  *out = NULL;
  if (!d || !job || strlen(job) > 900) return MPM_ERR_ARG;
  mpm_output* o = (mpm_output*)calloc(1, sizeof *o);
  if (!o) return MPM_ERR_OOM;
  o->d = d;
  snprintf(o->job, sizeof o->job, "%s", job);
  /* curves: the two defaults of DataOut.f90:46-54, then the deck's */
  o->ncurves = 2;
  o->curve_option[0] = 6;
  o->curve_option[1] = 7;
  o->curve_point[0] = o->curve_point[1] = 0;
  for (int i = 0; i < d->n_curves && o->ncurves < kMaxCurves; ++i) {
    o->curve_option[o->ncurves] = d->curve_option[i];
    o->curve_point[o->ncurves] = (int64_t)d->curve_point[i] - 1;
    o->ncurves++;
  }
  o->nanim = 1;
  o->anim_option[0] = 3; /* material number */
  for (int i = 0; i < d->n_anim && o->nanim < kMaxAnim; ++i) o->anim_option[o->nanim++] = d->anim_option[i];
  o->pv_step = 1;
  const int64_t np = d->nb_particle;
  o->xo = (double*)malloc(sizeof(double) * (size_t)(3 * (np > 0 ? np : 1)));
  if (!o->xo) {
    free(o);
    return MPM_ERR_OOM;
  }
  memcpy(o->xo, d->xp, sizeof(double) * (size_t)(3 * np));

  char path[1200], dir[1024];
  if (plot_dir) {
    snprintf(dir, sizeof dir, "%s", plot_dir);
  } else {
    snprintf(dir, sizeof dir, "%s", job);
    char* sl = strrchr(dir, '/');
    if (sl) sl[1] = 0;
    else dir[0] = 0;
  }
  int need_sep = dir[0] && dir[strlen(dir) - 1] != '/';
  snprintf(path, sizeof path, "%s_curv.dat", job);
  o->curv = open_w(path);
  snprintf(path, sizeof path, "%s%sEnergyPlot.dat", dir, need_sep ? "/" : "");
  o->energy = open_w(path);
  snprintf(path, sizeof path, "%s%sMomentumPlot.dat", dir, need_sep ? "/" : "");
  o->momentum = open_w(path);
  if (d->flags & MPM_F_CONTACT) { /* DataIn.f90:89 */
    snprintf(path, sizeof path, "%s%sContforcPlot.dat", dir, need_sep ? "/" : "");
    o->contact = open_w(path);
  }
  if (!o->curv || !o->energy || !o->momentum || ((d->flags & MPM_F_CONTACT) && !o->contact)) {
    mpm_output_close(o);
    return MPM_ERR_IO;
  }
  if (d->flags & MPM_F_TECPLOT) {
    snprintf(path, sizeof path, "%s_anim.dat", job);
    if (!(o->tec = open_w(path))) {
      mpm_output_close(o);
      return MPM_ERR_IO;
    }
  }
  if (d->flags & MPM_F_PARAVIEW) {
    snprintf(path, sizeof path, "%s_anim.pvd", job);
    if (!(o->pvd = open_w(path))) {
      mpm_output_close(o);
      return MPM_ERR_IO;
    }
    fputs("<?xml version=\"1.0\"?>\n", o->pvd);
    fputs("<VTKFile type=\"Collection\" version=\"0.1\" byte_order=\"BigEndian\" "
          "compressor=\"vtkZLibDataCompressor\">\n",
          o->pvd);
    fputs("    <Collection>\n", o->pvd);
    snprintf(path, sizeof path, "%s_Grid.vtu", job);
    grid_file(o, path);
  }
  *out = o;
  return MPM_OK;
}

void mpm_output_close(mpm_output* o) {
  if (!o) return;
  if (o->pvd) {
    fputs("    </Collection>\n", o->pvd);
    fputs("</VTKFile>\n", o->pvd);
    fclose(o->pvd);
  }
  if (o->tec) fclose(o->tec);
  if (o->curv) fclose(o->curv);
  if (o->energy) fclose(o->energy);
  if (o->momentum) fclose(o->momentum);
  if (o->contact) fclose(o->contact);
  free(o->xo);
  free(o);
}

int mpm_output_curve_count(const mpm_output* o) { return o ? o->ncurves : -1; }

/* ---------------------------------------------------------- OutCurve */
int mpm_output_curve_items(const mpm_output* o, int64_t* particle, int* field, int* component, int max) {
  if (!o) return -MPM_ERR_ARG;
  int n = 0;
#define ITEM(F, C)                 \
  do {                             \
    if (n < max) {                 \
      particle[n] = p;             \
      field[n] = (F);              \
      component[n] = (C);          \
    }                              \
    ++n;                           \
  } while (0)
  for (int i = 0; i < o->ncurves; ++i) {
    const int64_t p = o->curve_point[i];
    switch (o->curve_option[i]) {
      case 1: ITEM(MPM_P_SEQV, 0); break;
      case 2: case 3: ITEM(MPM_P_EPEFF, 0); break;
      case 4: ITEM(MPM_P_SM, 0); break;
      case 5: ITEM(MPM_P_VOL, 0); break;
      case 8: case 9: case 10: ITEM(MPM_P_VXP, o->curve_option[i] - 8); break;
      case 11: ITEM(MPM_P_CELSIUS, 0); break;
      case 12: ITEM(MPM_P_FAILURE, 0); break;
      case 13: ITEM(MPM_P_SD, 2); break; /* OutCurve writes SDzz for 'sspd' */
      case 14: ITEM(MPM_P_DMG, 0); break;
      case 15: ITEM(MPM_P_SD, 0); ITEM(MPM_P_SM, 0); break;
      case 16: case 17: case 18: ITEM(MPM_P_XP, o->curve_option[i] - 16); break;
      default: break; /* 6, 7: energies from the scalars */
    }
  }
#undef ITEM
  return n;
}

int mpm_output_curve(mpm_output* o, const double* s, const double* v) {
  if (!o || !s) return MPM_ERR_ARG;
  FILE* f = o->curv;
  if (o->ncurve_rows == 0) {
    fputs("Time ", f);
    for (int i = 0; i < o->ncurves; ++i) {
      char id[32];
      snprintf(id, sizeof id, "%lld", (long long)(o->curve_point[i] + 1));
      fputs(kOutName[o->curve_option[i]], f);
      fprintf(f, "%-8.8s", id);
    }
    fputc('\n', f);
  }
  const double t = s[1], ke = s[3], ie = s[4];
  put_e(f, 12, 4, t);
  int k = 0;
  for (int i = 0; i < o->ncurves; ++i) {
    const int opt = o->curve_option[i];
    double x = 0.0;
    switch (opt) {
      case 6: x = ke; break;
      case 7: x = ie; break;
      case 4: x = -v[k++]; break;
      case 15: x = v[k] + v[k + 1]; k += 2; break;
      case 16: case 17: case 18: x = v[k++] - o->xo[(opt - 16) * o->d->nb_particle + o->curve_point[i]]; break;
      case 12: fprintf(f, "%12d", v[k++] != 0.0 ? 1 : 0); continue;
      default: x = v[k++]; break;
    }
    put_e(f, 12, 4, x);
  }
  fputc('\n', f);
  put_e(o->energy, 12, 4, t);
  put_e(o->energy, 12, 4, ke + ie);
  put_e(o->energy, 12, 4, ke);
  put_e(o->energy, 12, 4, ie);
  fputc('\n', o->energy);
  put_e(o->momentum, 12, 4, t);
  for (int a = 0; a < 3; ++a) put_e(o->momentum, 12, 4, s[5 + a]);
  fputc('\n', o->momentum);
  o->ncurve_rows++;
  return ferror(f) || ferror(o->energy) || ferror(o->momentum) ? MPM_ERR_IO : MPM_OK;
}

int mpm_output_contact(mpm_output* o, double time, const double* force3) {
  if (!o || !force3) return MPM_ERR_ARG;
  if (!o->contact) return MPM_OK;
  put_e(o->contact, 12, 4, time);
  for (int a = 0; a < 3; ++a) put_e(o->contact, 12, 4, force3[a]);
  fputc('\n', o->contact);
  return ferror(o->contact) ? MPM_ERR_IO : MPM_OK;
}

/* ----------------------------------------------------------- OutAnim */
static int tecplot_frame(mpm_output* o, const double* s, const mpm_particle_view* v) {
  FILE* f = o->tec;
  const mpm_deck* d = o->d;
  const int64_t np = d->nb_particle;
  if (o->nanim_frames == 0) {
    fputs("TITLE = \"", f);
    char title[61];
    snprintf(title, sizeof title, "%-60.60s", d->title);
    fputs(title, f);
    fputs("\"\n", f);
    /* format ('VARIABLES= "X"   "Y"   "Z"  ', 50(A2, A4, A1)): each name is
       written with the next of A2, A4, A1 in turn (leftmost characters) */
    fputs("VARIABLES= \"X\"   \"Y\"   \"Z\"  ", f);
    static const int kw[3] = {2, 4, 1};
    for (int i = 0; i < o->nanim; ++i) {
      char q[16];
      char name[8];
      snprintf(name, sizeof name, "%s", kOutName[o->anim_option[i]]);
      for (int j = (int)strlen(name) - 1; j >= 0 && name[j] == ' '; --j) name[j] = 0; /* trim */
      snprintf(q, sizeof q, "\"%s\"", name);
      put_a(f, kw[i % 3], q);
    }
    fputc('\n', f);
  }
  fputs("ZONE T=\"time", f);
  put_e(f, 10, 3, s[1]);
  fputs("\"\n", f);
  for (int b = 0; b < d->nb_body; ++b) {
    const int mat = d->bodies[b].mat;
    for (int64_t p = d->bodies[b].par_begin; p < d->bodies[b].par_end; ++p) {
      if (v->icell && v->icell[p] < 0) continue;
      if (d->skip && d->skip[p]) continue;
      for (int a = 0; a < 3; ++a) put_e(f, 12, 4, v->xp[a * np + p]);
      for (int i = 0; i < o->nanim; ++i) {
        switch (o->anim_option[i]) {
          case 1: put_e(f, 12, 4, v->seqv[p]); break;
          case 2: put_e(f, 12, 4, v->epeff[p]); break;
          case 3: fprintf(f, "%3d", mat); break;
          case 4: put_e(f, 12, 4, -v->sm[p]); break;
          case 5: put_e(f, 12, 4, v->vol[p]); break;
          case 6: {
            const double vx = v->vxp[p], vy = v->vxp[np + p], vz = v->vxp[2 * np + p];
            put_e(f, 12, 4, 0.5 * v->mass[p] * (vx * vx + vy * vy + vz * vz));
            break;
          }
          case 7: put_e(f, 12, 4, v->ie[p]); break;
          case 8: case 9: case 10: put_e(f, 12, 4, v->vxp[(o->anim_option[i] - 8) * np + p]); break;
          case 11: put_e(f, 12, 4, v->celsius[p]); break;
          case 12: fprintf(f, "%3d", v->failure[p] != 0.0 ? 1 : 0); break;
          case 13: put_e(f, 12, 4, v->cp[p]); break;
          case 14: put_e(f, 12, 4, v->dmg[p]); break;
          case 15: put_e(f, 12, 4, v->sd[p] + v->sm[p]); break;
          case 16: put_e(f, 12, 4, v->xp[p] - o->xo[p]); break;
          default: break; /* 17, 18: not written by OutAnim */
        }
      }
      fputc('\n', f);
    }
  }
  return ferror(f) ? MPM_ERR_IO : MPM_OK;
}

/* --------------------------------------------------------- OutAnimPV */
static void pv_array(FILE* f, const char* name, int64_t np, const double* a, double sign, const double* minus) {
  fprintf(f, "            <DataArray type=\"Float32\" Name=\"%s\" Format=\"ascii\">\n", name);
  for (int64_t p = 0; p < np; ++p) {
    double x = a ? sign * a[p] : 0.0;
    if (minus) x -= minus[p];
    fputs("                ", f);
    put_e(f, 12, 4, x);
    fputc('\n', f);
  }
  fputs("            </DataArray>\n", f);
}

static int paraview_frame(mpm_output* o, const double* s, const mpm_particle_view* v) {
  const int64_t np = o->d->nb_particle;
  char path[1200], next[1200];
  snprintf(path, sizeof path, "%s_anim.vtu", o->job);
  snprintf(next, sizeof next, "%s_anim_%d.vtu", o->job, o->pv_step);
  FILE* f = open_w(path);
  if (!f) return MPM_ERR_IO;
  fputs("<?xml version=\"1.0\"?>\n", f);
  fputs("<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"BigEndian\">\n", f);
  fputs("<UnstructuredGrid>\n", f);
  fprintf(f, "    <Piece NumberOfPoints=\"%lld\" NumberOfCells=\"%lld\">\n", (long long)np, (long long)np);
  fputs("        <Points>\n", f);
  /* list-directed write: a leading blank, then the items */
  fputs("             <DataArray type=\"Float32\" NumberOfComponents=\"3\" Format=\"ascii\">\n", f);
  for (int64_t p = 0; p < np; ++p) {
    fputs("                ", f);
    put_e(f, 12, 4, v->xp[p]);
    fputs("  ", f);
    put_e(f, 12, 4, v->xp[np + p]);
    fputs("  ", f);
    put_e(f, 12, 4, v->xp[2 * np + p]);
    fputc('\n', f);
  }
  fputs("            </DataArray>\n", f);
  fputs("        </Points>\n", f);
  fputs("        <PointData Scalars=\"scalars\">\n", f);
  pv_array(f, "seqv", np, v->seqv, 1.0, NULL);
  pv_array(f, "epeff", np, v->epeff, 1.0, NULL);
  pv_array(f, "pressure", np, v->sm, -1.0, NULL);
  pv_array(f, "Smoothpressure", np, v->spre, 1.0, NULL);
  pv_array(f, "MeanNormalStress", np, v->sm, 1.0, NULL);
  pv_array(f, "SmoothMeanNormalStress", np, v->spre, -1.0, NULL);
  pv_array(f, "vx", np, v->vxp, 1.0, NULL);
  pv_array(f, "vy", np, v->vxp + np, 1.0, NULL);
  pv_array(f, "vz", np, v->vxp + 2 * np, 1.0, NULL);
  pv_array(f, "disx", np, v->xp, 1.0, o->xo);
  pv_array(f, "disy", np, v->xp + np, 1.0, o->xo + np);
  pv_array(f, "disz", np, v->xp + 2 * np, 1.0, o->xo + 2 * np);
  pv_array(f, "fxpx", np, v->fxp, 1.0, NULL);
  pv_array(f, "fxpy", np, v->fxp + np, 1.0, NULL);
  pv_array(f, "fxpz", np, v->fxp + 2 * np, 1.0, NULL);
  pv_array(f, "vol", np, v->vol, 1.0, NULL);
  pv_array(f, "celsius_t", np, v->celsius, 1.0, NULL);
  pv_array(f, "damage", np, v->dmg, 1.0, NULL);
  /* stressx = SDxx + SM */
  fputs("            <DataArray type=\"Float32\" Name=\"stressx\" Format=\"ascii\">\n", f);
  for (int64_t p = 0; p < np; ++p) {
    fputs("                ", f);
    put_e(f, 12, 4, v->sd[p] + v->sm[p]);
    fputc('\n', f);
  }
  fputs("            </DataArray>\n", f);
  pv_array(f, "disx", np, v->xp, 1.0, o->xo);
  fputs("        </PointData>\n", f);
  fputs("        <Cells>\n", f);
  fputs("            <DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n", f);
  for (int64_t p = 0; p < np; ++p) fprintf(f, "                %10lld\n", (long long)p);
  fputs("            </DataArray>\n", f);
  fputs("            <DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n", f);
  for (int64_t p = 0; p < np; ++p) fprintf(f, "                %10lld\n", (long long)(p + 1));
  fputs("            </DataArray>\n", f);
  fputs("            <DataArray type=\"Float32\" Name=\"types\" Format=\"ascii\">\n", f);
  for (int64_t p = 0; p < np; ++p) fprintf(f, "                %10d\n", 1);
  fputs("            </DataArray>\n", f);
  fputs("        </Cells>\n", f);
  fputs("    </Piece>\n", f);
  fputs("</UnstructuredGrid>\n", f);
  fputs("</VTKFile>\n", f);
  int bad = ferror(f);
  fclose(f);
  if (bad || rename(path, next) != 0) return MPM_ERR_IO;
  const char* base = strrchr(next, '/');
  fputs("    <DataSet timestep=\"", o->pvd);
  put_e(o->pvd, 12, 4, s[1]);
  fprintf(o->pvd, "\" group=\"\" part=\"0\" file=\"%s\"/>\n", next);
  (void)base;
  o->pv_step++;
  return ferror(o->pvd) ? MPM_ERR_IO : MPM_OK;
}

int mpm_output_anim(mpm_output* o, const double* s, const mpm_particle_view* v) {
  if (!o || !s || !v || !v->xp) return MPM_ERR_ARG;
  int r = MPM_OK;
  if (o->tec && (r = tecplot_frame(o, s, v))) return r;
  if (o->pvd && (r = paraview_frame(o, s, v))) return r;
  o->nanim_frames++;
  return MPM_OK;
}

/* ----------------------------------------------------------- OutGrid */
static void grid_file(const mpm_output* o, const char* path) {
  const mpm_deck* d = o->d;
  const double h = d->dcell;
  int64_t nc[3];
  for (int a = 0; a < 3; ++a) nc[a] = (int64_t)((d->span[a][1] - d->span[a][0]) / h + 0.5); /* SetGridData */
  const int64_t ng[3] = {nc[0] + 1, nc[1] + 1, nc[2] + 1};
  const int64_t nn = ng[0] * ng[1] * ng[2], ncell = nc[0] * nc[1] * nc[2];
  FILE* f = open_w(path);
  if (!f) return;
  fputs("<?xml version=\"1.0\"?>\n", f);
  fputs("<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"BigEndian\">\n", f);
  fputs("<UnstructuredGrid>\n", f);
  fprintf(f, "    <Piece NumberOfPoints=\"%lld\" NumberOfCells=\"%lld\">\n", (long long)nn, (long long)ncell);
  fputs("        <Points>\n", f);
  fputs("             <DataArray type=\"Float32\" NumberOfComponents=\"3\" Format=\"ascii\">\n", f);
  for (int64_t k = 0; k < ng[2]; ++k)
    for (int64_t j = 0; j < ng[1]; ++j)
      for (int64_t i = 0; i < ng[0]; ++i) {
        fputs("                ", f);
        put_e(f, 12, 4, d->span[0][0] + (double)i * h);
        fputs("  ", f);
        put_e(f, 12, 4, d->span[1][0] + (double)j * h);
        fputs("  ", f);
        put_e(f, 12, 4, d->span[2][0] + (double)k * h);
        fputc('\n', f);
      }
  fputs("            </DataArray>\n", f);
  fputs("        </Points>\n", f);
  fputs("        <Cells>\n", f);
  fputs("            <DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n", f);
  /* cell corners in the order 1, 2, 4, 3, 5, 6, 8, 7 of CellsNode (VTK voxel) */
  static const int corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0},
                                   {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
  for (int64_t k = 0; k < nc[2]; ++k)
    for (int64_t j = 0; j < nc[1]; ++j)
      for (int64_t i = 0; i < nc[0]; ++i) {
        fputs("                ", f);
        for (int c = 0; c < 8; ++c) {
          int64_t n = (k + corner[c][2]) * ng[0] * ng[1] + (j + corner[c][1]) * ng[0] + (i + corner[c][0]);
          fprintf(f, "%lld    ", (long long)n);
        }
        fputc('\n', f);
      }
  fputs("            </DataArray>\n", f);
  fputs("            <DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n", f);
  for (int64_t c = 1; c <= ncell; ++c) fprintf(f, "                %lld\n", (long long)(8 * c));
  fputs("            </DataArray>\n", f);
  fputs("            <DataArray type=\"Int32\" Name=\"types\" Format=\"ascii\">\n", f);
  for (int64_t c = 0; c < ncell; ++c) fprintf(f, "                %5d\n", 11);
  fputs("            </DataArray>\n", f);
  fputs("        </Cells>\n", f);
  fputs("    </Piece>\n", f);
  fputs("</UnstructuredGrid>\n", f);
  fputs("</VTKFile>\n", f);
  fclose(f);
}
