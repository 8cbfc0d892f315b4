/*
 * mpm_deck.c -- the .mpm keyword reader (see include/mpm_deck.h for the
 * reference routines it follows).
 *
 * Numeric semantics that matter for bit-for-bit set-up:
 *   - every real field is converted to a 32-bit float (strtof, round to
 *     nearest) and then widened to double, as GetReal (a default-REAL function,
 *     FFI.f90:110) does;
 *   - Fortran 'd'/'D' exponents are accepted (list-directed input);
 *   - derived values computed at parse time in the reference (block/sphere
 *     particle mass, the null-material wave speed, Gruneisen coefficients, the
 *     grid-mass CutOff) are computed here in double with the same operation
 *     order, and FP32 literals of the reference (1e-5, 0.06, 3.1415926535, ...)
 *     are used as float constants.
 */
#include "mpm_deck.h"

#include <ctype.h>
#include <errno.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define LINE_MAX_CHARS 256 /* character(256) sss, FFI.f90:39 */
#define FIELD_MAX_CHARS 20 /* character(20) cmd_line(15), FFI.f90:40 */
#define FIELDS_PER_LINE 15

typedef struct reader {
  const char* text; /* whole input */
  size_t pos;       /* next unread byte */
  int line_nb;
  char line[LINE_MAX_CHARS + 1];         /* processed line (GetString) */
  char field[FIELDS_PER_LINE][FIELD_MAX_CHARS + 1];
  int nfield;   /* fields in the current line */
  int next;     /* index of the next unread field */
  mpm_deck* d;
  char* err;    /* points at d->err */
  int64_t par_counter;
  int body_counter;
  int plot2d_on;
} reader;

static int fail(reader* r, int code, const char* fmt, ...) {
  char msg[200];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof msg, fmt, ap);
  va_end(ap);
  snprintf(r->err, 256, "line %d: %s", r->line_nb, msg);
  return code;
}

/* Split one physical line into fields (ReadLine, FFI.f90:177-253). Returns the
 * number of fields, 0 for a blank/comment line, -1 at end of input, -2 when the
 * line holds more fields than the reference's 15-entry field table. */
static int read_line(reader* r) {
  if (r->text[r->pos] == '\0') return -1;
  /* copy the record, keeping at most 256 characters (longer records are cut) */
  size_t n = 0;
  const char* s = r->text + r->pos;
  size_t len = strcspn(s, "\n");
  r->pos += len + (s[len] == '\n' ? 1 : 0);
  r->line_nb++;
  char buf[LINE_MAX_CHARS + 1];
  for (size_t i = 0; i < len && n < LINE_MAX_CHARS; ++i) buf[n++] = s[i];
  buf[n] = '\0';
  for (size_t i = 0; i < n; ++i) {
    if (buf[i] == '\t' || buf[i] == '\r') buf[i] = ' ';
    if (buf[i] == '!') { buf[i] = '\0'; n = i; break; }
  }
  /* adjustl + len_trim */
  size_t b = 0;
  while (b < n && buf[b] == ' ') ++b;
  size_t e = n;
  while (e > b && buf[e - 1] == ' ') --e;
  memcpy(r->line, buf + b, e - b);
  r->line[e - b] = '\0';
  r->nfield = 0;
  r->next = 0;
  if (e == b) return 0;
  /* Fields: comma-separated segments, each split on blank runs; an empty
   * segment between two commas is one empty field. */
  const char* p = r->line;
  for (;;) {
    const char* comma = strchr(p, ',');
    const char* segend = comma ? comma : p + strlen(p);
    const char* q = p;
    int words = 0;
    while (q < segend) {
      while (q < segend && *q == ' ') ++q;
      if (q >= segend) break;
      const char* w = q;
      while (q < segend && *q != ' ') ++q;
      if (r->nfield >= FIELDS_PER_LINE) return -2;
      size_t wl = (size_t)(q - w);
      if (wl > FIELD_MAX_CHARS) wl = FIELD_MAX_CHARS; /* character(20) truncation */
      memcpy(r->field[r->nfield], w, wl);
      r->field[r->nfield][wl] = '\0';
      r->nfield++;
      words++;
    }
    if (words == 0 && (comma || p != r->line)) {
      if (r->nfield >= FIELDS_PER_LINE) return -2;
      r->field[r->nfield][0] = '\0';
      r->nfield++;
    }
    if (!comma) break;
    p = comma + 1;
  }
  return r->nfield;
}

/* Make sure a field is available (the "do while(nb_word.eq.0)" loops). */
static int need_field(reader* r) {
  while (r->next >= r->nfield) {
    int k = read_line(r);
    if (k == -1) return fail(r, MPM_ERR_PARSE, "end of file reached before 'endi'");
    if (k == -2) return fail(r, MPM_ERR_PARSE, "more than %d fields on one line", FIELDS_PER_LINE);
  }
  return MPM_OK;
}

/* pcomp(a, b, 4): case-insensitive 4-character compare, blank padded. */
static int kw_match(const char* field, const char* kw4) {
  const int inc = 'A' - 'a';
  for (int i = 0; i < 4; ++i) {
    int ia = (unsigned char)(i < (int)strlen(field) ? field[i] : ' ');
    int ib = (unsigned char)kw4[i];
    if (ia != ib && ia + inc != ib && ia != ib + inc) return 0;
  }
  return 1;
}

/* KeyWord: returns the 1-based position of the matched keyword (consumed), or
 * an error when the field matches none of them. */
static int keyword(reader* r, const char* const* kw, int nkw, const char* what, int* out) {
  int st = need_field(r);
  if (st) return st;
  for (int i = 0; i < nkw; ++i) {
    if (kw_match(r->field[r->next], kw[i])) {
      r->next++;
      *out = i + 1;
      return MPM_OK;
    }
  }
  return fail(r, MPM_ERR_PARSE, "invalid %s keyword '%s'", what, r->field[r->next]);
}

static int is_number(const char* f) {
  unsigned char a = (unsigned char)f[0];
  return a == '-' || (a > 47 && a < 58);
}

static int get_real(reader* r, double* out) {
  int st = need_field(r);
  if (st) return st;
  const char* f = r->field[r->next];
  if (!is_number(f)) return fail(r, MPM_ERR_PARSE, "non-numeric field '%s'", f);
  char tmp[FIELD_MAX_CHARS + 1];
  size_t n = strlen(f);
  for (size_t i = 0; i <= n; ++i) {
    char c = f[i];
    tmp[i] = (c == 'd' || c == 'D' || c == 'q' || c == 'Q') ? 'e' : c;
  }
  char* end = NULL;
  errno = 0;
  float v = strtof(tmp, &end);
  if (end == tmp || *end != '\0') return fail(r, MPM_ERR_PARSE, "bad real '%s'", f);
  r->next++;
  *out = (double)v; /* REAL(4) result widened on assignment to REAL(8) */
  return MPM_OK;
}

static int get_int(reader* r, int64_t* out) {
  int st = need_field(r);
  if (st) return st;
  const char* f = r->field[r->next];
  if (!is_number(f)) return fail(r, MPM_ERR_PARSE, "non-numeric field '%s'", f);
  char* end = NULL;
  errno = 0;
  long long v = strtoll(f, &end, 10);
  if (end == f || *end != '\0' || errno) return fail(r, MPM_ERR_PARSE, "bad integer '%s'", f);
  r->next++;
  *out = (int64_t)v;
  return MPM_OK;
}

static int get_i32(reader* r, int32_t* out) {
  int64_t v = 0;
  int st = get_int(r, &v);
  if (st) return st;
  if (v > 2147483647LL || v < -2147483647LL) return fail(r, MPM_ERR_PARSE, "integer out of range");
  *out = (int32_t)v;
  return MPM_OK;
}

#define TRY(x)            \
  do {                    \
    int st__ = (x);       \
    if (st__) return st__; \
  } while (0)

static int on_off(reader* r, int* on) {
  static const char* const kw[] = {"on  ", "off "};
  int k = 0;
  TRY(keyword(r, kw, 2, "on/off", &k));
  *on = (k == 1);
  return MPM_OK;
}

static int res_option(reader* r, int32_t* out) {
  static const char* const kw[] = {"seqv", "epef", "mat ", "pres", "volu", "engk",
                                   "engi", "velx", "vely", "velz", "cels", "fail",
                                   "sspd", "damg", "stsx", "disx", "disy", "disz"};
  int k = 0;
  TRY(keyword(r, kw, 18, "result option", &k));
  *out = k;
  return MPM_OK;
}

/* ---------------------------------------------------------------- materials */
static int set_material(reader* r) {
  static const char* const kw[] = {"elas", "pla1", "pla2", "john", "sjc ", "sjcf",
                                   "jcf ", "hiex", "null", "dpm ", "neoh"};
  mpm_deck* d = r->d;
  if (d->nb_mat == 0 || d->nb_particle == 0)
    return fail(r, MPM_ERR_PARSE, "nmat and nbmp must precede 'mate'");
  int64_t i = 0;
  while (i < d->nb_mat) {
    TRY(get_int(r, &i));
    if (i > d->nb_mat || i <= 0) return fail(r, MPM_ERR_PARSE, "material set %lld out of range", (long long)i);
    mpm_material* m = &d->mats[i - 1];
    int t = 0;
    TRY(keyword(r, kw, 11, "material type", &t));
    m->mat_type = t;
    switch (t) {
      case 1:
        TRY(get_real(r, &m->density)); TRY(get_real(r, &m->young)); TRY(get_real(r, &m->poisson));
        break;
      case 2:
        TRY(get_real(r, &m->density)); TRY(get_real(r, &m->young)); TRY(get_real(r, &m->poisson));
        TRY(get_real(r, &m->yield0));
        break;
      case 3:
        TRY(get_real(r, &m->density)); TRY(get_real(r, &m->young)); TRY(get_real(r, &m->poisson));
        TRY(get_real(r, &m->yield0)); TRY(get_real(r, &m->tangmod));
        break;
      case 4:
      case 7:
        TRY(get_real(r, &m->density)); TRY(get_real(r, &m->young)); TRY(get_real(r, &m->poisson));
        TRY(get_real(r, &m->yield0)); TRY(get_real(r, &m->B_jc)); TRY(get_real(r, &m->n_jc));
        TRY(get_real(r, &m->C_jc)); TRY(get_real(r, &m->m_jc)); TRY(get_real(r, &m->roomt));
        TRY(get_real(r, &m->melt)); TRY(get_real(r, &m->specheat)); TRY(get_real(r, &m->epso));
        if (t == 7) TRY(get_real(r, &m->epf));
        break;
      case 5:
      case 6:
        TRY(get_real(r, &m->density)); TRY(get_real(r, &m->young)); TRY(get_real(r, &m->poisson));
        TRY(get_real(r, &m->yield0)); TRY(get_real(r, &m->B_jc)); TRY(get_real(r, &m->n_jc));
        TRY(get_real(r, &m->C_jc)); TRY(get_real(r, &m->epso));
        if (t == 6) TRY(get_real(r, &m->epf));
        break;
      case 8:
        TRY(get_real(r, &m->density)); TRY(get_real(r, &m->D));
        break;
      case 9:
        TRY(get_real(r, &m->density)); TRY(get_real(r, &m->bulk_modulus)); TRY(get_real(r, &m->miu));
        m->wavespd = sqrt(m->bulk_modulus / m->density);
        break;
      case 10:
        TRY(get_real(r, &m->density)); TRY(get_real(r, &m->young)); TRY(get_real(r, &m->poisson));
        TRY(get_real(r, &m->q_fai)); TRY(get_real(r, &m->k_fai)); TRY(get_real(r, &m->q_psi));
        TRY(get_real(r, &m->ten_f));
        break;
      case 11:
        TRY(get_real(r, &m->density)); TRY(get_real(r, &m->young)); TRY(get_real(r, &m->poisson));
        d->flags |= MPM_F_UVFP;
        break;
    }
  }
  /* grid-mass CutOff (DataIn.f90:517-524): the 1e-5 literal is a 32-bit REAL */
  double cut = 0.0;
  int matcount = 0;
  for (int k = 0; k < d->nb_mat; ++k) {
    cut = d->mats[k].density + cut;
    matcount++;
  }
  double dc3 = d->dcell * d->dcell * d->dcell;
  d->cutoff = cut * dc3 * (double)1e-5f / (double)matcount;
  return MPM_OK;
}

/* ---------------------------------------------------------------- particles */
static int new_particle(reader* r) {
  if (r->par_counter >= r->d->nb_particle)
    return fail(r, MPM_ERR_PARSE, "too many particles (nbmp = %lld)", (long long)r->d->nb_particle);
  r->par_counter++;
  return MPM_OK;
}

static void set_skip(reader* r, int64_t p) {
  mpm_deck* d = r->d;
  int64_t np = d->nb_particle;
  const double* pl = d->plot2d;
  double x = d->xp[p], y = d->xp[np + p], z = d->xp[2 * np + p];
  if (x < pl[0] || x > pl[1] || y < pl[2] || y > pl[3] || z < pl[4] || z > pl[5]) d->skip[p] = 1;
}

static int set_particle(reader* r) {
  static const char* const kw[] = {"poin", "bloc", "sphe", "blod", "cicl"};
  mpm_deck* d = r->d;
  const int64_t np = d->nb_particle;
  if (np == 0) return fail(r, MPM_ERR_PARSE, "nbmp must precede 'part'");
  int opt = 0;
  TRY(keyword(r, kw, 5, "particle generator", &opt));
  if (r->body_counter >= d->nb_body) return fail(r, MPM_ERR_PARSE, "more bodies than nbbo");
  mpm_body* bd = &d->bodies[r->body_counter++];
  TRY(get_i32(r, &bd->comID));
  if (opt == 1) { /* poin: comID, pnum, then (ID, mat, mass, x, y, z) per particle */
    int64_t pnum = 0;
    TRY(get_int(r, &pnum));
    if (pnum < 0) return fail(r, MPM_ERR_PARSE, "negative particle count");
    bd->par_begin = r->par_counter;
    bd->par_end = r->par_counter + pnum;
    int32_t mat = 0;
    for (int64_t k = 0; k < pnum; ++k) {
      int64_t newi = 0;
      TRY(get_int(r, &newi));
      TRY(new_particle(r));
      if (newi < r->par_counter) return fail(r, MPM_ERR_PARSE, "particle ID conflict");
      TRY(get_i32(r, &mat));
      if (mat > d->nb_mat || mat <= 0) return fail(r, MPM_ERR_PARSE, "improper material ID");
      int64_t p = r->par_counter - 1;
      TRY(get_real(r, &d->mass[p]));
      for (int c = 0; c < 3; ++c) TRY(get_real(r, &d->xp[c * np + p]));
      if (r->plot2d_on) set_skip(r, p);
    }
    bd->mat = mat;
    return MPM_OK;
  }
  int32_t mat = 0;
  TRY(get_i32(r, &mat));
  bd->mat = mat;
  bd->par_begin = r->par_counter;
  if (mat > d->nb_mat || mat <= 0) return fail(r, MPM_ERR_PARSE, "improper material ID");
  double pmass = 0, dp = 0, ox = 0, oy = 0, oz = 0;
  TRY(get_real(r, &pmass));
  TRY(get_real(r, &dp));
  pmass = pmass * (dp * dp * dp);
  TRY(get_real(r, &ox)); TRY(get_real(r, &oy)); TRY(get_real(r, &oz));
  if (opt == 2 || opt == 4) { /* bloc / blod */
    ox = ox + dp * 0.5;
    oy = oy + dp * 0.5;
    oz = oz + dp * 0.5;
    int64_t nx = 0, ny = 0, nz = 0, nr = 0;
    double oox = 0, ooy = 0, ooz = 0, radius2 = 0;
    TRY(get_int(r, &nx)); TRY(get_int(r, &ny)); TRY(get_int(r, &nz));
    if (opt == 4) {
      TRY(get_real(r, &oox)); TRY(get_real(r, &ooy)); TRY(get_real(r, &ooz));
      TRY(get_int(r, &nr));
      double t = (double)nr * dp;
      radius2 = t * t;
    }
    for (int64_t iz = 1; iz <= nz; ++iz)
      for (int64_t iy = 1; iy <= ny; ++iy)
        for (int64_t ix = 1; ix <= nx; ++ix) {
          double tx = (double)(ix - 1) * dp + ox;
          double ty = (double)(iy - 1) * dp + oy;
          double tz = (double)(iz - 1) * dp + oz;
          if (opt == 4) {
            double a = tx - oox, b = ty - ooy;
            if (!(a * a + b * b >= radius2)) continue;
          }
          TRY(new_particle(r));
          int64_t p = r->par_counter - 1;
          d->mass[p] = pmass;
          d->xp[p] = tx;
          d->xp[np + p] = ty;
          d->xp[2 * np + p] = tz;
          if (r->plot2d_on) set_skip(r, p);
        }
  } else if (opt == 3) { /* sphe: the radius count is read as a REAL into an INTEGER */
    double nxr = 0;
    TRY(get_real(r, &nxr));
    int64_t nx = (int64_t)nxr;
    double t = (double)nx * dp;
    double radius2 = t * t;
    for (int64_t ix = 1 - nx; ix <= nx; ++ix)
      for (int64_t iy = 1 - nx; iy <= nx; ++iy)
        for (int64_t iz = 1 - nx; iz <= nx; ++iz) {
          double tx = (double)(ix - 1) * dp + ox + 0.5 * dp;
          double ty = (double)(iy - 1) * dp + oy + 0.5 * dp;
          double tz = (double)(iz - 1) * dp + oz + 0.5 * dp;
          double a = tx - ox, b = ty - oy, c = tz - oz;
          if (!(a * a + b * b + c * c < radius2)) continue;
          TRY(new_particle(r));
          int64_t p = r->par_counter - 1;
          d->mass[p] = pmass;
          d->xp[p] = tx;
          d->xp[np + p] = ty;
          d->xp[2 * np + p] = tz;
          if (r->plot2d_on) set_skip(r, p);
        }
  } else { /* cicl: one layer of a disc */
    int64_t nx = 0;
    TRY(get_int(r, &nx));
    double t = (double)nx * dp;
    double radius2 = t * t;
    for (int64_t ix = 1 - nx; ix <= nx; ++ix)
      for (int64_t iy = 1 - nx; iy <= nx; ++iy) {
        double tx = (double)(ix - 1) * dp + ox + 0.5 * dp;
        double ty = (double)(iy - 1) * dp + oy + 0.5 * dp;
        double tz = oz + dp * 0.5;
        double a = tx - ox, b = ty - oy;
        if (!(a * a + b * b < radius2)) continue;
        TRY(new_particle(r));
        int64_t p = r->par_counter - 1;
        d->mass[p] = pmass;
        d->xp[p] = tx;
        d->xp[np + p] = ty;
        d->xp[2 * np + p] = tz;
        if (r->plot2d_on) set_skip(r, p);
      }
  }
  bd->par_end = r->par_counter;
  return MPM_OK;
}

/* -------------------------------------------------------- loads, velocities */
static int particle_id(reader* r, int64_t* p) {
  TRY(get_int(r, p));
  if (*p < 1 || *p > r->d->nb_particle) return fail(r, MPM_ERR_PARSE, "particle %lld out of range", (long long)*p);
  *p -= 1;
  return MPM_OK;
}

static int body_id(reader* r, int64_t* b) {
  TRY(get_int(r, b));
  if (*b < 1 || *b > r->d->nb_body) return fail(r, MPM_ERR_PARSE, "body %lld out of range", (long long)*b);
  *b -= 1;
  return MPM_OK;
}

static int set_load(reader* r) {
  static const char* const kw[] = {"endl", "part", "body", "grav", "node"};
  mpm_deck* d = r->d;
  const int64_t np = d->nb_particle;
  if (d->nb_body == 0) return fail(r, MPM_ERR_PARSE, "nbbo must precede 'load'");
  for (;;) {
    int k = 0;
    TRY(keyword(r, kw, 5, "load", &k));
    if (k == 1) return MPM_OK;
    if (k == 2) {
      int64_t p = 0;
      TRY(particle_id(r, &p));
      for (int c = 0; c < 3; ++c) TRY(get_real(r, &d->fxp[c * np + p]));
    } else if (k == 3) {
      int64_t b = 0;
      double f[3];
      TRY(body_id(r, &b));
      for (int c = 0; c < 3; ++c) TRY(get_real(r, &f[c]));
      for (int64_t p = d->bodies[b].par_begin; p < d->bodies[b].par_end; ++p)
        for (int c = 0; c < 3; ++c) d->fxp[c * np + p] = f[c];
    } else if (k == 4) {
      int64_t b = 0;
      d->flags |= MPM_F_GRAVITY;
      TRY(body_id(r, &b));
      for (int c = 0; c < 3; ++c) TRY(get_real(r, &d->bodies[b].gravp[c]));
    } else {
      /* 'node' is a legacy keyword the reference only warns about; its values
       * are then read as keywords and stop the run. Reject it up front. */
      return fail(r, MPM_ERR_PARSE, "legacy load keyword 'node' (use 'part')");
    }
  }
}

static int set_velocity(reader* r) {
  static const char* const kw[] = {"endv", "node", "body", "ksin", "nuli", "vsin"};
  mpm_deck* d = r->d;
  const int64_t np = d->nb_particle;
  if (d->nb_body == 0) return fail(r, MPM_ERR_PARSE, "nbbo must precede 'velo'");
  const double pi_f = (double)3.1415926535f; /* default-REAL literal */
  for (;;) {
    int k = 0;
    TRY(keyword(r, kw, 6, "velocity", &k));
    if (k == 1) return MPM_OK;
    if (k == 2) {
      int64_t p = 0;
      TRY(particle_id(r, &p));
      for (int c = 0; c < 3; ++c) TRY(get_real(r, &d->vxp[c * np + p]));
    } else if (k == 3) {
      int64_t b = 0;
      double v[3];
      TRY(body_id(r, &b));
      for (int c = 0; c < 3; ++c) TRY(get_real(r, &v[c]));
      for (int64_t p = d->bodies[b].par_begin; p < d->bodies[b].par_end; ++p)
        for (int c = 0; c < 3; ++c) d->vxp[c * np + p] = v[c];
    } else if (k == 4) { /* ksin: fixed 4 x 320 sine profile on body 1 */
      double v0 = 0;
      int64_t ib = 0;
      TRY(get_real(r, &v0));
      TRY(get_int(r, &ib));
      const int64_t n = 320;
      const double dc = (double)0.003125f;
      if (ib == 1) {
        if (4 * n > np) return fail(r, MPM_ERR_PARSE, "'ksin' needs at least 1280 particles");
        for (int64_t i = 1; i <= 4 * n; ++i) {
          int64_t m = i % n;
          if (m == 0) m = n;
          d->vxp[i - 1] = v0 * sin(pi_f * ((double)(m - 1) * dc + dc / 2.0));
          d->vxp[np + i - 1] = 0;
          d->vxp[2 * np + i - 1] = 0;
        }
      }
    } else if (k == 5) { /* nuli: Euler beam mode shape, 128 x 384 particles */
      double y = 0;
      TRY(get_real(r, &y));
      const int64_t n = 384;
      if (128 * n > np) return fail(r, MPM_ERR_PARSE, "'nuli' needs at least 49152 particles");
      const double dc = (double)0.00015625f;
      const double q = (double)78.83f;
      const double c006 = (double)0.06f;
      double c1 = cosh(q * c006) - cos(q * c006);
      double c2 = sinh(q * c006) - sin(q * c006);
      double A = y / (2 * c2);
      /* the constant under the root is folded in 32-bit REAL arithmetic */
      volatile float num = 318e9f * 0.01f;
      num = num * 0.01f;
      volatile float den = 12.0f * 1845.0f;
      volatile float nu2 = 0.054f * 0.054f;
      den = den * (1.0f - nu2);
      float rt = sqrtf(num / den);
      double W = q * q * (double)rt;
      for (int64_t i = 1; i <= 128 * n; ++i) {
        int64_t m = i % n;
        if (m == 0) m = n;
        double x = ((double)(m - 1) * dc + dc / 2.0);
        d->vxp[i - 1] = 0;
        d->vxp[np + i - 1] = A * W * (c1 * (sinh(q * x) + sin(q * x)) - c2 * (cosh(q * x) + cos(q * x)));
        d->vxp[2 * np + i - 1] = 0;
      }
    } else { /* vsin: sine profile along the initial y coordinate */
      double v0 = 0;
      TRY(get_real(r, &v0));
      for (int b = 0; b < d->nb_body; ++b)
        for (int64_t p = d->bodies[b].par_begin; p < d->bodies[b].par_end; ++p) {
          d->vxp[p] = v0 * sin(pi_f * d->xp[np + p] / 6);
          d->vxp[np + p] = 0;
          d->vxp[2 * np + p] = 0;
        }
    }
  }
}

static int set_eos(reader* r) {
  mpm_deck* d = r->d;
  int64_t mset = 0;
  TRY(get_int(r, &mset));
  if (mset < 1 || mset > d->nb_mat) return fail(r, MPM_ERR_PARSE, "EOS material %lld out of range", (long long)mset);
  mpm_material* m = &d->mats[mset - 1];
  TRY(get_i32(r, &m->eos_type));
  switch (m->eos_type) {
    case 1:
      for (int k = 0; k < 7; ++k) TRY(get_real(r, &m->cEos[k]));
      TRY(get_real(r, &m->cEos[9]));
      break;
    case 2: {
      double c0 = 0, lambda = 0, gamma0 = 0;
      TRY(get_real(r, &c0)); TRY(get_real(r, &lambda)); TRY(get_real(r, &gamma0));
      m->cEos[0] = m->density * (c0 * c0);
      m->cEos[1] = m->cEos[0] * (2 * lambda - 1);
      m->cEos[2] = m->cEos[0] * (lambda - 1) * (3 * lambda - 1);
      m->cEos[3] = m->density * gamma0;
      m->cEos[4] = gamma0;
      TRY(get_real(r, &m->cEos[9]));
      break;
    }
    case 3:
      for (int k = 0; k < 5; ++k) TRY(get_real(r, &m->cEos[k]));
      TRY(get_real(r, &m->cEos[9]));
      break;
    case 4:
      TRY(get_real(r, &m->cEos[0]));
      break;
    default:
      return fail(r, MPM_ERR_PARSE, "unknown EOS type %d", m->eos_type);
  }
  return MPM_OK;
}

static int set_curx(reader* r) {
  mpm_deck* d = r->d;
  const int64_t np = d->nb_particle;
  if (r->par_counter != np) return fail(r, MPM_ERR_PARSE, "'curx' must follow the particle input");
  if (d->n_curves >= MPM_MAX_CURVES) return fail(r, MPM_ERR_PARSE, "too many curves");
  int c = d->n_curves++;
  TRY(res_option(r, &d->curve_option[c]));
  double t[3];
  for (int k = 0; k < 3; ++k) TRY(get_real(r, &t[k]));
  for (int b = 0; b < d->nb_body; ++b)
    for (int64_t p = d->bodies[b].par_begin; p < d->bodies[b].par_end; ++p) {
      double m = fabs(d->xp[p] - t[0]);
      double m2 = fabs(d->xp[np + p] - t[1]);
      double m3 = fabs(d->xp[2 * np + p] - t[2]);
      if (m2 > m) m = m2;
      if (m3 > m) m = m3;
      if (m <= 0.25 * d->dcell) {
        d->curve_point[c] = (int32_t)(p + 1);
        break;
      }
    }
  return MPM_OK;
}

static int set_contact(reader* r) {
  static const char* const kw[] = {"lagr", "othe"};
  int k = 0;
  TRY(keyword(r, kw, 2, "contact", &k));
  r->d->contact_type = k;
  TRY(get_real(r, &r->d->fricfa));
  TRY(get_i32(r, &r->d->normbody));
  return MPM_OK;
}

static int alloc_particles(reader* r, int64_t n) {
  mpm_deck* d = r->d;
  if (d->mass) return fail(r, MPM_ERR_PARSE, "nbmp given twice");
  if (n <= 0) return fail(r, MPM_ERR_PARSE, "nbmp must be positive");
  d->nb_particle = n;
  d->mass = (double*)calloc((size_t)n, sizeof(double));
  d->xp = (double*)calloc((size_t)(3 * n), sizeof(double));
  d->vxp = (double*)calloc((size_t)(3 * n), sizeof(double));
  d->fxp = (double*)calloc((size_t)(3 * n), sizeof(double));
  d->skip = (uint8_t*)calloc((size_t)n, 1);
  if (!d->mass || !d->xp || !d->vxp || !d->fxp || !d->skip) return fail(r, MPM_ERR_OOM, "out of host memory");
  return MPM_OK;
}

/* ------------------------------------------------------------------ GetData */
static int get_data(reader* r) {
  static const char* const kw[] = {
      "endi", "mpm3", "nbmp", "endt", "grid", "spx ", "spy ", "spz ", "dcel", "dtsc", "outt",
      "rptt", "fixe", "nmat", "mate", "part", "musl", "jaum", "load", "velo", "outr", "curv",
      "seos", "pt2d", "curx", "deto", "tecp", "bulk", "gimp", "cont", "usf ", "usl ", "nbco",
      "nbbo", "para", "drda", "bimp", "sgmp", "smoo", "TLmp", "UVFp", "QuLo", "Damp"};
  mpm_deck* d = r->d;
  int update_method = 0;
  for (;;) {
    int key = 0;
    TRY(keyword(r, kw, 43, "input", &key));
    int on = 0;
    int64_t iv = 0;
    switch (key) {
      case 1:
        goto done;
      case 2:
        snprintf(d->title, sizeof d->title, "%s", r->line);
        r->next = r->nfield;
        break;
      case 3:
        TRY(get_int(r, &iv));
        TRY(alloc_particles(r, iv));
        break;
      case 4:
        TRY(get_real(r, &d->endtime));
        d->outtime = d->endtime;
        break;
      case 5:
        for (int a = 0; a < 3; ++a) { TRY(get_real(r, &d->span[a][0])); TRY(get_real(r, &d->span[a][1])); }
        break;
      case 6: case 7: case 8:
        TRY(get_real(r, &d->span[key - 6][0]));
        TRY(get_real(r, &d->span[key - 6][1]));
        break;
      case 9:
        TRY(get_real(r, &d->dcell));
        break;
      case 10:
        TRY(get_real(r, &d->dtscale));
        if (d->dtscale > 2.5) return fail(r, MPM_ERR_PARSE, "DTScale too large");
        break;
      case 11:
        TRY(get_real(r, &d->outtime));
        break;
      case 12:
        TRY(get_real(r, &d->reporttime));
        break;
      case 13:
        for (int k = 0; k < 6; ++k) TRY(get_i32(r, &d->fixs[k]));
        break;
      case 14:
        if (d->mats) return fail(r, MPM_ERR_PARSE, "nmat given twice");
        TRY(get_i32(r, &d->nb_mat));
        if (d->nb_mat <= 0) return fail(r, MPM_ERR_PARSE, "nmat must be positive");
        d->mats = (mpm_material*)calloc((size_t)d->nb_mat, sizeof(mpm_material));
        if (!d->mats) return fail(r, MPM_ERR_OOM, "out of host memory");
        break;
      case 15:
        TRY(set_material(r));
        break;
      case 16:
        TRY(set_particle(r));
        break;
      case 17:
        TRY(on_off(r, &on));
        if (on) { d->flags |= MPM_F_MUSL; update_method = 1; } else d->flags &= ~MPM_F_MUSL;
        break;
      case 18:
        TRY(on_off(r, &on));
        if (on) d->flags |= MPM_F_JAUM; else d->flags &= ~MPM_F_JAUM;
        break;
      case 19:
        TRY(set_load(r));
        break;
      case 20:
        TRY(set_velocity(r));
        break;
      case 21:
        if (d->n_anim >= MPM_MAX_ANIM) return fail(r, MPM_ERR_PARSE, "too many 'outr'");
        TRY(res_option(r, &d->anim_option[d->n_anim++]));
        break;
      case 22: {
        if (d->n_curves >= MPM_MAX_CURVES) return fail(r, MPM_ERR_PARSE, "too many curves");
        int c = d->n_curves++;
        TRY(res_option(r, &d->curve_option[c]));
        if (r->next < r->nfield) {
          TRY(get_int(r, &iv));
          if (iv <= 0 || iv > d->nb_particle) return fail(r, MPM_ERR_PARSE, "invalid curve particle ID");
          d->curve_point[c] = (int32_t)iv;
        } else {
          d->curve_point[c] = 1;
        }
        break;
      }
      case 23:
        TRY(set_eos(r));
        break;
      case 24:
        d->flags |= MPM_F_PLOT2D;
        r->plot2d_on = 1;
        for (int k = 0; k < 6; ++k) TRY(get_real(r, &d->plot2d[k]));
        break;
      case 25:
        TRY(set_curx(r));
        break;
      case 26:
        if (d->n_deto >= MPM_MAX_DETO) return fail(r, MPM_ERR_PARSE, "too many detonation points");
        for (int k = 0; k < 3; ++k) TRY(get_real(r, &d->deto[d->n_deto][k]));
        d->n_deto++;
        break;
      case 27:
        d->flags |= MPM_F_TECPLOT;
        break;
      case 28:
        TRY(get_real(r, &d->bq1));
        TRY(get_real(r, &d->bq2));
        break;
      case 29:
        d->flags |= MPM_F_GIMP;
        break;
      case 30:
        d->flags |= MPM_F_CONTACT;
        TRY(set_contact(r));
        break;
      case 31:
        TRY(on_off(r, &on));
        if (on) { d->flags |= MPM_F_USF; update_method = 1; } else d->flags &= ~MPM_F_USF;
        break;
      case 32:
        TRY(on_off(r, &on));
        if (on) { d->flags |= MPM_F_USL; update_method = 1; } else d->flags &= ~MPM_F_USL;
        break;
      case 33:
        TRY(get_i32(r, &d->nb_component));
        break;
      case 34:
        if (d->bodies) return fail(r, MPM_ERR_PARSE, "nbbo given twice");
        TRY(get_i32(r, &d->nb_body));
        if (d->nb_body <= 0) return fail(r, MPM_ERR_PARSE, "nbbo must be positive");
        d->bodies = (mpm_body*)calloc((size_t)d->nb_body, sizeof(mpm_body));
        if (!d->bodies) return fail(r, MPM_ERR_OOM, "out of host memory");
        break;
      case 35:
        d->flags |= MPM_F_PARAVIEW;
        break;
      case 36:
        d->flags |= MPM_F_DRDAMP;
        break;
      case 37:
        d->flags |= MPM_F_BSPLINE;
        break;
      case 38:
        d->flags |= MPM_F_SGMP;
        break;
      case 39:
        d->flags |= MPM_F_SMOOTH;
        break;
      case 40:
        d->flags |= MPM_F_TLMPM;
        break;
      case 41:
        d->flags |= MPM_F_UVFP;
        break;
      case 42:
        d->flags |= MPM_F_QUASILOAD;
        TRY(get_real(r, &d->quasi_load_time));
        break;
      case 43:
        d->flags |= MPM_F_QUASIDAMP;
        TRY(get_real(r, &d->damp_factor));
        break;
    }
  }
done:
  if (!update_method) d->flags |= MPM_F_MUSL; /* DataIn.f90:364 */
  if (d->nb_particle > 0 && r->par_counter != d->nb_particle)
    return fail(r, MPM_ERR_PARSE, "nbmp = %lld but %lld particles were defined",
                (long long)d->nb_particle, (long long)r->par_counter);
  return MPM_OK;
}

static void set_defaults(mpm_deck* d) {
  memset(d, 0, sizeof *d);
  d->nb_component = 1;
  d->dtscale = (double)0.9f;      /* real(8) initialised from the REAL literal 0.9 */
  d->bq1 = (double)1.5f;          /* Material.f90:65: FP32 literals */
  d->bq2 = (double)0.06f;
  d->flags = MPM_F_JAUM;          /* Jaum = .true. */
}

int mpm_deck_parse(const char* text, mpm_deck** out, char* errbuf, int errlen) {
  if (!out || !text) return MPM_ERR_ARG;
  *out = NULL;
  mpm_deck* d = (mpm_deck*)calloc(1, sizeof(mpm_deck));
  if (!d) return MPM_ERR_OOM;
  set_defaults(d);
  reader r;
  memset(&r, 0, sizeof r);
  r.text = text;
  r.d = d;
  r.err = d->err;
  int st = get_data(&r);
  d->line_nb = r.line_nb;
  if (st) {
    if (errbuf && errlen > 0) snprintf(errbuf, (size_t)errlen, "%s", d->err);
    mpm_deck_free(d);
    return st;
  }
  *out = d;
  return MPM_OK;
}

int mpm_deck_load(const char* path, mpm_deck** out, char* errbuf, int errlen) {
  if (!path || !out) return MPM_ERR_ARG;
  *out = NULL;
  FILE* f = fopen(path, "rb");
  if (!f) {
    if (errbuf && errlen > 0) snprintf(errbuf, (size_t)errlen, "cannot open %s", path);
    return MPM_ERR_IO;
  }
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  if (sz < 0) { fclose(f); return MPM_ERR_IO; }
  char* buf = (char*)malloc((size_t)sz + 1);
  if (!buf) { fclose(f); return MPM_ERR_OOM; }
  size_t got = fread(buf, 1, (size_t)sz, f);
  fclose(f);
  buf[got] = '\0';
  int st = mpm_deck_parse(buf, out, errbuf, errlen);
  free(buf);
  return st;
}

void mpm_deck_free(mpm_deck* d) {
  if (!d) return;
  free(d->mats);
  free(d->bodies);
  free(d->mass);
  free(d->xp);
  free(d->vxp);
  free(d->fxp);
  free(d->skip);
  free(d);
}

int64_t mpm_deck_nb_particle(const mpm_deck* d) { return d ? d->nb_particle : -1; }
int32_t mpm_deck_flags(const mpm_deck* d) { return d ? d->flags : 0; }

int mpm_deck_get_particles(const mpm_deck* d, double* mass, double* xp, double* vxp, double* fxp) {
  if (!d) return MPM_ERR_ARG;
  size_t n = (size_t)d->nb_particle;
  if (mass) memcpy(mass, d->mass, n * sizeof(double));
  if (xp) memcpy(xp, d->xp, 3 * n * sizeof(double));
  if (vxp) memcpy(vxp, d->vxp, 3 * n * sizeof(double));
  if (fxp) memcpy(fxp, d->fxp, 3 * n * sizeof(double));
  return MPM_OK;
}

/* span(6), dcell, cutoff, dtscale, endtime, outtime, reporttime,
 * quasi_load_time, damp_factor, bq1, bq2 */
int mpm_deck_scalars(const mpm_deck* d, double* o) {
  if (!d || !o) return MPM_ERR_ARG;
  for (int a = 0; a < 3; ++a) { o[2 * a] = d->span[a][0]; o[2 * a + 1] = d->span[a][1]; }
  o[6] = d->dcell; o[7] = d->cutoff; o[8] = d->dtscale; o[9] = d->endtime;
  o[10] = d->outtime; o[11] = d->reporttime; o[12] = d->quasi_load_time;
  o[13] = d->damp_factor; o[14] = d->bq1; o[15] = d->bq2;
  return MPM_OK;
}
