/*
 * mpm_deck.h -- reader for the MPM3D-F90 ".mpm" keyword input format.
 *
 * The reader reproduces the reference front end:
 *   FFI.f90:177-253      ReadLine   (tabs -> blanks, '!' comments, blank/comma fields,
 *                                    at most 15 fields per line, 20 characters per field)
 *   FFI.f90:110-138      GetReal    (every real is read as a 32-bit REAL, then widened)
 *   FFI.f90:140-175,255  KeyWord / pcomp (4-character, case-insensitive keywords)
 *   FFI.f90:287-299      isNumber   (a number starts with '-' or a digit)
 *   DataIn.f90:105-366   GetData    (keyword table and the "MUSL by default" rule)
 *   DataIn.f90:368-532   SetMaterial (material types and the grid-mass CutOff)
 *   DataIn.f90:534-865   SetParticle (point / block / sphere / blod / cicl generators)
 *   DataIn.f90:884-1042  SetLoad, SetVelocity
 *   DataIn.f90:1095-1156 SetEos
 * The derived set-up (Initial, SetGridData, SetDT in DataIn.f90:1211-1297 and
 * Grid.f90:222-418) is NOT done here: each consumer of a deck derives it.
 *
 * All functions return an mpm_status code; nothing aborts the process.
 */
#ifndef MPM_DECK_H
#define MPM_DECK_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes shared by every C-ABI entry point of this project. */
enum mpm_status {
  MPM_OK = 0,
  MPM_ERR_ARG = 1,          /* bad argument or bad call order                 */
  MPM_ERR_OOM = 2,          /* host or device allocation failed / over budget */
  MPM_ERR_PARSE = 3,        /* malformed .mpm input                           */
  MPM_ERR_UNSUPPORTED = 4,  /* option outside the explicit-step path          */
  MPM_ERR_CUDA = 5,         /* a CUDA runtime call failed                     */
  MPM_ERR_OUT_OF_GRID = 6,  /* a particle left the computational grid         */
  MPM_ERR_NONFINITE = 7,    /* non-finite particle state detected             */
  MPM_ERR_TIMEOUT = 8,      /* a bounded device-side wait gave up             */
  MPM_ERR_STATE = 9,        /* object is in the wrong state for this call     */
  MPM_ERR_IO = 10           /* file could not be opened / read               */
};

/* Option flags (ParticleData module logicals, Particle.f90:81-94, plus writers). */
enum mpm_flag {
  MPM_F_MUSL = 1 << 0,
  MPM_F_USL = 1 << 1,
  MPM_F_USF = 1 << 2,
  MPM_F_GIMP = 1 << 3,
  MPM_F_BSPLINE = 1 << 4,
  MPM_F_SGMP = 1 << 5,
  MPM_F_QUASILOAD = 1 << 6,
  MPM_F_QUASIDAMP = 1 << 7,
  MPM_F_SMOOTH = 1 << 8,
  MPM_F_UVFP = 1 << 9,
  MPM_F_TLMPM = 1 << 10,
  MPM_F_CONTACT = 1 << 11,
  MPM_F_GRAVITY = 1 << 12,
  MPM_F_DRDAMP = 1 << 13,
  MPM_F_JAUM = 1 << 14,
  MPM_F_TECPLOT = 1 << 15,
  MPM_F_PARAVIEW = 1 << 16,
  MPM_F_PLOT2D = 1 << 17
};

/* Material record (Material.f90:23-67). Fields a material type does not read stay 0. */
typedef struct mpm_material {
  int32_t mat_type;  /* 1 elas .. 11 neoh (DataIn.f90:379-382) */
  int32_t eos_type;  /* 0 none, 1 linear, 2 Gruneisen, 3 JWL, 4 weakly compressible */
  double density, miu, young, poisson, yield0, tangmod, roomt, melt, specheat;
  double B_jc, n_jc, C_jc, m_jc, epso, prd, epf, D;
  double cEos[10];
  double wavespd, bulk_modulus;
  double q_fai, k_fai, q_psi, ten_f;
} mpm_material;

/* Body record (Particle.f90:57-63). mat is 1-based like the reference; the
 * particle range is 0-based, [par_begin, par_end). */
typedef struct mpm_body {
  int32_t mat;
  int32_t comID;
  double gravp[3];
  int64_t par_begin;
  int64_t par_end;
} mpm_body;

#define MPM_MAX_DETO 10
#define MPM_MAX_CURVES 64
#define MPM_MAX_ANIM 64

typedef struct mpm_deck {
  char title[257];
  int64_t nb_particle;
  int32_t nb_component, nb_body, nb_mat;
  int32_t flags;          /* mpm_flag bits, after the "MUSL by default" rule   */
  mpm_material* mats;     /* nb_mat entries                                    */
  mpm_body* bodies;       /* nb_body entries                                   */
  /* particle inputs, component-major SoA: xp[d*nb_particle + p] */
  double* mass;
  double* xp;
  double* vxp;
  double* fxp;
  uint8_t* skip;          /* SkipThis (plot filter only)                       */
  double span[3][2];      /* SpanX/Y/Z as read (SetGridData re-derives the max) */
  double dcell, cutoff, dtscale, endtime, outtime, reporttime;
  double quasi_load_time, damp_factor, bq1, bq2;
  int32_t fixs[6];
  int32_t contact_type, normbody;
  double fricfa;
  int32_t n_deto;
  double deto[MPM_MAX_DETO][3];
  int32_t n_curves, n_anim;
  int32_t curve_option[MPM_MAX_CURVES], curve_point[MPM_MAX_CURVES];
  int32_t anim_option[MPM_MAX_ANIM];
  double plot2d[6];
  int32_t line_nb;        /* last line read (for error messages)               */
  char err[256];          /* message of the last error                         */
} mpm_deck;

/* Parse a deck file. On failure *out is NULL and, if errbuf is given, it
 * receives a one-line message (errlen bytes). */
int mpm_deck_load(const char* path, mpm_deck** out, char* errbuf, int errlen);
/* Parse a deck held in memory (NUL-terminated text). */
int mpm_deck_parse(const char* text, mpm_deck** out, char* errbuf, int errlen);
void mpm_deck_free(mpm_deck* d);

/* Plain accessors for FFI bindings (ctypes, ISO_C_BINDING) that do not want
 * to mirror the struct layout. */
int64_t mpm_deck_nb_particle(const mpm_deck* d);
int32_t mpm_deck_flags(const mpm_deck* d);
int mpm_deck_get_particles(const mpm_deck* d, double* mass, double* xp, double* vxp,
                           double* fxp);
int mpm_deck_scalars(const mpm_deck* d, double* out16);

#ifdef __cplusplus
}
#endif
#endif
