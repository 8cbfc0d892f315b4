/* mpm_output.h -- result files of MPM3D-F90 (DataOut.f90) written from host
 * arrays: the time-history curves (OutCurve: <job>_curv.dat, EnergyPlot.dat,
 * MomentumPlot.dat, ContforcPlot.dat with contact), the Tecplot animation
 * (OutAnim: <job>_anim.dat) and the ParaView animation (OutAnimPV: <job>_anim_<k>.vtu listed in <job>_anim.pvd,
 * plus the grid <job>_Grid.vtu from OutGrid), in the reference's file names,
 * layouts and Fortran edit descriptors (E12.4, E10.3, I3, I10, ...).
 *
 * The writer takes plain host arrays, so the same calls serve the GPU
 * library (curve values gathered from the device, mpm_gather*) and any other
 * producer of the step's state.
 */
#ifndef MPM_OUTPUT_H
#define MPM_OUTPUT_H

#include <stdint.h>

#include "mpm_deck.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mpm_output mpm_output;

/* Host view of the particle state in deck particle order (component-major
 * arrays of nb_particle doubles each; sd = SDxx, SDyy, SDzz, SDxy, SDyz,
 * SDxz). Fields the deck's animation options do not need may be NULL; icell
 * (1-based cell, <= 0 outside the grid) may be NULL when every particle is
 * inside the grid; spre (smoothed pressure, mpm_download MPM_P_SPRE) NULL
 * reads as 0, its value without stress smoothing. */
typedef struct mpm_particle_view {
  const double *xp, *vxp, *fxp, *mass;
  const double *seqv, *epeff, *sm, *vol, *ie, *celsius, *cp, *dmg, *sd;
  const double* failure; /* 0 / 1 */
  const double* icell;
  const double* spre;
} mpm_particle_view;

/* Opens the files of job `job` (a path prefix; the reference derives it
 * from the deck name without extension) as InputPara does (DataIn.f90:34-103):
 * <job>_curv.dat always; <job>_anim.dat with 'tecp'; <job>_anim.pvd and
 * <job>_Grid.vtu with 'para'. EnergyPlot.dat and MomentumPlot.dat go to
 * `plot_dir` (the reference writes them to the working directory; NULL =
 * the directory of `job`). The deck must stay valid while the writer is
 * open. */
int mpm_output_open(const mpm_deck* deck, const char* job, const char* plot_dir, mpm_output** out);
/* Closes the files (and the .pvd collection's tags). */
void mpm_output_close(mpm_output* o);

/* The curves of the run: the reference's two default curves (kinetic and
 * internal energy, particle 1) followed by the deck's 'curv' / 'curx' ones. */
int mpm_output_curve_count(const mpm_output* o);

/* The particle values one curve row needs, as (particle, field, component)
 * triples (0-based particle; mpm_field ids of mpm3d_gpu.h); returns their
 * count (at most 2 per curve). Gather these values, in this order, for
 * mpm_output_curve. */
int mpm_output_curve_items(const mpm_output* o, int64_t* particle, int* field, int* component, int max);

/* One OutCurve call (DataOut.f90:66-154): a row of <job>_curv.dat (the header
 * first), EnergyPlot.dat and MomentumPlot.dat. scalars16 as mpm_get_scalars
 * (time, energies, momentum); values as listed by mpm_output_curve_items. */
int mpm_output_curve(mpm_output* o, const double* scalars16, const double* values);

/* The contact-force row of OutCurve (DataOut.f90:148-152): with contact on,
 * a row of ContforcPlot.dat (next to EnergyPlot.dat) with the time and the
 * total contact force (mpm_contact_force); a no-op otherwise. */
int mpm_output_contact(mpm_output* o, double time, const double* force3);

/* One animation frame at an output time: OutAnim with 'tecp', OutAnimPV with
 * 'para' (DataOut.f90:157-247, 250-530). */
int mpm_output_anim(mpm_output* o, const double* scalars16, const mpm_particle_view* v);

/* Fortran edit descriptors as gfortran writes them (exposed for tests):
 * Ew.d -- [-]0.<d digits>E<+/-><2 digits>, right-justified in w. */
int mpm_format_e(char* buf, int bufsize, int w, int d, double x);

#ifdef __cplusplus
}
#endif
#endif
