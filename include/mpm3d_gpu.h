/*
 * mpm3d_gpu.h -- C ABI of the GB300 explicit MPM time step.
 *
 * This library replaces the bodies of the argument-less step subroutines that
 * MPM3D.f90's time loop calls (MPM3D.f90:66-160). A Fortran host binds these
 * functions with ISO_C_BINDING (mpm3d-f90_gb300/fortran/mpm3d_gpu_shim.f90);
 * any other host (C, C++, Python ctypes) binds them directly. Plain pointers,
 * sizes and int status codes only; no exception or C++ type crosses the ABI.
 *
 * Ownership: after mpm_create the device owns the live particle and grid
 * state. The host mirror is refreshed only by mpm_download / mpm_get_*.
 * Threading: one host thread per context; contexts are independent.
 * Errors: every function returns an mpm_status (mpm_deck.h). Device-side
 * health checks (non-finite state, particle outside the grid) are written to a
 * per-context status word and reported by mpm_check / mpm_sync.
 */
#ifndef MPM3D_GPU_H
#define MPM3D_GPU_H

#include <stdint.h>

#include "mpm_deck.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mpm_ctx mpm_ctx;

/* Arithmetic forms of the step. */
enum mpm_precision {
  MPM_FP64_STRICT = 0, /* FP64 throughout, reference summation order, no FMA,
                          project libm: bit-identical to the CPU oracle      */
  MPM_FP64_NATIVE = 1, /* as STRICT but CUDA libm for log/exp/pow           */
  MPM_MIXED = 2        /* FP32 shape functions, velocity gradient and
                          constitutive update; FP64 grid mass / momentum /
                          force accumulation, positions, velocities, energy  */
};

/* Step phases: one per reference subroutine, same order semantics.
 * A Fortran shim calls mpm_step_phase(ctx, MPM_PHASE_x) from the body of the
 * subroutine of the same name. */
enum mpm_phase {
  MPM_PHASE_GRID_MOMENTUM_INITIAL = 1,    /* update_step.f90:288  GridMomentumInitial     */
  MPM_PHASE_APPLY_BOUNDARY = 2,           /* update_step.f90:1795 ApplyBoundaryConditions */
  MPM_PHASE_PARTICLE_STRESS_UPDATE = 3,   /* update_step.f90:456  ParticleStressUpdate    */
  MPM_PHASE_GRID_MOMENTUM_UPDATE = 4,     /* update_step.f90:831  GridMomentumUpdate      */
  MPM_PHASE_INTEGRATE_MOMENTUM = 5,       /* update_step.f90:1194 IntegrateMomentum       */
  MPM_PHASE_PARTICLE_POSITION_UPDATE = 6, /* update_step.f90:1378 ParticlePositionUpdate  */
  MPM_PHASE_GRID_MOMENTUM_MUSL = 7,       /* update_step.f90:1668 GridMomentumMUSL        */
  MPM_PHASE_CALC_ENERGY = 8,              /* Particle.f90:204     calcEnergy              */
  MPM_PHASE_UPDATE_DT = 9,                /* update_step.f90:1833 UpdateDT                */
  MPM_PHASE_DR_DAMPING = 10,              /* Particle.f90:172     dynamicRelaxationDamping*/
  MPM_PHASE_BEGIN_STEP = 11,              /* MPM3D.f90:72-74: istep+1, time += DT         */
  MPM_PHASE_SMOOTH_STRESS = 12,           /* update_step.f90:1876 SmoothStressbyGrid      */
  MPM_PHASE_CONTACT = 13                  /* update_step.f90:1241 Lagr_NodContact         */
};

/* Field identifiers for mpm_download / oracle accessors. Particle fields are
 * component-major arrays of nb_particle doubles per component, in the input
 * particle order; grid fields are per node in the reference's flat order
 * (x fastest, MPM3D Grid.f90:299). */
enum mpm_field {
  MPM_P_XP = 1,      /* 3 */
  MPM_P_XX = 2,      /* 3 */
  MPM_P_VXP = 3,     /* 3 */
  MPM_P_FXP = 4,     /* 3 */
  MPM_P_XN = 5,      /* 3 */
  MPM_P_XXN = 6,     /* 3 */
  MPM_P_VOL = 7,
  MPM_P_VOL0 = 8,
  MPM_P_SIG_Y = 9,
  MPM_P_SM = 10,
  MPM_P_SEQV = 11,
  MPM_P_SD = 12,     /* 6: xx, yy, zz, xy, yz, xz */
  MPM_P_FP = 13,     /* 9: Fp(i,j) at i*3+j (0-based), Fp - I on the diagonal */
  MPM_P_EPEFF = 14,
  MPM_P_CELSIUS = 15,
  MPM_P_DMG = 16,
  MPM_P_LT = 17,
  MPM_P_IE = 18,
  MPM_P_MASS = 19,
  MPM_P_CP = 20,
  MPM_P_Q = 21,
  MPM_P_FAILURE = 22, /* 0 / 1 */
  MPM_P_ICELL = 23,   /* 1-based cell id, -1 outside */
  MPM_P_CENTERICELL = 24,
  MPM_P_INODE = 25,
  MPM_P_SPRE = 26,   /* smoothed pressure (SmoothStressbyGrid; 0 without 'smoo') */
  MPM_P_PK = 27,     /* 9: first Piola-Kirchhoff stress of TLMPM, xx yy zz yz xz xy zy zx yx */
  MPM_G_MG = 40,
  MPM_G_PX = 41,     /* 3 */
  MPM_G_FX = 42,     /* 3 */
  MPM_C_MG = 50,     /* SGMP auxiliary (cell-centre) grid mass */
  MPM_C_PX = 51      /* 3 */
};

/* Scalar block returned by mpm_get_scalars (16 doubles):
 * 0 istep, 1 CurrentTime, 2 DT, 3 EngKinetic, 4 EngInternal, 5-7 Momentum,
 * 8 EngKinetic_prev, 9 nb_gridnode, 10 nb_particle, 11 CutOff, 12 DCell,
 * 13 active nodes (Mg > 0) after the last P2G, 14 status word, 15 reserved. */
#define MPM_NSCALARS 16

/* Number of components a field has (1, 3, 6 or 9); 0 for an unknown id. */
int mpm_field_components(int field);

/* ------------------------------------------------------------- lifecycle */
/* Create a context from a parsed deck: derives the set-up (Initial,
 * SetGridData, SetDT, calcEnergy; DataIn.f90:1211-1297, Grid.f90:222-418,
 * MPM3D.f90:42) and uploads the particle state. device < 0 picks the
 * current device. */
int mpm_create(const mpm_deck* deck, int precision, int device, mpm_ctx** out);
void mpm_destroy(mpm_ctx* ctx);
/* Last error text of a context (or of the library when ctx is NULL). */
const char* mpm_last_error(const mpm_ctx* ctx);

/* ------------------------------------------------------------------ step */
/* One phase of the step (see enum mpm_phase). */
int mpm_step_phase(mpm_ctx* ctx, int phase);
/* One full step in the order of MPM3D.f90:69-118 (USF / USL / MUSL chosen by
 * the deck flags): begin-step, P2G, stress, forces, integration, G2P, MUSL
 * re-map, energies and the next DT. */
int mpm_step(mpm_ctx* ctx);
/* nsteps full steps, launched back to back without host synchronisation
 * (captured once into a CUDA graph when use_graph != 0). */
int mpm_run(mpm_ctx* ctx, int nsteps, int use_graph);
/* Wait for the context's stream and read the device status word. */
int mpm_sync(mpm_ctx* ctx);

/* -------------------------------------------------------------- data I/O */
int mpm_get_scalars(mpm_ctx* ctx, double* out16);
/* Copy a field to host memory (out holds components * count doubles). */
int mpm_download(mpm_ctx* ctx, int field, double* out);
/* Replace a particle field (component-major, nb_particle per component). */
int mpm_upload(mpm_ctx* ctx, int field, const double* in);
/* Page-locked host memory (no counterpart in the reference). Copies between
 * the device and page-locked buffers run at the link's bandwidth; pageable
 * buffers go through the driver's staging. mpm_host_alloc returns NULL on
 * failure (message in mpm_last_error); mpm_host_register locks an existing
 * buffer in place (undone by mpm_host_unregister, before the buffer is
 * freed); mpm_deck_pin locks (on != 0) or unlocks the particle arrays of a
 * deck, which mpm_create then uploads from. The locks are portable: they
 * count as page-locked for every device of the process, whichever device is
 * current when they are taken. */
void* mpm_host_alloc(int64_t bytes);
void mpm_host_free(void* p);
int mpm_host_register(void* p, int64_t bytes);
int mpm_host_unregister(void* p);
int mpm_deck_pin(mpm_deck* deck, int on);
int64_t mpm_nb_particle(const mpm_ctx* ctx);
int64_t mpm_nb_gridnode(const mpm_ctx* ctx);
int64_t mpm_nb_cell(const mpm_ctx* ctx);
/* Grid components (nbco): grid fields hold nb_component * nb_gridnode
 * nodes per vector component, component-major (DataIn.f90 'nbco',
 * Grid.f90:284 grid_list(nb_component, nb_gridnode)). */
int mpm_nb_component(const mpm_ctx* ctx);
/* Total contact force of the last step (tot_cont_for of Lagr_NodContact,
 * update_step.f90:1241-1376; written to ContforcPlot.dat by OutCurve); zero
 * without 'cont'. */
int mpm_contact_force(mpm_ctx* ctx, double f[3]);

/* ---------------------------------------------------- measurement hooks */
/* Time nsteps full steps with CUDA events on the context's stream;
 * returns milliseconds in *ms. */
int mpm_time_steps(mpm_ctx* ctx, int nsteps, int use_graph, double* ms);
/* Per-kernel event timing: when enabled, every launch of the step records a
 * start/stop event pair on the context's stream. mpm_kernel_stats returns,
 * for kernel index k, its name, launch count and total milliseconds. */
int mpm_profile_enable(mpm_ctx* ctx, int on);
int mpm_kernel_count(const mpm_ctx* ctx);
int mpm_kernel_stats(mpm_ctx* ctx, int k, char* name, int namelen, int64_t* launches,
                     double* total_ms);
/* Algorithmic bytes moved by the last step (particle fields read once and
 * modified fields written once, plus active-node grid traffic). */
int mpm_algorithmic_bytes(mpm_ctx* ctx, double* bytes_per_step);
/* Bytes of device memory the context holds. */
int64_t mpm_device_bytes(const mpm_ctx* ctx);

/* --------------------------------------------------- batched scenes */
/* No counterpart in the reference (which runs one scene per process): many
 * independent scenes advanced together on one GPU in the mixed-precision form,
 * one launch per kernel for the whole batch, indexed by per-scene offset
 * tables. Each scene keeps its own DT, time, energies and step count, and its
 * results do not depend on which other scenes share the batch.
 * mpm_batch_add stages a scene (steps = number of steps it runs, 0 = no
 * limit); mpm_batch_remove retires one; mpm_batch_commit lays the staged
 * composition out in device memory (moving resident scenes' state on the
 * device). Scene ids stay valid until removed. */
typedef struct mpm_batch mpm_batch;
int mpm_batch_create(int device, mpm_batch** out);
void mpm_batch_destroy(mpm_batch* b);
int mpm_batch_add(mpm_batch* b, const mpm_deck* deck, int steps, int* scene_id);
int mpm_batch_remove(mpm_batch* b, int scene_id);
int mpm_batch_commit(mpm_batch* b);
/* Device bytes a deck needs as a scene of a batch (admission by HBM budget). */
int64_t mpm_scene_device_bytes(const mpm_deck* deck);
int64_t mpm_batch_device_bytes(const mpm_batch* b);
int mpm_batch_scene_count(const mpm_batch* b);
/* nsteps steps of every resident scene (a scene stops at its step count);
 * use_graph replays a CUDA graph captured once per batch composition. */
int mpm_batch_run(mpm_batch* b, int nsteps, int use_graph);
/* Device-resident run loop (no counterpart in the reference, whose time
 * loop is one scene on the host, MPM3D.f90:66-160): one launch of a CUDA
 * graph whose WHILE node repeats two steps of the batch while a device-side
 * test passes, so the device steps the batch without a host round trip per
 * step or per chunk. The loop returns (and the call, after its last
 * reduction) once a scene has taken its last step, once max_steps steps are
 * taken, or after mpm_batch_interrupt; *steps receives the steps taken (at
 * least 1, at most max_steps). */
int mpm_batch_run_loop(mpm_batch* b, int max_steps, int* steps);
/* Ask a running device loop to return at its next test (two steps at most,
 * once MPM_BATCH_LOOP_MIN_STEPS steps are taken); callable from any thread.
 * The request is cleared when mpm_batch_run_loop returns. */
int mpm_batch_interrupt(mpm_batch* b);
int mpm_batch_sync(mpm_batch* b);
int mpm_batch_time_steps(mpm_batch* b, int nsteps, int use_graph, double* ms);
int mpm_batch_scene_scalars(mpm_batch* b, int scene_id, double* out16);
int mpm_batch_scene_download(mpm_batch* b, int scene_id, int field, double* out);
/* mpm_gather_async / mpm_gather_wait for one scene of a batch (particles in
 * the scene's deck order) */
int mpm_batch_scene_gather_async(mpm_batch* b, int scene_id, int n, const int64_t* particle, const int* field,
                                 const int* component);
int mpm_batch_scene_gather_wait(mpm_batch* b, double* out);
const char* mpm_batch_last_error(const mpm_batch* b);
/* Launch shape of the batch kernels (threads per block for particle and node
 * kernels; 0 keeps the current value). */
int mpm_batch_set_blocks(mpm_batch* b, int particle_block, int node_block);
/* Batch options (launch shapes; they change no result). */
enum mpm_batch_option {
  MPM_BATCH_PARTICLE_BLOCK = 1,
  MPM_BATCH_NODE_BLOCK = 2,
  MPM_BATCH_SCATTER_BLOCKS = 3, /* grid cap of the particle -> grid transfers, blocks per SM (1..64) */
  MPM_BATCH_LOOP_MIN_STEPS = 4  /* steps a device loop takes before it honours mpm_batch_interrupt (0) */
};
int mpm_batch_set_option(mpm_batch* b, int option, int value);
int mpm_batch_get_option(const mpm_batch* b, int option);
int mpm_batch_profile_enable(mpm_batch* b, int on);
int mpm_batch_kernel_stats(mpm_batch* b, int k, char* name, int namelen, int64_t* launches, double* total_ms);

/* ------------------------------------------------- particle value gather */
/* Values of a few particles (curve output, OutCurve): n (particle, field,
 * component) triples, particles 0-based in deck order, fields particle fields
 * of mpm_field. mpm_gather_async enqueues the gather behind the work already
 * on the context's stream and copies the values into pinned host memory;
 * mpm_gather_wait blocks until they have arrived and copies them to out
 * (n doubles); mpm_gather does both. At most MPM_GATHER_MAX items per call. */
#define MPM_GATHER_MAX 1024
int mpm_gather_async(mpm_ctx* ctx, int n, const int64_t* particle, const int* field, const int* component);
int mpm_gather_wait(mpm_ctx* ctx, double* out);
int mpm_gather(mpm_ctx* ctx, int n, const int64_t* particle, const int* field, const int* component, double* out);

/* ------------------------------------------------------ restart snapshot */
/* No counterpart in the reference: a full-precision restart file of a
 * context -- the device images of every persistent particle field and the
 * step's scalars (istep, time, DT, energies, the carried Johnson-Cook
 * depeff). For the mixed form the particle fields are stored at their
 * stored widths (FP64 positions, velocities, mass, energy; FP32 stress
 * state) in the batched engine's storage order, with the scene's step state.
 * Loading it into a context created from the same deck and precision
 * continues the run bit-identically. MPM_ERR_STATE for a file of another
 * deck or precision. */
int mpm_snapshot_save(mpm_ctx* ctx, const char* path);
int mpm_snapshot_load(mpm_ctx* ctx, const char* path);

/* ------------------------------------------------------ serving runtime */
/* No counterpart in the reference (a serial one-scene program): a server owns
 * one device and one batch (above). Client threads submit scenes; a server
 * thread admits them first-come first-served while their estimated device
 * bytes fit the budget, advances the batch in chunks of chunk_steps steps
 * (one CUDA graph replay per step, recaptured when the composition changes),
 * retires scenes that reached their step count (snapshotting the fields named
 * in field_mask to host memory) and admits the next ones. A scene's results
 * are the same as when it runs alone. */
typedef struct mpm_server mpm_server;
typedef struct mpm_serve_config {
  int device;               /* CUDA device, -1 = current                        */
  int chunk_steps;          /* steps between admission points (0 = 25): the device
                               loop returns when a scene finishes, or when a
                               submission is waiting and it has taken this many
                               steps                                            */
  int64_t hbm_budget_bytes; /* sum of the resident scenes' mpm_scene_device_bytes
                               (0 = 35% of free memory: a batch keeps two arenas) */
  int max_scenes;           /* resident scene cap (0 = 4096)                     */
  int autotune;             /* 1 = pick the batch launch shape by timing every
                               candidate on one frozen composition            */
  int policy;               /* admission order: MPM_SERVE_FIFO or MPM_SERVE_SHORTEST */
  int64_t max_resident_particles; /* admit while the resident particles stay below
                                     this (0 = no cap; a lone scene is always admitted) */
} mpm_serve_config;
/* FIFO admits in submission order; SHORTEST admits the queued scene with the
 * least work (particles x steps) first, which lowers the median latency when
 * the offered load exceeds the device's rate. */
enum mpm_serve_policy { MPM_SERVE_FIFO = 0, MPM_SERVE_SHORTEST = 1 };
/* bit (1u << field) of field_mask snapshots particle field `field` (mpm_field
 * ids 1..25) when the scene finishes */
#define MPM_SERVE_FIELD(f) (1u << (f))
int mpm_serve_create(const mpm_serve_config* cfg, mpm_server** out);
void mpm_serve_destroy(mpm_server* s); /* drains nothing: running scenes are dropped */
const char* mpm_serve_last_error(const mpm_server* s);
/* queue a scene for `steps` steps (>= 1); the deck may be freed on return */
int mpm_serve_submit(mpm_server* s, const mpm_deck* deck, int steps, uint32_t field_mask, int64_t* ticket);
/* wait up to timeout_ms (< 0: no limit) for a ticket: MPM_OK once finished,
 * MPM_ERR_TIMEOUT if still queued / running, MPM_ERR_OOM if the scene can
 * never fit the budget, MPM_ERR_ARG for an unknown ticket */
int mpm_serve_wait(mpm_server* s, int64_t ticket, int timeout_ms);
/* a finished ticket: scalars as mpm_get_scalars; times_ms[3] = queue wait,
 * time resident, total latency (submit to retirement) */
int mpm_serve_result(mpm_server* s, int64_t ticket, double* scalars16, double* times_ms3);
/* a snapshotted particle field of a finished ticket, in the deck's particle order */
int mpm_serve_field(mpm_server* s, int64_t ticket, int field, double* out);
int mpm_serve_release(mpm_server* s, int64_t ticket);
/* out[10]: submitted, finished, queued, resident, chunks run, particle-steps
 * run, device busy ms, particle block, node block, peak resident bytes */
int mpm_serve_stats(mpm_server* s, double* out10);
/* the launch shape in use (autotuned or default): MPM_ERR_STATE until the
 * autotuner has chosen */
int mpm_serve_launch_shape(mpm_server* s, int* particle_block, int* node_block, int* scatter_blocks);
/* block until no scene is queued or resident (or timeout_ms passes) */
int mpm_serve_drain(mpm_server* s, int timeout_ms);
/* The server's admission decision as a pure host function (no device needed;
 * also a capacity-planning aid). Queued scenes in submission order: particle
 * counts np, step counts, device-byte estimates (mpm_scene_device_bytes);
 * resident totals. Writes the queue positions admitted now, in admission
 * order, into admit and returns their count; writes into reject (count in
 * *nreject) the scenes that can never run (over the byte budget with nothing
 * resident). A budget of 0 is unlimited here. Negative return: -mpm_status. */
int mpm_serve_plan(const mpm_serve_config* cfg, int nqueued, const int64_t* np, const int* steps,
                   const int64_t* bytes, int resident_scenes, int64_t resident_particles, int64_t resident_bytes,
                   int* admit, int* reject, int* nreject);

/* ------------------------------------------------ FP64 pipe ceiling */
/* No counterpart in the reference: the measured FP64 arithmetic ceiling of a
 * device, the roofline of the FP64 forms (their kernels are bound by the FP64
 * pipe, not by HBM). A kernel of independent FP64 fused multiply-add chains
 * and one of FP64 divisions fill every SM; each is timed with CUDA events
 * (best of `repeats` launches after one warm-up launch). Outputs (any may be
 * NULL): dfma_per_s -- FP64 FMA instructions per second summed over the
 * device's threads (x 2 for flop/s); ddiv_per_s -- FP64 divisions (the
 * compiler's correctly rounded division) per second. Changes no device
 * setting; allocates 8 bytes of device memory per call for the kernels'
 * results (so that they cannot be optimised away). */
int mpm_fp64_ceiling(int device, int repeats, double* dfma_per_s, double* ddiv_per_s);

/* ------------------------------------------------ allocation-free call */
/* No counterpart in the reference: an extra entry point for hosts that may not
 * allocate device memory inside a solver call (a Fortran code passing device
 * arrays it manages itself, a host under a fixed memory pool, or a time loop
 * that must not allocate mid-run). It is the step's calcEnergy reduction
 * (Particle.f90:204-230) plus the maximum velocity component UpdateDT needs
 * (update_step.f90:1852), over caller-owned device arrays:
 *   vxp  : device, 3*np doubles, component-major (x block, y block, z block)
 *   mass : device, np doubles;  ie : device, np doubles (internal energy)
 *   out6 : device, 6 doubles written: kinetic energy, internal energy,
 *          momentum x, y, z, max |velocity component|
 *   stream : a cudaStream_t (NULL = default stream); the call is asynchronous.
 * It allocates nothing: its block partial sums live in a fixed 64 KiB
 * __device__ array that every GPU loading the library holds until the process
 * exits. np must be in 1..MPM_NOALLOC_MAX_PARTICLES, else MPM_ERR_ARG. The
 * first call on a device looks up that array's device address once (with that
 * device current), so make the first call before any stream capture. All
 * calls share the array: calls that overlap on the GPU (different streams or
 * threads at the same time) race and must be serialised by the caller.
 * It uses the block tree and combine order of the FP64 forms' calcEnergy
 * (mpm_step_phase MPM_PHASE_CALC_ENERGY) and gives the same bits on the same
 * arrays. */
#define MPM_NOALLOC_MAX_PARTICLES (1LL << 27)
int mpm_energy_reduce_noalloc(const double* vxp, const double* mass, const double* ie, int64_t np,
                              double* out6, void* stream);

#ifdef __cplusplus
}
#endif
#endif
