/*
 * cupic_gpu.h -- C-ABI of the GB300 (sm_103a) electrostatic PIC cycle.
 *
 * One handle (cupic_ctx) owns the device state of one probe/plasma slab:
 * particles of both species (FP32, float4 {x,y,vx,vy} per particle, grouped
 * by y cell row), the potential phi (FP32), the field E (FP32 pairs) and the
 * charge accumulator rho (int64 fixed point, 2^32 per unit macroparticle
 * charge).  Every call returns an int status (CUPIC_OK == 0); nothing calls
 * exit().  All pointers in this header are HOST pointers unless a name says
 * otherwise; no torch or CUDA types appear in the signatures.
 *
 * The entry points replace the reference's host functions, which have C++
 * linkage and global state (reference file:line given per function):
 *   charge_deposition   src/mesh.cu:15-51        -> cupic_charge_deposition
 *   poisson_solver      src/mesh.cu:55-120       -> cupic_poisson_solver
 *   field_solver        src/mesh.cu:124-154      -> cupic_field_solver
 *   particle_mover      src/particles.cu:15-102  -> cupic_particle_mover
 *   cc                  src/cc.cu:15-69          -> cupic_cc
 *   init_sim            src/init.cu:57-102       -> cupic_init_plasma
 *   read_input_file +   src/init.cu:424-789      -> cupic_params_from_input_data
 *     init_* getters
 *   read_particle_file  src/init.cu:348-420      -> cupic_load_particles
 *   particles_snapshot  src/diagnostic.cu:48-87  -> cupic_store_particles
 *   mesh_snapshot       src/diagnostic.cu:91-133 -> cupic_get_rho / cupic_get_phi
 *   number_of_particles src/diagnostic.cu:15-44  -> cupic_get_counts
 */
#ifndef CUPIC_GPU_H
#define CUPIC_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  CUPIC_OK = 0,
  CUPIC_ERR_ARG = 1,        /* invalid argument / parameter */
  CUPIC_ERR_CUDA = 2,       /* a CUDA runtime call failed */
  CUPIC_ERR_NOMEM = 3,      /* device or host allocation failed */
  CUPIC_ERR_IO = 4,         /* input_data / particle file could not be read */
  CUPIC_ERR_CAPACITY = 5,   /* a staging row or the injection buffer overflowed (full
                               rows are grown, not reported) */
  CUPIC_ERR_CFL = 6,        /* a particle moved more than one cell row in a step */
  CUPIC_ERR_NONFINITE = 7,  /* a NaN/Inf particle coordinate was seen */
  CUPIC_ERR_STATE = 8,      /* call out of order (e.g. step before init) */
  CUPIC_ERR_TIMEOUT = 9,    /* a bounded device-side wait gave up */
  CUPIC_ERR_NODEVICE = 10   /* no CUDA device visible */
};

/* device-side flag bits, as returned by cupic_get_flags() */
enum {
  CUPIC_FLAG_CFL = 1u << 0,
  CUPIC_FLAG_CAPACITY = 1u << 1,
  CUPIC_FLAG_STAGE = 1u << 2,
  CUPIC_FLAG_NONFINITE = 1u << 3,
  CUPIC_FLAG_TIMEOUT = 1u << 4,
  CUPIC_FLAG_XRANGE = 1u << 5
};

enum { CUPIC_ELECTRONS = 0, CUPIC_IONS = 1 };

/*
 * Normalised simulation parameters.  Units follow the reference
 * (src/init.cu:451-789): lengths in Debye lengths, time in 1/omega_pe,
 * masses in m_e, energies in kT_e, potential in kT_e/e, density in
 * particles per Debye-length cube.
 */
typedef struct cupic_params {
  int32_t ncx, ncy;         /* cells in x (periodic) and y (input_data lines 10, 11) */
  double ds;                /* cell size (line 12) */
  double dt;                /* time step (line 13) */
  double n;                 /* density n = ne*lambda_D^3 (init.cu:542-556) */
  double eps0;              /* permittivity (init.cu:612-630); equals n in exact arithmetic */
  double phi_p;             /* probe potential at y=0 (init.cu:523-538) */
  double me, mi;            /* masses (init.cu:473-494): 1, gamma */
  double kte, kti;          /* thermal energies (init.cu:498-519): 1, beta */
  double qe, qi;            /* charges (init.cu:451-469): -1, +1 */
  /* Jacobi control for each step (main.cu:64; mesh.cu:94-114).  A sweep
   * count s stops the solve when s >= min_sweeps and the max |delta phi| of
   * a checked sweep is < tol, or when s == max_sweeps.  A sweep is checked
   * when s % check_every == 0 or s == max_sweeps; the reported residual is
   * that of the last checked sweep.  (Checks before min_sweeps, which can
   * stop nothing, are not computed; the stop and the report are the same.) */
  double tol;
  int32_t min_sweeps, max_sweeps, check_every;
  /* the same for the initial solve (init.cu:254) */
  double init_tol;
  int32_t init_min_sweeps, init_max_sweeps;
  /* run control copied from input_data lines 1-4 (main.cu:33-36) */
  int32_t n_ini, n_prev, n_save, n_fin;
  /* particles per y row per species at t=0: int(n*Lx*ds*ds) (init.cu:136) */
  int32_t ppr;
  /* storage: row capacity = ceil(ppr*(1+row_slack)) + 64; movers staged per
   * row up to ceil(capacity*stage_frac) + 64.  A row that cannot take a
   * step's particles is grown to ceil(need*(1+row_slack)) + 64 (and the
   * staging rows with the largest row) before any particle is written. */
  double row_slack;
  double stage_frac;
  /* seed of the counter-based generator (Philox4x32-10) used for the
   * initial plasma and the injected flux */
  uint64_t seed;
  /* Precision form of the Poisson solve.  0: FP32 Jacobi with the stop rule
   * above.  m > 0: the potential is kept in FP64; every m FP32 Jacobi sweeps
   * solve for a correction from the FP64 residual b - A phi of the
   * 5-point operator, which is added in FP64.  The solve stops when that
   * residual's max norm (in the units of b = ds^2 rho / eps0) is below tol
   * (init_tol for the initial solve) after at least min_sweeps sweeps, or
   * at max_sweeps; the field is derived in FP64. */
  int32_t refine_every;
} cupic_params;

/* Per-step counters (absorbed = crossed y<0 into the probe; removed =
 * crossed y>=Ly; injected = half-Maxwellian flux at y=Ly). */
typedef struct cupic_step_stats {
  int64_t step;             /* index i of the step in the main loop */
  double t;                 /* time passed to the boundary stage */
  int64_t absorbed[2];      /* [electrons, ions] */
  int64_t removed[2];
  int64_t injected[2];
  int64_t live[2];          /* particles after the step */
  int32_t sweeps;           /* Jacobi sweeps of the step */
  float residual;           /* max |delta phi| of the last checked sweep */
  uint32_t flags;           /* CUPIC_FLAG_* raised during the step */
} cupic_step_stats;

/* ---- parameters -------------------------------------------------------- */

/* Fills *p with the 64x256-cell, 20-particles-per-cell plasma of the small
 * workload: ds=0.5, dt=0.05, n=160, mi=100, kti=1, phi_p=-5. */
int cupic_params_default(cupic_params *p);

/* Parses the reference's 13-parameter input_data file (header line then
 * "name = value;" lines, init.cu:424-447) and normalises it exactly as the
 * init_* getters do (init.cu:451-789). */
int cupic_params_from_input_data(const char *path, cupic_params *p);

/* Recomputes derived fields (ppr) after a caller edited *p. */
int cupic_params_finalize(cupic_params *p);

/* ---- lifetime ---------------------------------------------------------- */

int cupic_create(const cupic_params *p, int device, struct cupic_ctx **out);
int cupic_destroy(struct cupic_ctx *ctx);
const char *cupic_strerror(int status);

/* init_sim for n_ini == 0 (init.cu:57-83): seeded uniform/Maxwellian
 * plasma, linear phi, deposit, initial solve, field, leapfrog half-step. */
int cupic_init_plasma(struct cupic_ctx *ctx);

/* The same, enqueued on the context's stream without waiting for it (a
 * server admits a request while the device steps others).  Device-side
 * conditions are reported by the next call that waits (cupic_sync,
 * cupic_step's status, ...).  cupic_create itself never waits for the
 * device when the solver layout of its mesh shape is already known. */
int cupic_init_plasma_nowait(struct cupic_ctx *ctx);

/* Contexts take their device memory from the device's stream-ordered pool
 * (cudaMallocAsync), which keeps freed memory for later contexts, and their
 * streams from a per-device set that destroyed contexts return theirs to.
 * This grows the pool to at least `bytes` of free memory (it allocates
 * nothing when the pool already holds that much unused) and the set to
 * `contexts` streams' worth now, so that contexts created later (a server
 * admitting requests while the device steps others) neither map new pages
 * nor create streams, which can stall while the device is busy.  Both are
 * kept until the process exits. */
int cupic_reserve(int device, uint64_t bytes, int32_t contexts);

/* Replaces one species with n particles given as the reference's particle
 * struct (4 doubles x,y,vx,vy; stdh.h:30-36), in any order; they are binned
 * by y row keeping the given order within a row (init.cu:400-407).
 * Particles outside [0,Lx)x[0,Ly) are rejected with CUPIC_ERR_ARG. */
int cupic_load_particles(struct cupic_ctx *ctx, int species, const double *xyvv, int64_t n);

/* Sets the simulation clock t and the injection clocks (cc.cu:35-36).
 * tin < 0 means "first boundary call sets tin = t + dtin". */
int cupic_set_time(struct cupic_ctx *ctx, int64_t step, double t, double tin_e, double tin_i);
int cupic_get_time(struct cupic_ctx *ctx, int64_t *step, double *t, double *tin_e, double *tin_i);

/* init_sim for n_ini > 0 after the particles were loaded: initialize_mesh
 * (init.cu:202-260) -- linear phi, deposit, the initial solve (init_tol)
 * and field, no leapfrog half-step -- then the clock set to step n_ini+1 at
 * t = n_ini*dt + dt with the injection clocks unset (init.cu:86-93). */
int cupic_init_mesh(struct cupic_ctx *ctx);
/* The parameters the context was created with. */
int cupic_get_params(struct cupic_ctx *ctx, cupic_params *p);
/* The Jacobi solver's layout: CTAs of the cooperative grid, mesh rows each
 * CTA owns, and the halo depth (sweeps between neighbour exchanges). */
int cupic_get_solver_plan(struct cupic_ctx *ctx, int32_t *ctas, int32_t *rows_per_cta,
                          int32_t *depth);

/* ---- the cycle (reference entry points) -------------------------------- */

/* Deposits rho from the current particles (only needed after a load). */
int cupic_charge_deposition(struct cupic_ctx *ctx);
/* Jacobi solve; max_error<0 uses the per-step parameters of ctx. */
int cupic_poisson_solver(struct cupic_ctx *ctx, double max_error, int32_t min_sweeps,
                         int32_t max_sweeps, int32_t check_every);
int cupic_field_solver(struct cupic_ctx *ctx);
/* Gather + leapfrog + periodic wrap + y-row binning + probe absorption;
 * also deposits the moved particles into the next charge accumulator.
 * Rows that cannot take their arrivals are grown first. */
int cupic_particle_mover(struct cupic_ctx *ctx);
/* Injection of the half-Maxwellian flux at y=Ly for the step at time t and
 * end-of-step bookkeeping (cc.cu:134-272). */
int cupic_cc(struct cupic_ctx *ctx, double t);

/* nsteps full cycles (solve, field, push, bin, absorb, inject) with the
 * clock advancing by dt per step, replayed from a captured CUDA graph.
 * Returns once the steps are enqueued.  A step whose particles do not fit
 * their rows (checked on the device after the push) idles the rest of the
 * run; the next call that waits grows those rows, completes that step and
 * runs the remaining ones, with the results of a run with larger rows. */
int cupic_step(struct cupic_ctx *ctx, int32_t nsteps);
/* Waits for all work of ctx, completing a run that stopped for room. */
int cupic_sync(struct cupic_ctx *ctx);

/* Phases of a step, for cupic_step_timed. */
enum {
  CUPIC_PHASE_SOLVE = 0,  /* Jacobi sweeps + field (mesh.cu:55-154) */
  CUPIC_PHASE_ZERO = 1,   /* clearing the next charge accumulator (mesh.cu:35) */
  CUPIC_PHASE_PUSH = 2,   /* push + wrap + binning + deposition (particles.cu, cc.cu, mesh.cu) */
  CUPIC_PHASE_ARRIVE = 3, /* movers appended to their new rows (cc.cu:640-772); the draws
                             of the injected flux run on a side stream beside the push,
                             and this phase includes the wait for them and the room check */
  CUPIC_PHASE_INJECT = 4, /* append of the injected particles (cc.cu:134-272) */
  CUPIC_PHASE_FINAL = 5,  /* per-step counters and clock */
  CUPIC_NPHASE = 6
};
/* nsteps cycles of the step's own launch sequence (the one cupic_step's
 * graph captures), launched directly with a CUDA event after each phase on
 * the context's stream; phase_ms[k] = device ms of phase k summed over the
 * steps, *total_ms = device ms from the first to the last event.  A run that
 * the room check halts is completed inside the timed region (*total_ms then
 * runs to the end of the completion). */
int cupic_step_timed(struct cupic_ctx *ctx, int32_t nsteps, float *phase_ms, int32_t nphase,
                     float *total_ms);

/* ---- results ----------------------------------------------------------- */

int cupic_get_counts(struct cupic_ctx *ctx, int64_t *n_electrons, int64_t *n_ions);
/* Copies one species in row order as 4 doubles per particle. */
int cupic_store_particles(struct cupic_ctx *ctx, int species, double *xyvv, int64_t capacity,
                          int64_t *n_out);
/* Same, as 4 floats per particle (the device representation). */
int cupic_store_particles_f32(struct cupic_ctx *ctx, int species, float *xyvv, int64_t capacity,
                              int64_t *n_out);
/* Per-row [first,last] index pairs of the row-ordered particle list, -1 for
 * empty rows: the reference's bookmark array (init.cu:159-165). */
int cupic_get_bookmarks(struct cupic_ctx *ctx, int species, int32_t *bm);
/* Mesh arrays, nnx*nny doubles, index i + j*nnx.  which=0: the charge the
 * next solve will use; which=1: the charge used by the last solve. */
int cupic_get_rho(struct cupic_ctx *ctx, int which, double *rho);
int cupic_get_rho_fixed(struct cupic_ctx *ctx, int which, int64_t *acc);
int cupic_get_phi(struct cupic_ctx *ctx, double *phi);
int cupic_set_phi(struct cupic_ctx *ctx, const double *phi);
int cupic_get_field(struct cupic_ctx *ctx, double *ex, double *ey);
int cupic_get_phi_f32(struct cupic_ctx *ctx, float *phi);
int cupic_get_field_f32(struct cupic_ctx *ctx, float *ex, float *ey);
/* Stats of the last `count` steps (most recent last). */
int cupic_get_stats(struct cupic_ctx *ctx, cupic_step_stats *out, int32_t count);
int cupic_get_flags(struct cupic_ctx *ctx, uint32_t *flags);
/* Probe current: the net charge absorbed by the probe per step (qe times the
 * electrons plus qi times the ions crossing y<0), averaged over the last
 * `window` steps (at most 4096). */
int cupic_probe_current(struct cupic_ctx *ctx, int32_t window, double *current);
/* Density profile of one species: particles per unit volume in each cell
 * row, count / (ncx ds^3), ncy values; the initial plasma gives n. */
int cupic_density_profile(struct cupic_ctx *ctx, int species, double *density);
int cupic_clear_flags(struct cupic_ctx *ctx);
/* Fault-detection self-test, with no counterpart in the reference: one GPU
 * thread waits, through the solver's bounded wait, on a word that nothing
 * writes.  The wait gives up after its limit (under a second), raises
 * CUPIC_FLAG_TIMEOUT and the kernel returns; the call returns
 * CUPIC_ERR_TIMEOUT.  cupic_clear_flags makes the context usable again. */
int cupic_test_bounded_wait(struct cupic_ctx *ctx);

/* ---- solve without allocating ------------------------------------------ */

/* The Poisson solve (and field) on caller-owned DEVICE buffers, allocating
 * nothing.  It has no counterpart in the reference.  It is for callers that
 * cannot call cudaMalloc at solve time: real-time loops that forbid
 * allocation after start-up (an allocation can block for an unbounded
 * time), and hosts whose device memory all comes from their own pool.
 *   rho_dev  nnx*nny raw int64 fixed-point charge (2^32 per unit charge, the
 *            layout of cupic_get_rho_fixed, columns 0 and nnx-1 not folded)
 *   phi_dev  nnx*nny float potential, read as the initial guess, overwritten
 *   e_dev    nnx*nny {Ex, Ey} float pairs, written; NULL skips the field
 *   stream   a cudaStream_t, NULL for the default stream; the call waits for
 *            its own work before returning (it reads sweeps_out and
 *            residual_out back)
 * The solver's scratch (sweep counters, residual slots and the halo rows its
 * CTAs trade) lives in a static 8 MiB device array that every GPU loading
 * this library holds until exit.  The call lowers the halo depth, then the
 * CTA count, until the scratch fits; meshes for which nothing fits return
 * CUPIC_ERR_CAPACITY.  The largest ncy accepted is 5321 at ncx = 512, 2433
 * at ncx = 1024, 890 at ncx = 2048 and 127 at ncx = 4096.  The first call on a device
 * looks the array up (cudaGetSymbolAddress); make that first call before any
 * stream capture.  All calls share the array and it keeps the last call's
 * contents: calls that overlap on the GPU (other streams, other host
 * threads) race and must be serialised by the caller.  The environment
 * variable CUPIC_JACOBI_CTAS, when set, caps the number of solver CTAs, as
 * it does for a context's solve. */
int cupic_poisson_solver_static(const cupic_params *p, const int64_t *rho_dev, float *phi_dev,
                                float *e_dev, double max_error, int32_t min_sweeps,
                                int32_t max_sweeps, int32_t check_every, void *stream,
                                int32_t *sweeps_out, float *residual_out);

/* ---- batched form ------------------------------------------------------- */
/* Many independent contexts (probe-bias instances of any sizes) stepped
 * together.  It has no counterpart in the reference, which runs one
 * simulation per process.  A batched step is one launch per kernel for all
 * members: the solves run in one cooperative launch of CTA groups, each
 * group solving its list of instances in turn; push, arrive and the charge
 * clear run over work lists of {instance, row}.  Each member keeps its own
 * buffers, clocks and stats ring, and gets the same results as when stepped
 * alone.  Members must be initialised contexts of the batch's device in the
 * FP32 solve form; while they are members, step them only through the
 * batch, and call cupic_batch_sync before reading them. */
typedef struct cupic_batch cupic_batch;
int cupic_batch_create(int device, cupic_batch **out);
/* Sets the members (replacing the previous set); n == 0 empties the batch. */
int cupic_batch_set(cupic_batch *b, struct cupic_ctx *const *members, int32_t n);
/* nsteps batched cycles, replayed from a CUDA graph captured per member set. */
int cupic_batch_step(cupic_batch *b, int32_t nsteps);
/* Waits for the batch; returns the first member's error status, if any. */
int cupic_batch_sync(cupic_batch *b);
/* The batched solve's layout: each member's solve takes the fewest CTAs
 * whose shared memory holds its rows, times *cta_mult, with a halo depth of
 * at most *depth_cap; *ctas is the launch's CTA count.  When a member set
 * of 16 or more is built, an autotuner times every candidate (depth cap 1,
 * 2, 4, 8 x CTA multiple 1, 2) on the members' own meshes -- saving and
 * restoring their potential, field and solver status -- and keeps the
 * fastest; picks are cached per process by the members' mesh shapes and
 * sweep counts, and a batch keeps its pick while its member count stays
 * within a factor of two of the count it was tuned for.  Smaller sets, or
 * CUPIC_BATCH_TUNE=0, take depth cap 4 and multiple 1. */
int cupic_batch_plan(cupic_batch *b, int32_t *depth_cap, int32_t *cta_mult, int32_t *ctas);
int cupic_batch_destroy(cupic_batch *b);

/* ---- the reference's text files ---------------------------------------- */
/* Host-side only; paths are used as given (the reference's ".dat" suffix
 * and "../output/" prefix are the caller's).  The formats are the
 * reference's, character for character. */

/* particles_snapshot (diagnostic.cu:48-87): " %.17e %.17e %.17e %.17e \n"
 * per particle.  header != NULL first writes one line "# <header>", which
 * the reference's loader skips as its header line (D12, init.cu:372). */
int cupic_write_particles_file(const char *path, const double *xyvv, int64_t n,
                               const char *header);
/* read_particle_file (init.cu:348-420): every line holding four numbers is a
 * particle, in file order; other lines (a header, blank lines) are skipped.
 * Unlike the reference, the first particle of a header-less file is kept
 * (defect D12 fixed).  xyvv == NULL only counts into *n_out. */
int cupic_read_particles_file(const char *path, double *xyvv, int64_t capacity, int64_t *n_out);
/* mesh_snapshot (diagnostic.cu:91-133): " %d %d %.17e \n", i outer, j
 * inner, a blank line after each i; m is nnx*nny doubles, index i + j*nnx. */
int cupic_write_mesh_file(const char *path, const double *m, int32_t nnx, int32_t nny);
/* save_bm (diagnostic.cu:137-169): " %d %d %d \n" per cell row. */
int cupic_write_bookmarks_file(const char *path, const int32_t *bm, int32_t ncy);
/* save_bins (diagnostic.cu:173-215): " %d %d \n", index and int(y/ds). */
int cupic_write_bins_file(const char *path, const double *xyvv, int64_t n, double ds);
/* main.cu:98-113: line 1 of input_data becomes "n_ini = <n_ini>;", the
 * other lines are kept (a last line without '\n' is kept too). */
int cupic_rewrite_input_data(const char *path, int32_t n_ini);

/* The same files straight from a context. */
int cupic_particles_snapshot(struct cupic_ctx *ctx, int species, const char *path);
/* what: 0 the charge the next solve uses, 1 the charge of the last solve
 * (the reference's d_rho after a step), 2 phi, 3 Ex, 4 Ey */
int cupic_mesh_snapshot(struct cupic_ctx *ctx, int what, const char *path);
int cupic_save_bm(struct cupic_ctx *ctx, int species, const char *path);
int cupic_save_bins(struct cupic_ctx *ctx, int species, const char *path);
/* load_particles (init.cu:327-344) for one species from a particle file. */
int cupic_load_particles_file(struct cupic_ctx *ctx, int species, const char *path);

#ifdef __cplusplus
}
#endif

#endif /* CUPIC_GPU_H */
