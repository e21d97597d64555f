/*
 * pysph_gb300 -- C ABI of the GB300 (sm_103a) SPH particle-step hot path.
 *
 * Every entry point takes plain pointers and sizes, returns an int status
 * (SPH_OK = 0, negative on error; sph_last_error() gives the message) and is
 * asynchronous on the context's CUDA stream unless documented otherwise.
 * Particle data are DEVICE pointers owned by the caller (the Python facade
 * keeps them in torch tensors); the context owns only its scratch (cell
 * tables, sorted snapshots).  A context is not re-entrant.
 *
 * Reference interfaces replaced (paths relative to the reference's
 * source/pysph/):
 *   sph_nnps_build        base/cell.pyx:927-1015 CellManager.update/cells_update
 *                         (+ check_jump_tolerance :1422-1437) and
 *                         base/nnps.pyx:566-620 FixedDestNbrParticleLocator.update
 *   sph_nnps_count/fill   base/nnps.pyx:458-523,633-648 get_nearest_particles
 *   sph_density           sph/sph_calc.pyx:223-270 SPHCalc.sph over
 *                         sph/funcs/density_funcs.pyx:38-74 SPHRho (optionally
 *                         fused with sph/funcs/eos_funcs.pyx:105-116 TaitEquation)
 *   sph_rates             SPHCalc.sph over pressure_funcs.pyx:40-91,
 *                         viscosity_funcs.pyx:41-124, xsph_funcs.pyx:31-88,
 *                         boundary_funcs.pyx:54-110 (+ external_force.pyx:39-45,
 *                         position_funcs.pyx:32-60 folded in)
 *   sph_tait              sph/funcs/eos_funcs.pyx:105-116 TaitEquation.eval_single
 *   sph_const_rates       external_force.pyx:39-45 GravityForce,
 *                         position_funcs.pyx:32-60 PositionStepping
 *   sph_integrate         solver/integrator.py:339-912 set_initial_arrays /
 *                         step / final_step of Euler, RK2, RK4,
 *                         PredictorCorrector and LeapFrog
 *   sph_invariants        (no counterpart: FP64 mass/momentum/energy sums)
 */
#ifndef PYSPH_GB300_H
#define PYSPH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_OK 0
#define SPH_ERR_ARG (-1)      /* invalid argument (ValueError)                 */
#define SPH_ERR_CUDA (-2)     /* CUDA runtime error                            */
#define SPH_ERR_GRID (-3)     /* dense cell grid would exceed its capacity     */
#define SPH_ERR_JUMP (-4)     /* a particle moved by more than one cell width  */
#define SPH_ERR_STATE (-5)    /* call out of order (e.g. no neighbour build)   */
#define SPH_ERR_NOTSUP (-6)   /* unsupported configuration (NotImplementedError)*/

/* device error-word bits (sph_error_word) */
#define SPH_EFLAG_JUMP 1u
#define SPH_EFLAG_NONFINITE 2u
#define SPH_EFLAG_BOX 4u      /* batch: a particle left its instance's grid */
#define SPH_EFLAG_TIMEOUT 8u  /* a bounded device wait gave up               */

#define SPH_MAX_SOURCES 8

/* Particle tags (base/particle_array.pxd:20-26): only LocalReal (0)
 * destinations are evaluated; others get 0. */
#define SPH_TAG_LOCAL_REAL 0

typedef struct sph_ctx sph_ctx;

/* One particle array: FP64 device arrays of length n.  NULL = absent (read
 * as 0).  nx..tz are the wall normals/tangents MonaghanBoundaryForce reads. */
typedef struct {
    int64_t n;
    const double *x, *y, *z, *u, *v, *w, *m, *h, *rho, *p, *cs;
    const double *nx, *ny, *nz, *tx, *ty, *tz;
    const int64_t *tag; /* NULL: every particle LocalReal */
} sph_array_view;

/* term flags of one source in sph_rates */
#define SPH_TERM_PGRAD 1u   /* SPHPressureGradient            */
#define SPH_TERM_AVISC 2u   /* MonaghanArtificialVsicosity    */
#define SPH_TERM_XSPH 4u    /* XSPHCorrection                 */
#define SPH_TERM_BFORCE 8u  /* MonaghanBoundaryForce          */
#define SPH_TERM_DRHO 16u   /* SPHDensityRate (density_funcs.pyx:89-158): drho += m_j v_ij . grad W */
/* SPHVelocityDivergence (adke_funcs.pyx:152-226, hks off): div_i = (1/rho_i)
 * sum m_j (v_j - v_i) . grad W(r_ij, (h_i + h_j)/2), written to drho_out;
 * not combined with SPH_TERM_DRHO in one launch */
#define SPH_TERM_VDIV 32u
/* MomentumEquation (pressure_funcs.pyx:106-252) is PGRAD | AVISC with its own
 * eta (it stores eta, unlike MonaghanArtificialVsicosity) */

typedef struct {
    int src;           /* array slot of the source (index into the last build) */
    uint32_t flags;    /* SPH_TERM_* */
    double alpha, beta, eta; /* avisc (eta = 0 reproduces the reference)        */
    double eps;        /* xsph */
    double delp;       /* boundary force */
} sph_source_term;

typedef struct {
    int dim;              /* kernel dimension 1..3                              */
    int tait;             /* 1: also compute p, cs by the Tait equation           */
    double co, ro, gamma; /* Tait parameters                                    */
    double h0;            /* > 0: W at this fixed h for every pair, over the
                           * neighbours of the particles' own radius
                           * (ADKEPilotRho, adke_funcs.pyx:15-73); 0: the
                           * particles' own h (SPHRho)                          */
} sph_density_params;

typedef struct {
    int dim;
    int add_velocity;     /* PositionStepping: pos_out += (u, v, w) of the dest */
    double gx, gy, gz;    /* GravityForce: acc_out += g (when add_gravity)      */
    int add_gravity;
    double *drho_out;     /* density rate of SPH_TERM_DRHO sources (may be NULL) */
} sph_rates_params;

/* One line of an integrator update, applied elementwise over n particles:
 *   mode 0: t = base + c1 * (k1 (+ k2))          RK2 final (k2 may be NULL)
 *   mode 1: t = base + k1 * c1                   Euler / predictor step,
 *                                                LeapFrog position correction
 *   mode 2: t = base                             copy (set_initial_arrays)
 *   mode 3: t = 2 * base - k1                    PredictorCorrector final
 *   mode 4: t = base + c1 * (k2 - k1)            LeapFrog corrector
 *   mode 5: t = base + c1 * (k1 + 2 k2 + 2 k3 + k4)   RK4 final
 *   out[i] = t;  if (save) save[i] = t;
 * The FP64 operations are rounded exactly as the NumPy expressions of
 * solver/integrator.py:472-912 (left to right, no FMA contraction). */
typedef struct {
    double *out;
    double *save;
    const double *base;
    const double *k1;
    const double *k2;
    double c1;
    int mode;
    const double *k3; /* mode 5 only */
    const double *k4; /* mode 5 only */
} sph_axpy_line;

#define SPH_MAX_AXPY_LINES 12

/* context */
int sph_ctx_create(int dim, sph_ctx **out);
int sph_ctx_destroy(sph_ctx *ctx);
int sph_ctx_set_stream(sph_ctx *ctx, void *cuda_stream);
int sph_last_error(char *buf, size_t len);
int sph_version(void);
/* Number of kernels this library has launched in the process (diagnostic). */
int sph_launch_count(int64_t *out);

/* Neighbour structure for all arrays of one Particles collection.  Bins
 * every array on a dense grid of cells of size cell_size/subdiv (subdiv in
 * 1..3), sorts each array by cell (deterministic order within a cell) and
 * gathers the sorted FP32 snapshots.  Synchronises the stream once (to size
 * the grid).  check_jump: fail with SPH_ERR_JUMP if any particle's cell
 * (of size cell_size) moved by more than one since the previous build. */
int sph_nnps_build(sph_ctx *ctx, const sph_array_view *arrays, int narrays, double cell_size,
                   double radius_scale, int subdiv, int check_jump);

/* Neighbour-list skin as a fraction of the search radius (0 .. 0.5; 0 =
 * lists hold exactly the neighbours).  With a skin the grid cell is
 * cell_size (1 + fraction) / subdiv and every list keeps the sources within
 * radius_scale h + skin; the passes that stream a list keep the exact
 * neighbours, so results do not depend on the skin.  Takes effect at the
 * next build.  No reference counterpart (the reference rebuilds its lists
 * at every update, base/nnps.pyx:581-620). */
int sph_ctx_set_skin(sph_ctx *ctx, double skin_fraction);

/* Symmetric neighbour relation for per-particle smoothing lengths
 * (base/nnps.pyx:654-749 VarHNbrParticleLocator, used when
 * Particles(variable_h=True)): with on = 1, source j is a neighbour of
 * destination i when |x_i - x_j| < radius_scale h_i OR < radius_scale h_j
 * (each test exactly as the reference's FP64 one).  Takes effect at the
 * next build. */
int sph_ctx_set_symmetric(sph_ctx *ctx, int on);

/* Periodic x axis (base/cell.pyx:1277-1376 CellManager.create_ghost_cells,
 * cell.pyx:392-398 binning of the PeriodicDomain, which the reference
 * applies along x only): with on = 1, every neighbour search treats x as
 * periodic on [xmin, xmax).  Instead of appending ghost copies of the cells
 * near either end to the particle arrays, a particle is binned at its image
 * in the period and a stencil row that leaves the period continues at the
 * other end, where the sources are the images shifted by -+(xmax - xmin)
 * (added in FP64 exactly as the reference shifts its ghost copies); the
 * images carry the state of the particle they copy.  The period must span
 * at least 2K+1 grid cells.  Takes effect at the next build. */
int sph_ctx_set_periodic(sph_ctx *ctx, int on, double xmin, double xmax);
/* Particles.update() (base/particles.py:159-200 -> cell.pyx:927-1015):
 * with a skin and the same arrays, refresh the sorted snapshot in the
 * order of the last full build (one kernel, the reference's jump check
 * against the previous update) while every particle is within half the
 * skin of its build position, its h unchanged and no list overflowed;
 * otherwise a full sph_nnps_build.  *rebuilt (may be NULL) tells which.
 * Synchronises the stream once, unless the check is deferred (below). */
int sph_nnps_update(sph_ctx *ctx, const sph_array_view *arrays, int narrays, double cell_size,
                    double radius_scale, int subdiv, int check_jump, int *rebuilt);
/* Deferred check of light refreshes (on = 1): sph_nnps_update queues the
 * refresh and the copy of its status and returns without synchronising
 * (*rebuilt = 0).  The next sph_density / sph_rates / sph_features launches
 * its pass first, with a device test that makes the pass return at once
 * when the refresh found a particle past half the skin, a changed h, a
 * jump or a list past its capacity; it then reads the status (long since copied) and, in that case,
 * makes the full build and launches the pass again, or returns
 * SPH_ERR_JUMP.  Every other entry point of the context reads a pending
 * status first, synchronously.  Results are those of the synchronous
 * update; a jump is reported by the first pass after the update instead of
 * by the update itself.  No reference counterpart (the reference's update
 * runs on the host, base/cell.pyx:927-962). */
int sph_ctx_set_deferred(sph_ctx *ctx, int on);
/* out[0] = deferred light refreshes, out[1] = those of them found stale
 * (replaced by a full build at their first pass). */
int sph_nnps_deferred_stats(sph_ctx *ctx, int64_t *out);
/* out[0] = full builds, out[1] = light refreshes of this context. */
int sph_nnps_stats(sph_ctx *ctx, int64_t *out);

/* Step programs (no reference counterpart: the reference advances a
 * simulation by Python calls per calc and per NumPy update,
 * solver/integrator.py:432-645).  Between sph_step_begin and sph_step_end
 * the calls a time step is made of -- sph_nnps_update / sph_nnps_build,
 * sph_density, sph_rates, sph_tait, sph_const_rates, sph_integrate,
 * sph_refresh_state -- are recorded (with their pointers and parameters)
 * instead of run; the other entry points of the context fail with
 * SPH_ERR_STATE meanwhile.  sph_step_run runs the recorded step nsteps
 * times: while the neighbour build stays the same (light refreshes), as one
 * CUDA graph per step in which every launch after a light refresh returns
 * at once when the refresh found the lists stale; after each step it reads
 * the step's status (synchronises), reports a jump as the calls do, and
 * resumes a step whose refresh was stale with a full build and the rest of
 * the step's calls run eagerly.  A graph is captured once per build, after a
 * step that needed no full build; after a graph that never ran a whole step
 * the next 1, 2, 4 .. 64 capture chances are skipped (the flow's lists go
 * stale too soon for a graph to pay).  Results equal the recorded calls run
 * one by one.  Runs on the context's stream (on a stream of its own, ordered with
 * the legacy default stream, when the context's is that stream). */
typedef struct sph_step sph_step;
int sph_step_begin(sph_ctx *ctx);
int sph_step_end(sph_ctx *ctx, sph_step **out);
int sph_step_run(sph_step *step, int nsteps);
/* out[0] graph replays, out[1] eager steps, out[2] steps resumed after a
 * stale refresh, out[3] graph captures, out[4] recorded calls, out[5]
 * kernels of one replay, out[6] device time of all replays in microseconds
 * (CUDA events around each graph launch), out[7] capture attempts, out[8]
 * why the last attempt found no graph: 0 none failed, 1 an update needed a
 * full build, 2-5 a neighbour list needed building, 6 more than 32
 * updates, 7 a recorded full build, 8 a call failed while captured, 9 the
 * build changed, 10 the graph could not be made; out[9] captures that
 * updated the previous graph's executable in place (cudaGraphExecUpdate)
 * instead of instantiating a new one.  out holds 10 values. */
int sph_step_stats(sph_step *step, int64_t *out);
int sph_step_destroy(sph_step *step);

/* Brick-staged pair passes (on = 1, the default): for one source of uniform
 * h without a periodic axis or the variable-h relation, sph_density
 * (SPHRho, + Tait) and sph_rates with the terms PGRAD | AVISC (+ XSPH) run
 * kernels that stage, per brick of grid cells, the records of every source
 * within the stencil of the brick in shared memory once, and stream a
 * neighbour list of 16-bit indices into that staging.  Results are those of
 * the list-streaming kernels within FP32 rounding (positions relative to the
 * brick centre instead of the particle's cell); neighbour sets are the same.
 * on = 0 selects the list-streaming kernels everywhere.  Takes effect at the
 * next build.  The same reference routines as sph_density / sph_rates. */
int sph_ctx_set_bricks(sph_ctx *ctx, int on);
/* out[0] = pair passes run by the brick-staged kernels in this context. */
int sph_pair_pass_stats(sph_ctx *ctx, int64_t *out);

/* Neighbour lists of destination dst among source src (radius
 * radius_scale*h_dst, radius_scale no larger than the build's), as original particle
 * indices: counts[i] (device, int64, n_dst) then, given the exclusive prefix
 * offsets (device, n_dst+1), the index lists, each sorted ascending and then,
 * when dst == src, the destination itself swapped with the last entry (as
 * the reference's cache update does, base/nnps.pyx:609-616). */
int sph_nnps_count(sph_ctx *ctx, int dst, int src, double radius_scale, int64_t *counts);
int sph_nnps_fill(sph_ctx *ctx, int dst, int src, double radius_scale, const int64_t *offsets,
                  int64_t *index);

/* Build (if stale) the neighbour lists of destination dst among each of the
 * nsrc sources for the current neighbour build -- the counterpart of the
 * reference locator's cache update, base/nnps.pyx:566-620.  sph_density and
 * sph_rates build missing lists themselves; this entry point lets a caller
 * do it ahead of time. */
int sph_nbr_lists(sph_ctx *ctx, int dst, const int *srcs, int nsrc);

/* Re-gather the sorted FP32 snapshot of one array from (possibly new) device
 * pointers, keeping the cell order of the last build.  For data changed
 * since the build without moving particles across cells (velocities,
 * densities, pressures written outside sph_density). */
int sph_refresh_state(sph_ctx *ctx, int array, const sph_array_view *view);

int sph_density(sph_ctx *ctx, int dst, const int *srcs, int nsrc, const sph_density_params *prm,
                double *rho_out, double *p_out, double *cs_out);

/* acc_out[3] / pos_out[3]: FP64 outputs (entries may be NULL).  accumulate:
 * 0 stores the sum, 1 adds it to the outputs. */
int sph_rates(sph_ctx *ctx, int dst, const sph_source_term *terms, int nterms,
              const sph_rates_params *prm, double *const *acc_out, double *const *pos_out,
              int accumulate);

int sph_tait(sph_ctx *ctx, int64_t n, const double *rho, const int64_t *tag, double co,
             double ro, double gamma, double *p_out, double *cs_out);

/* ADKESmoothingUpdate.eval (sph/funcs/adke_funcs.pyx:118-147): over the
 * LocalReal particles among the first n, log g = (sum of log rhop) / nreal,
 * then h_out = h0 k (g / rhop)^eps for each of them (others untouched).  The
 * logarithms are summed in FP64 in a fixed order, so the result does not
 * depend on the launch; every step is rounded as the reference's C (no
 * fused multiply-add). */
int sph_adke_smoothing(sph_ctx *ctx, int64_t n, int64_t nreal, const int64_t *tag,
                       const double *rhop, double h0, double k, double eps, double *h_out);

/* ADKEConductionCoeffUpdate.eval (adke_funcs.pyx:256-291): for the
 * LocalReal particles among the first nreal, q_out = (g1 cs + g2 h
 * (|div| - div)) h (others untouched), rounded as the reference's C. */
int sph_adke_conduction(sph_ctx *ctx, int64_t nreal, const int64_t *tag, const double *cs,
                        const double *h, const double *div, double g1, double g2,
                        double *q_out);

/* kind 0: out_k = g_k (GravityForce); kind 1: out_k = (u, v, w)_k of src
 * (PositionStepping).  nout outputs, non-LocalReal get 0. */
int sph_const_rates(sph_ctx *ctx, int kind, int64_t n, const int64_t *tag, const double *g3,
                    const double *u, const double *v, const double *w, int nout,
                    double *const *out);

int sph_integrate(sph_ctx *ctx, int64_t n, const sph_axpy_line *lines, int nlines);

/* FP64 sums over LocalReal particles: out[0]=mass, out[1..3]=momentum,
 * out[4]=kinetic energy, out[5]=number of LocalReal particles.  out must
 * hold 6 doubles.  Synchronises. */
int sph_invariants(sph_ctx *ctx, const sph_array_view *a, double *out);

/* Allocation-free variant of sph_invariants (no counterpart in the
 * reference).  For callers that cannot allocate device memory: real-time
 * loops that forbid allocation after start-up (a cudaMalloc can block or
 * fail mid-run), and host applications whose own allocator reserves all
 * device memory up front.  Needs no context; its scratch is a fixed
 * file-scope device array (192 KiB per GPU that loads the library, held
 * until exit) that every call shares, so calls that overlap on the GPU race
 * and must be serialised by the caller.  The first call on a device looks
 * up the scratch's device address.  Rejects arrays of more than 16777216
 * particles with SPH_ERR_ARG.  stream: a cudaStream_t (NULL = default
 * stream).  out: 6 host doubles as for sph_invariants; the call copies them
 * to the host and synchronises the stream before it returns. */
int sph_invariants_noalloc(const sph_array_view *a, double *out, void *stream);

/* Self-check of the integer-operation conversions the light refresh uses in
 * place of FP64 instructions (no reference counterpart): FP64 -> FP32 round
 * to nearest against __double2float_rn, int -> FP64 against __int2double_rn
 * and the FP32-screened cell index against its FP64 form, over n hashed
 * inputs (all exponents, both signs) and edge values.  mismatches: host
 * int64, the number of differing results (0 expected).  Synchronises. */
int sph_selftest_conversions(int64_t n, int64_t *mismatches);

/* ---------------------------------------------------------------------
 * Batches of independent simulations (no counterpart in the reference,
 * which runs one simulation per Solver).  All instances share one
 * operation recipe -- SPHRho (+Tait) of each instance on itself, one set of
 * rate terms among its own particles, gravity / position stepping, Euler or
 * RK2 -- and their particles are concatenated in one set of arrays.  Every
 * instance gets its own dense grid (its own cell size and subdivision) over
 * a region around its particles, so a time step needs no host
 * synchronisation and no allocation: the step is captured into a CUDA graph
 * and replayed; the regions follow the instances as they deform.
 * --------------------------------------------------------------------- */
typedef struct sph_batch sph_batch;

typedef struct {
    int64_t offset, n;    /* particle range of the instance (instances tile [0, n) in order) */
    double cell_size;     /* reference cell size: radius_scale * max h of the instance */
    double lo[3], hi[3];  /* region the instance's particles may occupy at set-up */
    int uniform_h;        /* 1 if every particle of the instance has the same h */
    int subdiv;           /* grid cells per reference cell of this instance, 1..3
                             (0: the recipe's) */
} sph_batch_instance;

typedef struct {
    int dim;              /* kernel dimension 1..3 (also: integrated components) */
    int subdiv;           /* grid cells per reference cell, 1..3 */
    int scheme;           /* 0: Euler (integrator.py:525-573), 1: RK2 (:581-645) */
    int list_cap;         /* neighbour list capacity per particle (0: default) */
    double radius_scale;  /* 2 for the cubic spline */
    double dt;
    sph_density_params density;  /* SPHRho (+ Tait when density.tait) */
    sph_source_term term;        /* rate terms among an instance's particles (src unused) */
    sph_rates_params rates;      /* gravity and position stepping */
    double margin;        /* > 0: when a particle leaves its instance's region the
                             step is undone, every region is re-derived from the
                             current extent e as [lo - m e - 4 c, hi + m e + 4 c]
                             (c the instance's reference cell) and the step is
                             repeated; 0: leaving the region is an error */
} sph_batch_recipe;

int sph_batch_create(sph_batch **out);
int sph_batch_destroy(sph_batch *b);
/* Allocates everything the steps need and uploads the per-instance grids
 * (synchronises).  all: the concatenated particle arrays (device). */
int sph_batch_setup(sph_batch *b, const sph_array_view *all, const sph_batch_instance *inst,
                    int ninst, const sph_batch_recipe *recipe);
/* Advance every instance by nsteps time steps on the batch's own stream.
 * use_graph: capture the step into a CUDA graph on the first call (and after
 * the regions change) and replay it.  Every launch of a step that writes
 * the state is gated on the error word: when a particle leaves its
 * instance's region the step stops there, an RK2 step returns to the state
 * it started from, the regions are re-derived from the current extents
 * (recipe.margin) and the step is repeated.  Synchronises once at the end
 * (and once per re-derivation).  A jump leaves the state at the start of
 * the failing step and the error word set. */
int sph_batch_step(sph_batch *b, int nsteps, int use_graph);
/* Wait for the batch's stream. */
int sph_batch_sync(sph_batch *b);
/* The batch's CUDA stream (cudaStream_t), e.g. to record timing events. */
int sph_batch_stream(sph_batch *b, void **out);
/* Read and clear the batch's device error word (SPH_EFLAG_*; synchronises). */
int sph_batch_error_word(sph_batch *b, uint32_t *out);
/* out[0] regions re-derived so far, out[1] cells of the current grids,
 * out[2] steps completed, out[3] groups of instances of equal subdivision
 * (one pair launch each).  No reference counterpart. */
int sph_batch_stats(sph_batch *b, int64_t *out);
/* Neighbour counts (incl. self) of the batch's last evaluation, summed per
 * instance into out[ninst] (synchronises).  Used for pair-interaction
 * counts; the reference has no batch, its per-array counterpart is
 * NbrParticleLocatorBase.get_nearest_particles (base/nnps.pyx:311). */
int sph_batch_pair_counts(sph_batch *b, uint64_t *out);

/* Read and clear the device error word (synchronises). */
int sph_error_word(sph_ctx *ctx, uint32_t *out);

/* Mean neighbour count (incl. self) of dst among src from the last build,
 * computed on the device (synchronises).  Used for pair-interaction counts. */
int sph_mean_neighbours(sph_ctx *ctx, int dst, int src, double *out);

/* ------------------------------------------------------------------------
 * Learned momentum closure.  None of these has a counterpart in the
 * reference: the network stands in for the momentum pair loop of a fluid
 * array on itself (SPHPressureGradient, sph/funcs/pressure_funcs.pyx:40-91,
 * and MonaghanArtificialVsicosity, sph/funcs/viscosity_funcs.pyx:41-124).
 *
 * Network 192 -> 128 -> 128 -> 2, exact GELU on the hidden layers; BF16
 * weights and matrix-product inputs, FP32 accumulation (tensor memory).
 * Parameters: one FP32 vector of SPH_MLP_NPARAM values, W row-major
 * [out][in]; the BF16 copies (w1 [128][192], w2 [128][128], its transpose
 * w2t, w3 [2][128]) are written by sph_mlp_sync and sph_mlp_adam.
 * Buffers are device pointers; x, z1, z2, h1, h2 16-byte aligned.
 * ------------------------------------------------------------------------ */
#define SPH_MLP_NIN 192
#define SPH_MLP_NH 128
#define SPH_MLP_NOUT 2
#define SPH_MLP_NNBR 32       /* neighbours per feature row                  */
#define SPH_MLP_NCH 6         /* channels per neighbour                      */
#define SPH_MLP_OFF_W1 0
#define SPH_MLP_OFF_B1 (SPH_MLP_OFF_W1 + SPH_MLP_NH * SPH_MLP_NIN)
#define SPH_MLP_OFF_W2 (SPH_MLP_OFF_B1 + SPH_MLP_NH)
#define SPH_MLP_OFF_B2 (SPH_MLP_OFF_W2 + SPH_MLP_NH * SPH_MLP_NH)
#define SPH_MLP_OFF_W3 (SPH_MLP_OFF_B2 + SPH_MLP_NH)
#define SPH_MLP_OFF_B3 (SPH_MLP_OFF_W3 + SPH_MLP_NOUT * SPH_MLP_NH)
#define SPH_MLP_NPARAM (SPH_MLP_OFF_B3 + SPH_MLP_NOUT)

typedef struct {
    float *params;                 /* SPH_MLP_NPARAM FP32 master values */
    uint16_t *w1, *w2, *w2t, *w3;  /* BF16 copies                        */
} sph_mlp_model;

typedef struct {
    double c0;                     /* velocity scale                     */
    float mean[SPH_MLP_NCH];       /* per-channel standardisation        */
    float inv_std[SPH_MLP_NCH];
} sph_mlp_feature_params;

/* Feature rows of every particle of dst (by original index) from its
 * neighbours in src within radius_scale * h_i: the 32 nearest, self
 * included, ordered by squared distance then sorted source slot, each
 * ((x_i-x_j)/h_i, (y_i-y_j)/h_i, (u_j-u_i)/c0, (v_j-v_i)/c0, rho_j, p_j)
 * minus mean times inv_std; missing neighbours are zero rows.  Reads the
 * sorted state of the last density pass.  Output BF16 [n][192] and/or FP32
 * [n][192] (either may be NULL). */
int sph_mlp_features(sph_ctx *ctx, int dst, int src, const sph_mlp_feature_params *prm,
                     uint16_t *out_bf16, float *out_f32);
/* Write the BF16 copies from the FP32 parameters. */
int sph_mlp_sync(const sph_mlp_model *m, void *stream);
/* y[n][2] = network(x[n][192]).  z1, z2 (FP32 [n][128]) and h1, h2 (BF16
 * [n][128]) save the pre-activations and activations for sph_mlp_backward
 * (NULL: not saved).  err: device word, SPH_EFLAG_TIMEOUT on a wait that
 * gave up. */
int sph_mlp_forward(const sph_mlp_model *m, const uint16_t *x, int64_t n, float *y, float *z1,
                    float *z2, uint16_t *h1, uint16_t *h2, uint32_t *err, void *stream);
/* FP32 scratch values sph_mlp_backward needs for a batch of n samples. */
int sph_mlp_backward_scratch(int64_t n, int64_t *floats);
/* Gradient of loss = 0.5 * inv_count * sum (y - target)^2 into grad
 * [SPH_MLP_NPARAM] and the loss into *loss (device), from the saved
 * forward values.  Deterministic: fixed-order sums of per-CTA partials. */
int sph_mlp_backward(const sph_mlp_model *m, const uint16_t *x, const uint16_t *h1,
                     const uint16_t *h2, const float *z1, const float *z2, const float *y,
                     const float *target, int64_t n, float inv_count, float *grad, float *loss,
                     float *scratch, uint32_t *err, void *stream);
/* One Adam step (bias-corrected, step counts from 1) on the FP32
 * parameters with moment buffers mom, vel; rewrites the BF16 copies. */
int sph_mlp_adam(const sph_mlp_model *m, const float *grad, float *mom, float *vel, float lr,
                 float beta1, float beta2, float eps, int step, void *stream);
/* acc[c][i] = (or +=) (y[i][c] * scale[c] + mean[c]) * c0^2 / h_i for the
 * LocalReal particles of dst (acc[2], if given, is zeroed when not
 * accumulating), computed in FP32 and stored as FP64. */
int sph_mlp_apply(sph_ctx *ctx, int dst, const float *y, double c0, const double *scale,
                  const double *mean, double *const *acc, int accumulate);
/* out[i][c] = (a_c[i] * h_i / c0^2 - mean[c]) * inv_std[c]: standardised
 * training targets from accelerations. */
int sph_mlp_targets(int64_t n, const double *ax, const double *ay, const double *h, double c0,
                    const double *mean, const double *inv_std, float *out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PYSPH_GB300_H */
