/*
 * clbm.h -- C ABI of libclbm, the GB300-native cloning sampler over D2Q9
 * lattice-Boltzmann clones of a body-force-driven channel flow past a square.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, and
 * returns an int status (CLBM_OK == 0, negative on error; clbm_strerror and
 * clbm_last_error describe it).  There is no CPU fallback: without a CUDA
 * device the calls that compute return CLBM_ERR_CUDA.
 *
 * Two levels, mirroring the reference (tlestang/cloning-lbm-MPI):
 *
 *  1. Function level (clbm_ref_*): one clone in the reference's own FP64
 *     array-of-structures layout IDX(x,y,k) = k + 9*(y + Dy*x)
 *     (src/lbm_src/global.h:4), DEVICE pointers, geometry passed explicitly
 *     instead of through the reference's globals Dx, Dy, xmin, xmax, ymin, ymax
 *     (src/lbm_src/global.h:11-13).  Results are bit-identical to the
 *     reference functions named beside each declaration.
 *
 *  2. Sampler level (clbm_ctx): every clone of one or several independent runs
 *     lives in one device-resident structure-of-arrays population buffer; one
 *     call advances them all by a cloning interval, one call performs the
 *     cloning step (weights, normaliser, resampling, clone copy,
 *     perturbation of new clones).  This replaces the MPI drivers' per-rank
 *     clone loops and point-to-point clone transfers
 *     (src/mpi_LBM_GK_pops_perturb.cpp:387-701).
 *
 * Threading: a context is used by one host thread at a time; its work is
 * ordered on the context's own CUDA stream.
 */
#ifndef CLBM_H
#define CLBM_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define CLBM_OK 0
#define CLBM_ERR_INVALID (-1) /* bad argument or call order */
#define CLBM_ERR_CUDA (-2)    /* CUDA runtime error, or no device */
#define CLBM_ERR_DEVICE (-3)  /* the device error word was set (see below) */
#define CLBM_ERR_NOMEM (-4)   /* device or pinned host allocation failed */
#define CLBM_ERR_IO (-5)      /* file I/O (drivers) */

/* device error word bits (clbm_error_word) */
#define CLBM_DEV_NONFINITE_DRAG 0x1u  /* a drag value was NaN or Inf */
#define CLBM_DEV_WEIGHT_OVERFLOW 0x2u /* exp(alpha*s) or the normaliser overflowed */
#define CLBM_DEV_BAD_DENSITY 0x4u     /* rho <= 0 or NaN at some node */
#define CLBM_DEV_BAD_PARENT 0x8u      /* resampling produced an invalid parent */
#define CLBM_DEV_RESAMPLE 0x10u       /* copy numbers could not be corrected */
#define CLBM_DEV_TIMEOUT 0x20u        /* a bounded wait of the random-field
                                         tensor-core kernel gave up */

/* arithmetic of the populations */
#define CLBM_FP64 0 /* FP64, reference operation order, no fused multiply-add */
#define CLBM_FP32 1 /* FP32 populations stored as f - w[k]; FP64 drag integral,
                       weights, normaliser and SCGF */

/* resampling of the cloning step */
#define CLBM_RESAMPLE_REFERENCE 0  /* floor(s_j/R + drand48()) + glibc rand()
                                      kill/duplicate correction, the reference's
                                      random streams emulated bit for bit */
#define CLBM_RESAMPLE_SYSTEMATIC 1 /* systematic resampling, one Philox uniform
                                      per interval, log-domain weights */

/* drag on the square, the observable of the weights (clbm_run_desc.drag_mode) */
#define CLBM_DRAG_STRESS 0   /* the reference's stress integration over the
                                perimeter nodes (src/lbm_src/force.cpp:8-144) */
#define CLBM_DRAG_MOMENTUM 1 /* momentum exchange of the links bounced back on
                                the square: F = sum -2 c_kx f_k over the slots
                                the square reflects (no counterpart in the
                                reference; a different estimator of the same
                                force, see clbm_run_interval) */

/* perturbation of newly created clones (at the start of the next interval) */
#define CLBM_PERTURB_NONE 0
#define CLBM_PERTURB_MIX 1     /* snapshot mix, prefactors from drand48 */
#define CLBM_PERTURB_UNIFORM 2 /* f <- f (1 + eps (2u-1)), u Philox4x32-10 */

/* context creation flags */
#define CLBM_FLAG_GRAPH 0x1 /* capture each interval in a CUDA graph */

typedef struct {
  int nx, ny;                 /* Dx, Dy */
  int xmin, xmax, ymin, ymax; /* square, perimeter nodes inclusive */
} clbm_geom;

typedef struct {
  int width, height;          /* Dx, Dy */
  int xmin, xmax, ymin, ymax; /* square, perimeter nodes inclusive */
  int nclones;                /* Nc */
  int ranks;                  /* virtual MPI ranks of the reference's random
                                 streams (>= 1, divides nclones) */
  double tau;                 /* BGK relaxation time */
  double beta;                /* body force beta0 */
  double alpha;               /* bias k */
  double force_scale;         /* F <- F*force_scale - force_shift */
  double force_shift;         /*   (1/F0 and AVG=1.775 under ZERO_MEAN) */
  double dt;                  /* weight integral: s = dt * sum F */
  int perturb_mode;           /* CLBM_PERTURB_* */
  int resample_mode;          /* CLBM_RESAMPLE_* */
  double eps;                 /* perturbation amplitude */
  unsigned long long seed;    /* counter-based random streams */
  int nsnap;                  /* snapshots for CLBM_PERTURB_MIX (<= 64) */
  int drag_mode;              /* CLBM_DRAG_* (0: the reference's) */
  /* spatially random body force of the forcing variant
   * (src/mpi_LBM_GK_forcing.cpp:333-364): at the start of every interval
   * each clone draws a Gaussian random field `map` with covariance
   * exp(-r^2 / (2 field_sigma^2)) (circulant embedding,
   * src/perturbation_routines/generate_random_field.cpp:9-181, generalised
   * from the reference's square domain to W x H), and its first field_steps
   * steps use beta(x,y) = (1 + field_eps * map(x,y)) * beta. */
  int field_mode;             /* 0 off, 1 Gaussian random field */
  int field_steps;            /* T1 of the interval (steps under the field) */
  double field_eps;           /* amplitude eps */
  double field_sigma;         /* correlation length (reference: 32) */
} clbm_run_desc;

typedef struct clbm_ctx clbm_ctx;

const char *clbm_strerror(int status);
/* last error message of the calling thread (CUDA error text included) */
const char *clbm_last_error(void);
int clbm_version(void);
/* number of CUDA devices visible (0 without a GPU); never fails */
int clbm_device_count(void);

/* ---- function level: reference functions on one clone, device pointers ---- */

/* streamingAndCollisionComputeMacroBodyForce(fin, fout, rho, ux, uy, beta,
 * tau), src/lbm_src/streamCollCompute.h:1 / streamCollCompute.cpp:7-48.
 * fin is overwritten with the post-collision populations; rho/ux/uy may be
 * NULL. stream is a cudaStream_t (NULL = default stream). */
int clbm_ref_stream_collide(const clbm_geom *g, double *fin, double *fout,
                            double *rho, double *ux, double *uy, double beta,
                            double tau, void *stream);
/* streamingAndCollisionComputeMacroBodyForceSpatial(fin, fout, rho, ux, uy,
 * beta0, map, tau, eps), streamCollCompute.h:2 / streamCollCompute.cpp:50-93 */
int clbm_ref_stream_collide_spatial(const clbm_geom *g, double *fin,
                                    double *fout, double *rho, double *ux,
                                    double *uy, double beta0, const double *map,
                                    double tau, double eps, void *stream);
/* computeDomainNoSlipWalls_BB(fout, fin), boundaryConditions.h:1 */
int clbm_ref_walls_bb(const clbm_geom *g, double *fout, const double *fin,
                      void *stream);
/* computeSquareBounceBack_TEST(fout, fin), boundaryConditions.h:5 */
int clbm_ref_square_bb(const clbm_geom *g, double *fout, const double *fin,
                       void *stream);
/* interior reset to w[k], src/mpi_LBM_GK_pops_perturb.cpp:430-439 */
int clbm_ref_interior_reset(const clbm_geom *g, double *fout, void *stream);
/* computeForceOnSquare(f, omega), src/lbm_src/force.h:1; the result is
 * written to *result (HOST pointer) after a stream synchronisation. */
int clbm_ref_force_on_square(const clbm_geom *g, const double *f,
                             double omega, double *result, void *stream);
/* generatePerturbedState(fin, snaps, eps, NN, N),
 * src/perturbation.h:5 / generatePerturbedState.cpp:4-38, with the NN
 * drand48() prefactors supplied by the caller (HOST array).  snaps is one
 * DEVICE array of NN*N doubles.  Returns a status (the reference returns an
 * undefined value). */
int clbm_ref_perturbed_state(double *fin, const double *snaps, double eps,
                             int nsnap, int n, const double *prefactors,
                             void *stream);
/* Same computation and result as clbm_ref_perturbed_state, for callers that
 * cannot allocate device memory (an allocator owns the whole device, or an
 * allocation's implicit synchronisation is not allowed in their loop).  No
 * counterpart in the reference.  It allocates nothing: its scratch (the
 * prefactors and the per-block norm partials) lives in one fixed device array
 * of 66 KB that every GPU loading the library holds until exit, so n (the
 * values of one state, 9*Dx*Dy) is limited to 1048576 and nsnap to 64; larger
 * sizes return CLBM_ERR_INVALID.  The first call on a device looks up the
 * array's device address, so make that first call before any stream capture
 * (the address is kept for the process: do not call it again after a
 * cudaDeviceReset of that device).
 * Each call synchronises `stream` before it returns.  All calls share the
 * array: calls that overlap on the GPU (other streams, other host threads)
 * race and must be serialised by the caller. */
int clbm_ref_perturbed_state_noalloc(double *fin, const double *snaps,
                                     double eps, int nsnap, int n,
                                     const double *prefactors, void *stream);

/* generate_random_field (src/perturbation_routines/generate_random_field.cpp:9-181):
 * one Gaussian random field with covariance exp(-r^2 / (2 sigma^2)) on a
 * dx x dy lattice by circulant embedding, written to the HOST array map in
 * the reference's order y + dy*x (dx*dy values).  The reference draws its
 * normals from rand() (randNormal.cpp:4-22) and takes dx = dy; here any dx,
 * dy <= 1024 (dy >= 4), and the normals come from a counter-based stream:
 * (seed, draw) selects the field, and it equals the field the sampler draws
 * for clone 0 of run 0 in interval `draw` of a context with the same seed and
 * lattice.  Parity with the reference is statistical (same covariance).
 * *negative (nullable) = eigenvalues of the embedding below -1e-15 (clamped
 * to 0, the reference's `error`). */
int clbm_ref_random_field(int dx, int dy, double sigma, unsigned long long seed,
                          int draw, double *map, int *negative);

/* ---- sampler level ------------------------------------------------------- */

/* max_steps bounds the steps of one interval (drag-term storage). */
int clbm_create(const clbm_run_desc *runs, int nruns, int precision,
                int max_steps, int flags, clbm_ctx **out);
int clbm_destroy(clbm_ctx *ctx);

/* HOST FP64 arrays in the reference AoS layout, N = 9*Dx*Dy values per clone.
 * Loading replaces the clone's state (reference: the popfiles read at pops
 * driver :251-310). */
int clbm_load_pops_aos_f64(clbm_ctx *ctx, int run, int clone,
                           const double *aos);
/* all clones of a run at once: aos holds nclones*N values */
int clbm_load_run_aos_f64(clbm_ctx *ctx, int run, const double *aos);
/* the clone's current state (after a clone step: its parent's state, before
 * the pending perturbation) */
int clbm_dump_pops_aos_f64(clbm_ctx *ctx, int run, int clone, double *aos);
/* perturbation snapshots of a run, nsnap*N values (pops driver :321-364) */
int clbm_set_snapshots_aos_f64(clbm_ctx *ctx, int run, int nsnap,
                               const double *aos);
/* synthetic initial state of every clone of a run, generated on the device:
 * equilibrium at rho = 1, u = (u0, 0), times (1 + noise (2u-1)) with a
 * Philox uniform per population; w[k] inside the square. */
int clbm_init_equilibrium(clbm_ctx *ctx, int run, double u0, double noise,
                          unsigned long long seed);

/* one cloning interval of `steps` LB steps for every clone of every run:
 * pending perturbation of new clones, then per step stream-collide with wall
 * and square bounce-back and interior reset, the drag on the square after
 * every step, and the weight integral s_j = dt * sum F (pops driver :399-469).
 * The drag F is the run's drag_mode: the reference's stress integration, or
 * the momentum exchange of the links the square bounces back, evaluated in
 * the same pass from the populations the step already holds in registers and
 * summed per clone by a warp-shuffle reduction in a fixed order. */
int clbm_run_interval(clbm_ctx *ctx, int steps);
/* drag series of the last interval, [nclones][steps] F values of a run */
int clbm_get_drag(clbm_ctx *ctx, int run, double *out);
/* the cloning step of every run (pops driver :487-701): weights, mean weight
 * R_t, copy numbers, kill/duplicate correction, copy table, labels; copies
 * take effect (and new clones are marked for perturbation) for the next
 * interval. */
int clbm_clone_step(clbm_ctx *ctx);
/* results of the last clone step of a run; any pointer may be NULL.
 * labels[Nc] int32 (parent slot of each slot), *rvalue = R_t,
 * weights[Nc] = exp(alpha*s_j), copies_pre/post[Nc] int32 copy numbers before
 * and after the correction (forcing driver :461,:510). */
int clbm_get_clone_result(clbm_ctx *ctx, int run, int *labels, double *rvalue,
                          double *weights, int *copies_pre, int *copies_post);
/* R_t and log R_t of intervals [first, first+count) of a run (history of up
 * to 65536 cloning steps; log R_t stays finite where R_t overflows, e.g.
 * under systematic resampling at a large bias).  Either pointer may be NULL. */
int clbm_get_rvalues(clbm_ctx *ctx, int run, int first, int count,
                     double *rvalues, double *log_rvalues);
/* SCGF estimate psi = sum_t log R_t / (count * dT) over the recorded
 * intervals [first, first+count), in FP64 on the device; dT is the cloning
 * interval in the weight's time unit (steps * dt).  The reference computes
 * it offline (post_processing/read_rvalue.py:14-20, with a hard-coded dT). */
int clbm_scgf(clbm_ctx *ctx, int run, int first, int count, double dT,
              double *psi);
/* Replace the pending copy table of a run (labels[j] = parent slot of slot
 * j, parents must map to themselves); slots with labels[j] != j become new
 * clones.  Used to drive two contexts (FP32 and FP64) along one genealogy. */
int clbm_set_pending_labels(clbm_ctx *ctx, int run, const int *labels);
/* number of cloning steps a run has completed */
int clbm_intervals_done(clbm_ctx *ctx, int run, int *done);
/* `intervals` x (run_interval + clone_step) without host round trips, as
 * CUDA graphs when the context was created with CLBM_FLAG_GRAPH.  rvalues
 * (nullable, [nruns][intervals]) receives R_t of every interval. */
int clbm_run_sampler(clbm_ctx *ctx, int steps, int intervals, double *rvalues);
/* clbm_run_sampler that also delivers every interval's outputs to host
 * arrays without stalling the device: after each interval and its cloning
 * step the outputs are copied to pinned staging memory on the context's
 * stream, and from there into the caller's arrays on the host while the
 * device runs the next interval (the reference writes them per interval:
 * data_force.datout from the drag series, labels.dat, the weights;
 * src/mpi_LBM_GK_pops_perturb.cpp:445-520).  With T = steps and N = the
 * total clones of all runs, interval i writes (any pointer nullable):
 * drag + i*N*T the drag series, run after run and clone after clone, T
 * values each (clbm_get_drag's layout); labels + i*N the cloning step's
 * parent labels and weights + i*N the weights (clbm_get_clone_result's);
 * rvalues as clbm_run_sampler.  The caller's arrays may be pageable. */
int clbm_run_sampler_outputs(clbm_ctx *ctx, int steps, int intervals, double *rvalues,
                             double *drag, int *labels, double *weights);

/* Timing of the interval kernels: while enabled, every interval enqueued
 * eagerly (run_interval, or run_sampler without CUDA graphs) records a CUDA
 * event pair around its LB steps on the context's stream (the T step
 * launches, or the cluster-resident kernel's one launch per run).  Enabling
 * resets the accumulators; clbm_profile_read returns the summed milliseconds
 * and the number of LB steps they cover (and resets them). */
int clbm_profile(clbm_ctx *ctx, int enable);
int clbm_profile_read(clbm_ctx *ctx, double *step_ms, int *nsteps);
/* the same for the random-field kernels (forcing variant): summed
 * milliseconds of the field draws of the profiled intervals and their number
 * (and resets them) */
int clbm_profile_read_fields(clbm_ctx *ctx, double *field_ms, int *nintervals);

/* Autotuner of the FP32 interval: times each candidate on this context's
 * workload at an interval boundary without touching the sampler state, and
 * selects the fastest.  Candidates: the streaming step kernel's launch
 * variants (block size, registers per thread, store caching; one launch per
 * step), then the cluster-resident interval kernel (every clone's populations
 * in the shared memory of one thread-block cluster for all the steps of an
 * interval, one launch per interval) for cluster sizes 1, 2, 4, 8, 16, 3, 5,
 * 6, 7, 9, 10 (numbered in that order) and three thread counts (1024, 512,
 * 256), where every lattice fits: at most 8 + 33 uniform variants.  For the fastest
 * cluster-resident shapes it then times band splits balanced for the extra
 * cost of the square's rows and the walls (clbm_band_rows).  With several runs
 * it then times each run alone on every shape that fits its lattice (and its
 * best shape balanced) and, when the runs' own bests differ,
 * the per-run plan as a whole: each cluster-resident run is one launch per
 * interval on its own stream, concurrent with one step launch per step of
 * the streaming runs (a CUDA-graph interval holds them as parallel
 * branches).  *best = the chosen uniform variant, or CLBM_VARIANT_PER_RUN for
 * a per-run plan (clbm_get_run_variants); ms_per_variant (nullable,
 * *nvariants entries, -1 = not runnable here) = milliseconds per step of the
 * uniform variants.  With ms_per_variant NULL a result cached for the same
 * lattices and clone counts is reused.  FP64 contexts have one variant.
 * Every variant and plan gives bit-identical results. */
#define CLBM_VARIANT_PER_RUN (-1)
int clbm_autotune(clbm_ctx *ctx, int launches, int *best,
                  double *ms_per_variant, int *nvariants);
/* one variant (autotuner numbering) for every run */
int clbm_set_step_variant(clbm_ctx *ctx, int variant);
/* a variant per run (nruns entries): runs given a cluster-resident variant run
 * it concurrently, each on its own stream; the runs given a streaming variant
 * share one step launch per step and must name the same streaming variant */
int clbm_set_run_variants(clbm_ctx *ctx, const int *variants);
/* the variant each run uses now (nruns entries) */
int clbm_get_run_variants(clbm_ctx *ctx, int *variants);
/* Band split of a cluster-resident run: cluster rank b holds rows[b]
 * consecutive lattice rows (from the bottom wall up) of every clone.  An even
 * split (H / cs rows, the first H % cs bands one more) is the default and what
 * a variant change restores; the autotuner also times splits balanced for the
 * extra cost of the square's rows and the walls and keeps the fastest.  The
 * results do not depend on the split (bit-identical).
 * clbm_band_rows: the split of a lattice balanced for weight gamma (a node on
 * the general update path, the square's box, counts 1 + gamma, a node of a
 * wall or band-edge row 1 + gamma / 4; gamma <= 0: the even split), cs
 * entries, host-only.  clbm_set_band_rows: nbands = the run's cluster size
 * (a cluster-resident variant must be set), every band at least one row,
 * rows summing to the height, the largest band within shared memory; nbands 0
 * restores the even split.  clbm_get_band_rows: *nbands = the run's cluster
 * size (0 for a streaming run) and that many rows. */
int clbm_band_rows(const clbm_run_desc *run, int cluster_size, double gamma, int *rows);
int clbm_set_band_rows(clbm_ctx *ctx, int run, const int *rows, int nbands);
int clbm_get_band_rows(clbm_ctx *ctx, int run, int *rows, int *nbands);

/* Macroscopic fields of a clone's current pre-collision state, HOST arrays of
 * Dx*Dy values in the reference's node order y + Dy*x: rho, ux (shifted by
 * beta/(2 rho), as streamCollCompute.cpp:28 computes it) and uy -- what
 * write_fluid_vtk prints (src/lbm_src/write_vtk.cpp:8-53). */
int clbm_macro_fields(clbm_ctx *ctx, int run, int clone, double *rho,
                      double *ux, double *uy);

/* The random body-force field a clone used in the last interval, as FP64 in
 * the reference's map order y + Dy*x (Dx*Dy values; map may be NULL), and
 * the number of circulant-embedding eigenvalues below -1e-15 that were set to
 * zero (*negative, nullable; the reference flags them as an error,
 * generate_random_field.cpp:145-151). */
int clbm_get_field_map(clbm_ctx *ctx, int run, int clone, double *map,
                       int *negative);

/* ---- lineage reconstruction (post_processing/reconstruction.cpp:35-109) ----
 * clbm_enable_history(ctx, max_intervals), before the first interval, keeps
 * every interval's drag series and the labels of its clone step on the
 * device (max_intervals * clones * max_steps doubles).
 * clbm_reconstruct_lineages then traces each final slot j back through its
 * ancestors (slot_t = labels_t[slot_{t+1}]) and returns, for the n recorded
 * intervals (*nintervals), out[j][t*steps + s] = drag of j's ancestor in
 * interval t, step s, and ancestors[j][t] (either pointer may be NULL). */
int clbm_enable_history(clbm_ctx *ctx, int max_intervals);
int clbm_reconstruct_lineages(clbm_ctx *ctx, int run, int *nintervals,
                              double *out, int *ancestors);

/* ---- differentiation: adjoint of the interval-integrated drag ------------
 * J_j = dt * sum_{t<steps} (F_t*force_scale - force_shift) of every clone j
 * (the weight integral s_j of the sampler, pops driver :445-465), started
 * from the clones' current states S_0.  clbm_drag_fwd runs the forward in the
 * context's precision, keeping the post-collision populations every `every`
 * steps as checkpoints, and returns J (HOST array, all clones of all runs in
 * run order; nullable).  It does not change the sampler state; it needs no
 * pending clone step (run an interval first).  clbm_drag_bwd runs the
 * hand-written adjoint backwards, recomputing each checkpoint segment, and
 * leaves dJ/dS_0 on the device; clbm_get_drag_grad_aos_f64 returns one
 * clone's gradient in the reference AoS layout (FP64, 9*Dx*Dy values; zero
 * inside the square).  dJ/dS_0 is the gradient with respect to an additive
 * perturbation of the populations.  Runs with a random body-force field
 * (field_mode) step, forward and backward, under the fields of the last
 * interval (the ones clbm_get_field_map returns). */
int clbm_drag_fwd(clbm_ctx *ctx, int steps, int every, double *J);
int clbm_drag_bwd(clbm_ctx *ctx);
int clbm_get_drag_grad_aos_f64(clbm_ctx *ctx, int run, int clone, double *aos);

/* device error word (CLBM_DEV_* bits) accumulated since the last clear */
int clbm_error_word(clbm_ctx *ctx, unsigned *word, int clear);
/* ---- clones split over processes (one GPU each) ---------------------------
 * Replaces the MPI clone exchange of the pops driver
 * (src/mpi_LBM_GK_pops_perturb.cpp:650-699): clones in contiguous blocks of
 * nclones / nshards per shard; after a cloning step slot j takes the state of
 * slot labels[j] (labels[j] == j keeps it; a parent keeps its own state).
 * For shard `shard` the plan lists (global slots, peer shard) the copies it
 * sends, receives and does locally, each list in ascending destination slot
 * (both ends of a transfer see it at the same position).  Any list pointer
 * may be NULL (counts only); each holds at most nclones entries.  Host only:
 * no device is needed. */
typedef struct {
  int src_slot; /* global index of the parent slot */
  int dst_slot; /* global index of the slot that takes its state */
  int peer;     /* the other shard (this shard for local copies) */
} clbm_copy;
int clbm_shard_plan(const int *labels, int nclones, int nshards, int shard,
                    clbm_copy *sends, int *nsends, clbm_copy *recvs,
                    int *nrecvs, clbm_copy *locals, int *nlocals);

/* block until the context's stream is idle */
int clbm_sync(clbm_ctx *ctx);
/* the context's cudaStream_t */
void *clbm_stream(clbm_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
