/*
 * geostat_gb300.h -- C ABI of the GB300-native kriging / Vecchia library.
 *
 * Every entry point is plain C: pointers, sizes and status codes, no CUDA or
 * torch types (streams are passed as `void*` holding a cudaStream_t, NULL for
 * the handle's own stream).  Each declaration names the geostat-rs interface
 * it replaces (paths relative to the geostat-rs workspace); the Rust-side
 * binding lives behind a `cuda` cargo feature next to
 * crates/geostat-core/src/parallel.rs.
 *
 * Threading: handles are immutable after creation and may be used from
 * several host threads at once (each call takes its own stream); the only
 * mutable shared state is the per-thread last-error message.
 */
#ifndef GEOSTAT_GB300_H
#define GEOSTAT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GS_ABI_VERSION 2
#define GS_MAX_STRUCTURES 4
/* Largest conditioning set the mixed-precision kernel holds on chip, and the
 * largest neighbourhood (neighbours + drift terms) any GPU kernel accepts. */
#define GS_MIXED_MAX_NEIGHBORS 64
#define GS_MAX_SYSTEM 256

/* Return codes: 1..6 mirror GeostatError (crates/geostat-core/src/error.rs:14-39). */
enum {
  GS_OK = 0,
  GS_ERR_INSUFFICIENT_DATA = 1,
  GS_ERR_DIMENSION_MISMATCH = 2,
  GS_ERR_SINGULAR_SYSTEM = 3,
  GS_ERR_INVALID_PARAMETER = 4,
  GS_ERR_NO_NEIGHBORS = 5,
  GS_ERR_DUPLICATE_POINTS = 6,
  GS_ERR_CUDA = 100,
  GS_ERR_OUT_OF_MEMORY = 101,
  GS_ERR_IO = 102, /* file input/output (the CLI's anyhow errors) */
  GS_ERR_CANCELLED = 103 /* a serving request cancelled before it started */
};

/* ModelKind (crates/geostat-core/src/variogram/model.rs:50-101).  The CUDA
 * path evaluates the closed-form kinds 0..4; others are rejected with
 * GS_ERR_INVALID_PARAMETER so the caller keeps them on the generic path. */
enum {
  GS_KIND_SPHERICAL = 0,
  GS_KIND_EXPONENTIAL = 1,
  GS_KIND_GAUSSIAN = 2,
  GS_KIND_MATERN15 = 3,
  GS_KIND_MATERN25 = 4,
  GS_KIND_CIRCULAR = 5,
  GS_KIND_STABLE = 6,
  GS_KIND_HOLE = 7,
  GS_KIND_WAVE = 8,
  GS_KIND_POWER = 9
};

/* KrigingMethod (crates/geostat-core/src/kriging.rs:24-44). */
enum { GS_SIMPLE = 0, GS_ORDINARY = 1, GS_UNIVERSAL = 2, GS_EXTERNAL_DRIFT = 3 };

/* Arithmetic of the per-target solve. */
enum {
  GS_PREC_MIXED = 0, /* FP32 factorisation, double-float refinement, FP64 outputs */
  GS_PREC_FP64 = 1   /* plain FP64, one system per thread */
};

/* Per-target status byte.  Low bits: 0 or a GeostatError code (the
 * reference maps every per-target error to a NaN estimate,
 * kriging.rs:648-652).  GS_ST_FP64_RESOLVED is OR-ed in when the mixed
 * kernel handed the system to the FP64 solver (refinement stalled or a
 * pivot was too small). */
enum {
  GS_ST_OK = 0,
  GS_ST_INSUFFICIENT_DATA = 1,
  GS_ST_SINGULAR = 3,
  GS_ST_NO_NEIGHBORS = 5,
  GS_ST_INVALID_PARAMETER = 4, /* block grids: a method or model blocks do not support */
  GS_ST_CAPACITY = 7, /* neighbourhood larger than GS_MAX_SYSTEM */
  GS_ST_FP64_RESOLVED = 0x40
};

/* Structure / Anisotropy (model.rs:288-519); ratio/ratio_z/dip/rake are
 * read only when has_anis != 0. */
typedef struct {
  int32_t kind;
  int32_t has_anis;
  double param; /* Stable alpha / Power theta; unused by the CUDA path */
  double sill;
  double range;
  double azimuth_deg, ratio, ratio_z, dip_deg, rake_deg;
} gs_structure;

/* VariogramModel (model.rs:542-552). */
typedef struct {
  double nugget;
  int32_t n_structures;
  int32_t pad_;
  gs_structure s[GS_MAX_STRUCTURES];
} gs_model;

/* KrigingConfig (kriging.rs:73-115).  Negative integers and has_* == 0
 * encode Option::None. */
typedef struct {
  int64_t method;
  double sk_mean;
  int64_t uk_degree;
  int64_t ked_nvars;
  int64_t max_neighbors;
  int64_t min_neighbors;
  int64_t max_per_octant;
  int64_t has_search_radius;
  double search_radius;
  int64_t has_anisotropic_search;
  double search_azimuth_deg, search_ratio, search_ratio_z, search_dip_deg, search_rake_deg;
} gs_kcfg;

typedef struct gs_pointset gs_pointset;
typedef struct gs_kriging gs_kriging;
typedef struct gs_vecchia_plan gs_vecchia_plan;

/* Message of the last failing call on this host thread. */
const char* gs_last_error(void);
int gs_abi_version(void);

/* PointSet::from_xyz / from_xyzv + PointSet::new validation
 * (crates/geostat-core/src/data.rs:15-83).  Copies coordinates and values
 * into device memory; z is ignored when dim == 2. */
int gs_pointset_create(int dim, int64_t n, const double* x, const double* y, const double* z,
                       const double* values, gs_pointset** out);
void gs_pointset_destroy(gs_pointset* ps);
/* PointSet::duplicate_pair (data.rs:171-173, 384-397): 1 and (i, j) when
 * two points share coordinates, else 0. */
int gs_pointset_duplicate_pair(const gs_pointset* ps, int64_t* i, int64_t* j);

/* Kriging::new / with_external_drift / with_measurement_error
 * (kriging.rs:166-260) including Kriging::build's validation
 * (kriging.rs:262-340).  drift is n x ked_nvars row-major; errors has n
 * entries.  The device bucket grid for the search frame is built here. */
int gs_kriging_new(const gs_pointset* ps, const gs_model* model, const gs_kcfg* cfg,
                   gs_kriging** out);
int gs_kriging_with_external_drift(const gs_pointset* ps, const gs_model* model,
                                   const gs_kcfg* cfg, const double* drift, gs_kriging** out);
int gs_kriging_with_measurement_error(const gs_pointset* ps, const gs_model* model,
                                      const gs_kcfg* cfg, const double* errors,
                                      gs_kriging** out);
void gs_kriging_destroy(gs_kriging* k);

/* Kriging::predict_many / predict_many_with_drift (kriging.rs:648-672):
 * host buffers in and out (copied inside the call).  tz ignored in 2-D;
 * tdrift is nt x ked_nvars (external drift only).  lagrange and status may
 * be NULL.  Failed targets get NaN value/variance as in the reference. */
int gs_kriging_predict_many(const gs_kriging* k, int64_t nt, const double* tx, const double* ty,
                            const double* tz, const double* tdrift, double* value,
                            double* variance, double* lagrange, uint8_t* status, int precision,
                            void* stream);
/* Same, with every buffer already in device memory (no host copies). */
int gs_kriging_predict_many_device(const gs_kriging* k, int64_t nt, const double* tx,
                                   const double* ty, const double* tz, const double* tdrift,
                                   double* value, double* variance, double* lagrange,
                                   uint8_t* status, int precision, void* stream);
/* Same as gs_kriging_predict_many_device, but the call only enqueues its
 * work on `stream` (NULL: the predictor's stream) and never waits for the
 * device: no phase timings and no re-solve count are recorded.  Targets whose
 * double-float refinement fails are re-solved in FP64 with the length of
 * their list read on the device, so the whole pass can be captured into a
 * CUDA graph (stream capture) and replayed; its temporary buffers are
 * stream-ordered allocations.  Make one ordinary call before capturing
 * (it sets up constant tables and kernel attributes).  No counterpart in the
 * reference: the batching entry of predict_many for serving loops. */
int gs_kriging_predict_many_async(const gs_kriging* k, int64_t nt, const double* tx,
                                  const double* ty, const double* tz, const double* tdrift,
                                  double* value, double* variance, double* lagrange,
                                  uint8_t* status, int precision, void* stream);
/* Cross-validation of a built predictor over its own data points
 * (validation.rs:136-253): nfolds = 0 is leave_one_out (each point predicted
 * from all the others), nfolds = k >= 2 is k_fold with the reference's seeded
 * fold assignment (each fold predicted from the other folds).  Every point's
 * estimate and variance are written (status may be NULL); as in the reference
 * the call fails -- with the error of the first failing point -- if any
 * prediction fails.  Neighbour sets are those of a predictor built on the
 * remaining points; drift bases keep the full data's normalisation, which
 * changes estimates and variances only by rounding.  Errors: fewer than 3
 * points (InsufficientData), k outside [2, n] (InvalidParameter). */
int gs_kriging_cross_validate(const gs_kriging* k, int64_t nfolds, uint64_t seed,
                              double* predicted, double* variance, uint8_t* status, int precision);
/* block_cv (validation.rs:348-374): labels from spatial_block_assignment
 * (validation.rs:298-328, a blocks_per_dim[0] x ... grid over the bounding
 * box, dimension 0 fastest), each point predicted from the points outside
 * its block, otherwise as gs_kriging_cross_validate.  Errors: fewer than 3
 * points (InsufficientData), an entry of 0 or fewer than 2 blocks in all
 * (InvalidParameter). */
int gs_kriging_block_cv(const gs_kriging* k, const int64_t* blocks_per_dim, double* predicted,
                        double* variance, uint8_t* status, int precision);
/* Launch shapes of the mixed solver (no counterpart in the reference).  The
 * first call of at least 65,536 targets on a predictor times the candidate
 * shapes -- runs of 16/32/64/128 consecutive targets per system; warps per
 * system for neighbourhoods of at most 32 points (bins 1: uneven
 * neighbourhoods split onto the one-warp and two-warp solvers, bins 0: every
 * system on the two-warp solver); one or two systems per block -- on its
 * first 131,072 targets and keeps the fastest for every later call of at
 * least 65,536 targets; smaller and asynchronous calls before that use a
 * default.  A tuned shape is also kept for the process under the systems'
 * shape (device, dimension, neighbour slots, drift terms, nested structures,
 * binning, cross-validation or not): a later predictor of the same shape
 * takes it on its first call instead of timing the candidates again.
 * Results of different shapes agree within the parity tolerance (the order
 * of roundings differs), and a predictor's results are reproducible once its
 * shapes are fixed.
 * gs_kriging_set_tiles pins one shape for every call (run a power of two in
 * [1, 1024], bins 0/1, systems_per_block 1/2; run 0 unpins).
 * gs_kriging_tiles reports the shape this predictor has fixed for calls
 * with nt targets: tuned = 0 none yet (its first call may still take one
 * kept for the process), 1 tuned, 2 pinned. */
int gs_kriging_set_tiles(gs_kriging* k, int run, int bins, int systems_per_block);
int gs_kriging_tiles(const gs_kriging* k, int64_t nt, int* run, int* bins,
                     int* systems_per_block, int* tuned);
/* Allocation-free FP64 prediction (no counterpart in the reference).  The
 * same results as gs_kriging_predict_many_device with GS_PREC_FP64, for
 * callers that may not allocate device memory while they predict: the
 * neighbour lists and FP64 scratch live in one static device array of
 * GS_NOALLOC_SCRATCH_BYTES per device.  At most GS_NOALLOC_MAX_TARGETS
 * targets per call (more: GS_ERR_INVALID_PARAMETER).  All pointers are device
 * memory; the call returns once its kernels are enqueued on `stream` (NULL:
 * the predictor's stream).  The first call on a device sets up the array's
 * address; make it before any section that cannot afford set-up work.  Calls
 * whose work overlaps in time on one device (other streams, unordered host
 * threads) share the array and race; calls ordered on one stream are safe. */
#define GS_NOALLOC_SCRATCH_BYTES (64ll << 20)
#define GS_NOALLOC_MAX_TARGETS 16384
int gs_kriging_predict_fp64_noalloc(const gs_kriging* k, int64_t nt, const double* tx,
                                    const double* ty, const double* tz, const double* tdrift,
                                    double* value, double* variance, double* lagrange,
                                    uint8_t* status, void* stream);
/* Kriging::predict_grid (kriging.rs:783-786) for Grid2D / Grid3D cell
 * centres (grid.rs:80-96, 188-203), generated on the device. */
int gs_kriging_predict_grid(const gs_kriging* k, const double* bbox_min, const double* bbox_max,
                            const int64_t* ncell, double* value, double* variance,
                            uint8_t* status, int precision, void* stream);
/* block_offsets (kriging.rs:815-838): out receives n[0] * n[1] offsets
 * (x, y pairs, x fastest) of the cell centres of a block of `size`. */
int gs_block_offsets(const double* size, const int64_t* n, double* out);
/* Kriging::predict_block (kriging.rs:674-779) for nb blocks sharing one
 * discretisation (offsets: noff x dim, row-major); simple and ordinary
 * kriging, FP64; host buffers.  A per-block failure is NaN with its
 * status; lagrange and status may be NULL. */
int gs_kriging_predict_block(const gs_kriging* k, int64_t nb, const double* cx, const double* cy,
                             const double* cz, const double* offsets, int64_t noff, double* value,
                             double* variance, double* lagrange, uint8_t* status, void* stream);
/* Kriging::predict_block_grid (kriging.rs:787-805), 2-D grids: one block of
 * block_size (discretised by block_offsets(block_size, discr)) per cell. */
int gs_kriging_predict_block_grid(const gs_kriging* k, const double* bbox_min,
                                  const double* bbox_max, const int64_t* ncell,
                                  const double* block_size, const int64_t* discr, double* value,
                                  double* variance, uint8_t* status, void* stream);
/* Kriging::neighbors (kriging.rs:441-490): the conditioning indices the
 * path uses, in the reference's (squared distance, index) order; host
 * buffers, kcap slots per target, -1 padded.  count may be NULL. */
int gs_kriging_neighbors(const gs_kriging* k, int64_t nt, const double* tx, const double* ty,
                         const double* tz, int64_t kcap, int32_t* idx, int32_t* count,
                         void* stream);

/* vecchia::maxmin_order (crates/geostat-core/src/vecchia.rs:144-215), on
 * the host as in the reference: the same order (first the point nearest the
 * centroid, then the largest squared distance to the selected points, ties
 * to the larger index), found by an exact eager search instead of the
 * reference's lazily refreshed heap.  Non-finite coordinates (which point
 * sets reject) still give a permutation. */
int gs_maxmin_order(int dim, int64_t n, const double* x, const double* y, const double* z,
                    int64_t* order);
/* vecchia_plan (vecchia.rs:232-282): order == NULL uses maxmin_order; the
 * predecessor search runs on the device. */
int gs_vecchia_plan_create(const gs_pointset* ps, int64_t m, const int64_t* order,
                           gs_vecchia_plan** out);
/* Copies the plan out: order[n], neighbours[n*m] (-1 padded), count[n]. */
int gs_vecchia_plan_get(const gs_vecchia_plan* plan, int64_t* order, int64_t* neighbours,
                        int32_t* count);
void gs_vecchia_plan_destroy(gs_vecchia_plan* plan);
/* loglik_with_plan (vecchia.rs:285-336) for ncand parameter candidates in
 * one launch (the batched Nelder-Mead objective).  status[c] is 0 or a
 * GeostatError code (a singular conditioning system). */
int gs_vecchia_loglik_batch(const gs_vecchia_plan* plan, int64_t ncand, const gs_model* models,
                            double* loglik, int32_t* status, int precision, void* stream);
/* The terms of loglik_with_plan's per-point loop (vecchia.rs:285-336) for
 * the ordered positions [lo, hi) only, summed per candidate: one shard of
 * the likelihood when the points are split across GPUs.  Position k is the
 * k-th point of the plan's max-min order (position 0 contributes the
 * unconditional N(0, sill) term).  Each range's sum is a fixed-order tree
 * over 8192-position chunks starting at lo, so it does not depend on
 * scheduling; sums over consecutive ranges covering [0, n), added in range
 * order, equal gs_vecchia_loglik_batch's total up to re-association
 * (relative differences near 1e-16).  lo = hi gives 0; a range outside
 * [0, n) is InvalidParameter. */
int gs_vecchia_loglik_batch_range(const gs_vecchia_plan* plan, int64_t lo, int64_t hi,
                                  int64_t ncand, const gs_model* models, double* loglik,
                                  int32_t* status, int precision, void* stream);
/* loglik_with_plan_grouped (vecchia.rs:604-668, Guinness 2018 grouping) for
 * ncand candidates: blocks of up to group_size consecutive ordered points
 * (guinness_blocks, vecchia.rs:570-602) conditioned jointly on the union of
 * their predecessor sets, one FP64 factorisation per block and candidate.
 * group_size <= 1 is gs_vecchia_loglik_batch.  The blocks of a group size
 * are built once per plan.  A joint set too large for one shared-memory
 * frame (about 190 points with its data rows): InvalidParameter. */
int gs_vecchia_loglik_grouped_batch(const gs_vecchia_plan* plan, int64_t ncand,
                                    const gs_model* models, int64_t group_size, double* loglik,
                                    int32_t* status, void* stream);
/* Vecchia REML log-likelihood (reml_loglik_with_plan, vecchia.rs:1278-1357,
 * for group_size <= 1; reml_loglik_with_blocks, vecchia.rs:1366-1457,
 * otherwise) for ncand candidates: the mean is a GLS trend over the basis of
 * vecchia_reml (drift NULL: poly_basis of drift_degree, vecchia.rs:1199-1233)
 * or of vecchia_reml_drift (drift: plan's n x ncov covariates, row-major;
 * standardized_drift_basis, vecchia.rs:1246-1272).  Per-block FP64 sums on
 * the device; the p x p GLS solve on the host. */
int gs_vecchia_reml_loglik_batch(const gs_vecchia_plan* plan, int64_t ncand, const gs_model* models,
                                 int32_t drift_degree, const double* drift, int64_t ncov,
                                 int64_t group_size, double* loglik, int32_t* status,
                                 void* stream);
/* vecchia_loglik (vecchia.rs:874-884). */
int gs_vecchia_loglik(const gs_pointset* ps, const gs_model* model, int64_t m,
                      const int64_t* order, double* loglik);
/* loglik_grad_with_plan (vecchia.rs:416-530): log-likelihood and its
 * gradient with respect to (nugget, psill, range), grad[c * 3 + q], for
 * ncand single-structure isotropic models of the closed-form kinds
 * (g_and_dg, vecchia.rs:353-389) in one launch.  status[c] is 0, a singular
 * conditioning system, or GS_ERR_INVALID_PARAMETER for a model without a
 * closed-form gradient. */
int gs_vecchia_loglik_grad_batch(const gs_vecchia_plan* plan, int64_t ncand,
                                 const gs_model* models, double* loglik, double* grad,
                                 int32_t* status, int precision, void* stream);
/* vecchia_mle (vecchia.rs:921-1081 mle_fit_with_plan): the reference's fit
 * -- its three starts, BFGS (optim.rs:207-289, 200 iterations) with the
 * analytical gradient for the closed-form kinds, which are all the kinds the
 * CUDA path evaluates.  The three starts advance in lock-step: each round's
 * objective requests go to the device in one gs_vecchia_loglik_batch launch
 * and its gradient requests in one gs_vecchia_loglik_grad_batch launch.
 * out_x receives the optimum in x = (sqrt nugget, ln psill, ln range). */
int gs_vecchia_mle(const gs_pointset* ps, int32_t kind, int64_t m, const int64_t* order,
                   gs_model* out_model, double* out_loglik, double* out_x, int64_t* n_evals);
/* Multi-start Nelder-Mead fit (the reference's gradient-free path,
 * optim.rs:6-123, step and max_iter as given) with every start's pending
 * simplex evaluations batched into one launch per round -- the form for
 * many starts.  starts (nstarts x 3, in x) may be NULL: nstarts <= 3 gives
 * the reference's three starts, more a deterministic spread. */
int gs_vecchia_mle_nm(const gs_pointset* ps, int32_t kind, int64_t m, const int64_t* order,
                      int64_t nstarts, const double* starts, double step, int64_t max_iter,
                      gs_model* out_model, double* out_loglik, double* out_x, int64_t* n_evals);
/* Batched objective launches (rounds) of the last lock-step Nelder-Mead fit
 * on this host thread (gs_vecchia_mle_nm and the grouped / REML fits). */
int64_t gs_last_fit_rounds(void);
/* Diagnostics of the last mixed Vecchia likelihood evaluation on this host
 * thread: out2[0] = (candidate, point) systems accepted when their
 * double-float refinement reached its noise floor (corrections at most
 * 1e-10 of |w|), out2[1] = systems refined with FP64 residuals.  Systems
 * re-solved by the FP64 kernel are gs_last_fallbacks(). */
void gs_last_vecchia_tiers(int64_t* out2);
/* vecchia_mle_grouped (vecchia.rs:939-950): group_size <= 1 is
 * gs_vecchia_mle; otherwise Nelder-Mead (step 0.3, 2000 iterations) from
 * the reference's three starts over the grouped likelihood, each round's
 * simplex points batched into one launch. */
int gs_vecchia_mle_grouped(const gs_pointset* ps, int32_t kind, int64_t m, const int64_t* order,
                           int64_t group_size, gs_model* out_model, double* out_loglik,
                           double* out_x, int64_t* n_evals);
/* vecchia_reml / vecchia_reml_grouped (vecchia.rs:1460-1493,
 * reml_fit_with_basis 1572-1644): polynomial trend of drift_degree.
 * InsufficientData when n <= p + 1. */
int gs_vecchia_reml(const gs_pointset* ps, int32_t kind, int64_t m, int32_t drift_degree,
                    const int64_t* order, int64_t group_size, gs_model* out_model,
                    double* out_loglik, double* out_x, int64_t* n_evals);
/* vecchia_reml_drift / vecchia_reml_drift_grouped (vecchia.rs:1500-1568):
 * drift is n_rows x ncov, row-major; n_rows != n: DimensionMismatch, ncov
 * == 0: InvalidParameter. */
int gs_vecchia_reml_drift(const gs_pointset* ps, int32_t kind, int64_t m, const double* drift,
                          int64_t n_rows, int64_t ncov, const int64_t* order, int64_t group_size,
                          gs_model* out_model, double* out_loglik, double* out_x,
                          int64_t* n_evals);
/* vecchia_predict (vecchia.rs:748-866): level-scheduled on the device. */
int gs_vecchia_predict(const gs_pointset* ps, const gs_model* model, int64_t nt,
                       const double* tx, const double* ty, const double* tz, int64_t m,
                       double* value, double* variance);

/* optim::nelder_mead_multistart (crates/geostat-core/src/optim.rs:6-123)
 * over a host callback: the same state machine gs_vecchia_mle_nm drives with
 * batched device evaluations, exposed for driver parity checks. */
typedef double (*gs_objective_fn)(const double* x, int64_t n, void* ctx);
int gs_nelder_mead_multistart(gs_objective_fn f, void* ctx, int64_t n, int64_t nstarts,
                              const double* starts, double step, int64_t max_iter, double* x_out,
                              double* f_out);

/* Serving loop (no counterpart in the reference, which serves one call at a
 * time): data sets stay resident as built predictors and Vecchia plans;
 * callers on any thread submit prediction and log-likelihood requests;
 * `executors` threads, each with its own stream, take pending requests once
 * device memory admits them -- their bytes within mem_budget_bytes and within
 * the device's current headroom (free memory plus what the stream-ordered
 * pool holds unused, less 512 MiB) -- coalesce every pending request of the
 * same data set and kind into the same launch, and scatter the results.
 * Size-aware admission: predictions of 131,072 targets or more are large;
 * executor 0 serves large requests in arrival order (and small ones when no
 * large request waits), the other executors serve small requests only, so a
 * small request never waits behind a large one.  A request whose device
 * bytes exceed mem_budget_bytes is refused at submission
 * (GS_ERR_OUT_OF_MEMORY).  Host buffers of a request must stay valid until
 * gs_server_wait returns for it; every request is waited for exactly once.
 * gs_server_cancel removes a request that has not started (its wait then
 * returns GS_ERR_CANCELLED); a running or finished request cannot be
 * cancelled (GS_ERR_INVALID_PARAMETER).
 * gs_server_stats reports the median and 99th-percentile submit-to-finish
 * latency of the completed requests and the number of launches formed. */
typedef struct gs_server gs_server;
int gs_server_create(int64_t mem_budget_bytes, int32_t executors, gs_server** out);
int gs_server_add_kriging(gs_server* s, const gs_kriging* k, int32_t* dataset);
int gs_server_add_vecchia(gs_server* s, const gs_vecchia_plan* plan, int32_t* dataset);
int gs_server_submit_predict(gs_server* s, int32_t dataset, int64_t nt, const double* tx,
                             const double* ty, const double* tz, double* value, double* variance,
                             uint8_t* status, int64_t* request_id);
int gs_server_submit_loglik(gs_server* s, int32_t dataset, const gs_model* model, double* loglik,
                            int32_t* status, int64_t* request_id);
/* Precision of the launches formed from now on (GS_PREC_MIXED by default;
 * GS_PREC_FP64 serves the same requests through the plain FP64 build). */
int gs_server_set_precision(gs_server* s, int precision);
int gs_server_cancel(gs_server* s, int64_t request_id);
int gs_server_wait(gs_server* s, int64_t request_id, double* latency_ms);
int gs_server_stats(gs_server* s, double* p50_ms, double* p99_ms, int64_t* completed,
                    int64_t* batches);
void gs_server_destroy(gs_server* s);

/* Seeded xoshiro256++ streams (crates/geostat-core/src/rng.rs): uniforms in
 * [0, 1) and standard normals, the generator behind seeded k-fold
 * assignments. */
void gs_rng_uniform(uint64_t seed, int64_t count, double* out);
void gs_rng_normal(uint64_t seed, int64_t count, double* out);

/* Timing of the last gs_kriging_predict_* or Vecchia log-likelihood call on
 * this host thread (ms of device time per phase, measured with CUDA events on
 * the call's stream): [0] search, [1] mixed solve, [2] FP64 re-solve,
 * [3] whole call. */
int gs_last_timings(double* ms4);
/* Systems the last gs_kriging_predict_* or Vecchia log-likelihood call on
 * this host thread solved with the FP64 kernels (mixed-precision systems
 * the refinement could not certify, or all of them at GS_PREC_FP64). */
int64_t gs_last_fallbacks(void);
/* Of those, the systems of the last gs_kriging_predict_* call on this host
 * thread that went on from the FP64 LDL^T re-solve to the partial-pivoting
 * LU (near-singular systems, more than 64 neighbours; all of them at
 * GS_PREC_FP64; 0 after a Vecchia call). */
int64_t gs_last_lu_resolves(void);

/* Diagnostics (no reference counterpart): the number of kernels this library
 * has launched since it was loaded, and the number of device allocations it
 * has made (cudaMalloc and stream-ordered allocations alike). */
int64_t gs_launch_count(void);
int64_t gs_debug_device_allocations(void);
/* Failure injection for tests (host side; no device fault): the next
 * `count` stream-ordered allocations the library makes fail as if the device
 * were out of memory (the calls return GS_ERR_OUT_OF_MEMORY); 0 ends it. */
int gs_debug_refuse_allocations(int64_t count);

/* CSV input and output (crates/geostat-cli/src/io_utils.rs), host only.
 * gs_csv_read reads the named numeric columns of a CSV file (header row,
 * csv crate 1.4.0 quoting) into a table, skipping rows where a requested
 * field is empty, "na", "nan" or not a number (io_utils.rs:12-18, 37-75);
 * a missing column is InvalidParameter naming the available ones, a record
 * whose field count differs from the header's is GS_ERR_IO.  nthreads <= 0
 * uses the host's threads.  gs_csv_write writes `header` then nrows rows of
 * ncols columns, each number as Rust's Display for f64 prints it (shortest
 * round-trip digits, no exponent, NaN / inf / -inf). */
typedef struct gs_csv_table gs_csv_table;
int gs_csv_read(const char* path, const char* const* cols, int ncols, int nthreads,
                gs_csv_table** out);
int gs_csv_table_info(const gs_csv_table* t, int64_t* rows, int64_t* skipped);
int gs_csv_table_copy(const gs_csv_table* t, double* out); /* rows x ncols, row-major */
void gs_csv_table_destroy(gs_csv_table* t);
int gs_csv_write(const char* path, const char* header, int ncols, const double* const* columns,
                 int64_t nrows, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
