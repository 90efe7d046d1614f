/*
 * geostat_oracle.h -- C interface of the FP64 CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a line-by-line restatement of
 * the reference's CPU algorithms (geostat-rs, crates/geostat-core) and is
 * used exclusively as the parity checker by tests/, by __graft_entry__.smoke()
 * and by bench.py's CPU-baseline / reference arm.  The product
 * (libgeostat_gb300.so) never links, loads or calls it.
 *
 * The struct layouts below are byte-identical to the product's public
 * structs in include/geostat_gb300.h so one ctypes definition serves both.
 */
#ifndef GEOSTAT_ORACLE_H
#define GEOSTAT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Model kinds (crates/geostat-core/src/variogram/model.rs:50-101). */
enum {
  OR_SPHERICAL = 0,
  OR_EXPONENTIAL = 1,
  OR_GAUSSIAN = 2,
  OR_MATERN15 = 3,
  OR_MATERN25 = 4,
  OR_CIRCULAR = 5,
  OR_STABLE = 6,
  OR_HOLE = 7,
  OR_WAVE = 8,
  OR_POWER = 9
};

/* Error codes mirror GeostatError (crates/geostat-core/src/error.rs:14-39). */
enum {
  OR_OK = 0,
  OR_INSUFFICIENT_DATA = 1,
  OR_DIMENSION_MISMATCH = 2,
  OR_SINGULAR_SYSTEM = 3,
  OR_INVALID_PARAMETER = 4,
  OR_NO_NEIGHBORS = 5,
  OR_DUPLICATE_POINTS = 6
};

typedef struct {
  int32_t kind;     /* OR_* kind */
  int32_t has_anis; /* 0: isotropic */
  double param;     /* Stable alpha / Power theta (unused otherwise) */
  double sill;
  double range;
  double azimuth_deg, ratio, ratio_z, dip_deg, rake_deg;
} or_structure;

typedef struct {
  double nugget;
  int32_t n_structures; /* <= 4 */
  int32_t pad_;
  or_structure s[4];
} or_model;

/* KrigingConfig (crates/geostat-core/src/kriging.rs:73-115); negative
 * integers and has_* == 0 encode Option::None. */
typedef struct {
  int64_t method; /* 0 simple, 1 ordinary, 2 universal, 3 external drift */
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
} or_kcfg;

const char* or_last_error(void);

/* model.rs:636 gamma_dh / model.rs:554 VariogramModel::new validation. */
int or_model_validate(const or_model* m);
double or_gamma_dh(const or_model* m, int dim, const double* dh);

/* linalg.rs: LU solve (A row-major n x n), Cholesky solve, ln|det|. */
int or_lu_solve(int64_t n, const double* a, const double* b, double* x);
int or_cholesky_solve(int64_t n, const double* a, const double* b, double* x);

/* search.rs: kd-tree k-nearest and brute force; returns the count. */
int64_t or_kdtree_knn(int dim, int64_t n, const double* coords, const double* target, int64_t k,
                      int has_radius, double radius, int64_t* out);
int64_t or_knn_brute(int dim, int64_t n, const double* coords, const double* target, int64_t k,
                     int has_radius, double radius, int64_t* out);
/* Incremental BucketGrid: inserts points 0..n-1 one at a time and, after
 * inserting point q_after[i], queries target q_target[i]; outputs are
 * written at out[i*k], counts at cnt[i]. */
int or_bucketgrid_queries(int dim, int64_t n, const double* coords, const double* bbox_min,
                          const double* bbox_max, int64_t expected, int64_t nq,
                          const int64_t* q_after, const double* q_target, int64_t k,
                          int has_radius, double radius, int64_t* out, int64_t* cnt,
                          int64_t* grid_dims);

/* data.rs:384 duplicate_coord_pair; returns 1 and (i, j) when found. */
int or_duplicate_pair(int dim, int64_t n, const double* coords, int64_t* i, int64_t* j);

/* grid.rs Grid2D/Grid3D centres. */
int or_grid_centers(int dim, const double* bmin, const double* bmax, const int64_t* ncell,
                    double* out);

/* kriging.rs: Kriging::{new,with_external_drift,with_measurement_error} +
 * predict_many / predict_many_with_drift.  ctor: 0 new, 1 external drift,
 * 2 measurement error.  Per-target status: 0 ok, else the error code
 * (the reference maps every per-target error to NaN).  nb_out (optional):
 * up to kcap neighbour indices per target in the reference's order.
 * boundary_ties (optional): number of targets whose k-th and (k+1)-th
 * candidates tie on squared distance (kd-tree tie order is
 * traversal-dependent in the reference). */
int or_krige(int dim, int64_t n, const double* coords, const double* values, const double* drift,
             const double* meas_err, int ctor, const or_model* model, const or_kcfg* cfg,
             int64_t nt, const double* targets, const double* tdrift, double* value,
             double* variance, double* lagrange, int8_t* status, int32_t* nb_out, int64_t kcap,
             int32_t* nb_count, int64_t* boundary_ties, int nthreads);

/* vecchia.rs */
int or_maxmin_order(int dim, int64_t n, const double* coords, int64_t* order);
int or_maxmin_order_brute(int dim, int64_t n, const double* coords, int64_t* order);
int or_vecchia_plan(int dim, int64_t n, const double* coords, int64_t m, const int64_t* order_in,
                    int64_t* order_out, int64_t* nb, int32_t* nb_count);
int or_vecchia_loglik_grouped(int dim, int64_t n, const double* coords, const double* values,
                              const or_model* model, int64_t m, const int64_t* order,
                              const int64_t* nb, const int32_t* nb_count, int64_t group_size,
                              double* ll);
int or_vecchia_loglik_plan(int dim, int64_t n, const double* coords, const double* values,
                           const or_model* model, int64_t m, const int64_t* order,
                           const int64_t* nb, const int32_t* nb_count, double* ll,
                           double* terms);
int or_vecchia_loglik(int dim, int64_t n, const double* coords, const double* values,
                      const or_model* model, int64_t m, const int64_t* order, double* ll);
int or_exact_loglik(int dim, int64_t n, const double* coords, const double* values,
                    const or_model* model, double* ll);
int or_vecchia_predict(int dim, int64_t n, const double* coords, const double* values,
                       const or_model* model, int64_t nt, const double* targets, int64_t m,
                       double* value, double* variance);
/* Vecchia MLE objective (vecchia.rs:999-1016) evaluated at x=(sqrt nugget,
 * ln psill, ln range) for a single isotropic structure of `kind`. */
int or_vecchia_mle_objective(int dim, int64_t n, const double* coords, const double* values,
                             int32_t kind, double param, int64_t m, const int64_t* order,
                             const int64_t* nb, const int32_t* nb_count, double range_max,
                             int64_t nx, const double* x, double* fx);
/* Start points of vecchia.rs:1021-1024 plus var0/extent/range_max. */
int or_vecchia_mle_setup(int dim, int64_t n, const double* coords, const double* values,
                         double* starts9, double* range_max);
/* Nelder-Mead multistart over the MLE objective (optim.rs:6-123). */
int or_vecchia_mle_nm(int dim, int64_t n, const double* coords, const double* values,
                      int32_t kind, double param, int64_t m, const int64_t* order_in,
                      int64_t nstarts, const double* starts, double step, int64_t max_iter,
                      double* x_out, double* f_out, int64_t* n_evals);

/* kriging.rs:674-779 Kriging::predict_block for nc blocks sharing offsets
 * (noff x dim); per-block status as or_krige. */
int or_krige_block(int dim, int64_t n, const double* coords, const double* values,
                   const double* meas_err, int ctor, const or_model* model, const or_kcfg* cfg,
                   int64_t nc, const double* centers, const double* offsets, int64_t noff,
                   double* value, double* variance, double* lagrange, int8_t* status);
/* validation.rs:298-328 spatial_block_assignment (fold index per point). */
int or_spatial_block_assignment(int dim, int64_t n, const double* coords, const int64_t* bpd,
                                int64_t* fold_of);
/* vecchia.rs:577-602 guinness_blocks: block ends k1[0 .. *nblocks). */
int or_guinness_blocks(int64_t n, int64_t m, const int64_t* order, const int64_t* nb,
                       const int32_t* nb_count, int64_t group_size, int64_t* k1,
                       int64_t* nblocks);
/* vecchia.rs:1181-1233 poly_basis (row-major n x p, p = or_poly_basis_terms)
 * and vecchia.rs:1246-1272 standardized_drift_basis (n x (1 + ncov)). */
int64_t or_poly_basis_terms(int dim, int32_t degree);
int or_poly_basis(int dim, int64_t n, const double* coords, int32_t degree, double* out);
int or_drift_basis(int64_t n, int64_t ncov, const double* drift, double* out);
/* vecchia.rs:1278-1457 REML log-likelihood on a plan given as arrays, with a
 * trend basis (row-major n x p); group_size <= 1 ungrouped. */
int or_vecchia_reml_loglik(int dim, int64_t n, const double* coords, const double* values,
                           const or_model* model, int64_t m, const int64_t* order,
                           const int64_t* nb, const int32_t* nb_count, const double* basis,
                           int64_t p, int64_t group_size, double* ll);
/* Nelder-Mead multistart fit: basis null = grouped ML (vecchia.rs:939-1081
 * with blocks), else REML (vecchia.rs:1572-1644). */
int or_vecchia_fit_nm(int dim, int64_t n, const double* coords, const double* values, int32_t kind,
                      int64_t m, const int64_t* order_in, const double* basis, int64_t p,
                      int64_t group_size, int64_t nstarts, const double* starts, double step,
                      int64_t max_iter, double* x_out, double* f_out, int64_t* n_evals);

/* optim.rs nelder_mead_multistart over a C callback (for driver parity). */
typedef double (*or_objective_fn)(const double* x, int64_t n, void* ctx);
/* vecchia.rs:353-389 g_and_dg; vecchia.rs:428-530 loglik_grad_inner on a plan
 * given as arrays; vecchia.rs:1018-1061 + optim.rs:207-289: the BFGS path of
 * mle_fit_with_plan (three reference starts, max_iter iterations). */
int or_g_and_dg(int32_t kind, double d, double* g, double* dg);
int or_vecchia_loglik_grad(int dim, int64_t n, const double* coords, const double* values,
                           int32_t kind, double nugget, double psill, double range, int64_t m,
                           const int64_t* order, const int64_t* nb, const int32_t* nb_count,
                           double* ll, double* grad3);
int or_vecchia_mle_bfgs(int dim, int64_t n, const double* coords, const double* values,
                        int32_t kind, int64_t m, const int64_t* order_in, int64_t max_iter,
                        double* x_out, double* f_out, int64_t* n_evals);
/* optim.rs:281-289 bfgs_multistart over host callbacks. */
typedef void (*or_gradient_fn)(const double* x, int64_t n, double* g, void* ctx);
int or_bfgs_multistart(or_objective_fn f, or_gradient_fn g, void* ctx, int64_t n, int64_t nstarts,
                       const double* starts, int64_t max_iter, double* x_out, double* f_out);
int or_nelder_mead_multistart(or_objective_fn f, void* ctx, int64_t n, int64_t nstarts,
                              const double* starts, double step, int64_t max_iter, double* x_out,
                              double* f_out);

/* rng.rs xoshiro256++ streams and the reference tests' field helpers. */
void or_rng_u64(uint64_t seed, int64_t count, uint64_t* out);
void or_rng_uniform(uint64_t seed, int64_t count, double* out);
void or_rng_normal(uint64_t seed, int64_t count, double* out);
void or_rng_draw(uint64_t seed, int64_t n_uniform, int64_t n_normal, double* out);
/* vecchia.rs:1941 `field(n, seed)` and tests/three_d.rs:12 `synthetic_3d`. */
void or_test_field_2d(int64_t n, uint64_t seed, double* coords, double* values);
void or_test_field_3d(int64_t n, uint64_t seed, double* coords, double* values);

#ifdef __cplusplus
}
#endif
#endif
