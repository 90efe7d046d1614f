// gs_krige.cuh -- per-target kriging solves (K3 mixed, K3' FP64).
#pragma once

#include <stdint.h>

#include "gs_common.cuh"

namespace gs {

#define GS_MAX_KED_VARS 8
#define GS_MIXED_MAX_DRIFT 10

struct KrigeArgs {
  int dim;
  int method;     // GS_SIMPLE .. GS_EXTERNAL_DRIFT
  int p;          // number of drift terms (KrigingMethod::n_drift)
  int nv;         // external-drift variables
  int uk_degree;
  int min_nb;     // min_neighbors (1 when unset)
  int kout;       // neighbour slots per target
  int nmax;       // largest N = n + p in this launch (shared-memory sizing)
  double sk_mean;
  double center[3];
  double scale;
  double dmean[GS_MAX_KED_VARS];
  double dscale[GS_MAX_KED_VARS];
  const double* x;
  const double* y;
  const double* z;
  const double* val;
  const df* cdf;             // coordinates as df, axis-major (dim x n)
  const df* vdf;             // values as df
  const df* basis_df;        // p x n drift basis of the data points (df), or null
  const df* err_df;          // n measurement-error variances (df), or null
  int64_t n;                 // data points
  const double* meas_err;    // n or null
  const double* drift;       // n x nv raw covariates or null
  const double* tx;
  const double* ty;
  const double* tz;
  const double* tdrift;      // nt x nv or null
  const int32_t* nb;
  const int32_t* nbc;
  double* out_v;
  double* out_var;
  double* out_lag;           // may be null
  uint8_t* out_st;
  const int64_t* tlist;      // targets to process (null: 0..nt-1)
  int64_t ntl;               // number of them (an upper bound when ntl_dev is set)
  const int64_t* ntl_dev;    // the number on the device, read by the kernel, or null
  int run;                   // consecutive targets per block sequence (0: 64)
  int spc;                   // systems per block of the mixed solver (1 or 2; 0: 1)
  const int* route_fp64;     // when set and nonzero: flag every valid system
                             // for the FP64 re-solve without attempting it
  const double* boff;        // block kriging: nboff x dim discretisation offsets
  int nboff;                 // (FP64 kernel only; 0 = point kriging)
  const double* cbb;         // block kriging: the within-block covariance (device)
};

// Mixed-precision kernel for systems with n <= 64 neighbours and at most
// GS_MIXED_MAX_DRIFT drift terms.  Systems it cannot certify are marked in
// `flag` (1 = re-solve in FP64).
// force_rows: 0 picks the block size from the neighbour slots (32 or 64
// threads), 32 / 64 forces it (binned launches).
int krige_mixed_launch(const KrigeArgs& a, const DevModel& m, uint8_t* flag, int force_rows,
                       cudaStream_t stream);
// Routing for the rest of a call: *route = 1 when more than three quarters
// of the first n systems were flagged (the FP32 attempt then costs more
// than it saves), else 0.
int route_launch(const uint8_t* flag, int64_t n, int* route, cudaStream_t stream);
// FP64 re-solve of the flagged systems (bordered LDL^T, one system per
// warp); clears the flag of every system it solves.  Systems left flagged
// (near-singular, or beyond 64 neighbours) go to krige_fp64_launch.
// scratch: chol_scratch_doubles(scratch_warps) doubles (the grid is capped
// at scratch_warps warps; 16 warps per SM fill the device).
int krige_chol_launch(const KrigeArgs& a, const DevModel& m, uint8_t* flag, double* scratch,
                      int64_t scratch_warps, cudaStream_t stream);
int64_t chol_scratch_doubles(int64_t warps);
// Plain FP64 kernel, one system per thread (the reference's partial-pivoting
// LU; the FP64 build and the last re-solve tier).
// scratch must hold fp64_scratch_doubles(nmax, threads) doubles.
int krige_fp64_launch(const KrigeArgs& a, const DevModel& m, double* scratch, int64_t threads,
                      cudaStream_t stream);
int64_t fp64_scratch_doubles(int nmax, int64_t threads);
// Global neighbourhood (kriging.rs:396-406): build_lhs over all points and
// lu_factor on the device into A (N x N, row-major), pivots piv[N];
// *state = 1 factored, 2 singular (as lu_factor's error).  Synchronises.
int global_factor(const KrigeArgs& a, const DevModel& m, int N, double* A, int32_t* piv,
                  int* state, cudaStream_t stream);
// Per-target Lu::solve with the factors (perm: the row order after the
// pivots' swaps); scratch: 2 N doubles per warp, at most scratch_warps warps.
int global_solve_launch(const KrigeArgs& a, const DevModel& m, int N, const double* LU,
                        const int32_t* perm, int state, double* scratch, int64_t scratch_warps,
                        cudaStream_t stream);
int64_t fp64_threads_for(int nmax, int64_t budget_bytes);
// Matrix-product form of the factored global system (the mixed-precision
// predict path): at build, R (row j = A^{-1} e_j, from the LU factors) split
// into hi / lo floats Rh, Rl (N x N), lambda = R z and arow = R e_n (N
// doubles each); synchronises.  Per call, estimates and Lagrange
// multipliers as FP64 dot products with lambda and arow, variances
// C(0) - b^T R b through a double-float GEMM over tiles of targets.
int global_gemm_prepare(const KrigeArgs& a, int N, const double* LU, const int32_t* perm,
                        float* Rh, float* Rl, double* lambda, double* arow, cudaStream_t stream);
int global_gemm_launch(const KrigeArgs& a, const DevModel& m, int N, const float* Rh,
                       const float* Rl, const double* lambda, const double* arow,
                       cudaStream_t stream);


// Block kriging's within-block covariance (kriging.rs:742-756): the mean of
// C(u - v) over all discretisation pairs, with c0 - nugget for u = v; one
// thread, the reference's summation order.
int block_cbb_launch(int dim, const DevModel& m, const double* off, int noff, double nugget,
                     double* out, cudaStream_t stream);

// Grid2D / Grid3D cell centres (grid.rs:80-96, 188-203) on the device.
int grid_centers_launch(int dim, const double* bmin, const double* step, const int64_t* ncell,
                        double* x, double* y, double* z, cudaStream_t stream);

}  // namespace gs
