// gs_kriging_handle.h -- the predictor behind the opaque gs_kriging handle,
// shared by the C-ABI translation units.
#pragma once

#include <map>
#include <mutex>

#include "gs_common.cuh"
#include "gs_internal.h"
#include "gs_krige.cuh"
#include "gs_search.cuh"

namespace gs {
// Launch shape of the mixed solver: consecutive targets per system's run
// (longer runs share more matrix entries between neighbouring targets,
// shorter ones spread small calls over more SMs), warps per system for
// neighbourhoods of at most 32 points (bins 1: such systems go to the
// one-warp solver, bins 0: every system uses the two-warp solver) and
// systems per block (spc 1 or 2).
struct Tiles {
  int run = 64;
  int bins = 0;
  int spc = 1;
};
}  // namespace gs

struct gs_kriging {
  const gs_pointset* ps = nullptr;
  gs_kcfg cfg{};
  gs_model model{};
  gs::DevModel dm{};
  int p = 0;
  int nv = 0;
  double center[3] = {0, 0, 0};
  double scale = 1.0;
  double dmean[GS_MAX_KED_VARS] = {0};
  double dscale[GS_MAX_KED_VARS] = {0};
  double* d_drift = nullptr;
  double* d_err = nullptr;
  gs::df* d_basis_df = nullptr;  // p x n drift basis of the data points
  gs::df* d_err_df = nullptr;    // measurement errors as df
  bool use_tree = false;
  gs::SearchFrame frame{};
  gs::Grid grid;
  cudaStream_t stream = nullptr;
  int device = 0;  // the device the predictor's data and stream live on
  // autotuned launch shapes per size class of a call (floor(log2(nt))),
  // and a shape pinned by the caller (run 0: none)
  mutable std::mutex tiles_mu;
  mutable std::map<int, gs::Tiles> tiles;
  gs::Tiles pinned{0, 0, 1};
  // global neighbourhood: LU factors of the (n + p) system (row-major), the
  // solve's row order; lu_state 0 none, 1 factored, 2 singular
  double* d_lu = nullptr;
  int32_t* d_perm = nullptr;
  int lu_n = 0;
  int lu_state = 0;
  // its matrix-product form (mixed precision): R = A^{-T} split into hi / lo
  // floats, lambda = R z, arow = R e_n, prepared by the first mixed-precision
  // call that needs it (gemm_state 0: not yet, 1: ready, 2: no room for it)
  mutable std::mutex gemm_mu;
  mutable int gemm_state = 0;
  mutable float* d_rh = nullptr;
  mutable float* d_rl = nullptr;
  mutable double* d_lambda = nullptr;
  mutable double* d_arow = nullptr;
  ~gs_kriging() {
    cudaFree(d_lu);
    cudaFree(d_perm);
    cudaFree(d_rh);
    cudaFree(d_rl);
    cudaFree(d_lambda);
    cudaFree(d_arow);
    cudaFree(d_drift);
    cudaFree(d_err);
    cudaFree(d_basis_df);
    cudaFree(d_err_df);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace gs {
// The predictor's part of the kernel arguments (targets, neighbour lists and
// outputs are filled in by the caller).
KrigeArgs base_args(const gs_kriging* k);

// Search + solves for nt targets whose coordinates are already on the device
// (outputs in device memory); synchronises `stream` before returning.
int predict_device(const gs_kriging* k, int64_t nt, const double* tx, const double* ty,
                   const double* tz, const double* tdrift, double* value, double* variance,
                   double* lagrange, uint8_t* status, int precision, cudaStream_t stream);
}  // namespace gs
