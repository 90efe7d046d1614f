// gs_search.cuh -- device bucket grid (K1) and neighbour search (K2).
#pragma once

#include <stdint.h>

#include "gs_common.cuh"

namespace gs {

// Search-frame transform of KrigingConfig::anisotropic_search
// (kriging.rs:16-21 search_point -> model.rs:353-367 transform_vector).
struct SearchFrame {
  int aniso;
  double s, c, ratio;  // 2-D: sin/cos of the azimuth in radians, ratio
  double rot[9];       // 3-D: GSLIB setrot matrix
};

// Uniform bucket grid over the search-frame coordinates, points sorted by
// cell (stable in the original index).
struct GridDev {
  double origin[3];
  double inv_cell;
  double cell;
  int n[3];
  int64_t ncells;
  const double* sx;
  const double* sy;
  const double* sz;
  const uint32_t* sidx;    // original index of each sorted point
  const uint32_t* cstart;  // ncells + 1 offsets
  // FP32 copies of the sorted coordinates relative to the origin, for the
  // distance prefilter; ext[d] bounds |coordinate - origin| per axis.
  const float* fx;
  const float* fy;
  const float* fz;
  double ext[3];
  float extf[3];   // ext rounded up to FP32
  float cellf_lo;  // cell rounded down to FP32
};

struct SearchParams {
  int k;           // neighbours kept per buffer (kNN: k; octant: per-octant cap)
  int kout;        // output slots per target
  int octant;      // 1: GSLIB octant search
  int unbounded;   // 1: radius-only search, report overflow beyond kout
  int capb;        // buffer capacity (power of two >= k + 32)
  int has_radius;
  double r2;
  // Ranked mode (Vecchia): query t has rank rank0 + t and only candidates
  // whose grid payload (store rank) is below it are admitted; queries with
  // rank <= brute_below scan ranks [0, rank) directly from px/py/pz.
  int ranked;
  int64_t rank0;
  int64_t brute_below;
  const double* px;
  const double* py;
  const double* pz;
  // Cross-validation: when set, candidates j with excl_label[j] equal to the
  // target's target_label[t] do not exist for it (its own point for
  // leave-one-out, its fold for k-fold).
  const int32_t* excl_label;
  const int32_t* target_label;
};

// Owns the device buffers of one grid.
struct Grid {
  GridDev dev{};
  int dim = 2;
  int64_t n = 0;
  double* d_sx = nullptr;
  double* d_sy = nullptr;
  double* d_sz = nullptr;
  uint32_t* d_sidx = nullptr;
  uint32_t* d_cstart = nullptr;
  float* d_f = nullptr;  // 3 x n FP32 prefilter coordinates
  ~Grid();
};

// Builds the grid of `n` points (x, y, z device arrays, original frame) in
// the given search frame.  points_per_cell sets the cell size.
int grid_build(Grid* g, int dim, int64_t n, const double* x, const double* y, const double* z,
               const SearchFrame& frame, double points_per_cell, cudaStream_t stream);

// kNN / radius / octant search for nt targets (original-frame device
// arrays).  Writes kout indices per target (original indices, sorted by
// (squared distance, index), -1 padded) and the count (-1 on overflow of an
// unbounded radius search).
int search_launch(const Grid& g, const SearchFrame& frame, const SearchParams& p, int64_t nt,
                  const double* tx, const double* ty, const double* tz, int32_t* nb,
                  int32_t* nbc, cudaStream_t stream);

// Builds a grid whose payload is the store rank: point r of the store is
// (x[r], y[r], z[r]).  Used by the Vecchia predecessor searches.
int grid_build_ranked(Grid* g, int dim, int64_t n, const double* x, const double* y,
                      const double* z, double points_per_cell, cudaStream_t stream);

}  // namespace gs
