// gs_solve.cuh -- device helpers shared by the per-system kernels: packed
// lower-triangular indexing (entry (i, j), j <= i, at i(i+1)/2 + j), warp
// reductions, coordinate frames and double-float covariances.  Triangular
// numbers modulo 32 form a permutation of 0..31, so column accesses of the
// packed layout are free of shared-memory bank conflicts.
#pragma once

#include "gs_common.cuh"

namespace gs {

__device__ __forceinline__ int pk(int i, int j) { return ((i * (i + 1)) >> 1) + j; }

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_max_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_max_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Coordinate frames of a model: frame 0 is the identity, each anisotropic
// structure adds its own rotated/scaled frame.
struct Frames {
  int nf;
  int fid[GS_MAX_STRUCTURES];
};

__device__ __forceinline__ Frames frames_of(const DevModel& m) {
  Frames f;
  f.nf = 1;
  for (int s = 0; s < m.ns; ++s) f.fid[s] = m.s[s].aniso ? f.nf++ : 0;
  return f;
}

// Covariance in df from per-frame separation norms h[frame] (all > 0).
__device__ __forceinline__ df cov_from_h(const DevModel& m, const Frames& fr, const df* h,
                                         const ExpTable& tab, const DfConsts& k) {
  df c = df_make(0.0f, 0.0f);
  for (int s = 0; s < m.ns; ++s) {
    const DevStruct& st = m.s[s];
    df d = df_mul(h[fr.fid[s]], st.inv_range_df);
    df r = rho_df(st.kind, d, tab, k);
    c = df_add_fast(c, df_mul(r, st.sill_df));  // non-negative terms
  }
  return c;
}

// |a - b| in df.  Coordinates are target-relative (a few ranges at most), so
// the fast difference keeps ~2^-46 relative accuracy on the separation; the
// squares are non-negative, so their sum needs no extra renormalisation.
template <int D>
__device__ __forceinline__ df norm_df(const df* a, const df* b) {
  df q = df_sqr(df_add_fast(a[0], df_neg(b[0])));
#pragma unroll
  for (int d = 1; d < D; ++d) q = df_add_fast(q, df_sqr(df_add_fast(a[d], df_neg(b[d]))));
  return df_sqrt(q);
}

template <int D>
__device__ __forceinline__ df norm0_df(const df* a) {
  df q = df_sqr(a[0]);
#pragma unroll
  for (int d = 1; d < D; ++d) q = df_add_fast(q, df_sqr(a[d]));
  return df_sqrt(q);
}

// Frame coordinates of one point (identity frame in ud already): writes the
// transformed coordinates of every anisotropic structure's frame to
// V[(f * stride + i) * D + r] and the norms to h[f].
template <int D>
__device__ __forceinline__ void frame_coords(const DevModel& m, const Frames& fr, const df* ud,
                                             df* V, int stride, int i, df* h) {
#pragma unroll
  for (int d = 0; d < D; ++d) V[(0 * stride + i) * D + d] = ud[d];
  h[0] = norm0_df<D>(ud);
  for (int s = 0; s < m.ns; ++s) {
    if (!m.s[s].aniso) continue;
    const int f = fr.fid[s];
    df vv[3];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      df acc = df_make(0.0f, 0.0f);
#pragma unroll
      for (int c = 0; c < D; ++c) acc = df_add(acc, df_mul(m.s[s].rot_df[r * 3 + c], ud[c]));
      vv[r] = acc;
      V[(f * stride + i) * D + r] = acc;
    }
    h[f] = norm0_df<D>(vv);
  }
}

}  // namespace gs
