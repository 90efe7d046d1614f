// gs_solve.cuh -- in-warp factor / solve / refine of one small symmetric
// system held in shared memory, shared by the kriging and Vecchia kernels.
//
// The matrix is packed lower-triangular (entry (i, j), j <= i, at
// i(i+1)/2 + j) in double-float.  Its FP32 hi parts are factored
// A = L D L^T without pivoting -- valid for a positive-definite covariance
// block bordered by drift rows (the Schur complement is negative definite) --
// and the solution is refined with residuals b - A x taken against the
// double-float entries in compensated FP32 (Ogita, Rump & Oishi, "Accurate
// sum and dot product", SIAM J. Sci. Comput. 26(6), 2005), accumulated in
// FP64.  Triangular numbers modulo 32 form a permutation of 0..31, so the
// column accesses of the packed layout are free of bank conflicts.
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
    c = df_add(c, df_mul(r, st.sill_df));
  }
  return c;
}

template <int D>
__device__ __forceinline__ df norm_df(const df* a, const df* b) {
  df q = df_make(0.0f, 0.0f);
#pragma unroll
  for (int d = 0; d < D; ++d) q = df_add(q, df_sqr(df_sub(a[d], b[d])));
  return df_sqrt(q);
}

template <int D>
__device__ __forceinline__ df norm0_df(const df* a) {
  df q = df_make(0.0f, 0.0f);
#pragma unroll
  for (int d = 0; d < D; ++d) q = df_add(q, df_sqr(a[d]));
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

// L D L^T w = w in place (unit-lower packed L, inverse pivots DI).
__device__ __forceinline__ void ldl_solve(const float* L, const float* DI, float* w, int N,
                                          int lane) {
  for (int k = 0; k < N - 1; ++k) {
    const float wk = w[k];
    for (int i = k + 1 + lane; i < N; i += 32) w[i] = fmaf(-L[pk(i, k)], wk, w[i]);
    __syncwarp();
  }
  for (int i = lane; i < N; i += 32) w[i] *= DI[i];
  __syncwarp();
  for (int k = N - 1; k > 0; --k) {
    const float wk = w[k];
    for (int i = lane; i < k; i += 32) w[i] = fmaf(-L[pk(k, i)], wk, w[i]);
    __syncwarp();
  }
}

}  // namespace gs
