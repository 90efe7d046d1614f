// gs_rows.cuh -- block-level pieces of the register-row kriging solver: one
// system per block of R threads (R = 32: one warp, R = 64: two warps), thread
// i holding row i of the covariance block (R columns) and of the drift block
// (PC columns) in registers.
//
// Reductions over the block run as warp butterflies; with two warps the
// per-warp partials meet in shared memory.  Each reduction writes one of two
// alternating slots and ends with a barrier, so a slot is only rewritten after
// every thread has passed the barrier of the reduction that used the other
// slot -- i.e. after every thread has read it.
#pragma once

#include "gs_solve.cuh"

namespace gs {

template <int R>
__device__ __forceinline__ void rows_bar() {
  if constexpr (R == 32) __syncwarp();
  else __syncthreads();
}

// Sum of K floats over the block; every thread receives the sums.  The
// per-warp partials are added in warp order (deterministic).
template <int R, int K>
__device__ __forceinline__ void rows_sum(float (&v)[K], float* red, int& slot) {
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  if constexpr (R > 32) {
    constexpr int NW = R / 32;
    float* r = red + slot * NW * K;
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
      for (int k = 0; k < K; ++k) r[(threadIdx.x >> 5) * K + k] = v[k];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
      float s = r[k];
#pragma unroll
      for (int w = 1; w < NW; ++w) s += r[w * K + k];
      v[k] = s;
    }
    slot ^= 1;
  }
}

template <int R>
__device__ __forceinline__ float rows_max(float v, float* red, int& slot) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  if constexpr (R > 32) {
    constexpr int NW = R / 32;
    float* r = red + slot * NW;
    if ((threadIdx.x & 31) == 0) r[threadIdx.x >> 5] = v;
    __syncthreads();
    v = r[0];
#pragma unroll
    for (int w = 1; w < NW; ++w) v = fmaxf(v, r[w]);
    slot ^= 1;
  }
  return v;
}

// Double-float sum of K values over the block (compensated at every step).
template <int R, int K>
__device__ __forceinline__ void rows_sum_df(df (&v)[K], df* red, int& slot) {
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      df w;
      w.hi = __shfl_xor_sync(0xffffffffu, v[k].hi, o);
      w.lo = __shfl_xor_sync(0xffffffffu, v[k].lo, o);
      v[k] = df_add(v[k], w);
    }
  if constexpr (R > 32) {
    constexpr int NW = R / 32;
    df* r = red + slot * NW * K;
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
      for (int k = 0; k < K; ++k) r[(threadIdx.x >> 5) * K + k] = v[k];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
      df s = r[k];
#pragma unroll
      for (int w = 1; w < NW; ++w) s = df_add(s, r[w * K + k]);
      v[k] = s;
    }
    slot ^= 1;
  }
}

// In-place sweep inverse of the register rows: after pivots 0..n-1 the
// covariance block holds -C^{-1} with +2 on its diagonal (rows < n) and the
// drift block holds C^{-1} F.
//
// Pivot k: thread k publishes its row with the pivot entry replaced by d - 1
// (d = a_kk, also stored after the row); every thread then applies
//     t[j] -= l * row_k[j]   for every column j,
// with l = a_ik / d (a_ik read from the published row by symmetry) and
// l = 1 - 1/d on thread k.  That single update is the sweep operator
// (a_ij -= a_ik a_kj / d, a_ik /= d, a_kj /= d) except on the pivot's own
// diagonal, which becomes 2 - 1/d instead of -1/d; later pivots change that
// entry linearly, so every swept diagonal ends exactly 2 too large.  Rows
// beyond n are identity rows and never change (their published columns are
// zero).  The row buffer is double-buffered, so one barrier per pivot
// suffices.  Returns false (uniformly) when a pivot is not above tol.
template <int R, int W>
__device__ __forceinline__ bool rows_sweep(float (&t)[W], int n, float tol, float* rowbuf) {
  const int i = threadIdx.x;
  for (int k = 0; k < n; ++k) {
    float* rb = rowbuf + (k & 1) * (W + 4);
    if (i == k) {
#pragma unroll
      for (int j = 0; j < W; j += 4)
        *reinterpret_cast<float4*>(rb + j) = make_float4(t[j], t[j + 1], t[j + 2], t[j + 3]);
      const float d = rb[k];  // this thread's own store
      rb[k] = d - 1.0f;
      rb[W] = d;
    }
    rows_bar<R>();
    const float d = rb[W];
    if (!(fabsf(d) > tol)) return false;
    const float invd = __frcp_rn(d);
    const float l = i == k ? 1.0f - invd : rb[i] * invd;
#pragma unroll
    for (int j = 0; j < W; j += 4) {
      const float4 r = *reinterpret_cast<const float4*>(rb + j);
      t[j] = fmaf(-l, r.x, t[j]);
      t[j + 1] = fmaf(-l, r.y, t[j + 1]);
      t[j + 2] = fmaf(-l, r.z, t[j + 2]);
      t[j + 3] = fmaf(-l, r.w, t[j + 3]);
    }
  }
  return true;
}

// y_i = (C^{-1} v)_i for row i < n from the swept rows (v broadcast through
// shared memory, zero beyond n).
template <int R, int W>
__device__ __forceinline__ float rows_cinv_apply(const float (&t)[W], const float* v, int n) {
  const int i = threadIdx.x;
  float s = 0.0f;
#pragma unroll
  for (int j = 0; j < R; j += 4) {
    const float4 q = *reinterpret_cast<const float4*>(v + j);
    s = fmaf(t[j], q.x, s);
    s = fmaf(t[j + 1], q.y, s);
    s = fmaf(t[j + 2], q.z, s);
    s = fmaf(t[j + 3], q.w, s);
  }
  return i < n ? fmaf(2.0f, v[i], -s) : 0.0f;
}

}  // namespace gs
