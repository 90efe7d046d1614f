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

// A block holds S systems side by side (R threads each); thread i of a
// system is rows_tid<R, S>() and its system within the block rows_sys<R, S>().
template <int R, int S>
__device__ __forceinline__ int rows_tid() {
  if constexpr (S == 1) return (int)threadIdx.x;
  else return (int)(threadIdx.x & (unsigned)(R - 1));
}
template <int R, int S>
__device__ __forceinline__ int rows_sys() {
  if constexpr (S == 1) return 0;
  else return (int)(threadIdx.x / (unsigned)R);
}

// Barrier over one system's threads: the warp for R = 32; for R = 64 the
// block's barrier with one system per block, else the named barrier
// 1 + (system in the block) over the system's two warps.
template <int R, int S>
__device__ __forceinline__ void rows_bar() {
  if constexpr (R == 32) {
    __syncwarp();
  } else if constexpr (S == 1) {
    __syncthreads();
  } else {
    static_assert(R == 64, "one or two warps per system");
    asm volatile("bar.sync %0, %1;" ::"r"(1 + rows_sys<R, S>()), "r"(R) : "memory");
  }
}

// Sum of K floats over the block; every thread receives the sums.  The
// per-warp partials are added in warp order (deterministic).
template <int R, int K, int S = 1>
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
      for (int k = 0; k < K; ++k) r[(rows_tid<R, S>() >> 5) * K + k] = v[k];
    }
    rows_bar<R, S>();
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

template <int R, int S = 1>
__device__ __forceinline__ float rows_max(float v, float* red, int& slot) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  if constexpr (R > 32) {
    constexpr int NW = R / 32;
    float* r = red + slot * NW;
    if ((threadIdx.x & 31) == 0) r[rows_tid<R, S>() >> 5] = v;
    rows_bar<R, S>();
    v = r[0];
#pragma unroll
    for (int w = 1; w < NW; ++w) v = fmaxf(v, r[w]);
    slot ^= 1;
  }
  return v;
}

// Double-float sum of K values over the block (compensated at every step).
template <int R, int K, int S = 1>
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
      for (int k = 0; k < K; ++k) r[(rows_tid<R, S>() >> 5) * K + k] = v[k];
    }
    rows_bar<R, S>();
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

// rows_sum_df of two values, as one packed double-float pair.
template <int R, int S = 1>
__device__ __forceinline__ dfp rows_sum_dfp(dfp v, df* red, int& slot) {
  v = warp_sum_dfp(v);
  if constexpr (R > 32) {
    constexpr int NW = R / 32;
    df* r = red + slot * NW * 2;
    if ((threadIdx.x & 31) == 0) {
      const int w = rows_tid<R, S>() >> 5;
      r[2 * w] = dp_first(v);
      r[2 * w + 1] = dp_second(v);
    }
    rows_bar<R, S>();
    v = dp_pack(r[0], r[1]);
#pragma unroll
    for (int w = 1; w < NW; ++w) v = dp_add(v, dp_pack(r[2 * w], r[2 * w + 1]));
    slot ^= 1;
  }
  return v;
}

// Element j of a register row stored as float4 quads (j compile-time after
// unrolling).  Quads keep each published row's 16-byte stores on aligned
// register quads, and their halves are the FP32x2 operand pairs.
template <int W4>
__device__ __forceinline__ float row_elt(const float4 (&t)[W4], int j) {
  const float4 q = t[j >> 2];
  return (j & 3) == 0 ? q.x : (j & 3) == 1 ? q.y : (j & 3) == 2 ? q.z : q.w;
}

// In-place sweep inverse of the register rows (4 * W4 columns as quads)
// over the pivots piv[0..npiv): afterwards the covariance block holds
// -C^{-1} with +2 on its diagonal (pivot rows) and the drift block holds
// C^{-1} F.
//
// Pivot k: thread k publishes its row with the pivot entry replaced by d - 1
// (d = a_kk, also stored after the row); every thread then applies
//     t[j] -= l * row_k[j]   for every column j,
// with l = a_ik / d (a_ik read from the published row by symmetry) and
// l = 1 - 1/d on thread k.  That single update is the sweep operator
// (a_ij -= a_ik a_kj / d, a_ik /= d, a_kj /= d) except on the pivot's own
// diagonal, which becomes 2 - 1/d instead of -1/d; later pivots change that
// entry linearly, so every swept diagonal ends exactly 2 too large.  Rows
// that are not pivots are identity rows and never change (their published
// columns are zero).  The update runs as packed FP32x2 FMAs (two columns per
// instruction).  The row buffer is double-buffered, so one barrier per pivot
// suffices.  Returns false (uniformly) when a pivot is not above tol.
template <int R, int W4, int S = 1>
__device__ __forceinline__ bool rows_sweep(float4 (&t)[W4], const int* piv, int npiv, float tol,
                                           float* rowbuf) {
  constexpr int W = 4 * W4;
  const int i = rows_tid<R, S>();
  for (int kk = 0; kk < npiv; ++kk) {
    const int k = piv[kk];
    float* rb = rowbuf + (kk & 1) * (W + 4);
    if (i == k) {
#pragma unroll
      for (int q = 0; q < W4; ++q) *reinterpret_cast<float4*>(rb + 4 * q) = t[q];
      const float d = rb[k];  // this thread's own store
      rb[k] = d - 1.0f;
      rb[W] = d;
    }
    rows_bar<R, S>();
    const float d = rb[W];
    if (!(fabsf(d) > tol)) return false;
    const float invd = __fdividef(1.0f, d);  // an approximate inverse suffices
    const float l = i == k ? 1.0f - invd : rb[i] * invd;
    const float2 nl = make_float2(-l, -l);
#pragma unroll
    for (int q = 0; q < W4; ++q) {
      const float4 r = *reinterpret_cast<const float4*>(rb + 4 * q);
      const float2 u0 = __ffma2_rn(nl, make_float2(r.x, r.y), make_float2(t[q].x, t[q].y));
      const float2 u1 = __ffma2_rn(nl, make_float2(r.z, r.w), make_float2(t[q].z, t[q].w));
      t[q] = make_float4(u0.x, u0.y, u1.x, u1.y);
    }
  }
  return true;
}

// y_i = (M^{-1} v)_i for a pivot row i (act) from the rows swept on M (v
// broadcast through shared memory, zero off the pivots); packed FP32x2
// products.
template <int R, int W4, int S = 1>
__device__ __forceinline__ float rows_cinv_apply(const float4 (&t)[W4], const float* v, bool act) {
  const int i = rows_tid<R, S>();
  float2 a0 = make_float2(0.0f, 0.0f), a1 = make_float2(0.0f, 0.0f);
#pragma unroll
  for (int q4 = 0; q4 < R / 4; ++q4) {
    const float4 q = *reinterpret_cast<const float4*>(v + 4 * q4);
    a0 = __ffma2_rn(make_float2(t[q4].x, t[q4].y), make_float2(q.x, q.y), a0);
    a1 = __ffma2_rn(make_float2(t[q4].z, t[q4].w), make_float2(q.z, q.w), a1);
  }
  const float s = (a0.x + a1.x) + (a0.y + a1.y);
  return act ? fmaf(2.0f, v[i], -s) : 0.0f;
}

// 64-bit masks of two predicates over the block's threads (bit i = thread
// i), identical in every thread.  sh: 4 words of shared scratch not read by
// anyone else until the next barrier after this call.
template <int R, int S = 1>
__device__ __forceinline__ void rows_ballot2(bool p0, bool p1, unsigned long long& m0,
                                             unsigned long long& m1, unsigned* sh) {
  const unsigned b0 = __ballot_sync(0xffffffffu, p0), b1 = __ballot_sync(0xffffffffu, p1);
  if constexpr (R == 32) {
    m0 = b0;
    m1 = b1;
  } else {
    static_assert(R == 64, "one or two warps");
    const int w = rows_tid<R, S>() >> 5;
    if ((threadIdx.x & 31) == 0) {
      sh[2 * w] = b0;
      sh[2 * w + 1] = b1;
    }
    rows_bar<R, S>();
    m0 = (unsigned long long)sh[0] | ((unsigned long long)sh[2] << 32);
    m1 = (unsigned long long)sh[1] | ((unsigned long long)sh[3] << 32);
  }
}

// Number of set bits of m below bit i.
__device__ __forceinline__ int rank_below(unsigned long long m, int i) {
  return __popcll(m & ((1ull << i) - 1ull));
}

}  // namespace gs
