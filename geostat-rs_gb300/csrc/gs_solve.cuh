// gs_solve.cuh -- device helpers shared by the per-system kernels: packed
// lower-triangular indexing (entry (i, j), j <= i, at i(i+1)/2 + j), warp
// reductions, coordinate frames and double-float covariances.  Triangular
// numbers modulo 32 form a permutation of 0..31, so column accesses of the
// packed layout are free of shared-memory bank conflicts.
#pragma once

#include "gs_common.cuh"
#include "gs_pair.cuh"

namespace gs {

__device__ __forceinline__ int pk(int i, int j) { return ((i * (i + 1)) >> 1) + j; }

// Exact coordinate coincidence (reference: gamma(0) = 0 only when every
// separation component is exactly zero, -0 == +0), on the 64-bit patterns.
__device__ __forceinline__ bool same_double(double a, double b) {
  const unsigned long long x = (unsigned long long)__double_as_longlong(a);
  const unsigned long long y = (unsigned long long)__double_as_longlong(b);
  return x == y || ((x | y) << 1) == 0ull;
}

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

// Covariance of one structure at separation norm h (> 0), df.
__device__ __forceinline__ df cov_struct(const DevStruct& st, df h, const ExpTable& tab,
                                         const DfConsts& k) {
  const df d = df_mul(h, st.inv_range_df);
  return df_mul(rho_df(st.kind, d, tab, k), st.sill_df);
}

// Covariance from a single norm shared by every (isotropic) structure.
__device__ __forceinline__ df cov_from_norm(const DevModel& m, df h, const ExpTable& tab,
                                            const DfConsts& k) {
  df c = df_make(0.0f, 0.0f);
#pragma unroll 1
  for (int s = 0; s < m.ns; ++s) c = df_add_fast(c, cov_struct(m.s[s], h, tab, k));  // >= 0 terms
  return c;
}

// Frame coordinates are stored structure-of-arrays: coordinate d of point i in
// frame f at V[(f * D + d) * stride + i].
template <int D>
__device__ __forceinline__ df vget(const df* V, int stride, int f, int d, int i) {
  return V[(f * D + d) * stride + i];
}

// |a - b| in df for points i, j of frame f.  Coordinates are target-relative
// (a few ranges at most), so the fast difference keeps ~2^-46 relative
// accuracy on the separation; the squares are non-negative, so their sum needs
// no extra renormalisation.
template <int D>
__device__ __forceinline__ df norm_pair(const df* V, int stride, int f, int i, int j) {
  df q = df_sqr(df_add_fast(vget<D>(V, stride, f, 0, i), df_neg(vget<D>(V, stride, f, 0, j))));
#pragma unroll
  for (int d = 1; d < D; ++d)
    q = df_add_fast(q, df_sqr(df_add_fast(vget<D>(V, stride, f, d, i),
                                          df_neg(vget<D>(V, stride, f, d, j)))));
  return df_sqrt(q);
}

template <int D>
__device__ __forceinline__ df norm_origin(const df* V, int stride, int f, int i) {
  df q = df_sqr(vget<D>(V, stride, f, 0, i));
#pragma unroll
  for (int d = 1; d < D; ++d) q = df_add_fast(q, df_sqr(vget<D>(V, stride, f, d, i)));
  return df_sqrt(q);
}

// Writes point i's coordinates (identity frame ud) in every frame of the
// model: frame 0 = identity, frame fr.fid[s] = anisotropic structure s.
template <int D>
__device__ __forceinline__ void frame_coords(const DevModel& m, const Frames& fr, const df* ud,
                                             df* V, int stride, int i) {
#pragma unroll
  for (int d = 0; d < D; ++d) V[(0 * D + d) * stride + i] = ud[d];
#pragma unroll
  for (int s = 0; s < GS_MAX_STRUCTURES; ++s) {
    if (s >= m.ns || !m.s[s].aniso) continue;
    const int f = fr.fid[s];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      df acc = df_mul(m.s[s].rot_df[r * 3 + 0], ud[0]);
#pragma unroll
      for (int c = 1; c < D; ++c) acc = df_add(acc, df_mul(m.s[s].rot_df[r * 3 + c], ud[c]));
      V[(f * D + r) * stride + i] = acc;
    }
  }
}

// Covariance between stored points i and j (all frames of the model).
template <int D>
__device__ __forceinline__ df cov_pair(const DevModel& m, const Frames& fr, const df* V,
                                       int stride, int i, int j, const ExpTable& tab,
                                       const DfConsts& k) {
  df c = df_make(0.0f, 0.0f);
  df hiso = df_make(-1.0f, 0.0f);
#pragma unroll 1
  for (int s = 0; s < m.ns; ++s) {
    df h;
    if (m.s[s].aniso) {
      h = norm_pair<D>(V, stride, fr.fid[s], i, j);
    } else {
      if (hiso.hi < 0.0f) hiso = norm_pair<D>(V, stride, 0, i, j);
      h = hiso;
    }
    c = df_add_fast(c, cov_struct(m.s[s], h, tab, k));
  }
  return c;
}

// Covariances at two separation norms (isotropic models), side by side in
// packed FP32x2 arithmetic.
__device__ __forceinline__ void cov_from_norm2(const DevModel& m, df h0, df h1,
                                               const ExpTable& tab, const DfConsts& k, df& c0,
                                               df& c1) {
  const dfp h = dp_pack(h0, h1);
  auto term = [&](const DevStruct& st) {
    return dp_mul(dp_rho(st.kind, dp_mul(h, dp_splat(st.inv_range_df)), tab, k),
                  dp_splat(st.sill_df));
  };
  // the first structure's term as is (adding it to zero would return it
  // unchanged), the others summed onto it (>= 0 terms); a pure nugget model
  // has no structure and covariance 0 off the origin
  dfp c = dp_zero();
  if (m.ns > 0) {
    c = term(m.s[0]);
#pragma unroll 1
    for (int s = 1; s < m.ns; ++s) c = dp_add_fast(c, term(m.s[s]));
  }
  c0 = dp_first(c);
  c1 = dp_second(c);
}

// Visits this thread's pairs (i, j), i > j, of the strict lower triangle of
// an n x n matrix -- pair numbers first, first + stride, first + 2 stride,
// ... in packed order -- two at a time: fn(i0, j0, i1, j1, two).  When the
// second pair does not exist, (i1, j1) repeats the first and two is false.
template <class Fn>
__device__ __forceinline__ void for_pairs2(int n, int first, int stride, Fn&& fn) {
  const int npairs = (n * (n - 1)) >> 1;
  int ii = 1, jj = first;
  while (jj >= ii && ii < n) {
    jj -= ii;
    ++ii;
  }
  for (int q = first; q < npairs; q += 2 * stride) {
    int ii2 = ii, jj2 = jj + stride;
    while (jj2 >= ii2 && ii2 < n) {
      jj2 -= ii2;
      ++ii2;
    }
    const bool two = q + stride < npairs;
    if (!two) {
      ii2 = ii;
      jj2 = jj;
    }
    fn(ii, jj, ii2, jj2, two);
    ii = ii2;
    jj = jj2 + stride;
    while (jj >= ii && ii < n) {
      jj -= ii;
      ++ii;
    }
  }
}

// |a - b| of the pairs (i0, j0) and (i1, j1) of frame f, side by side
// (norm_pair lane by lane).
template <int D>
__device__ __forceinline__ dfp norm_pair2(const df* V, int stride, int f, int i0, int j0, int i1,
                                          int j1) {
  auto diff = [&](int d) {
    return dp_sub_fast(dp_pack(vget<D>(V, stride, f, d, i0), vget<D>(V, stride, f, d, i1)),
                       dp_pack(vget<D>(V, stride, f, d, j0), vget<D>(V, stride, f, d, j1)));
  };
  dfp q = dp_sqr(diff(0));
#pragma unroll
  for (int d = 1; d < D; ++d) q = dp_add_fast(q, dp_sqr(diff(d)));
  return dp_sqrt(q);
}

// Covariances of two pairs (i0, j0) and (i1, j1) of stored points, evaluated
// side by side in packed FP32x2 arithmetic (cov_pair lane by lane).
template <int D>
__device__ __forceinline__ void cov_pair2(const DevModel& m, const Frames& fr, const df* V,
                                          int stride, int i0, int j0, int i1, int j1,
                                          const ExpTable& tab, const DfConsts& k, df& c0,
                                          df& c1) {
  dfp c = dp_zero();
  dfp hiso = dp_make(p_splat(-1.0f), p_splat(0.0f));
#pragma unroll 1
  for (int s = 0; s < m.ns; ++s) {
    const DevStruct& st = m.s[s];
    dfp h;
    if (st.aniso) {
      h = norm_pair2<D>(V, stride, fr.fid[s], i0, j0, i1, j1);
    } else {
      if (hiso.hi.x < 0.0f) hiso = norm_pair2<D>(V, stride, 0, i0, j0, i1, j1);
      h = hiso;
    }
    const dfp r = dp_rho(st.kind, dp_mul(h, dp_splat(st.inv_range_df)), tab, k);
    c = dp_add_fast(c, dp_mul(r, dp_splat(st.sill_df)));
  }
  c0 = dp_first(c);
  c1 = dp_second(c);
}

// Covariance between stored point i and the frame origin (the target).
template <int D>
__device__ __forceinline__ df cov_origin(const DevModel& m, const Frames& fr, const df* V,
                                         int stride, int i, const ExpTable& tab,
                                         const DfConsts& k) {
  df c = df_make(0.0f, 0.0f);
  df hiso = df_make(-1.0f, 0.0f);
#pragma unroll 1
  for (int s = 0; s < m.ns; ++s) {
    df h;
    if (m.s[s].aniso) {
      h = norm_origin<D>(V, stride, fr.fid[s], i);
    } else {
      if (hiso.hi < 0.0f) hiso = norm_origin<D>(V, stride, 0, i);
      h = hiso;
    }
    c = df_add_fast(c, cov_struct(m.s[s], h, tab, k));
  }
  return c;
}

// Compensated accumulation of df products: acc += a * b.
__device__ __forceinline__ df df_fma_acc(df acc, df a, df b) { return df_add(acc, df_mul(a, b)); }

__device__ __forceinline__ df warp_sum_df(df v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    df w;
    w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
    w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
    v = df_add(v, w);
  }
  return v;
}

// Two warp_sum_df side by side (packed FP32x2 additions).
__device__ __forceinline__ dfp warp_sum_dfp(dfp v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    dfp w;
    w.hi.x = __shfl_xor_sync(0xffffffffu, v.hi.x, o);
    w.hi.y = __shfl_xor_sync(0xffffffffu, v.hi.y, o);
    w.lo.x = __shfl_xor_sync(0xffffffffu, v.lo.x, o);
    w.lo.y = __shfl_xor_sync(0xffffffffu, v.lo.y, o);
    v = dp_add(v, w);
  }
  return v;
}

}  // namespace gs
