// gs_pair.cuh -- two double-float numbers side by side, in packed FP32x2
// arithmetic (FADD2 / FMUL2 / FFMA2 on sm_100 and later).
//
// Each function repeats the operation sequence of its scalar counterpart in
// gs_common.cuh lane by lane.  A packed add, multiply or fused multiply-add
// rounds each lane as the scalar instruction does, and a - b is formed as
// fma(b, -1, a) (a - b rounded once, signed zeros included) and -a as
// a * -1, so a pair
// evaluation gives the two scalar results with about half the issued
// instructions.  Table lookups, rounding to an integer and the per-lane
// selects of the branch-free kinds stay scalar.
#pragma once

#include "gs_common.cuh"

namespace gs {

struct dfp {
  float2 hi, lo;
};

__device__ __forceinline__ float2 p_splat(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
}
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// -a as one packed multiply (exact); a per-lane sign flip would take two
// instructions
__device__ __forceinline__ float2 p_neg(float2 a) {
  return __fmul2_rn(a, make_float2(-1.0f, -1.0f));
}
__device__ __forceinline__ float2 p_sel(bool cx, bool cy, float2 a, float2 b) {
  return make_float2(cx ? a.x : b.x, cy ? a.y : b.y);
}

__device__ __forceinline__ dfp dp_make(float2 h, float2 l) {
  dfp r;
  r.hi = h;
  r.lo = l;
  return r;
}
__device__ __forceinline__ dfp dp_pack(df a, df b) {
  return dp_make(make_float2(a.hi, b.hi), make_float2(a.lo, b.lo));
}
__device__ __forceinline__ dfp dp_splat(df a) { return dp_make(p_splat(a.hi), p_splat(a.lo)); }
__device__ __forceinline__ df dp_first(dfp a) { return df_make(a.hi.x, a.lo.x); }
__device__ __forceinline__ df dp_second(dfp a) { return df_make(a.hi.y, a.lo.y); }
__device__ __forceinline__ dfp dp_zero() { return dp_make(p_splat(0.0f), p_splat(0.0f)); }
__device__ __forceinline__ dfp dp_neg(dfp a) { return dp_make(p_neg(a.hi), p_neg(a.lo)); }
__device__ __forceinline__ dfp dp_sel(bool cx, bool cy, dfp a, dfp b) {
  return dp_make(p_sel(cx, cy, a.hi, b.hi), p_sel(cx, cy, a.lo, b.lo));
}

// two_sum, fast_two_sum, two_prod
__device__ __forceinline__ dfp p_two_sum(float2 a, float2 b) {
  const float2 s = p_add(a, b);
  const float2 bb = p_sub(s, a);
  return dp_make(s, p_add(p_sub(a, p_sub(s, bb)), p_sub(b, bb)));
}
// two_sum(a, -b): the same sum and the same (exact) error term
__device__ __forceinline__ dfp p_two_diff(float2 a, float2 b) {
  const float2 s = p_sub(a, b);
  const float2 bb = p_sub(s, a);
  return dp_make(s, p_sub(p_sub(a, p_sub(s, bb)), p_add(b, bb)));
}
__device__ __forceinline__ dfp p_fast_two_sum(float2 a, float2 b) {
  const float2 s = p_add(a, b);
  return dp_make(s, p_sub(b, p_sub(s, a)));
}
__device__ __forceinline__ dfp p_two_prod(float2 a, float2 b) {
  const float2 p = p_mul(a, b);
  return dp_make(p, p_fma(a, b, p_neg(p)));
}

// df_add, df_add_fast, df_add_f, df_mul, df_sqr
__device__ __forceinline__ dfp dp_add(dfp a, dfp b) {
  dfp s = p_two_sum(a.hi, b.hi);
  const dfp t = p_two_sum(a.lo, b.lo);
  s.lo = p_add(s.lo, t.hi);
  s = p_fast_two_sum(s.hi, s.lo);
  s.lo = p_add(s.lo, t.lo);
  return p_fast_two_sum(s.hi, s.lo);
}
// df_add(a, df_neg(b)): two_sum is exact in either operand order, so this is
// the same computation with the negation folded into the subtractions.
__device__ __forceinline__ dfp dp_sub(dfp a, dfp b) {
  dfp s = p_two_diff(a.hi, b.hi);
  const dfp t = p_two_diff(a.lo, b.lo);
  s.lo = p_add(s.lo, t.hi);
  s = p_fast_two_sum(s.hi, s.lo);
  s.lo = p_add(s.lo, t.lo);
  return p_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dfp dp_add_fast(dfp a, dfp b) {
  const dfp s = p_two_sum(a.hi, b.hi);
  return p_fast_two_sum(s.hi, p_add(s.lo, p_add(a.lo, b.lo)));
}
// df_add_fast(a, df_neg(b))
__device__ __forceinline__ dfp dp_sub_fast(dfp a, dfp b) {
  const dfp s = p_two_diff(a.hi, b.hi);
  return p_fast_two_sum(s.hi, p_add(s.lo, p_sub(a.lo, b.lo)));
}
__device__ __forceinline__ dfp dp_add_f(dfp a, float2 b) {
  dfp s = p_two_sum(a.hi, b);
  s.lo = p_add(s.lo, a.lo);
  return p_fast_two_sum(s.hi, s.lo);
}
// df_add_f(df_neg(a), b) = b - a
__device__ __forceinline__ dfp dp_rsub_f(float2 b, dfp a) {
  dfp s = p_two_diff(b, a.hi);
  s.lo = p_sub(s.lo, a.lo);
  return p_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dfp dp_mul(dfp a, dfp b) {
  dfp p = p_two_prod(a.hi, b.hi);
  p.lo = p_fma(a.hi, b.lo, p.lo);
  p.lo = p_fma(a.lo, b.hi, p.lo);
  return p_fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ dfp dp_sqr(dfp a) {
  dfp p = p_two_prod(a.hi, a.hi);
  p.lo = p_fma(p_add(a.hi, a.hi), a.lo, p.lo);  // 2 a.hi is exact
  return p_fast_two_sum(p.hi, p.lo);
}

// df_sqrt (Karp & Markstein correction), per lane 0 for s <= 0.
__device__ __forceinline__ dfp dp_sqrt(dfp s) {
  const bool px = s.hi.x > 0.0f, py = s.hi.y > 0.0f;
  const float2 sh = p_sel(px, py, s.hi, p_splat(1.0f));
  float2 r = make_float2(rsqrtf(sh.x), rsqrtf(sh.y));
  r = p_mul(r, p_fma(p_mul(p_mul(p_splat(-0.5f), sh), r), r, p_splat(1.5f)));
  const float2 y = p_mul(sh, r);
  const dfp yy = p_two_prod(y, y);
  const float2 e = p_add(p_sub(p_sub(sh, yy.hi), yy.lo), p_sel(px, py, s.lo, p_splat(0.0f)));
  const dfp res = p_fast_two_sum(y, p_mul(e, p_mul(p_splat(0.5f), r)));
  return dp_sel(px, py, res, dp_zero());
}

// df_expneg (Tang's table-driven exp(-d)), lane by lane.
__device__ __forceinline__ dfp dp_expneg(dfp din, const ExpTable& tab, const ExpConsts& k) {
  const bool ix = din.hi.x < 87.0f, iy = din.hi.y < 87.0f;
  const dfp d = dp_sel(ix, iy, din, dp_zero());
  const float2 prod = p_mul(d.hi, p_splat(k.inv));
  const float2 nf = make_float2(rintf(prod.x), rintf(prod.y));
  const int nx = (int)nf.x, ny = (int)nf.y;
  const float2 t1 = p_sub(d.hi, p_mul(nf, p_splat(k.l1)));  // exact (Sterbenz)
  const dfp nl2 = p_two_prod(nf, p_splat(k.l2));
  dfp r = p_two_diff(t1, nl2.hi);
  r = p_fast_two_sum(r.hi, p_add(r.lo, p_sub(p_sub(d.lo, nl2.lo), p_mul(nf, p_splat(k.l3)))));
  const float2 t = r.hi;
  const dfp r2 = p_two_prod(t, t);  // exact
  const float2 small = p_fma(p_mul(p_mul(t, t), t),
                             p_fma(t, p_splat(1.0f / 24.0f), p_splat(-(1.0f / 6.0f))), p_mul(t, r.lo));
  const dfp half = p_fast_two_sum(p_mul(p_splat(0.5f), r2.hi), p_fma(p_splat(0.5f), r2.lo, small));
  const dfp q = dp_sub(half, r);  // df_add(-r, half)
  const dfp e = dp_add_f(q, p_splat(1.0f));
  const dfp tv = dp_pack(tab.v[nx & 255], tab.v[ny & 255]);
  const dfp res = dp_mul(e, tv);
  const float2 sc = make_float2(__int_as_float((127 - (nx >> 8)) << 23),
                                __int_as_float((127 - (ny >> 8)) << 23));
  return dp_sel(ix, iy, dp_make(p_mul(res.hi, sc), p_mul(res.lo, sc)), dp_zero());
}

// rho_sph_df / exp_arg_df / exp_factor_df / rho_df, lane by lane.
__device__ __forceinline__ dfp dp_rho_sph(dfp d) {
  const bool inx = !(d.hi.x > 1.0f || (d.hi.x == 1.0f && d.lo.x >= 0.0f));
  const bool iny = !(d.hi.y > 1.0f || (d.hi.y == 1.0f && d.lo.y >= 0.0f));
  const dfp d2 = dp_sqr(d);
  const dfp t = dp_add_f(dp_make(p_mul(p_splat(-0.5f), d2.hi), p_mul(p_splat(-0.5f), d2.lo)),
                         p_splat(1.5f));
  const dfp u = dp_mul(d, t);
  const dfp r = dp_rsub_f(p_splat(1.0f), u);
  return dp_sel(inx, iny, r, dp_zero());
}
__device__ __forceinline__ dfp dp_exp_arg(int kind, dfp d, const ExpConsts& k) {
  if (kind == GS_KIND_GAUSSIAN) return dp_sqr(d);
  if (kind == GS_KIND_MATERN15) return dp_mul(d, dp_splat(df_make(k.s3h, k.s3l)));
  if (kind == GS_KIND_MATERN25) return dp_mul(d, dp_splat(df_make(k.s5h, k.s5l)));
  return d;
}
__device__ __forceinline__ dfp dp_exp_factor(int kind, dfp s, dfp e) {
  if (kind == GS_KIND_MATERN15) return dp_mul(dp_add_f(s, p_splat(1.0f)), e);
  if (kind == GS_KIND_MATERN25) {
    const dfp s2 = dp_sqr(s);
    // 1 + s + s^2/3: s^2/3 as df via FP32 reciprocal correction
    const float2 q = p_mul(s2.hi, p_splat(1.0f / 3.0f));
    const dfp q3 = p_two_prod(q, p_splat(3.0f));
    const float2 rq = p_mul(p_add(p_sub(p_sub(s2.hi, q3.hi), q3.lo), s2.lo), p_splat(1.0f / 3.0f));
    const dfp third = p_fast_two_sum(q, rq);
    const dfp p = dp_add(dp_add_f(s, p_splat(1.0f)), third);
    return dp_mul(p, e);
  }
  return e;
}
__device__ __forceinline__ dfp dp_rho(int kind, dfp d, const ExpTable& tab, const ExpConsts& k) {
  if (kind == GS_KIND_SPHERICAL) return dp_rho_sph(d);
  const dfp s = dp_exp_arg(kind, d, k);
  return dp_exp_factor(kind, s, dp_expneg(s, tab, k));
}

}  // namespace gs
