// gs_common.cuh -- shared types, error plumbing, double-float arithmetic and
// the device variogram model.
//
// Precision design (GB300 has ~1/64-rate FP64): matrix entries are formed in
// double-float ("df": an unevaluated FP32 pair hi+lo, ~2^-48 relative), the
// hi parts feed an FP32 factorisation, and the df entries feed the residuals
// of the iterative refinement.  Only O(N) per-system work (variances,
// log-likelihood terms, coordinate differences) uses FP64.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/geostat_gb300.h"

namespace gs {

// ---------------------------------------------------------------- errors --
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define GS_CUDA(call)                                                       \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) return ::gs::cuda_fail(e_, #call, __FILE__, __LINE__); \
  } while (0)

#define GS_TRY(call)           \
  do {                         \
    int rc_ = (call);          \
    if (rc_ != GS_OK) return rc_; \
  } while (0)

// ------------------------------------------------------------ df numbers --
struct df {
  float hi, lo;
};

__host__ __device__ inline df df_make(float h, float l) {
  df r;
  r.hi = h;
  r.lo = l;
  return r;
}

__device__ __forceinline__ df two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df_make(s, e);
}
// |a| >= |b| (or a == 0)
__device__ __forceinline__ df fast_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return df_make(s, e);
}
__device__ __forceinline__ df two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  float e = __fmaf_rn(a, b, -p);
  return df_make(p, e);
}
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  df t = two_sum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = fast_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return fast_two_sum(s.hi, s.lo);
}
// Double-float sum without the second renormalisation: error <= ~2^-46
// (|a| + |b|); used for sums of same-sign terms (no cancellation) and for
// differences of nearby coordinates whose magnitudes bound the error.
__device__ __forceinline__ df df_add_fast(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  const float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, e);
}
__device__ __forceinline__ df df_neg(df a) { return df_make(-a.hi, -a.lo); }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df df_add_f(df a, float b) {
  df s = two_sum(a.hi, b);
  s.lo = __fadd_rn(s.lo, a.lo);
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_mul(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
  p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df df_mul_f(df a, float b) {
  df p = two_prod(a.hi, b);
  p.lo = __fmaf_rn(a.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df df_sqr(df a) {
  df p = two_prod(a.hi, a.hi);
  p.lo = __fmaf_rn(2.0f * a.hi, a.lo, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
__host__ __device__ inline df df_from_double(double x) {
  float h = (float)x;
  float l = (float)(x - (double)h);
  return df_make(h, l);
}
__host__ __device__ inline double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

// sqrt of a non-negative df: an FP32 reciprocal square root refined by one
// Newton step, then one correction with the exact residual s - y*y
// (Karp & Markstein, ACM TOMS 23(4), 1997): relative error ~2^-47.  Branch
// free (0 for s <= 0), so independent evaluations interleave.
__device__ __forceinline__ df df_sqrt(df s) {
  const bool pos = s.hi > 0.0f;
  const float sh = pos ? s.hi : 1.0f;
  float r = rsqrtf(sh);
  r = r * fmaf(-0.5f * sh * r, r, 1.5f);
  const float y = sh * r;
  const df yy = two_prod(y, y);
  const float e = __fadd_rn(__fsub_rn(__fsub_rn(sh, yy.hi), yy.lo), pos ? s.lo : 0.0f);
  const df res = fast_two_sum(y, e * (0.5f * r));
  return pos ? res : df_make(0.0f, 0.0f);
}

// exp(-d) for d >= 0, table-driven after P. T. P. Tang, "Table-driven
// implementation of the exponential function in IEEE floating-point
// arithmetic", ACM TOMS 15(2), 1989: d = n*ln2/256 + r with |r| <= ln2/512,
// exp(-d) = 2^(-n/256) * exp(-r).  2^(-j/256) comes from a 256-entry df table;
// exp(-r) = 1 - r + r^2/2 - r^3/6 + r^4/24 with r^2/2 in double-float.  ln2/256 is split as l1 (9 significant bits, so
// n*l1 is exact for n < 2^15, i.e. d < 88) + l2 + l3; n*l2 is formed exactly.
struct ExpTable {
  df v[256];  // 2^(-j/256) as (hi, lo) pairs: one 8-byte load per lookup
};
// Uniform df constants, filled on the host (df_consts_host).
struct DfConsts {
  float l1, l2, l3, inv;  // ln2/256 in three parts, 256/ln2
  float s3h, s3l, s5h, s5l;  // sqrt(3), sqrt(5) as df
};
typedef DfConsts ExpConsts;

__device__ __forceinline__ df df_expneg(df din, const ExpTable& tab, const ExpConsts& k) {
  // branch free: out-of-range (or NaN) arguments are evaluated at 0 and
  // replaced by 0 at the end
  const bool in = din.hi < 87.0f;
  const df d = in ? din : df_make(0.0f, 0.0f);
  const float nf = rintf(__fmul_rn(d.hi, k.inv));
  const int n = (int)nf;
  const float t1 = __fsub_rn(d.hi, __fmul_rn(nf, k.l1));  // exact (Sterbenz)
  const df nl2 = two_prod(nf, k.l2);
  df r = two_sum(t1, -nl2.hi);
  r = fast_two_sum(r.hi, __fadd_rn(r.lo, __fsub_rn(__fsub_rn(d.lo, nl2.lo), __fmul_rn(nf, k.l3))));
  // exp(-r) = 1 - r + r^2/2 - r^3/6 + r^4/24 for |r| <= ln2/512 (the next
  // term is below 4e-17).  r^2/2 (up to ~9e-7) is formed as a double-float --
  // its FP32 rounding alone would cost ~5e-14 -- and the cubic and quartic
  // terms (below 4e-10) go in FP32.
  const float t = r.hi;
  const df r2 = two_prod(t, t);  // exact
  const float small = __fmaf_rn(t * t * t, -(1.0f / 6.0f) + t * (1.0f / 24.0f), t * r.lo);
  const df half = fast_two_sum(0.5f * r2.hi, __fmaf_rn(0.5f, r2.lo, small));
  const df q = df_add(df_neg(r), half);
  const df e = df_add_f(q, 1.0f);
  const int j = n & 255;
  const int kk = n >> 8;
  const df res = df_mul(e, tab.v[j]);
  const float sc = __int_as_float((127 - kk) << 23);  // 2^-kk, kk <= 126 for d < 88
  return in ? df_make(res.hi * sc, res.lo * sc) : df_make(0.0f, 0.0f);
}

void df_consts_host(ExpTable* tab, DfConsts* k);

// ------------------------------------------------------------ the model --
struct DevStruct {
  int kind;
  int aniso;
  double sill;
  double inv_range;
  double rot[9];  // covariance-frame rotation+scaling, row-major 3x3
  df sill_df;
  df inv_range_df;
  df rot_df[9];
};

struct DevModel {
  int ns;
  int dim;
  double nugget;
  double c0;  // total sill = C(0)
  df c0_df;
  DevStruct s[GS_MAX_STRUCTURES];
};

// Host: converts and validates a gs_model for the device path.
int make_dev_model(const gs_model& m, int dim, DevModel* out, bool gpu_kinds_only);
int validate_model(const gs_model& m);
double total_sill(const gs_model& m);
bool has_power(const gs_model& m);
// Host rotation matrix of model.rs:407-433 (3-D) / 353-367 (2-D as matrix).
void rotation_matrix(const gs_structure& s, int dim, double rot[9]);

// Unit-sill correlation rho(d) = 1 - g(d) in FP64 (model.rs:122-141).
__device__ __forceinline__ double rho_fp64(int kind, double d) {
  switch (kind) {
    case GS_KIND_SPHERICAL:
      return d >= 1.0 ? 0.0 : 1.0 - (1.5 * d - 0.5 * d * d * d);
    case GS_KIND_EXPONENTIAL:
      return exp(-d);
    case GS_KIND_GAUSSIAN:
      return exp(-(d * d));
    case GS_KIND_MATERN15: {
      double s = 1.7320508075688772 * d;
      return (1.0 + s) * exp(-s);
    }
    default: {  // GS_KIND_MATERN25
      double s = 2.23606797749979 * d;
      return (1.0 + s + s * s / 3.0) * exp(-s);
    }
  }
}

// FP64 exp(-x) by Tang's table-driven method (P. T. P. Tang, "Table-driven
// implementation of the exponential function in IEEE floating-point
// arithmetic", ACM TOMS 15(2), 1989), for the re-solve kernels' covariances:
// x = (64 m + j) ln2/64 + r with |r| <= ln2/128, so
//     exp(-x) = 2^-m * 2^(-j/64) * exp(-r),
// exp(-r) - 1 from its Taylor polynomial through r^5 (remainder < 4e-17),
// 2^(-j/64) as a two-double table entry, ln2/64 in two parts (the first with
// 36 significant bits, so k * part1 is exact).  About 1 ulp; x >= 708 gives 0.
struct Exp64Table {
  double hi[64], lo[64];  // 2^(-j/64) = hi + lo
  double l1, l2, inv;     // ln2/64 = l1 + l2, 64/ln2
};
void exp64_table_host(Exp64Table* t);

__device__ __forceinline__ double expneg_fp64(double x, const Exp64Table& T) {
  const double magic = 6755399441055744.0;  // 1.5 * 2^52: integer part in the low word
  const bool in = x < 708.0;
  const double xc = in ? x : 0.0;
  const double km = fma(xc, T.inv, magic);
  const int k = __double2loint(km);
  const double kd = km - magic;
  const double r = fma(-kd, T.l2, fma(-kd, T.l1, xc));
  double p = fma(r, -1.0 / 120.0, 1.0 / 24.0);
  p = fma(r, p, -1.0 / 6.0);
  p = fma(r, p, 0.5);
  p = fma(r, p, -1.0);
  p *= r;
  const int j = k & 63, mexp = k >> 6;
  const double th = T.hi[j];
  const double res = th + fma(th, p, T.lo[j]);  // in (0.49, 1.01): exponent 1022 or 1023
  const double scaled = __hiloint2double(__double2hiint(res) - (mexp << 20), __double2loint(res));
  return in ? scaled : 0.0;
}

// rho_fp64 with expneg_fp64 in place of exp.
__device__ __forceinline__ double rho_fp64x(int kind, double d, const Exp64Table& T) {
  switch (kind) {
    case GS_KIND_SPHERICAL:
      return d >= 1.0 ? 0.0 : 1.0 - (1.5 * d - 0.5 * d * d * d);
    case GS_KIND_EXPONENTIAL:
      return expneg_fp64(d, T);
    case GS_KIND_GAUSSIAN:
      return expneg_fp64(d * d, T);
    case GS_KIND_MATERN15: {
      double s = 1.7320508075688772 * d;
      return (1.0 + s) * expneg_fp64(s, T);
    }
    default: {  // GS_KIND_MATERN25
      double s = 2.23606797749979 * d;
      return (1.0 + s + s * s / 3.0) * expneg_fp64(s, T);
    }
  }
}

// Covariance C(h) = c0 - gamma(h) in FP64 for a separation vector.
template <int D>
__device__ __forceinline__ double cov_fp64(const DevModel& m, const double* h) {
  bool zero = true;
#pragma unroll
  for (int d = 0; d < D; ++d) zero = zero && (h[d] == 0.0);
  if (zero) return m.c0;
  double acc = 0.0;
  for (int k = 0; k < m.ns; ++k) {
    const DevStruct& s = m.s[k];
    double q = 0.0;
    if (s.aniso) {
#pragma unroll
      for (int r = 0; r < D; ++r) {
        double e = 0.0;
#pragma unroll
        for (int c = 0; c < D; ++c) e += s.rot[r * 3 + c] * h[c];
        q += e * e;
      }
    } else {
#pragma unroll
      for (int d = 0; d < D; ++d) q += h[d] * h[d];
    }
    acc += s.sill * rho_fp64(s.kind, sqrt(q) * s.inv_range);
  }
  return acc;
}

// cov_fp64 with the table-driven exp (the same operation order otherwise).
template <int D>
__device__ __forceinline__ double cov_fp64x(const DevModel& m, const double* h,
                                            const Exp64Table& T) {
  bool zero = true;
#pragma unroll
  for (int d = 0; d < D; ++d) zero = zero && (h[d] == 0.0);
  if (zero) return m.c0;
  double acc = 0.0;
  for (int k = 0; k < m.ns; ++k) {
    const DevStruct& s = m.s[k];
    double q = 0.0;
    if (s.aniso) {
#pragma unroll
      for (int r = 0; r < D; ++r) {
        double e = 0.0;
#pragma unroll
        for (int c = 0; c < D; ++c) e += s.rot[r * 3 + c] * h[c];
        q += e * e;
      }
    } else {
#pragma unroll
      for (int d = 0; d < D; ++d) q += h[d] * h[d];
    }
    acc += s.sill * rho_fp64x(s.kind, sqrt(q) * s.inv_range, T);
  }
  return acc;
}

// Unit-sill correlations in df for d >= 0, branch free.
__device__ __forceinline__ df rho_sph_df(df d) {
  // 1 - d (1.5 - 0.5 d^2) for d < 1, else 0
  const bool inside = !(d.hi > 1.0f || (d.hi == 1.0f && d.lo >= 0.0f));
  const df d2 = df_sqr(d);
  const df t = df_add_f(df_make(-0.5f * d2.hi, -0.5f * d2.lo), 1.5f);
  const df u = df_mul(d, t);
  const df r = df_add_f(df_neg(u), 1.0f);
  return inside ? r : df_make(0.0f, 0.0f);
}
__device__ __forceinline__ df rho_mat15_df(df d, const ExpTable& tab, const ExpConsts& k) {
  const df s = df_mul(d, df_make(k.s3h, k.s3l));
  const df e = df_expneg(s, tab, k);
  return df_mul(df_add_f(s, 1.0f), e);
}
__device__ __forceinline__ df rho_mat25_df(df d, const ExpTable& tab, const ExpConsts& k) {
  const df s = df_mul(d, df_make(k.s5h, k.s5l));
  const df e = df_expneg(s, tab, k);
  const df s2 = df_sqr(s);
  // 1 + s + s^2/3: s^2/3 as df via FP32 reciprocal correction
  const float q = s2.hi * (1.0f / 3.0f);
  const df q3 = two_prod(q, 3.0f);
  const float rq = (s2.hi - q3.hi - q3.lo + s2.lo) * (1.0f / 3.0f);
  const df third = fast_two_sum(q, rq);
  const df p = df_add(df_add_f(s, 1.0f), third);
  return df_mul(p, e);
}

// rho(d) in df for d >= 0.
// Argument of the exponential of kind `kind` at d = h / range (Exponential:
// d, Gaussian: d^2, Matern 3/2: sqrt(3) d, Matern 5/2: sqrt(5) d), and the
// factor that multiplies it (1, 1, 1 + s, 1 + s + s^2/3); Spherical has no
// exponential.  Splitting each kind this way gives one copy of df_expneg per
// call site instead of one per kind, with the same operations per kind as
// rho_mat15_df / rho_mat25_df.
__device__ __forceinline__ df exp_arg_df(int kind, df d, const ExpConsts& k) {
  if (kind == GS_KIND_GAUSSIAN) return df_sqr(d);
  if (kind == GS_KIND_MATERN15) return df_mul(d, df_make(k.s3h, k.s3l));
  if (kind == GS_KIND_MATERN25) return df_mul(d, df_make(k.s5h, k.s5l));
  return d;
}
__device__ __forceinline__ df exp_factor_df(int kind, df s, df e) {
  if (kind == GS_KIND_MATERN15) return df_mul(df_add_f(s, 1.0f), e);
  if (kind == GS_KIND_MATERN25) {
    const df s2 = df_sqr(s);
    // 1 + s + s^2/3: s^2/3 as df via FP32 reciprocal correction
    const float q = s2.hi * (1.0f / 3.0f);
    const df q3 = two_prod(q, 3.0f);
    const float rq = (s2.hi - q3.hi - q3.lo + s2.lo) * (1.0f / 3.0f);
    const df third = fast_two_sum(q, rq);
    const df p = df_add(df_add_f(s, 1.0f), third);
    return df_mul(p, e);
  }
  return e;
}

__device__ __forceinline__ df rho_df(int kind, df d, const ExpTable& tab, const ExpConsts& k) {
  if (kind == GS_KIND_SPHERICAL) return rho_sph_df(d);
  const df s = exp_arg_df(kind, d, k);
  return exp_factor_df(kind, s, df_expneg(s, tab, k));
}

// 1/d to FP64 accuracy: FP32 estimate, two Newton steps (e = 1 - d r,
// r += r e).  sc (a power of two) scales d into FP32's range first when the
// system's scale is outside [1e-20, 1e20] (scaled = true).
__device__ __forceinline__ double rcp_fp64(double d, double sc, bool scaled) {
  double r = scaled ? (double)__frcp_rn((float)(d * sc)) * sc : (double)__frcp_rn((float)d);
  double e = fma(-d, r, 1.0);
  r = fma(r, e, r);
  e = fma(-d, r, 1.0);
  return fma(r, e, r);
}

}  // namespace gs
