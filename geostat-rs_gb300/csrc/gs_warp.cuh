// gs_warp.cuh -- one small symmetric system (N <= 32) per warp, rows in
// registers: FP32 inversion by the sweep operator and double-float refinement.
//
// Lane i holds row i of the working matrix in registers.  Pivot k: lane k
// publishes its row through shared memory, with its pivot entry replaced by
// d - 1 (d = a_kk); every lane then applies the same update
//     t[j] -= l * row_k[j]   for all j,
// with l = a_ik / d on lane i != k and l = 1 - 1/d on lane k.  This single
// uniform update is the sweep operator (a_ij -= a_ik a_kj / d, a_ik = a_ik/d,
// a_kj = a_kj/d) except on lane k's own diagonal, which ends at 2 - 1/d instead
// of -1/d.  Later pivots change that entry linearly, so after all N pivots
// every lane's diagonal is exactly 2 too large and the rows hold -A^{-1}
// (diagonal corrected once).  No per-element selects and no register-array
// indexing are needed.  Symmetry gives a_ik as row_k[i].
//
// Refinement residuals b - A x use the double-float entries held in registers
// (compensated FP32 dot products, Ogita, Rump & Oishi 2005); corrections are
// register GEMVs with -A^{-1}.  One factorisation serves any number of
// right-hand sides (warp_refine).
#pragma once

#include "gs_solve.cuh"
#include "gs_pair.cuh"

namespace gs {

constexpr int kWarpN = 32;
constexpr int kWarpN2 = kWarpN / 2;  // column pairs of a register row
// Floats of the published-row buffer: two alternating rows of kWarpN
// entries plus the pivot (padded to 16 bytes).
constexpr int kWarpRowFloats = 2 * (kWarpN + 4);

struct WarpScratch {
  float* row;  // kWarpRowFloats floats: the published pivot rows
  float* vec;  // 32 floats: broadcast vector
  df* xd;      // 32 df: solution (during a refinement: its hi parts, then its lo parts)
};

constexpr int kWarpN4 = kWarpN / 4;  // column quads of a register row

// The factorisation one lane holds: its row of the double-float matrix
// (ah + al) as column pairs and of -(sc A)^{-1} + 2I (t) as column quads
// (so a published row is stored straight from aligned registers), with the
// power-of-two scale sc.
struct WarpFactor {
  float2 ah[kWarpN2], al[kWarpN2];
  float4 t[kWarpN4];
  float sc;
};

// Loads row `lane` of a packed symmetric df matrix (N x N; at(e) returns
// packed entry e) into registers; rows and columns beyond N hold the
// identity.
template <class At>
__device__ __forceinline__ void warp_load_rows(At&& at, int N, int lane, float2 (&ah)[kWarpN2],
                                               float2 (&al)[kWarpN2]) {
  auto elt = [&](int j) {
    df v = df_make(j == lane ? 1.0f : 0.0f, 0.0f);
    if (lane < N && j < N) v = at(lane >= j ? pk(lane, j) : pk(j, lane));
    return v;
  };
#pragma unroll
  for (int j2 = 0; j2 < kWarpN2; ++j2) {
    const df v0 = elt(2 * j2), v1 = elt(2 * j2 + 1);
    ah[j2] = make_float2(v0.hi, v1.hi);
    al[j2] = make_float2(v0.lo, v1.lo);
  }
}

__device__ __forceinline__ void warp_gemv_neg_inv(const float4 (&t)[kWarpN4], const float* vec,
                                                  int lane, float& y) {
  // y = (-A^{-1}) v with the +2 diagonal offset removed; packed FP32x2
  // products into two accumulator pairs
  float2 a0 = make_float2(0.0f, 0.0f), a1 = make_float2(0.0f, 0.0f);
#pragma unroll
  for (int q = 0; q < kWarpN4; ++q) {
    const float4 v = *reinterpret_cast<const float4*>(vec + 4 * q);
    a0 = __ffma2_rn(make_float2(t[q].x, t[q].y), make_float2(v.x, v.y), a0);
    a1 = __ffma2_rn(make_float2(t[q].z, t[q].w), make_float2(v.z, v.w), a1);
  }
  y = fmaf(-2.0f, vec[lane], (a0.x + a1.x) + (a0.y + a1.y));
}

// FP32 inverse of the packed df matrix A (N <= 32 unknowns).  Returns false
// (uniformly in the warp) when a pivot is too small for FP32.
//
// Pivot k: lane k publishes its row in one of two alternating buffers, with
// the pivot entry replaced by d - 1 and d stored after the row; one
// __syncwarp, then every lane applies its packed FP32x2 update.  Lane k's
// next write to the same buffer (pivot k + 2) comes after the next pivot's
// __syncwarp, which every lane reaches only after reading this row.
template <class At>
__device__ __forceinline__ bool warp_factor_at(At&& at, int N, int lane, WarpFactor& f,
                                               const WarpScratch& W) {
  warp_load_rows(at, N, lane, f.ah, f.al);
  float amax = 0.0f;
#pragma unroll
  for (int j2 = 0; j2 < kWarpN2; ++j2)
    amax = fmaxf(amax, lane < N ? fmaxf(fabsf(f.ah[j2].x), fabsf(f.ah[j2].y)) : 0.0f);
  amax = warp_max_f(amax);
  f.sc = 1.0f;
  if (!(amax > 0.0f)) return false;
  // power-of-two scale: sc * max|A| in [0.5, 1), so every pivot is <= 1 and
  // the pivot lane's multiplier 1 - 1/d never cancels; the swept rows then
  // hold -(sc A)^{-1}, i.e. -A^{-1} / sc
  int ex = 0;
  frexpf(amax, &ex);
  f.sc = ldexpf(1.0f, -ex);
  auto scaled = [&](int j) {
    const float v = (j & 1) ? f.ah[j >> 1].y : f.ah[j >> 1].x;
    return (lane < N && j < N) ? v * f.sc : v;
  };
#pragma unroll
  for (int q = 0; q < kWarpN4; ++q)
    f.t[q] = make_float4(scaled(4 * q), scaled(4 * q + 1), scaled(4 * q + 2), scaled(4 * q + 3));
  const float tol = 1e-6f * amax * f.sc;
  __syncwarp();  // the previous user of W.row is done with it
  for (int k = 0; k < N; ++k) {
    float* rb = W.row + (k & 1) * (kWarpN + 4);
    if (lane == k) {
#pragma unroll
      for (int q = 0; q < kWarpN4; ++q) *reinterpret_cast<float4*>(rb + 4 * q) = f.t[q];
      const float d = rb[k];  // this lane's own store
      rb[k] = d - 1.0f;
      rb[kWarpN] = d;
    }
    __syncwarp();
    const float d = rb[kWarpN];
    if (!(fabsf(d) > tol)) return false;  // the same value in every lane
    const float invd = __fdividef(1.0f, d);  // an approximate inverse suffices
    const float l = lane == k ? 1.0f - invd : rb[lane] * invd;
    const float2 nl = make_float2(-l, -l);
#pragma unroll
    for (int q = 0; q < kWarpN4; ++q) {
      const float4 r = *reinterpret_cast<const float4*>(rb + 4 * q);
      const float2 u0 = __ffma2_rn(nl, make_float2(r.x, r.y), make_float2(f.t[q].x, f.t[q].y));
      const float2 u1 = __ffma2_rn(nl, make_float2(r.z, r.w), make_float2(f.t[q].z, f.t[q].w));
      f.t[q] = make_float4(u0.x, u0.y, u1.x, u1.y);
    }
  }
  __syncwarp();
  return true;
}

// The matrix as packed df entries.
__device__ __forceinline__ bool warp_factor(const df* A, int N, int lane, WarpFactor& f,
                                            const WarpScratch& W) {
  return warp_factor_at([&](int e) { return A[e]; }, N, lane, f, W);
}
// The matrix as packed entries split into hi parts Ah[e] and lo parts Al[e].
__device__ __forceinline__ bool warp_factor(const float* Ah, const float* Al, int N, int lane,
                                            WarpFactor& f, const WarpScratch& W) {
  return warp_factor_at([&](int e) { return df_make(Ah[e], Al[e]); }, N, lane, f, W);
}

// Refinement sweeps before a system is handed to the FP64 solver; a sweep
// that no longer halves the correction ends the refinement earlier (the
// double-float residual of an ill-conditioned system has reached its limit).
constexpr int kMaxRefineSweeps = 8;

// Solves A x = B with the factorisation f and refines to ~1e-13 relative; on
// success W.xd[i] holds x_i.  Returns false (uniformly) when the refinement
// stalls.
//
// accept_floor > 0: a refinement that stops contracting (or runs out of
// sweeps) once its corrections are at most accept_floor |x| is accepted as
// well, with *at_floor set.  The residual b - A x is then limited by the
// double-float entries (about 2^-48 of each entry and product), not by the
// FP32 inverse.  A linear functional g.x of the last iterate then differs
// from g.A^{-1}b by v.(r~ - r) + (v - v32).r, with v = A^{-1} g, v32 its FP32
// approximation and r~ the computed residual of the previous iterate: the
// first term is the effect of the entries' rounding, the same for a
// refinement that converges (it converges to the double-float system's
// solution), and the second is a product of two small factors.  Callers
// whose outputs are such functionals (the Vecchia conditional mean and
// variance) may use it.
__device__ __forceinline__ bool warp_refine(const WarpFactor& f, const df* B, int N, int lane,
                                            const WarpScratch& W, float accept_floor = 0.0f,
                                            bool* at_floor = nullptr) {
  // x0 = A^{-1} b_hi = -(-A^{-1}) b_hi
  __syncwarp();
  W.vec[lane] = lane < N ? B[lane].hi : 0.0f;
  __syncwarp();
  float y;
  warp_gemv_neg_inv(f.t, W.vec, lane, y);
  y *= f.sc;
  df x = df_make(lane < N ? -y : 0.0f, 0.0f);
  const float nx = warp_max_f(fabsf(x.hi));
  float nd_prev = nx;
  for (int sweep = 1; sweep <= kMaxRefineSweeps; ++sweep) {
    // residual of row `lane`: b - A x, compensated (Dot2) in packed FP32x2
    // over column pairs: two accumulator lanes (even and odd columns) with
    // their compensations, joined by one more error-free sum.  x is
    // broadcast negated and split (hi parts, then lo parts) so a 16-byte load
    // gives the operands of two column pairs.
    float* xs = reinterpret_cast<float*>(W.xd);
    __syncwarp();
    xs[lane] = -x.hi;
    xs[kWarpN + lane] = -x.lo;
    __syncwarp();
    float2 s2 = make_float2(lane < N ? B[lane].hi : 0.0f, 0.0f);
    float2 c2 = make_float2(lane < N ? B[lane].lo : 0.0f, 0.0f);
    auto acc = [&](float2 ah, float2 al, float2 xh, float2 xl) {
      const float2 ph = __fmul2_rn(ah, xh);
      float2 pe = __ffma2_rn(ah, xh, p_neg(ph));
      pe = __ffma2_rn(ah, xl, pe);
      pe = __ffma2_rn(al, xh, pe);
      const dfp ts = p_two_sum(s2, ph);
      s2 = ts.hi;
      c2 = p_add(c2, p_add(ts.lo, pe));
    };
#pragma unroll
    for (int j = 0; j < kWarpN; j += 4) {
      const float4 xh = *reinterpret_cast<const float4*>(xs + j);
      const float4 xl = *reinterpret_cast<const float4*>(xs + kWarpN + j);
      acc(f.ah[j >> 1], f.al[j >> 1], make_float2(xh.x, xh.y), make_float2(xl.x, xl.y));
      acc(f.ah[(j >> 1) + 1], f.al[(j >> 1) + 1], make_float2(xh.z, xh.w), make_float2(xl.z, xl.w));
    }
    const df st = two_sum(s2.x, s2.y);
    const float s = st.hi, c = (c2.x + c2.y) + st.lo;
    const float r = lane < N ? s + c : 0.0f;
    __syncwarp();
    W.vec[lane] = r;
    __syncwarp();
    warp_gemv_neg_inv(f.t, W.vec, lane, y);
    y *= f.sc;
    if (lane < N) x = df_add_f(x, -y);
    const float nd = warp_max_f(lane < N ? fabsf(y) : 0.0f);
    bool done = nd <= 1e-15f * nx;
    if (!done && sweep >= 2) {
      const float rho = nd / nd_prev;
      done = rho < 0.5f && rho * nd <= 1e-13f * nx;
    }
    const bool stalled = sweep >= 2 && !(nd < 0.5f * nd_prev);  // no longer contracting
    const bool floor_ok = (stalled || sweep == kMaxRefineSweeps) && nd <= accept_floor * nx;
    if (done || floor_ok) {
      __syncwarp();
      W.xd[lane] = x;
      __syncwarp();
      if (at_floor) *at_floor = !done;
      return true;
    }
    if (stalled) {
      __syncwarp();
      W.xd[lane] = x;  // the last iterate, for a caller that refines further
      __syncwarp();
      return false;
    }
    nd_prev = nd;
  }
  __syncwarp();
  W.xd[lane] = x;
  __syncwarp();
  return false;
}

// Factor and solve one right-hand side.
__device__ __forceinline__ bool warp_solve(const df* A, const df* B, int N, int lane,
                                           const WarpScratch& W) {
  WarpFactor f;
  if (!warp_factor(A, N, lane, f, W)) return false;
  return warp_refine(f, B, N, lane, W);
}

}  // namespace gs
