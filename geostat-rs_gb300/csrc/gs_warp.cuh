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
// Refinement residuals b - A x use the double-float entries read from shared
// memory (compensated FP32 dot products, Ogita, Rump & Oishi 2005);
// corrections are register GEMVs with -A^{-1}.  One factorisation serves any
// number of right-hand sides (warp_refine).
#pragma once

#include "gs_solve.cuh"
#include "gs_pair.cuh"

namespace gs {

constexpr int kWarpN = 32;
// Floats of the published-row buffer: two alternating rows of kWarpN
// entries plus the pivot (padded to 16 bytes).
constexpr int kWarpRowFloats = 2 * (kWarpN + 4);

struct WarpScratch {
  float* row;  // kWarpRowFloats floats: the published pivot rows
  float* vec;  // 32 floats: broadcast vector
  df* xd;      // 32 df: solution (during a refinement: its hi parts, then its lo parts)
};

constexpr int kWarpN4 = kWarpN / 4;  // column quads of a register row

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

// Refinement sweeps before a system is handed to the FP64 solver; a sweep
// that no longer halves the correction ends the refinement earlier (the
// double-float residual of an ill-conditioned system has reached its limit).
constexpr int kMaxRefineSweeps = 8;

// The factorisation one lane holds: its row of -(sc A)^{-1} + 2I as column
// quads (so a published row is stored straight from aligned registers) and
// the power-of-two scale sc.  The matrix's own entries stay in shared memory
// (read through an accessor at(e) -> df of packed entry e), which keeps the
// lane's registers for the inverse.
struct WarpFactor {
  float4 t[kWarpN4];
  float sc;
};

// Entry (lane, j) of the packed symmetric matrix; rows and columns beyond N
// hold the identity.
template <class At>
__device__ __forceinline__ df warp_entry(At&& at, int N, int lane, int j) {
  df v = df_make(j == lane ? 1.0f : 0.0f, 0.0f);
  if (lane < N && j < N) v = at(lane >= j ? pk(lane, j) : pk(j, lane));
  return v;
}

// The lane's matrix row as the refinement reads it: pair(j, ah, al) gives
// the hi and lo parts of entries j and j + 1 (j even).  SharedRow reads them
// from shared memory at every use (registers stay free for the inverse);
// RegisterRow loads the row once, for a factorisation that serves several
// right-hand sides.
template <class At>
struct SharedRow {
  At at;
  int N, lane;
  __device__ __forceinline__ void pair(int j, float2& ah, float2& al) const {
    const df a0 = warp_entry(at, N, lane, j), a1 = warp_entry(at, N, lane, j + 1);
    ah = make_float2(a0.hi, a1.hi);
    al = make_float2(a0.lo, a1.lo);
  }
  __device__ __forceinline__ float hi(int j) const { return warp_entry(at, N, lane, j).hi; }
};
template <class At>
__device__ __forceinline__ SharedRow<At> shared_row(At at, int N, int lane) {
  return SharedRow<At>{at, N, lane};
}
struct RegisterRow {
  float2 h[kWarpN / 2], l[kWarpN / 2];
  template <class At>
  __device__ __forceinline__ void load(At&& at, int N, int lane) {
#pragma unroll
    for (int j = 0; j < kWarpN; j += 2) {
      const df a0 = warp_entry(at, N, lane, j), a1 = warp_entry(at, N, lane, j + 1);
      h[j >> 1] = make_float2(a0.hi, a1.hi);
      l[j >> 1] = make_float2(a0.lo, a1.lo);
    }
  }
  __device__ __forceinline__ void pair(int j, float2& ah, float2& al) const {
    ah = h[j >> 1];
    al = l[j >> 1];
  }
  __device__ __forceinline__ float hi(int j) const { return (j & 1) ? h[j >> 1].y : h[j >> 1].x; }
};

// FP32 inverse of the packed df matrix (N <= 32 unknowns; the lane's row
// `row`) by the sweep operator.  Returns false (uniformly in the warp) when a
// pivot is too small for FP32.
//
// Pivot k: lane k publishes its row in one of two alternating buffers, with
// the pivot entry replaced by d - 1 and d stored after the row; one
// __syncwarp, then every lane applies its packed FP32x2 update.  Lane k's
// next write to the same buffer (pivot k + 2) comes after the next pivot's
// __syncwarp, which every lane reaches only after reading this row.
template <class Row>
__device__ __forceinline__ bool warp_factor(const Row& row, int N, int lane, WarpFactor& f,
                                            const WarpScratch& W) {
  float amax = 0.0f;
#pragma unroll
  for (int q = 0; q < kWarpN4; ++q) {
    f.t[q] = make_float4(row.hi(4 * q), row.hi(4 * q + 1), row.hi(4 * q + 2), row.hi(4 * q + 3));
    if (lane < N)
      amax = fmaxf(amax, fmaxf(fmaxf(fabsf(f.t[q].x), fabsf(f.t[q].y)),
                               fmaxf(fabsf(f.t[q].z), fabsf(f.t[q].w))));
  }
  amax = warp_max_f(amax);
  f.sc = 1.0f;
  if (!(amax > 0.0f)) return false;
  // power-of-two scale: sc * max|A| in [0.5, 1), so every pivot is <= 1 and
  // the pivot lane's multiplier 1 - 1/d never cancels; the swept rows then
  // hold -(sc A)^{-1}, i.e. -A^{-1} / sc
  int ex = 0;
  frexpf(amax, &ex);
  f.sc = ldexpf(1.0f, -ex);
#pragma unroll
  for (int q = 0; q < kWarpN4; ++q) {
    if (lane < N && 4 * q < N) f.t[q].x *= f.sc;
    if (lane < N && 4 * q + 1 < N) f.t[q].y *= f.sc;
    if (lane < N && 4 * q + 2 < N) f.t[q].z *= f.sc;
    if (lane < N && 4 * q + 3 < N) f.t[q].w *= f.sc;
  }
  const float tol = 1e-6f * amax * f.sc;
  __syncwarp();  // the previous user of W.row is done with it
  for (int k = 0; k < N; ++k) {
    float* rb = W.row + (k & 1) * (kWarpN + 4);
    if (lane == k) {
#pragma unroll
      for (int q = 0; q < kWarpN4; ++q) *reinterpret_cast<float4*>(rb + 4 * q) = f.t[q];
      const float d = rb[k];
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

// Solves A x = B with the factorisation f and refines to ~1e-13 relative
// (residuals from the lane's matrix row `row`); on success W.xd[i] holds x_i.
// Returns false (uniformly) when the refinement stalls.
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
template <class Row>
__device__ __forceinline__ bool warp_refine(const WarpFactor& f, const Row& row, const df* B,
                                            int N, int lane, const WarpScratch& W,
                                            float accept_floor = 0.0f, bool* at_floor = nullptr) {
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
#pragma unroll
    for (int j = 0; j < kWarpN; j += 4) {
      const float4 xh = *reinterpret_cast<const float4*>(xs + j);
      const float4 xl = *reinterpret_cast<const float4*>(xs + kWarpN + j);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float2 ah, al;
        row.pair(j + 2 * h, ah, al);
        const float2 xh2 = h ? make_float2(xh.z, xh.w) : make_float2(xh.x, xh.y);
        const float2 xl2 = h ? make_float2(xl.z, xl.w) : make_float2(xl.x, xl.y);
        const float2 ph = __fmul2_rn(ah, xh2);
        float2 pe = __ffma2_rn(ah, xh2, p_neg(ph));
        pe = __ffma2_rn(ah, xl2, pe);
        pe = __ffma2_rn(al, xh2, pe);
        const dfp ts = p_two_sum(s2, ph);
        s2 = ts.hi;
        c2 = p_add(c2, p_add(ts.lo, pe));
      }
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

// Factor and solve one right-hand side (packed df matrix A).
__device__ __forceinline__ bool warp_solve(const df* A, const df* B, int N, int lane,
                                           const WarpScratch& W) {
  auto at = [&](int e) { return A[e]; };
  const auto row = shared_row(at, N, lane);
  WarpFactor f;
  if (!warp_factor(row, N, lane, f, W)) return false;
  return warp_refine(f, row, B, N, lane, W);
}

}  // namespace gs
