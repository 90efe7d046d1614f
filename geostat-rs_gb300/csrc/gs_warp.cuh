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

namespace gs {

constexpr int kWarpN = 32;

struct WarpScratch {
  float* row;  // 32 (+1 for d) floats: the published pivot row
  float* vec;  // 32 floats: broadcast vector
  df* xd;      // 32 df: solution
};

// The factorisation one lane holds: its row of the double-float matrix
// (ah + al) and of -(sc A)^{-1} + 2I (t), with the power-of-two scale sc.
struct WarpFactor {
  float ah[kWarpN], al[kWarpN], t[kWarpN];
  float sc;
};

// Loads row `lane` of the packed df matrix A (N x N) into registers; rows and
// columns beyond N hold the identity.
__device__ __forceinline__ void warp_load_rows(const df* A, int N, int lane, float (&ah)[kWarpN],
                                               float (&al)[kWarpN]) {
#pragma unroll
  for (int j = 0; j < kWarpN; ++j) {
    df v = df_make(j == lane ? 1.0f : 0.0f, 0.0f);
    if (lane < N && j < N) v = lane >= j ? A[pk(lane, j)] : A[pk(j, lane)];
    ah[j] = v.hi;
    al[j] = v.lo;
  }
}

__device__ __forceinline__ void warp_gemv_neg_inv(const float (&t)[kWarpN], const float* vec,
                                                  int lane, float& y) {
  // y = (-A^{-1}) v with the +2 diagonal offset removed
  float s = 0.0f;
#pragma unroll
  for (int j = 0; j < kWarpN; j += 4) {
    const float4 v = *reinterpret_cast<const float4*>(vec + j);
    s = fmaf(t[j], v.x, s);
    s = fmaf(t[j + 1], v.y, s);
    s = fmaf(t[j + 2], v.z, s);
    s = fmaf(t[j + 3], v.w, s);
  }
  y = fmaf(-2.0f, vec[lane], s);
}

// FP32 inverse of the packed df matrix A (N <= 32 unknowns).  Returns false
// (uniformly in the warp) when a pivot is too small for FP32.
__device__ __forceinline__ bool warp_factor(const df* A, int N, int lane, WarpFactor& f,
                                            const WarpScratch& W) {
  warp_load_rows(A, N, lane, f.ah, f.al);
  float amax = 0.0f;
#pragma unroll
  for (int j = 0; j < kWarpN; ++j) amax = fmaxf(amax, lane < N ? fabsf(f.ah[j]) : 0.0f);
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
  for (int j = 0; j < kWarpN; ++j) f.t[j] = (lane < N && j < N) ? f.ah[j] * f.sc : f.ah[j];
  const float tol = 1e-6f * amax * f.sc;
  for (int k = 0; k < N; ++k) {
    if (lane == k) {
#pragma unroll
      for (int j = 0; j < kWarpN; j += 4)
        *reinterpret_cast<float4*>(W.row + j) =
            make_float4(f.t[j], f.t[j + 1], f.t[j + 2], f.t[j + 3]);
    }
    __syncwarp();
    const float d = W.row[k];
    __syncwarp();
    if (lane == k) W.row[k] = d - 1.0f;
    __syncwarp();
    if (!(fabsf(d) > tol)) return false;  // the same value in every lane
    const float invd = __fdividef(1.0f, d);  // an approximate inverse suffices
    const float l = lane == k ? 1.0f - invd : W.row[lane] * invd;
#pragma unroll
    for (int j = 0; j < kWarpN; j += 4) {
      const float4 r = *reinterpret_cast<const float4*>(W.row + j);
      f.t[j] = fmaf(-l, r.x, f.t[j]);
      f.t[j + 1] = fmaf(-l, r.y, f.t[j + 1]);
      f.t[j + 2] = fmaf(-l, r.z, f.t[j + 2]);
      f.t[j + 3] = fmaf(-l, r.w, f.t[j + 3]);
    }
    __syncwarp();
  }
  return true;
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
    // residual of row `lane`: b - A x, compensated, x broadcast as df
    __syncwarp();
    W.xd[lane] = x;
    __syncwarp();
    float s = lane < N ? B[lane].hi : 0.0f, c = lane < N ? B[lane].lo : 0.0f;
#pragma unroll
    for (int j = 0; j < kWarpN; ++j) {
      const df xj = W.xd[j];
      const float ph = __fmul_rn(-f.ah[j], xj.hi);
      float pe = __fmaf_rn(-f.ah[j], xj.hi, -ph);
      pe = __fmaf_rn(-f.ah[j], xj.lo, pe);
      pe = __fmaf_rn(-f.al[j], xj.hi, pe);
      const float tsum = __fadd_rn(s, ph);
      const float bb = __fsub_rn(tsum, s);
      const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(tsum, bb)), __fsub_rn(ph, bb));
      s = tsum;
      c += e + pe;
    }
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
    if (stalled) return false;
    nd_prev = nd;
  }
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
