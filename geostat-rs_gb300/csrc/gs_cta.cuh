// gs_cta.cuh -- one small symmetric system per thread block: register-tiled
// FP32 inversion and double-float iterative refinement.
//
// The packed lower-triangular double-float matrix A (entry (i, j), j <= i, at
// i(i+1)/2 + j) lives in shared memory.  Each thread owns one 4x4 tile of the
// lower triangle (tile (ib, jb), ib >= jb, numbered row by row) in registers.
// The FP32 hi parts are inverted in place with the symmetric sweep operator
// applied one 4x4 block at a time (block Gauss-Jordan without pivoting: for
// pivot block K with P = A_KK, A_IJ -= A_IK P^{-1} A_KJ off block row/column
// K, A_IK = A_IK P^{-1}, A_KK = -P^{-1}; after every block the tiles hold
// -A^{-1}).  No pivoting is needed for a positive-definite covariance block
// bordered by drift rows: the pivots are those of A = L D L^T, positive for
// the covariance block and negative for the drift block.  Per block step the
// diagonal-tile owner inverts P in registers, the panel owners publish A_IK
// and A_IK P^{-1}, and every other tile applies a 64-FMA update -- two
// barriers per four pivots.
//
// The solution and its corrections are tile-parallel matrix-vector products
// from the registers, reduced in a fixed order (deterministic).  Refinement
// residuals b - A x use the double-float entries in compensated FP32
// (Ogita, Rump & Oishi, "Accurate sum and dot product", 2005), two threads per
// row; the solution accumulates in FP64.
#pragma once

#include "gs_solve.cuh"

namespace gs {

// Panel blocks are 4x4 floats padded to a 20-float stride, so the float4 rows
// of blocks read by one warp fall on distinct banks.
#define GS_PB 20

struct CtaScratch {
  float* W;      // FP32 work vector (residual)
  float* pan;    // 2 x nbr x PB: panel blocks A_IK, by block-step parity
  float* lp;     // 2 x nbr x PB: A_IK P^{-1}, by parity
  float* pinv;   // 2 x 16: P^{-1}, by parity
  float* P;      // nbr x nbr x 4 partial products
  df* XD;        // solution (double-float)
  float* red;    // block reduction scratch (>= 2 * warps floats)
  int* flag;     // shared decision word
};

// Tile (ib, jb) of thread t in the row-by-row numbering of the lower
// triangle of an nbr x nbr tile grid; returns false for idle threads.
__device__ __forceinline__ bool tile_of(int t, int nbr, int& ib, int& jb) {
  if (t >= nbr * (nbr + 1) / 2) return false;
  int r = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
  while ((r + 1) * (r + 2) / 2 <= t) ++r;
  while (r * (r + 1) / 2 > t) --r;
  ib = r;
  jb = t - r * (r + 1) / 2;
  return true;
}

// row[c] for a runtime c in 0..3 without indexing the register array
__device__ __forceinline__ float sel4(const float* row, int c) {
  float v = row[0];
  v = c == 1 ? row[1] : v;
  v = c == 2 ? row[2] : v;
  v = c == 3 ? row[3] : v;
  return v;
}

__device__ __forceinline__ void block_max2(float& a, float& b, float* red) {
  a = warp_max_f(a);
  b = warp_max_f(b);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) {
    red[2 * w] = a;
    red[2 * w + 1] = b;
  }
  __syncthreads();
  a = 0.0f;
  b = 0.0f;
  const int nw = blockDim.x >> 5;
  for (int i = 0; i < nw; ++i) {
    a = fmaxf(a, red[2 * i]);
    b = fmaxf(b, red[2 * i + 1]);
  }
}

// In-register sweep of a symmetric 4x4 block: P -> -P^{-1}.  Returns false
// when a pivot is not larger than tol in magnitude.
__device__ __forceinline__ bool inv4_sweep(float (&P)[4][4], float tol) {
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float d = P[k][k];
    ok = ok && (fabsf(d) > tol);
    const float invd = __fdividef(1.0f, d);
    float u[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) u[i] = P[i][k];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (i == k && j == k) P[i][j] = -invd;
        else if (i == k) P[i][j] = u[j] * invd;
        else if (j == k) P[i][j] = u[i] * invd;
        else P[i][j] = fmaf(-u[i] * invd, u[j], P[i][j]);
      }
  }
  return ok;
}

// Writes this tile's share of y = T_full r (T symmetric, lower tiles) to P.
__device__ __forceinline__ void tile_gemv_partial(const float (&T)[4][4], bool own, int ib, int jb,
                                                  int nbr, const float* r, float* P) {
  if (!own) return;
  float rc[4], rr[4];
#pragma unroll
  for (int b = 0; b < 4; ++b) rc[b] = r[4 * jb + b];
#pragma unroll
  for (int a = 0; a < 4; ++a) rr[a] = r[4 * ib + a];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    float s = 0.0f;
#pragma unroll
    for (int b = 0; b < 4; ++b) s = fmaf(T[a][b], rc[b], s);
    P[(ib * nbr + jb) * 4 + a] = s;
  }
  if (ib != jb) {
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      float s = 0.0f;
#pragma unroll
      for (int a = 0; a < 4; ++a) s = fmaf(T[a][b], rr[a], s);
      P[(jb * nbr + ib) * 4 + b] = s;
    }
  }
}

// Solves A X = B (N unknowns) and refines to ~1e-13 relative.  Returns false
// (uniformly) when a pivot is too small for FP32 or the refinement stalls;
// the caller then re-solves in FP64.  S.pan and S.lp need 2 * nbr * GS_PB
// floats (GS_PB = 20), S.pinv 32, S.P nbr * nbr * 4, S.W 4 * nbr.
static __device__ bool cta_solve(const df* A, const df* B, int N, const CtaScratch& S) {
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const int nbr = (N + 3) >> 2;
  const int stride = nbr * 4;
  int ib = 0, jb = 0;
  const bool own = tile_of(tid, nbr, ib, jb);
  float T[4][4];
  float amax = 0.0f, dummy = 0.0f;
  if (tid == 0) S.flag[0] = 0;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int i = 4 * ib + a, j = 4 * jb + b;
      float v = 0.0f;
      if (own) {
        if (i < N && j < N) v = i >= j ? A[pk(i, j)].hi : A[pk(j, i)].hi;
        else if (i == j) v = 1.0f;  // padding: decoupled unit pivots
      }
      T[a][b] = v;
      amax = fmaxf(amax, fabsf(v));
    }
  block_max2(amax, dummy, S.red);
  const float tol = 1e-6f * amax;
  for (int K = 0; K < nbr; ++K) {
    const int par = K & 1;
    float* pan = S.pan + par * nbr * GS_PB;
    float* lp = S.lp + par * nbr * GS_PB;
    float* pinv = S.pinv + par * 16;
    // A: invert the diagonal block; publish the panel blocks A_IK (I != K)
    if (own) {
      if (ib == K && jb == K) {
        const bool ok = inv4_sweep(T, tol);
        if (!ok) S.flag[0] = 1;
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) pinv[a * 4 + b] = -T[a][b];
      } else if (jb == K) {
#pragma unroll
        for (int a = 0; a < 4; ++a)
          *reinterpret_cast<float4*>(pan + ib * GS_PB + a * 4) =
              make_float4(T[a][0], T[a][1], T[a][2], T[a][3]);
      } else if (ib == K) {
#pragma unroll
        for (int b = 0; b < 4; ++b)
          *reinterpret_cast<float4*>(pan + jb * GS_PB + b * 4) =
              make_float4(T[0][b], T[1][b], T[2][b], T[3][b]);
      }
    }
    __syncthreads();
    if (S.flag[0]) return false;  // the same value in every thread
    // B: panel owners form A_IK P^{-1}
    if (own && (jb == K || ib == K) && !(ib == K && jb == K)) {
      const int I = jb == K ? ib : jb;
      float pv[4][4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const float4 r = *reinterpret_cast<const float4*>(pinv + c * 4);
        pv[c][0] = r.x; pv[c][1] = r.y; pv[c][2] = r.z; pv[c][3] = r.w;
      }
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const float4 r = *reinterpret_cast<const float4*>(pan + I * GS_PB + a * 4);
        const float ra[4] = {r.x, r.y, r.z, r.w};
        float o[4];
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          float acc = 0.0f;
#pragma unroll
          for (int c = 0; c < 4; ++c) acc = fmaf(ra[c], pv[c][b], acc);
          o[b] = acc;
        }
        *reinterpret_cast<float4*>(lp + I * GS_PB + a * 4) = make_float4(o[0], o[1], o[2], o[3]);
      }
    }
    __syncthreads();
    // C: update every tile
    if (own && !(ib == K && jb == K)) {
      if (jb == K) {
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const float4 r = *reinterpret_cast<const float4*>(lp + ib * GS_PB + a * 4);
          T[a][0] = r.x; T[a][1] = r.y; T[a][2] = r.z; T[a][3] = r.w;
        }
      } else if (ib == K) {
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const float4 r = *reinterpret_cast<const float4*>(lp + jb * GS_PB + b * 4);
          T[0][b] = r.x; T[1][b] = r.y; T[2][b] = r.z; T[3][b] = r.w;
        }
      } else {
        // T -= (A_IK P^{-1}) A_JK^T
        float li[4][4], pj[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const float4 r = *reinterpret_cast<const float4*>(lp + ib * GS_PB + a * 4);
          li[a][0] = r.x; li[a][1] = r.y; li[a][2] = r.z; li[a][3] = r.w;
          const float4 q = *reinterpret_cast<const float4*>(pan + jb * GS_PB + a * 4);
          pj[a][0] = q.x; pj[a][1] = q.y; pj[a][2] = q.z; pj[a][3] = q.w;
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            float acc = T[a][b];
#pragma unroll
            for (int c = 0; c < 4; ++c) acc = fmaf(-li[a][c], pj[b][c], acc);
            T[a][b] = acc;
          }
      }
    }
  }
  // T now holds -A^{-1}.  x0 = A^{-1} b_hi
  float* w = S.W;
  for (int i = tid; i < stride; i += nthr) w[i] = i < N ? B[i].hi : 0.0f;
  __syncthreads();
  tile_gemv_partial(T, own, ib, jb, nbr, w, S.P);
  __syncthreads();
  // |x| from the FP32 first solution; refinement moves x by ~1e-4 relative
  float nx = 0.0f;
  for (int i = tid; i < N; i += nthr) {
    float s = 0.0f;
    for (int q = 0; q < nbr; ++q) s += S.P[((i >> 2) * nbr + q) * 4 + (i & 3)];
    S.XD[i] = df_make(-s, 0.0f);
    nx = fmaxf(nx, fabsf(s));
  }
  block_max2(nx, dummy, S.red);
  float nd_prev = nx;
  for (int sweep = 1; sweep <= 4; ++sweep) {
    // residual r = b - A x: two threads per row, each over half the columns
    for (int rbase = 0; rbase < N; rbase += nthr / 2) {
      const int row = rbase + (tid >> 1), half = tid & 1;
      float s = 0.0f, c = 0.0f;
      if (row < N) {
        const int j0 = half ? (N >> 1) : 0, j1 = half ? N : (N >> 1);
        if (!half) {
          s = B[row].hi;
          c = B[row].lo;
        }
        // entries (row, jj): packed row for jj <= row, packed column after
        const int jmid = min(j1, row + 1);
        int idx = pk(row, 0) + j0;
        int idx2 = pk(max(j0, row + 1), row);
        for (int jj = j0; jj < j1; ++jj) {
          const bool lower = jj < jmid;
          const df aij = A[lower ? idx : idx2];
          if (lower) ++idx;
          else idx2 += jj + 1;
          const df xj = S.XD[jj];
          // TwoProduct / TwoSum with explicit roundings (no contraction)
          const float ph = __fmul_rn(-aij.hi, xj.hi);
          float pe = __fmaf_rn(-aij.hi, xj.hi, -ph);
          pe = __fmaf_rn(-aij.hi, xj.lo, pe);
          pe = __fmaf_rn(-aij.lo, xj.hi, pe);
          const float tsum = __fadd_rn(s, ph);
          const float bb = __fsub_rn(tsum, s);
          const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(tsum, bb)), __fsub_rn(ph, bb));
          s = tsum;
          c += e + pe;
        }
      }
      const float s2 = __shfl_down_sync(0xffffffffu, s, 1);
      const float c2 = __shfl_down_sync(0xffffffffu, c, 1);
      if (row < N && !half) {
        const float tsum = __fadd_rn(s, s2);
        const float bb = __fsub_rn(tsum, s);
        const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(tsum, bb)), __fsub_rn(s2, bb));
        w[row] = tsum + (c + c2 + e);
      }
    }
    __syncthreads();
    tile_gemv_partial(T, own, ib, jb, nbr, w, S.P);
    __syncthreads();
    float nd = 0.0f;
    for (int i = tid; i < N; i += nthr) {
      float s = 0.0f;
      for (int q = 0; q < nbr; ++q) s += S.P[((i >> 2) * nbr + q) * 4 + (i & 3)];
      S.XD[i] = df_add_f(S.XD[i], -s);
      nd = fmaxf(nd, fabsf(s));
    }
    block_max2(nd, dummy, S.red);
    if (nd <= 1e-15f * nx) return true;
    if (sweep >= 2) {
      const float rho = nd / nd_prev;
      if (rho < 0.5f && rho * nd <= 1e-13f * nx) return true;
    }
    nd_prev = nd;
  }
  return false;
}

}  // namespace gs
