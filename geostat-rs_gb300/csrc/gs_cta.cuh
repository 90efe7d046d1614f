// gs_cta.cuh -- one small symmetric system per thread block: register-tiled
// L D L^T factorisation, triangular solves and double-float refinement.
//
// The packed lower-triangular double-float matrix A (entry (i, j), j <= i, at
// i(i+1)/2 + j) lives in shared memory.  For the factorisation each thread
// owns one 4x4 tile of the lower triangle in registers (tile (ib, jb),
// ib >= jb, numbered row by row); step k reads column k from a small shared
// buffer, applies the rank-1 update A_ij -= (A_ik / d_k) A_jk to its tile and
// the owners of column k+1 publish it -- one barrier per column.  The unit-
// lower factor is written packed (FP32) for the solves, which one warp runs
// while the others wait; refinement residuals b - A x are formed from the
// double-float entries in compensated FP32 (Ogita, Rump & Oishi 2005), two
// threads per row, and the solution is accumulated in FP64.
#pragma once

#include "gs_solve.cuh"

namespace gs {

struct CtaScratch {
  float* L;      // packed unit-lower factor
  float* DI;     // inverse pivots
  float* W;      // FP32 work vector
  float* colU;   // 2 x (4 * nbr) column buffers
  double* X;     // FP64 solution
  df* XD;        // solution as df
  double* red;   // block reduction scratch (>= 2 * warps doubles)
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

template <int BLOCK>
__device__ __forceinline__ float block_max_f(float v, double* red) {
  v = warp_max_f(v);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[w] = (double)v;
  __syncthreads();
  float r = 0.0f;
#pragma unroll
  for (int i = 0; i < BLOCK / 32; ++i) r = fmaxf(r, (float)red[i]);
  return r;
}

// Factors hi(A) (N x N) into S.L / S.DI.  Returns false (uniformly) when a
// pivot is too small for FP32.
template <int BLOCK>
__device__ bool cta_ldl(const df* A, int N, const CtaScratch& S) {
  const int tid = threadIdx.x;
  const int nbr = (N + 3) >> 2;
  const int stride = nbr * 4;
  int ib = 0, jb = 0;
  const bool own = tile_of(tid, nbr, ib, jb);
  float T[4][4];
  float amax = 0.0f;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int i = 4 * ib + a, j = 4 * jb + b;
      float v = 0.0f;
      if (own) {
        if (i < N && j < N) v = i >= j ? A[pk(i, j)].hi : A[pk(j, i)].hi;
        else if (i == j) v = 1.0f;
      }
      T[a][b] = v;
      amax = fmaxf(amax, fabsf(v));
    }
  amax = block_max_f<BLOCK>(amax, S.red);
  const float tol = 1e-6f * amax;
  if (own && jb == 0) {
#pragma unroll
    for (int a = 0; a < 4; ++a) S.colU[4 * ib + a] = T[a][0];
  }
  __syncthreads();
  for (int k = 0; k < N; ++k) {
    const float* cu = S.colU + (k & 1) * stride;
    const float d = cu[k];
    if (!(fabsf(d) > tol)) return false;  // same value for every thread
    const float invd = 1.0f / d;
    const int kb = k >> 2, kc = k & 3;
    if (own && jb >= kb) {
      if (jb == kb) {
        // column k is final: publish the scaled multipliers of this tile
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const int i = 4 * ib + a;
          if (i > k && i < N) S.L[pk(i, k)] = sel4(T[a], kc) * invd;
        }
        if (ib == kb && tid == (kb * (kb + 1) / 2 + kb)) S.DI[k] = invd;
      }
      float lr[4], cc[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) lr[a] = cu[4 * ib + a] * invd;
#pragma unroll
      for (int b = 0; b < 4; ++b) cc[b] = cu[4 * jb + b];
      const bool edge = (ib == kb) || (jb == kb);
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const bool upd = !edge || ((4 * ib + a) > k && (4 * jb + b) > k);
          if (upd) T[a][b] = fmaf(-lr[a], cc[b], T[a][b]);
        }
    }
    const int kn = k + 1;
    if (own && kn < N && jb == (kn >> 2)) {
      float* cn = S.colU + (kn & 1) * stride;
      const int kcn = kn & 3;
#pragma unroll
      for (int a = 0; a < 4; ++a) cn[4 * ib + a] = sel4(T[a], kcn);
    }
    __syncthreads();
  }
  return true;
}

// Solves A X = B with the factor from cta_ldl and refines; returns false
// (uniformly) when the refinement does not contract to ~1e-13 relative.
template <int BLOCK>
__device__ bool cta_refine(const df* A, const df* B, int N, const CtaScratch& S) {
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const bool w0 = tid < 32;
  if (w0) {
    for (int i = lane; i < N; i += 32) S.W[i] = B[i].hi;
    __syncwarp();
    ldl_solve(S.L, S.DI, S.W, N, lane);
    double nx = 0.0;
    for (int i = lane; i < N; i += 32) {
      const double xi = (double)S.W[i];
      S.X[i] = xi;
      S.XD[i] = df_from_double(xi);
      nx = fmax(nx, fabs(xi));
    }
    nx = warp_max_d(nx);
    if (lane == 0) S.red[0] = nx;
  }
  __syncthreads();
  double nd_prev = S.red[0];
  for (int sweep = 1; sweep <= 4; ++sweep) {
    // residual: two threads per row, each over half the columns
    for (int rbase = 0; rbase < N; rbase += BLOCK / 2) {
      const int row = rbase + (tid >> 1), half = tid & 1;
      float s = 0.0f, c = 0.0f;
      if (row < N) {
        const int j0 = half ? (N >> 1) : 0, j1 = half ? N : (N >> 1);
        if (!half) {
          s = B[row].hi;
          c = B[row].lo;
        }
        for (int jj = j0; jj < j1; ++jj) {
          const df aij = jj <= row ? A[pk(row, jj)] : A[pk(jj, row)];
          const df xj = S.XD[jj];
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
      // combine the two halves (same pairing and order every time)
      const float s2 = __shfl_down_sync(0xffffffffu, s, 1);
      const float c2 = __shfl_down_sync(0xffffffffu, c, 1);
      if (row < N && !half) {
        const float tsum = __fadd_rn(s, s2);
        const float bb = __fsub_rn(tsum, s);
        const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(tsum, bb)), __fsub_rn(s2, bb));
        S.W[row] = tsum + (c + c2 + e);
      }
    }
    __syncthreads();
    if (w0) {
      ldl_solve(S.L, S.DI, S.W, N, lane);
      double nd = 0.0, nx = 0.0;
      for (int i = lane; i < N; i += 32) {
        const double dlt = (double)S.W[i];
        const double xi = S.X[i] + dlt;
        S.X[i] = xi;
        S.XD[i] = df_from_double(xi);
        nd = fmax(nd, fabs(dlt));
        nx = fmax(nx, fabs(xi));
      }
      nd = warp_max_d(nd);
      nx = warp_max_d(nx);
      if (lane == 0) {
        int dec = 0;  // 0 continue, 1 converged
        if (nd <= 1e-15 * nx) dec = 1;
        else if (sweep >= 2) {
          const double rho = nd / nd_prev;
          if (rho < 0.5 && rho * nd <= 1e-13 * nx) dec = 1;
        }
        S.flag[0] = dec;
        S.red[1] = nd;
      }
    }
    __syncthreads();
    const int dec = S.flag[0];
    nd_prev = S.red[1];
    __syncthreads();
    if (dec) return true;
  }
  return false;
}

}  // namespace gs
