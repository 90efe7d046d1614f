// gs_krige.cu -- per-target kriging solves.
//
// K3 (krige_mixed_kernel): one warp per target system.  The system
// (kriging.rs:527-567 build_lhs + the right-hand side of predict_inner,
// kriging.rs:569-612) is assembled in shared memory as packed lower-triangular
// double-float entries; the FP32 hi parts are factored A = L D L^T without
// pivoting (the covariance block is positive definite, the drift block's
// Schur complement negative definite); the solution is refined with
// residuals b - A x formed from the double-float entries in compensated FP32
// (Ogita-Rump-Oishi Dot2) and accumulated in FP64; the outputs
// (kriging.rs:614-643) are FP64 sums.  A system whose refinement does not
// contract to ~1e-13 relative, or whose pivot is too small for FP32, is
// flagged for the FP64 solver.
//
// K3' (krige_fp64_kernel): one system per thread, the reference's own
// algorithm in FP64 -- build_lhs, LU with partial pivoting and its singular
// test (linalg.rs:27-111), the same summation order for the outputs.  Each
// thread's matrix lives in a global scratch slab, interleaved across threads
// so neighbouring threads touch neighbouring addresses.
#include <algorithm>
#include <cmath>

#include "gs_internal.h"
#include "gs_krige.cuh"
#include "gs_solve.cuh"

namespace gs {

namespace {

// fill_basis (kriging.rs:410-439) in FP64.
template <int D>
__device__ __forceinline__ void fill_basis(const KrigeArgs& a, const double* pt,
                                           const double* drow, double* out) {
  switch (a.method) {
    case GS_ORDINARY:
      out[0] = 1.0;
      break;
    case GS_UNIVERSAL: {
      double xn[3];
#pragma unroll
      for (int d = 0; d < D; ++d) xn[d] = (pt[d] - a.center[d]) / a.scale;
      out[0] = 1.0;
#pragma unroll
      for (int d = 0; d < D; ++d) out[1 + d] = xn[d];
      if (a.uk_degree == 2) {
        int idx = 1 + D;
#pragma unroll
        for (int u = 0; u < D; ++u)
#pragma unroll
          for (int v = u; v < D; ++v) out[idx++] = xn[u] * xn[v];
      }
      break;
    }
    case GS_EXTERNAL_DRIFT:
      out[0] = 1.0;
      for (int k = 0; k < a.nv; ++k) out[1 + k] = (drow[k] - a.dmean[k]) / a.dscale[k];
      break;
    default:
      break;
  }
}

template <int D>
__global__ void __launch_bounds__(128) krige_mixed_kernel(KrigeArgs a, DevModel m, ExpTable tab_g,
                                                          DfConsts kc, uint8_t* flag,
                                                          size_t per_warp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ ExpTable tab;
  for (int i = threadIdx.x; i < 64; i += blockDim.x) {
    tab.hi[i] = tab_g.hi[i];
    tab.lo[i] = tab_g.lo[i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const int NMAX = a.nmax;
  const int NP = (NMAX * (NMAX + 1)) >> 1;
  const Frames fr = frames_of(m);
  const int NBMAX = GS_MIXED_MAX_NEIGHBORS;
  unsigned char* base = smem_raw + (size_t)wib * per_warp;
  df* A = reinterpret_cast<df*>(base);
  df* V = A + NP;                                   // [frame][i][d]
  df* B = V + fr.nf * NBMAX * D;                    // rhs
  df* XD = B + NMAX;                                // x as df
  double* X = reinterpret_cast<double*>(XD + NMAX); // FP64 solution
  double* Z = X + NMAX;                             // neighbour values
  float* L = reinterpret_cast<float*>(Z + NBMAX);
  float* W = L + NP;
  float* DI = W + NMAX;

  for (int64_t it = (int64_t)blockIdx.x * wpb + wib; it < a.ntl; it += (int64_t)gridDim.x * wpb) {
    const int64_t t = a.tlist ? a.tlist[it] : it;
    const int n = a.nbc[t];
    const int p = a.p;
    uint8_t st = GS_ST_OK;
    if (n < 0) st = GS_ST_CAPACITY;
    else if (n < a.min_nb) st = GS_ST_NO_NEIGHBORS;
    else if (n < p) st = GS_ST_INSUFFICIENT_DATA;
    if (st != GS_ST_OK) {
      if (lane == 0) {
        a.out_v[t] = __longlong_as_double(0x7ff8000000000000ll);
        a.out_var[t] = __longlong_as_double(0x7ff8000000000000ll);
        if (a.out_lag) a.out_lag[t] = __longlong_as_double(0x7ff8000000000000ll);
        a.out_st[t] = st;
        flag[t] = 0;
      }
      continue;
    }
    if (n > NBMAX) {
      if (lane == 0) flag[t] = 1;
      __syncwarp();
      continue;
    }
    const int N = n + p;
    double tp[3] = {a.tx[t], a.ty[t], D == 3 ? a.tz[t] : 0.0};
    // --- per-neighbour data: frames, values, rhs, drift rows -----------
    for (int i = lane; i < n; i += 32) {
      const int idx = a.nb[t * (int64_t)a.kout + i];
      double pp[3] = {a.x[idx], a.y[idx], D == 3 ? a.z[idx] : 0.0};
      double u[3];
      bool zero = true;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        u[d] = pp[d] - tp[d];
        zero = zero && (u[d] == 0.0);
      }
      df ud[3];
#pragma unroll
      for (int d = 0; d < D; ++d) ud[d] = df_from_double(u[d]);
      df h[GS_MAX_STRUCTURES + 1];
      frame_coords<D>(m, fr, ud, V, NBMAX, i, h);
      B[i] = zero ? m.c0_df : cov_from_h(m, fr, h, tab, kc);
      Z[i] = a.val[idx];
      // diagonal and drift entries of row i
      df diag = m.c0_df;
      if (a.meas_err) diag = df_add(diag, df_from_double(a.meas_err[idx]));
      A[pk(i, i)] = diag;
      if (p > 0) {
        double f[GS_MIXED_MAX_DRIFT];
        fill_basis<D>(a, pp, a.drift ? a.drift + (int64_t)idx * a.nv : nullptr, f);
        for (int k = 0; k < p; ++k) A[pk(n + k, i)] = df_from_double(f[k]);
      }
    }
    if (lane < p) {
      double f[GS_MIXED_MAX_DRIFT];
      fill_basis<D>(a, tp, a.tdrift ? a.tdrift + t * a.nv : nullptr, f);
      B[n + lane] = df_from_double(f[lane]);
    }
    for (int q = lane; q < p * (p + 1) / 2; q += 32) {
      int r = 0;
      while ((r + 1) * (r + 2) / 2 <= q) ++r;
      int c = q - r * (r + 1) / 2;
      A[pk(n + r, n + c)] = df_make(0.0f, 0.0f);
    }
    __syncwarp();
    // --- covariance block, strictly lower part -------------------------
    {
      const int npairs = (n * (n - 1)) >> 1;
      int i = 1, j = lane;
      while (j >= i && i < n) {
        j -= i;
        ++i;
      }
      for (int q = lane; q < npairs; q += 32) {
        df h[GS_MAX_STRUCTURES + 1];
        for (int f = 0; f < fr.nf; ++f)
          h[f] = norm_df<D>(&V[(f * NBMAX + i) * D], &V[(f * NBMAX + j) * D]);
        A[pk(i, j)] = cov_from_h(m, fr, h, tab, kc);
        j += 32;
        while (j >= i && i < n) {
          j -= i;
          ++i;
        }
      }
    }
    __syncwarp();
    // --- FP32 L D L^T, FP64-accumulated refinement --------------------
    const bool bad = !ldl_refine_solve(A, B, L, DI, W, X, XD, N, lane);
    if (bad) {
      if (lane == 0) flag[t] = 1;
      __syncwarp();
      continue;
    }
    // --- outputs (FP64) ------------------------------------------------
    double sv = 0.0, sr = 0.0;
    if (a.method == GS_SIMPLE) {
      for (int i = lane; i < n; i += 32) {
        sv += X[i] * (Z[i] - a.sk_mean);
        sr += X[i] * df_to_double(B[i]);
      }
    } else {
      for (int i = lane; i < n; i += 32) sv += X[i] * Z[i];
      for (int i = lane; i < N; i += 32) sr += X[i] * df_to_double(B[i]);
    }
    sv = warp_sum_d(sv);
    sr = warp_sum_d(sr);
    if (lane == 0) {
      const double val = a.method == GS_SIMPLE ? a.sk_mean + sv : sv;
      const double var = fmax(m.c0 - sr, 0.0);
      a.out_v[t] = val;
      a.out_var[t] = var;
      if (a.out_lag)
        a.out_lag[t] = a.method == GS_SIMPLE ? __longlong_as_double(0x7ff8000000000000ll) : X[n];
      a.out_st[t] = GS_ST_OK;
      flag[t] = 0;
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------- FP64 path --
template <int D>
__global__ void __launch_bounds__(128) krige_fp64_kernel(KrigeArgs a, DevModel m, double* scratch,
                                                         int64_t T) {
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (tid >= T) return;
  const int NMAX = a.nmax;
  // element e of this thread's slab lives at S[e * T]
  double* S = scratch + tid;
  auto AT = [&](int r, int c, int N) -> double& { return S[(int64_t)(r * N + c) * T]; };
  double* Bv = scratch + (int64_t)NMAX * NMAX * T + tid;  // rhs / solution
  double* B0 = Bv + (int64_t)NMAX * T;                     // original rhs
  const double kNaN = __longlong_as_double(0x7ff8000000000000ll);
  for (int64_t it = tid; it < a.ntl; it += T) {
    const int64_t t = a.tlist ? a.tlist[it] : it;
    const int n = a.nbc[t];
    const int p = a.p;
    uint8_t st = GS_ST_OK;
    if (n < 0) st = GS_ST_CAPACITY;
    else if (n < a.min_nb) st = GS_ST_NO_NEIGHBORS;
    else if (n < p) st = GS_ST_INSUFFICIENT_DATA;
    else if (n + p > NMAX) st = GS_ST_CAPACITY;
    const uint8_t fb = a.tlist ? GS_ST_FP64_RESOLVED : 0;
    if (st != GS_ST_OK) {
      a.out_v[t] = kNaN;
      a.out_var[t] = kNaN;
      if (a.out_lag) a.out_lag[t] = kNaN;
      a.out_st[t] = st;
      continue;
    }
    const int N = n + p;
    const int32_t* nbt = a.nb + t * (int64_t)a.kout;
    double tp[3] = {a.tx[t], a.ty[t], D == 3 ? a.tz[t] : 0.0};
    // build_lhs (kriging.rs:527-567)
    for (int r = 0; r < N; ++r)
      for (int c = 0; c < N; ++c) AT(r, c, N) = 0.0;
    for (int ii = 0; ii < n; ++ii) {
      const int i = nbt[ii];
      double pi[3] = {a.x[i], a.y[i], D == 3 ? a.z[i] : 0.0};
      AT(ii, ii, N) = m.c0 + (a.meas_err ? a.meas_err[i] : 0.0);
      for (int jj = ii + 1; jj < n; ++jj) {
        const int j = nbt[jj];
        double h[3] = {pi[0] - a.x[j], pi[1] - a.y[j], D == 3 ? pi[2] - a.z[j] : 0.0};
        const double c = cov_fp64<D>(m, h);
        AT(ii, jj, N) = c;
        AT(jj, ii, N) = c;
      }
      if (p > 0) {
        double f[GS_MIXED_MAX_DRIFT];
        fill_basis<D>(a, pi, a.drift ? a.drift + (int64_t)i * a.nv : nullptr, f);
        for (int k = 0; k < p; ++k) {
          AT(ii, n + k, N) = f[k];
          AT(n + k, ii, N) = f[k];
        }
      }
      double h[3] = {pi[0] - tp[0], pi[1] - tp[1], D == 3 ? pi[2] - tp[2] : 0.0};
      const double bi = cov_fp64<D>(m, h);
      Bv[(int64_t)ii * T] = bi;
      B0[(int64_t)ii * T] = bi;
    }
    if (p > 0) {
      double f[GS_MIXED_MAX_DRIFT];
      fill_basis<D>(a, tp, a.tdrift ? a.tdrift + t * a.nv : nullptr, f);
      for (int k = 0; k < p; ++k) {
        Bv[(int64_t)(n + k) * T] = f[k];
        B0[(int64_t)(n + k) * T] = f[k];
      }
    }
    // lu_factor (linalg.rs:27-76) fused with Lu::solve's row swaps
    double scale = 0.0;
    for (int r = 0; r < N; ++r)
      for (int c = 0; c < N; ++c) scale = fmax(scale, fabs(AT(r, c, N)));
    scale = fmax(scale, 2.2250738585072014e-308);
    bool singular = false;
    for (int k = 0; k < N && !singular; ++k) {
      int pv = k;
      double mx = fabs(AT(k, k, N));
      for (int i = k + 1; i < N; ++i) {
        const double v = fabs(AT(i, k, N));
        if (v > mx) {
          mx = v;
          pv = i;
        }
      }
      if (mx < 1e-12 * scale) {
        singular = true;
        break;
      }
      if (pv != k) {
        for (int c = 0; c < N; ++c) {
          const double tmp = AT(k, c, N);
          AT(k, c, N) = AT(pv, c, N);
          AT(pv, c, N) = tmp;
        }
        const double tb = Bv[(int64_t)k * T];
        Bv[(int64_t)k * T] = Bv[(int64_t)pv * T];
        Bv[(int64_t)pv * T] = tb;
      }
      const double pivot = AT(k, k, N);
      for (int i = k + 1; i < N; ++i) {
        const double f = AT(i, k, N) / pivot;
        AT(i, k, N) = f;
        if (f != 0.0)
          for (int c = k + 1; c < N; ++c) AT(i, c, N) -= f * AT(k, c, N);
      }
    }
    if (singular) {
      a.out_v[t] = kNaN;
      a.out_var[t] = kNaN;
      if (a.out_lag) a.out_lag[t] = kNaN;
      a.out_st[t] = GS_ST_SINGULAR | fb;
      continue;
    }
    for (int i = 0; i < N; ++i) {
      double s = Bv[(int64_t)i * T];
      for (int j = 0; j < i; ++j) s -= AT(i, j, N) * Bv[(int64_t)j * T];
      Bv[(int64_t)i * T] = s;
    }
    for (int i = N - 1; i >= 0; --i) {
      double s = Bv[(int64_t)i * T];
      for (int j = i + 1; j < N; ++j) s -= AT(i, j, N) * Bv[(int64_t)j * T];
      Bv[(int64_t)i * T] = s / AT(i, i, N);
    }
    // outputs (kriging.rs:614-643)
    double v, var, lag = kNaN;
    if (a.method == GS_SIMPLE) {
      v = a.sk_mean;
      double red = 0.0;
      for (int ii = 0; ii < n; ++ii) {
        const double w = Bv[(int64_t)ii * T];
        v += w * (a.val[nbt[ii]] - a.sk_mean);
        red += w * B0[(int64_t)ii * T];
      }
      var = m.c0 - red;
    } else {
      v = 0.0;
      for (int ii = 0; ii < n; ++ii) v += Bv[(int64_t)ii * T] * a.val[nbt[ii]];
      double red = 0.0;
      for (int i = 0; i < N; ++i) red += Bv[(int64_t)i * T] * B0[(int64_t)i * T];
      var = m.c0 - red;
      lag = Bv[(int64_t)n * T];
    }
    a.out_v[t] = v;
    a.out_var[t] = fmax(var, 0.0);
    if (a.out_lag) a.out_lag[t] = lag;
    a.out_st[t] = GS_ST_OK | fb;
  }
}

template <int D>
__global__ void grid_centers_kernel(double x0, double y0, double z0, double dx, double dy,
                                    double dz, int64_t nx, int64_t ny, int64_t total, double* x,
                                    double* y, double* z) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ix = i % nx;
    const int64_t iy = (i / nx) % ny;
    const int64_t iz = i / (nx * ny);
    x[i] = x0 + ((double)ix + 0.5) * dx;
    y[i] = y0 + ((double)iy + 0.5) * dy;
    if (D == 3) z[i] = z0 + ((double)iz + 0.5) * dz;
  }
}

}  // namespace

static ExpTable g_tab;
static DfConsts g_kc;
static bool g_tab_ready = false;

static void ensure_tables() {
  if (!g_tab_ready) {
    df_consts_host(&g_tab, &g_kc);
    g_tab_ready = true;
  }
}

size_t mixed_per_warp_bytes(int nmax, int nf, int dim) {
  const int NP = nmax * (nmax + 1) / 2;
  size_t bytes = 0;
  bytes += (size_t)NP * sizeof(df);                                 // A
  bytes += (size_t)nf * GS_MIXED_MAX_NEIGHBORS * dim * sizeof(df);  // V
  bytes += (size_t)nmax * sizeof(df) * 2;                           // B, XD
  bytes += (size_t)nmax * sizeof(double);                           // X
  bytes += (size_t)GS_MIXED_MAX_NEIGHBORS * sizeof(double);         // Z
  bytes += (size_t)NP * sizeof(float);                              // L
  bytes += (size_t)nmax * sizeof(float) * 2;                        // W, DI
  return (bytes + 15) & ~(size_t)15;
}

int krige_mixed_launch(const KrigeArgs& a, const DevModel& m, uint8_t* flag, int warps_per_block,
                       cudaStream_t stream) {
  if (a.ntl == 0) return GS_OK;
  ensure_tables();
  int nf = 1;
  for (int s = 0; s < m.ns; ++s) nf += m.s[s].aniso ? 1 : 0;
  const size_t per_warp = mixed_per_warp_bytes(a.nmax, nf, a.dim);
  int wpb = std::max(1, warps_per_block);
  while (wpb > 1 && per_warp * wpb > 200 * 1024) --wpb;
  const size_t smem = per_warp * wpb;
  if (smem > 220 * 1024) return fail(GS_ERR_INVALID_PARAMETER, "system too large for the mixed kernel");
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  auto kern = a.dim == 2 ? krige_mixed_kernel<2> : krige_mixed_kernel<3>;
  GS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, wpb * 32, smem));
  per_sm = std::max(per_sm, 1);
  const int64_t want = (a.ntl + wpb - 1) / wpb;
  const int blocks = (int)std::min<int64_t>(want, (int64_t)sms * per_sm * 8);
  kern<<<blocks, wpb * 32, smem, stream>>>(a, m, g_tab, g_kc, flag, per_warp);
  GS_CUDA(cudaGetLastError());
  count_launch(1);
  return GS_OK;
}

int64_t fp64_scratch_doubles(int nmax, int64_t threads) {
  return ((int64_t)nmax * nmax + 2 * (int64_t)nmax) * threads;
}

int64_t fp64_threads_for(int nmax, int64_t budget_bytes) {
  const int64_t per = ((int64_t)nmax * nmax + 2 * (int64_t)nmax) * 8;
  int64_t t = budget_bytes / std::max<int64_t>(per, 1);
  t = std::min<int64_t>(t, 152 * 1024);
  t = (t / 128) * 128;
  return std::max<int64_t>(t, 128);
}

int krige_fp64_launch(const KrigeArgs& a, const DevModel& m, double* scratch, int64_t threads,
                      cudaStream_t stream) {
  if (a.ntl == 0) return GS_OK;
  const int tpb = 128;
  const int64_t T = ((std::min<int64_t>(threads, std::max<int64_t>(a.ntl, 1)) + tpb - 1) / tpb) * tpb;
  const int64_t Tl = std::min<int64_t>(T, threads);
  const int blocks = (int)((Tl + tpb - 1) / tpb);
  if (a.dim == 2) krige_fp64_kernel<2><<<blocks, tpb, 0, stream>>>(a, m, scratch, Tl);
  else krige_fp64_kernel<3><<<blocks, tpb, 0, stream>>>(a, m, scratch, Tl);
  GS_CUDA(cudaGetLastError());
  count_launch(1);
  return GS_OK;
}

int grid_centers_launch(int dim, const double* bmin, const double* step, const int64_t* ncell,
                        double* x, double* y, double* z, cudaStream_t stream) {
  int64_t total = ncell[0] * ncell[1] * (dim == 3 ? ncell[2] : 1);
  if (total == 0) return GS_OK;
  const int tpb = 256;
  const int blocks = (int)std::min<int64_t>((total + tpb - 1) / tpb, 152 * 64);
  if (dim == 2)
    grid_centers_kernel<2><<<blocks, tpb, 0, stream>>>(bmin[0], bmin[1], 0.0, step[0], step[1], 0.0,
                                                       ncell[0], ncell[1], total, x, y, z);
  else
    grid_centers_kernel<3><<<blocks, tpb, 0, stream>>>(bmin[0], bmin[1], bmin[2], step[0], step[1],
                                                       step[2], ncell[0], ncell[1], total, x, y, z);
  GS_CUDA(cudaGetLastError());
  return GS_OK;
}

}  // namespace gs
