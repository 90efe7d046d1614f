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
#include "gs_cta.cuh"
#include "gs_solve.cuh"

namespace gs {

namespace {

// Basis function k of fill_basis (kriging.rs:410-439) at point pt, FP64.
template <int D>
__device__ __forceinline__ double basis_at(const KrigeArgs& a, const double* pt,
                                           const double* drow, int k) {
  if (k == 0) return 1.0;
  if (a.method == GS_EXTERNAL_DRIFT) return (drow[k - 1] - a.dmean[k - 1]) / a.dscale[k - 1];
  // universal: normalised coordinates, then their degree-2 monomials
  if (k <= D) return (pt[k - 1] - a.center[k - 1]) / a.scale;
  int idx = 1 + D;
  for (int u = 0; u < D; ++u)
    for (int v = u; v < D; ++v) {
      if (idx == k)
        return ((pt[u] - a.center[u]) / a.scale) * ((pt[v] - a.center[v]) / a.scale);
      ++idx;
    }
  return 0.0;
}

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

// Shared-memory layout of one system.
struct MixedLayout {
  int np, nbr;
  size_t off_a, off_v, off_b, off_xd, off_z, off_red, off_w, off_pan, off_lp, off_pinv, off_p, off_t, off_flag,
      total;
};

__host__ __device__ inline MixedLayout mixed_layout(int nmax, int nf, int dim) {
  MixedLayout L;
  L.np = nmax * (nmax + 1) / 2;
  L.nbr = (nmax + 3) / 4;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t r = o;
    o += (bytes + 15) & ~(size_t)15;
    return r;
  };
  L.off_a = take((size_t)L.np * sizeof(df));
  L.off_v = take((size_t)nf * dim * GS_MIXED_MAX_NEIGHBORS * sizeof(df));
  L.off_b = take((size_t)nmax * sizeof(df));
  L.off_xd = take((size_t)4 * L.nbr * sizeof(df));
  L.off_z = take((size_t)GS_MIXED_MAX_NEIGHBORS * sizeof(df));
  L.off_red = take(32 * sizeof(float));
  L.off_w = take((size_t)4 * L.nbr * sizeof(float));
  L.off_pan = take((size_t)2 * L.nbr * GS_PB * sizeof(float));
  L.off_lp = take((size_t)2 * L.nbr * GS_PB * sizeof(float));
  L.off_pinv = take(32 * sizeof(float));
  L.off_p = take((size_t)L.nbr * L.nbr * 4 * sizeof(float));
  L.off_t = take(8 * sizeof(df));
  L.off_flag = take(16);
  L.total = o;
  return L;
}

// Exact coordinate coincidence (reference: gamma(0) = 0 only when every
// separation component is exactly zero, -0 == +0), on the 64-bit patterns.
__device__ __forceinline__ bool same_double(double a, double b) {
  const unsigned long long x = (unsigned long long)__double_as_longlong(a);
  const unsigned long long y = (unsigned long long)__double_as_longlong(b);
  return x == y || ((x | y) << 1) == 0ull;
}

template <int D, int BLOCK>
__global__ void __launch_bounds__(BLOCK, 4) krige_mixed_kernel(KrigeArgs a, DevModel m, ExpTable tab_g,
                                                               DfConsts kc, uint8_t* flag) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ ExpTable tab;
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    tab.v[i] = tab_g.v[i];
  }
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const Frames fr = frames_of(m);
  const int NB = GS_MIXED_MAX_NEIGHBORS;
  const MixedLayout lay = mixed_layout(a.nmax, fr.nf, D);
  df* A = reinterpret_cast<df*>(smem_raw + lay.off_a);
  df* V = reinterpret_cast<df*>(smem_raw + lay.off_v);
  df* B = reinterpret_cast<df*>(smem_raw + lay.off_b);
  df* ZV = reinterpret_cast<df*>(smem_raw + lay.off_z);
  df* TD = reinterpret_cast<df*>(smem_raw + lay.off_t);  // target coordinates, sk mean
  CtaScratch S;
  S.XD = reinterpret_cast<df*>(smem_raw + lay.off_xd);
  S.red = reinterpret_cast<float*>(smem_raw + lay.off_red);
  S.W = reinterpret_cast<float*>(smem_raw + lay.off_w);
  S.pan = reinterpret_cast<float*>(smem_raw + lay.off_pan);
  S.lp = reinterpret_cast<float*>(smem_raw + lay.off_lp);
  S.pinv = reinterpret_cast<float*>(smem_raw + lay.off_pinv);
  S.P = reinterpret_cast<float*>(smem_raw + lay.off_p);
  S.flag = reinterpret_cast<int*>(smem_raw + lay.off_flag);
  const double* coord[3] = {a.x, a.y, a.z};
  __syncthreads();

  for (int64_t it = blockIdx.x; it < a.ntl; it += gridDim.x) {
    const int64_t t = a.tlist ? a.tlist[it] : it;
    const int n = a.nbc[t];
    const int p = a.p;
    uint8_t st = GS_ST_OK;
    if (n < 0) st = GS_ST_CAPACITY;
    else if (n < a.min_nb) st = GS_ST_NO_NEIGHBORS;
    else if (n < p) st = GS_ST_INSUFFICIENT_DATA;
    if (st != GS_ST_OK) {
      if (tid == 0) {
        a.out_v[t] = __longlong_as_double(0x7ff8000000000000ll);
        a.out_var[t] = __longlong_as_double(0x7ff8000000000000ll);
        if (a.out_lag) a.out_lag[t] = __longlong_as_double(0x7ff8000000000000ll);
        a.out_st[t] = st;
        flag[t] = 0;
      }
      continue;
    }
    if (n > NB) {
      if (tid == 0) flag[t] = 1;
      continue;
    }
    const int N = n + p;
    const double tp[3] = {a.tx[t], a.ty[t], D == 3 ? a.tz[t] : 0.0};
    // target coordinates (and the simple-kriging mean) as df, once per system
    if (tid < D) TD[tid] = df_from_double(tp[tid]);
    if (tid == 3) TD[3] = df_from_double(a.sk_mean);
    // drift basis of the target: one basis function per thread
    if (tid >= 32 && tid - 32 < p) {
      const int k = tid - 32;
      B[n + k] = df_from_double(basis_at<D>(a, tp, a.tdrift ? a.tdrift + t * a.nv : nullptr, k));
    }
    __syncthreads();
    // --- per-neighbour data: frames, values, rhs, diagonal, drift rows ---
    for (int i = tid; i < n; i += nthr) {
      const int idx = a.nb[t * (int64_t)a.kout + i];
      df ud[3];
      bool zero = true;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        ud[d] = df_sub(a.cdf[(int64_t)d * a.n + idx], TD[d]);
        zero = zero && same_double(coord[d][idx], tp[d]);
      }
      frame_coords<D>(m, fr, ud, V, NB, i);
      B[i] = zero ? m.c0_df : cov_origin<D>(m, fr, V, NB, i, tab, kc);
      ZV[i] = a.vdf[idx];
      A[pk(i, i)] = a.err_df ? df_add(m.c0_df, a.err_df[idx]) : m.c0_df;
      for (int k = 0; k < p; ++k) A[pk(n + k, i)] = a.basis_df[(int64_t)k * a.n + idx];
    }
    for (int q = tid; q < p * (p + 1) / 2; q += nthr) {
      int r = 0;
      while ((r + 1) * (r + 2) / 2 <= q) ++r;
      const int c = q - r * (r + 1) / 2;
      A[pk(n + r, n + c)] = df_make(0.0f, 0.0f);
    }
    __syncthreads();
    // --- covariance block, strictly lower part ---------------------------
    {
      const int npairs = (n * (n - 1)) >> 1;
      int i = 1, j = tid;
      while (j >= i && i < n) {
        j -= i;
        ++i;
      }
      for (int q = tid; q < npairs; q += nthr) {
        A[pk(i, j)] = cov_pair<D>(m, fr, V, NB, i, j, tab, kc);
        j += nthr;
        while (j >= i && i < n) {
          j -= i;
          ++i;
        }
      }
    }
    __syncthreads();
    // --- FP32 inverse, double-float refinement ----------------------------
    const bool ok = cta_solve(A, B, N, S);
    if (!ok) {
      if (tid == 0) flag[t] = 1;
      __syncthreads();
      continue;
    }
    // --- outputs: double-float dot products, FP64 at the end -------------
    if (tid < 32) {
      df sv = df_make(0.0f, 0.0f), sr = df_make(0.0f, 0.0f);
      if (a.method == GS_SIMPLE) {
        const df mean = TD[3];
        for (int i = tid; i < n; i += 32) {
          sv = df_fma_acc(sv, S.XD[i], df_sub(ZV[i], mean));
          sr = df_fma_acc(sr, S.XD[i], B[i]);
        }
      } else {
        for (int i = tid; i < n; i += 32) sv = df_fma_acc(sv, S.XD[i], ZV[i]);
        for (int i = tid; i < N; i += 32) sr = df_fma_acc(sr, S.XD[i], B[i]);
      }
      sv = warp_sum_df(sv);
      sr = warp_sum_df(sr);
      if (tid == 0) {
        const double val = a.method == GS_SIMPLE ? a.sk_mean + df_to_double(sv) : df_to_double(sv);
        a.out_v[t] = val;
        a.out_var[t] = fmax(df_to_double(df_sub(m.c0_df, sr)), 0.0);
        if (a.out_lag)
          a.out_lag[t] = a.method == GS_SIMPLE ? __longlong_as_double(0x7ff8000000000000ll)
                                               : df_to_double(S.XD[n]);
        a.out_st[t] = GS_ST_OK;
        flag[t] = 0;
      }
    }
    __syncthreads();
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

int krige_mixed_launch(const KrigeArgs& a, const DevModel& m, uint8_t* flag, int /*unused*/,
                       cudaStream_t stream) {
  if (a.ntl == 0) return GS_OK;
  ensure_tables();
  int nf = 1;
  for (int s = 0; s < m.ns; ++s) nf += m.s[s].aniso ? 1 : 0;
  const MixedLayout lay = mixed_layout(a.nmax, nf, a.dim);
  const size_t smem = lay.total;
  if (smem > 200 * 1024) return fail(GS_ERR_INVALID_PARAMETER, "system too large for the mixed kernel");
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int nbr = lay.nbr;
  const int tiles = nbr * (nbr + 1) / 2;
  const int block = std::min(256, std::max(64, ((tiles + 31) / 32) * 32));
  auto kern = a.dim == 2 ? krige_mixed_kernel<2, 256> : krige_mixed_kernel<3, 256>;
  GS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem));
  per_sm = std::max(per_sm, 1);
  const int blocks = (int)std::min<int64_t>(a.ntl, (int64_t)sms * per_sm);
  kern<<<blocks, block, smem, stream>>>(a, m, g_tab, g_kc, flag);
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
