// gs_vecchia.cu -- Vecchia plan, log-likelihood, MLE driver and joint
// prediction (crates/geostat-core/src/vecchia.rs).
//
// Plan (vecchia.rs:232-282): the max-min order is computed on the host (as
// in the reference); the m nearest predecessors of every ordered point come
// from the ranked device search (store rank = order position), sorted by
// (squared distance, position) like the reference's incremental BucketGrid.
//
// Log-likelihood (vecchia.rs:285-336): one warp per ordered point runs every
// parameter candidate of the batch against the point's conditioning set:
// double-float covariances, FP32 L D L^T with FP64-accumulated refinement,
// FP64 mean/variance/log terms.  Points whose refinement stalls are redone
// by an FP64 one-thread-per-point Cholesky that follows linalg.rs:123-203.
// Per-point terms are summed per candidate in a fixed tree order (FP64), so
// results do not depend on scheduling.
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "gs_common.cuh"
#include "gs_host.h"
#include "gs_internal.h"
#include "gs_search.cuh"
#include "gs_cta.cuh"
#include "gs_solve.cuh"
#include "gs_warp.cuh"
#include "gs_vecchia.h"

struct gs_vecchia_plan {
  const gs_pointset* ps = nullptr;
  int64_t n = 0;
  int64_t m = 0;
  std::vector<int64_t> order;
  int64_t* d_order = nullptr;  // position -> point id
  int32_t* d_nb = nullptr;     // n x m point ids, -1 padded
  int32_t* d_cnt = nullptr;
  double mean = 0.0;
  cudaStream_t stream = nullptr;
  // grouped likelihood blocks per group size: block b's joint set (the
  // members' predecessors, then the members) at vid[off[b] .. off[b + 1]),
  // the first slen[b] of them predecessors; vmax = the largest set
  struct Groups {
    int64_t nblocks = 0;
    int vmax = 0;
    int64_t* d_off = nullptr;
    int32_t* d_vid = nullptr;
    int32_t* d_slen = nullptr;
    // blocks of more than one member: their indices, the largest of their
    // sets, and per ordered position whether it belongs to one of them
    int64_t nmulti = 0;
    int vmax_multi = 0;
    int64_t* d_multi = nullptr;
    uint8_t* d_in_multi = nullptr;
  };
  mutable std::mutex groups_mu;
  mutable std::map<int64_t, Groups> groups;
  ~gs_vecchia_plan() {
    for (auto& g : groups) {
      cudaFree(g.second.d_off);
      cudaFree(g.second.d_vid);
      cudaFree(g.second.d_slen);
      cudaFree(g.second.d_multi);
      cudaFree(g.second.d_in_multi);
    }
    cudaFree(d_order);
    cudaFree(d_nb);
    cudaFree(d_cnt);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace gs {
namespace {

__global__ void gather_by_order(int64_t n, const int64_t* order, const double* x, const double* y,
                                const double* z, double* ox, double* oy, double* oz) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = order[k];
    ox[k] = x[i];
    oy[k] = y[i];
    if (oz) oz[k] = z[i];
  }
}

__global__ void positions_to_ids(int64_t total, const int64_t* order, int32_t* nb) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int32_t pos = nb[q];
    if (pos >= 0) nb[q] = (int32_t)order[pos];
  }
}

struct VArgs {
  int dim;
  int64_t n;
  int m;
  int ncand;
  int iso_shared;  // every candidate isotropic: cache separation norms
  const double* x;
  const double* y;
  const double* z;
  const double* v;
  double mean;
  const df* cdf;   // coordinates as df, axis-major
  const df* vdf;   // values as df
  df mean_df;
  const int64_t* order;
  const int32_t* nb;
  const int32_t* cnt;
  const DevModel* models;  // device array of ncand models
  double* terms;           // ncand x n (position order)
  uint8_t* flag;           // ncand x n
  // ordered positions evaluated: [k0, k1) (the whole plan unless a
  // point-range call asks for part of it)
  int64_t k0, k1;
  // REML (reml_loglik_with_plan, vecchia.rs:1278-1345): the trend basis
  // (p x n, column-major), and per (candidate, position) the record
  // (var, r, g_0 .. g_{p-1}) at rec[(c * n + k) * (2 + p)], with r and g the
  // raw value's and the basis rows' residuals after the conditioning solve
  const double* basis;
  int p;
  double* rec;
  // likelihood systems accepted at the double-float floor [0] and refined
  // with FP64 residuals [1] (one add per warp; may be null)
  unsigned long long* tiers;
};

constexpr double kLn2Pi = 1.8378770664093453;  // ln(2*pi)

struct VLayout {
  int np, nbr;
  size_t off_a, off_h, off_v, off_b, off_xd, off_h0, off_z, off_red, off_w, off_pan, off_lp, off_pinv, off_p,
      off_flag, total;
};

__host__ __device__ inline VLayout vecchia_layout(int m, int dim) {
  VLayout L;
  L.np = m * (m + 1) / 2;
  L.nbr = (m + 3) / 4;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t r = o;
    o += (bytes + 15) & ~(size_t)15;
    return r;
  };
  L.off_a = take((size_t)L.np * sizeof(df));
  L.off_h = take((size_t)L.np * sizeof(df));
  L.off_v = take((size_t)(GS_MAX_STRUCTURES + 1) * dim * m * sizeof(df));
  L.off_b = take((size_t)m * sizeof(df));
  L.off_xd = take((size_t)4 * L.nbr * sizeof(df));
  L.off_h0 = take((size_t)m * sizeof(df));
  L.off_z = take((size_t)m * sizeof(df));
  L.off_red = take(32 * sizeof(float));
  L.off_w = take((size_t)4 * L.nbr * sizeof(float));
  L.off_pan = take((size_t)2 * L.nbr * GS_PB * sizeof(float));
  L.off_lp = take((size_t)2 * L.nbr * GS_PB * sizeof(float));
  L.off_pinv = take(32 * sizeof(float));
  L.off_p = take((size_t)L.nbr * L.nbr * 4 * sizeof(float));
  L.off_flag = take(16);
  L.total = o;
  return L;
}

template <int D, int BLOCK>
__global__ void __launch_bounds__(BLOCK, 4) vecchia_loglik_kernel(VArgs a, ExpTable tab_g,
                                                                  DfConsts kc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ ExpTable tab;
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    tab.v[i] = tab_g.v[i];
  }
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const int M = a.m;
  const VLayout lay = vecchia_layout(M, D);
  df* A = reinterpret_cast<df*>(smem_raw + lay.off_a);
  df* H = reinterpret_cast<df*>(smem_raw + lay.off_h);
  df* V = reinterpret_cast<df*>(smem_raw + lay.off_v);
  df* B = reinterpret_cast<df*>(smem_raw + lay.off_b);
  df* H0 = reinterpret_cast<df*>(smem_raw + lay.off_h0);
  df* ZV = reinterpret_cast<df*>(smem_raw + lay.off_z);
  CtaScratch S;
  S.XD = reinterpret_cast<df*>(smem_raw + lay.off_xd);
  S.red = reinterpret_cast<float*>(smem_raw + lay.off_red);
  S.W = reinterpret_cast<float*>(smem_raw + lay.off_w);
  S.pan = reinterpret_cast<float*>(smem_raw + lay.off_pan);
  S.lp = reinterpret_cast<float*>(smem_raw + lay.off_lp);
  S.pinv = reinterpret_cast<float*>(smem_raw + lay.off_pinv);
  S.P = reinterpret_cast<float*>(smem_raw + lay.off_p);
  S.flag = reinterpret_cast<int*>(smem_raw + lay.off_flag);
  __syncthreads();

  for (int64_t k = a.k0 + blockIdx.x; k < a.k1; k += gridDim.x) {
    const int64_t i = a.order[k];
    const int s = a.cnt[k];
    const df zi = df_sub(a.vdf[i], a.mean_df);
    if (s == 0) {
      // first point: marginal N(0, sill)
      const double z = df_to_double(zi);
      for (int c = tid; c < a.ncand; c += nthr) {
        const double sill = a.models[c].c0;
        a.terms[(int64_t)c * a.n + k] = -0.5 * (kLn2Pi + log(sill) + z * z / sill);
        a.flag[(int64_t)c * a.n + k] = 0;
      }
      continue;
    }
    for (int q = tid; q < s; q += nthr) {
      const int j = a.nb[k * (int64_t)M + q];
#pragma unroll
      for (int d = 0; d < D; ++d)
        V[d * M + q] = df_sub(a.cdf[(int64_t)d * a.n + j], a.cdf[(int64_t)d * a.n + i]);
      ZV[q] = df_sub(a.vdf[j], a.mean_df);
    }
    __syncthreads();
    const int npairs = (s * (s - 1)) >> 1;
    if (a.iso_shared) {
      for (int q = tid; q < s; q += nthr) H0[q] = norm_origin<D>(V, M, 0, q);
      int ii = 1, jj = tid;
      while (jj >= ii && ii < s) {
        jj -= ii;
        ++ii;
      }
      for (int q = tid; q < npairs; q += nthr) {
        H[pk(ii, jj)] = norm_pair<D>(V, M, 0, ii, jj);
        jj += nthr;
        while (jj >= ii && ii < s) {
          jj -= ii;
          ++ii;
        }
      }
      __syncthreads();
    }
    for (int c = 0; c < a.ncand; ++c) {
      const DevModel& mdl = a.models[c];
      const Frames fr = frames_of(mdl);
      if (a.iso_shared) {
        for (int q = tid; q < s; q += nthr) {
          B[q] = cov_from_norm(mdl, H0[q], tab, kc);
          A[pk(q, q)] = mdl.c0_df;
        }
        int ii = 1, jj = tid;
        while (jj >= ii && ii < s) {
          jj -= ii;
          ++ii;
        }
        for (int q = tid; q < npairs; q += nthr) {
          A[pk(ii, jj)] = cov_from_norm(mdl, H[pk(ii, jj)], tab, kc);
          jj += nthr;
          while (jj >= ii && ii < s) {
            jj -= ii;
            ++ii;
          }
        }
      } else {
        for (int q = tid; q < s; q += nthr) {
          df ud[3];
#pragma unroll
          for (int d = 0; d < D; ++d) ud[d] = V[d * M + q];
          frame_coords<D>(mdl, fr, ud, V, M, q);
          B[q] = cov_origin<D>(mdl, fr, V, M, q, tab, kc);
          A[pk(q, q)] = mdl.c0_df;
        }
        __syncthreads();
        int ii = 1, jj = tid;
        while (jj >= ii && ii < s) {
          jj -= ii;
          ++ii;
        }
        for (int q = tid; q < npairs; q += nthr) {
          A[pk(ii, jj)] = cov_pair<D>(mdl, fr, V, M, ii, jj, tab, kc);
          jj += nthr;
          while (jj >= ii && ii < s) {
            jj -= ii;
            ++ii;
          }
        }
      }
      __syncthreads();
      const bool ok = cta_solve(A, B, s, S);
      if (!ok) {
        if (tid == 0) a.flag[(int64_t)c * a.n + k] = 1;
        __syncthreads();
        continue;
      }
      if (tid < 32) {
        df mu = df_make(0.0f, 0.0f), red = df_make(0.0f, 0.0f);
        for (int q = tid; q < s; q += 32) {
          mu = df_fma_acc(mu, S.XD[q], ZV[q]);
          red = df_fma_acc(red, S.XD[q], B[q]);
        }
        mu = warp_sum_df(mu);
        red = warp_sum_df(red);
        if (tid == 0) {
          const double var = fmax(df_to_double(df_sub(mdl.c0_df, red)), 1e-12);
          const double r = df_to_double(df_sub(zi, mu));
          a.terms[(int64_t)c * a.n + k] = -0.5 * (kLn2Pi + log(var) + r * r / var);
          a.flag[(int64_t)c * a.n + k] = 0;
        }
      }
      __syncthreads();
    }
  }
}

// Per-warp shared-memory layout of vecchia_warp_kernel (conditioning sets of
// at most 32 points).
struct VWLayout {
  size_t off_a, off_h, off_v, off_b, off_z, off_row, off_vec, off_xd, off_lt, total;
};

// Entries of the split (hi parts, then lo parts) arrays of the likelihood
// kernel's assembly: the packed triangle of m points, then the m covariances
// with the point, rounded up to an even count (entries go in pairs).
__host__ __device__ inline int vw_split_entries(int m) { return (m * (m + 1) / 2 + m + 1) & ~1; }

__host__ __device__ inline VWLayout vecchia_warp_layout(int m, int dim, int lt_width = 2) {
  VWLayout L;
  const int np = m * (m + 1) / 2;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t r = o;
    o += (bytes + 15) & ~(size_t)15;
    return r;
  };
  const int ne = vw_split_entries(m);
  L.off_a = take((size_t)(np > ne ? np : ne) * sizeof(df));
  L.off_h = take((size_t)ne * sizeof(df));
  L.off_v = take((size_t)(GS_MAX_STRUCTURES + 1) * dim * m * sizeof(df));
  L.off_b = take((size_t)m * sizeof(df));
  L.off_z = take((size_t)m * sizeof(df));
  L.off_row = take(kWarpRowFloats * sizeof(float));
  L.off_vec = take(kWarpN * sizeof(float));
  L.off_xd = take(kWarpN * sizeof(df));
  // (variance, residual[, basis residuals]) of 32 candidates
  L.off_lt = take((size_t)lt_width * kWarpN * sizeof(double));
  L.total = o;
  return L;
}

constexpr int kVWarps = 4;  // warps (ordered points in flight) per block

// Likelihood systems whose double-float refinement stops contracting with its
// corrections at most this fraction of |w| are accepted (warp_refine's
// accept_floor): the conditional mean and variance are linear functionals of
// w, so their error at that floor is the double-float entries' rounding, as
// for a converged refinement.  Larger stalls take the FP64-residual
// refinement below.
constexpr float kVecchiaFloor = 1e-10f;

// Refinement with residuals formed in FP64, for a likelihood system whose
// double-float refinement stalled (its residual is limited by the 48-bit
// entries): the warp evaluates the covariances of the conditioning set S and
// of the point in FP64 (the table-driven exp of the FP64 re-solve kernel,
// K64 packed lower over S, k64 per neighbour), starts from the stalled
// solution in W.xd, and repeats w += C32^{-1} (k - K w) with the FP32 inverse
// it already holds (the sweep rows of f) and the residual in FP64.  It
// accepts when a correction falls below 1e-14 of |w|, or when the
// corrections stop shrinking at or below 1e-12 of |w| -- the fixed point of
// FP64-residual refinement, whose forward error is the size of that last
// correction (cond(K) 2^-53, as for an FP64 factorisation; larger stalls go
// to the FP64 re-solve kernel).  On success lane 0 receives the conditional
// variance and residual of loglik_with_plan (vecchia.rs:302-330) from FP64
// dot products; returns false (uniformly) otherwise.
template <int D, class Factor>
__device__ bool vecchia_refine_fp64(const VArgs& a, const DevModel& mdl, const Exp64Table& et,
                                    int64_t k, int64_t pt, int s, int lane, const Factor& f,
                                    const WarpScratch& W, double* K64, double* k64,
                                    double& var, double& r) {
  const int M = a.m;
  const int32_t* nbk = a.nb + k * (int64_t)M;
  const double* xs[3] = {a.x, a.y, a.z};
  // the stalled double-float iterate, before the buffers are reused
  __syncwarp();
  double w = lane < s ? (double)W.xd[lane].hi + (double)W.xd[lane].lo : 0.0;
  __syncwarp();
  for (int e = lane; e < (s * (s + 1)) / 2; e += 32) {
    // (q, p), p <= q < s, packed order
    int q = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
    while ((q * (q + 1)) / 2 > e) --q;
    while (((q + 1) * (q + 2)) / 2 <= e) ++q;
    const int p = e - (q * (q + 1)) / 2;
    double v = mdl.c0;
    if (p != q) {
      const int ip = nbk[p], iq = nbk[q];
      double h[3];
#pragma unroll
      for (int d = 0; d < D; ++d) h[d] = xs[d][ip] - xs[d][iq];
      v = cov_fp64x<D>(mdl, h, et);
    }
    K64[pk(q, p)] = v;
  }
  double zl = 0.0;
  if (lane < s) {
    const int j = nbk[lane];
    double h[3];
#pragma unroll
    for (int d = 0; d < D; ++d) h[d] = xs[d][pt] - xs[d][j];
    k64[lane] = cov_fp64x<D>(mdl, h, et);
    zl = a.v[j] - a.mean;
  }
  double* wb = reinterpret_cast<double*>(W.xd);  // broadcast of w
  bool ok = false;
  float nd_prev = 0.0f;
  for (int sweep = 1; sweep <= 4; ++sweep) {
    __syncwarp();
    wb[lane] = w;
    __syncwarp();
    double rho = 0.0;
    if (lane < s) {
      rho = k64[lane];
      for (int j = 0; j < s; ++j) rho = fma(-K64[lane >= j ? pk(lane, j) : pk(j, lane)], wb[j], rho);
    }
    W.vec[lane] = (float)rho;
    __syncwarp();
    float y;
    warp_gemv_neg_inv(f.t, W.vec, lane, y);
    y *= f.sc;
    if (lane < s) w -= (double)y;
    const float nd = warp_max_f(lane < s ? fabsf(y) : 0.0f);
    const float nw = warp_max_f(lane < s ? (float)fabs(w) : 0.0f);
    if (nd <= 1e-14f * nw) {
      ok = true;
      break;
    }
    if (sweep >= 2 && !(nd < 0.5f * nd_prev)) {
      ok = nd <= 1e-12f * nw;
      break;
    }
    nd_prev = nd;
  }
  if (!ok) return false;
  double red = lane < s ? k64[lane] * w : 0.0, mu = lane < s ? zl * w : 0.0;
  red = warp_sum_d(red);
  mu = warp_sum_d(mu);
  var = fmax(mdl.c0 - red, 1e-12);
  r = (a.v[pt] - a.mean) - mu;
  return true;
}


// One warp per ordered point for conditioning sets of at most 32 points: the
// same assembly and certification as vecchia_loglik_kernel, with the
// register-row solver of gs_warp.cuh (no block barriers).  The likelihood
// form is compiled for four blocks (16 warps) per SM (128 registers: the
// matrix entries stay in shared memory); the REML form keeps the default.
constexpr int kVWBlocksPerSm = 4;
template <int D, bool REML>
__global__ void __launch_bounds__(32 * kVWarps, REML ? 1 : kVWBlocksPerSm)
    vecchia_warp_kernel(VArgs a, ExpTable tab_g, DfConsts kc, Exp64Table et_g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ ExpTable tab;
  __shared__ Exp64Table et;  // FP64 covariances of the FP64-residual refinement
  for (int i = threadIdx.x; i < 256; i += blockDim.x) tab.v[i] = tab_g.v[i];
  for (int q = threadIdx.x; q < 64; q += blockDim.x) {
    et.hi[q] = et_g.hi[q];
    et.lo[q] = et_g.lo[q];
  }
  if (threadIdx.x == 0) {
    et.l1 = et_g.l1;
    et.l2 = et_g.l2;
    et.inv = et_g.inv;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int M = a.m;
  const int LW = REML ? 2 + a.p : 2;  // doubles per candidate in LT
  const VWLayout lay = vecchia_warp_layout(M, D, LW);
  unsigned char* base = smem_raw + (size_t)wib * lay.total;
  // the matrix's packed entries and the point's covariances, split: hi parts
  // at Ah[e], lo parts at Al[e] (e < np: packed triangle, np + q: point q);
  // the separations of the isotropic form in the same split layout
  const int NE = vw_split_entries(M);
  float* Ah = reinterpret_cast<float*>(base + lay.off_a);
  float* Al = Ah + NE;
  float* Hh = reinterpret_cast<float*>(base + lay.off_h);
  float* Hl = Hh + NE;
  df* V = reinterpret_cast<df*>(base + lay.off_v);
  df* B = reinterpret_cast<df*>(base + lay.off_b);
  df* ZV = reinterpret_cast<df*>(base + lay.off_z);
  WarpScratch W;
  W.row = reinterpret_cast<float*>(base + lay.off_row);
  W.vec = reinterpret_cast<float*>(base + lay.off_vec);
  W.xd = reinterpret_cast<df*>(base + lay.off_xd);
  // per-candidate (variance, residual), -1 variance: flagged; the log terms
  // of up to 32 candidates are then evaluated by one lane each
  double* LT = reinterpret_cast<double*>(base + lay.off_lt);
  auto flush_terms = [&](int64_t k, int c0, int cnt) {
    __syncwarp();
    if (lane < cnt) {
      const int c = c0 + lane;
      const double var = LT[LW * lane], r = LT[LW * lane + 1];
      if (REML) {
        if (var >= 0.0) {
          double* rc = a.rec + ((int64_t)c * a.n + k) * LW;
          for (int q = 0; q < LW; ++q) rc[q] = LT[LW * lane + q];
        }
      } else if (var >= 0.0) {
        a.terms[(int64_t)c * a.n + k] = -0.5 * (kLn2Pi + log(var) + r * r / var);
      }
      a.flag[(int64_t)c * a.n + k] = var >= 0.0 ? 0 : 1;
    }
    __syncwarp();
  };
  const int64_t nwarps = (int64_t)gridDim.x * kVWarps;
  unsigned n_floor = 0, n_fp64res = 0;
  for (int64_t k = a.k0 + (int64_t)blockIdx.x * kVWarps + wib; k < a.k1; k += nwarps) {
    const int64_t i = a.order[k];
    const int s = a.cnt[k];
    // REML works on the raw values (vecchia.rs:1296-1337)
    const df zi = REML ? a.vdf[i] : df_sub(a.vdf[i], a.mean_df);
    if (s == 0) {
      const double z = df_to_double(zi);
      for (int c = lane; c < a.ncand; c += 32) {
        const double sill = a.models[c].c0;
        if (REML) {
          double* rc = a.rec + ((int64_t)c * a.n + k) * LW;
          rc[0] = sill;
          rc[1] = z;
          for (int q = 0; q < a.p; ++q) rc[2 + q] = a.basis[(int64_t)q * a.n + i];
        } else {
          a.terms[(int64_t)c * a.n + k] = -0.5 * (kLn2Pi + log(sill) + z * z / sill);
        }
        a.flag[(int64_t)c * a.n + k] = 0;
      }
      continue;
    }
    __syncwarp();
    if (lane < s) {
      const int j = a.nb[k * (int64_t)M + lane];
      // separations from the FP64 coordinates (exact for nearby points), so
      // short lags keep their full relative precision
      const double* xs[3] = {a.x, a.y, a.z};
#pragma unroll
      for (int d = 0; d < D; ++d) V[d * M + lane] = df_from_double(xs[d][j] - xs[d][i]);
      ZV[lane] = REML ? a.vdf[j] : df_sub(a.vdf[j], a.mean_df);
    }
    __syncwarp();
    // entries of this set: packed triangle, then the point's covariances
    const int np = (s * (s + 1)) >> 1;
    const int ne = (np + s + 1) & ~1;
    if (a.iso_shared) {
      // separation norms once per point (diagonal positions 0; the padding
      // entry, if any, a harmless 0 too)
      for_pairs2(s, lane, 32, [&](int i0, int j0, int i1, int j1, bool two) {
        const df h0 = norm_pair<D>(V, M, 0, i0, j0);
        const df h1 = norm_pair<D>(V, M, 0, i1, j1);
        Hh[pk(i0, j0)] = h0.hi;
        Hl[pk(i0, j0)] = h0.lo;
        if (two) {
          Hh[pk(i1, j1)] = h1.hi;
          Hl[pk(i1, j1)] = h1.lo;
        }
      });
      if (lane < s) {
        const df h = norm_origin<D>(V, M, 0, lane);
        Hh[np + lane] = h.hi;
        Hl[np + lane] = h.lo;
        Hh[pk(lane, lane)] = 0.0f;
        Hl[pk(lane, lane)] = 0.0f;
      }
      if (lane == 0 && ne > np + s) {
        Hh[np + s] = 0.0f;
        Hl[np + s] = 0.0f;
      }
      __syncwarp();
    }
    for (int c = 0; c < a.ncand; ++c) {
      const DevModel& mdl = a.models[c];
      const Frames fr = frames_of(mdl);
      if (a.iso_shared) {
        // every entry of the set, two adjacent ones per lane and step, by
        // packed position: no pair indices, 8-byte loads and stores of
        // aligned hi / lo pairs
        for (int e = 2 * lane; e < ne; e += 64) {
          df c0, c1;
          const float2 hh = *reinterpret_cast<const float2*>(Hh + e);
          const float2 hl = *reinterpret_cast<const float2*>(Hl + e);
          cov_from_norm2(mdl, df_make(hh.x, hl.x), df_make(hh.y, hl.y), tab, kc, c0, c1);
          *reinterpret_cast<float2*>(Ah + e) = make_float2(c0.hi, c1.hi);
          *reinterpret_cast<float2*>(Al + e) = make_float2(c0.lo, c1.lo);
        }
        __syncwarp();
        if (lane < s) {
          B[lane] = df_make(Ah[np + lane], Al[np + lane]);
          Ah[pk(lane, lane)] = mdl.c0_df.hi;  // C(0), nugget included
          Al[pk(lane, lane)] = mdl.c0_df.lo;
        }
      } else {
        if (lane < s) {
          df ud[3];
#pragma unroll
          for (int d = 0; d < D; ++d) ud[d] = V[d * M + lane];
          frame_coords<D>(mdl, fr, ud, V, M, lane);
          B[lane] = cov_origin<D>(mdl, fr, V, M, lane, tab, kc);
          Ah[pk(lane, lane)] = mdl.c0_df.hi;
          Al[pk(lane, lane)] = mdl.c0_df.lo;
        }
        __syncwarp();
        for_pairs2(s, lane, 32, [&](int i0, int j0, int i1, int j1, bool two) {
          df c0, c1;
          cov_pair2<D>(mdl, fr, V, M, i0, j0, i1, j1, tab, kc, c0, c1);
          Ah[pk(i0, j0)] = c0.hi;
          Al[pk(i0, j0)] = c0.lo;
          if (two) {
            Ah[pk(i1, j1)] = c1.hi;
            Al[pk(i1, j1)] = c1.lo;
          }
        });
      }
      __syncwarp();
      bool ok, ok64 = false;
      {
        const auto row = shared_row([&](int e) { return df_make(Ah[e], Al[e]); }, s, lane);
        WarpFactor fct;
        const bool fok = warp_factor(row, s, lane, fct, W);
        // REML keeps the strict test: its records feed further sums
        bool at_floor = false;
        ok = fok && warp_refine(fct, row, B, s, lane, W, REML ? 0.0f : kVecchiaFloor, &at_floor);
        n_floor += ok && at_floor;
        if (!REML && fok && !ok) {
          // stalled: refine with FP64 residuals (A's and B's storage take the
          // FP64 entries; this candidate's double-float system is done with)
          double v64 = 0.0, r64 = 0.0;
          ok64 = vecchia_refine_fp64<D>(a, mdl, et, k, i, s, lane, fct, W,
                                        reinterpret_cast<double*>(Ah),
                                        reinterpret_cast<double*>(B), v64, r64);
          if (ok64 && lane == 0) {
            LT[LW * (c & 31)] = v64;
            LT[LW * (c & 31) + 1] = r64;
          }
          n_fp64res += ok64;
        }
      }
      if (ok64) {
        // outputs written by the FP64-residual refinement
      } else if (!ok) {
        if (lane == 0) LT[LW * (c & 31)] = -1.0;
      } else {
        // (w . z, w . k) as one packed double-float product and sum
        dfp pr = dp_zero();
        if (lane < s) pr = dp_mul(dp_splat(W.xd[lane]), dp_pack(ZV[lane], B[lane]));
        pr = warp_sum_dfp(pr);
        const df mu = dp_first(pr), red = dp_second(pr);
        if (lane == 0) {
          LT[LW * (c & 31)] = fmax(df_to_double(df_sub(mdl.c0_df, red)), 1e-12);
          LT[LW * (c & 31) + 1] = df_to_double(df_sub(zi, mu));
        }
        if (REML) {
          // the basis rows' residuals f_i - w . f_S
          const int j = lane < s ? a.nb[k * (int64_t)M + lane] : 0;
          for (int q = 0; q < a.p; ++q) {
            df g = df_make(0.0f, 0.0f);
            if (lane < s) g = df_fma_acc(g, W.xd[lane], df_from_double(a.basis[(int64_t)q * a.n + j]));
            g = warp_sum_df(g);
            if (lane == 0)
              LT[LW * (c & 31) + 2 + q] =
                  df_to_double(df_sub(df_from_double(a.basis[(int64_t)q * a.n + i]), g));
          }
        }
      }
      if ((c & 31) == 31 || c == a.ncand - 1) flush_terms(k, c & ~31, (c & 31) + 1);
      __syncwarp();
    }
  }
  if (lane == 0 && a.tiers) {
    if (n_floor) atomicAdd(&a.tiers[0], (unsigned long long)n_floor);
    if (n_fp64res) atomicAdd(&a.tiers[1], (unsigned long long)n_fp64res);
  }
}

// cholesky_solve_in_place (linalg.rs:123-203) on an s x s row-major matrix
// whose element e lives at S[e * T] (one slab per thread, interleaved): the
// unpivoted factor with the reference's failure test !(d > 1e-12 max diag),
// then the forward and back substitutions of W in place.
__device__ bool chol_factor_strided(double* S, int s, int64_t T) {
  double scale = 0.0;
  for (int q = 0; q < s; ++q) scale = fmax(scale, S[(int64_t)(q * s + q) * T]);
  scale = fmax(scale, 2.2250738585072014e-308);
  for (int kk = 0; kk < s; ++kk) {
    double d = S[(int64_t)(kk * s + kk) * T];
    for (int j = 0; j < kk; ++j) d -= S[(int64_t)(kk * s + j) * T] * S[(int64_t)(kk * s + j) * T];
    if (!(d > 1e-12 * scale)) return false;
    d = sqrt(d);
    S[(int64_t)(kk * s + kk) * T] = d;
    for (int r = kk + 1; r < s; ++r) {
      double acc = S[(int64_t)(r * s + kk) * T];
      for (int j = 0; j < kk; ++j) acc -= S[(int64_t)(r * s + j) * T] * S[(int64_t)(kk * s + j) * T];
      S[(int64_t)(r * s + kk) * T] = acc / d;
    }
  }
  return true;
}
// cholesky_forward_solve + cholesky_back_solve (linalg.rs:160-180) of W in place.
__device__ void chol_subst_strided(const double* S, double* W, int s, int64_t T) {
  for (int r = 0; r < s; ++r) {
    double acc = W[(int64_t)r * T];
    for (int j = 0; j < r; ++j) acc -= S[(int64_t)(r * s + j) * T] * W[(int64_t)j * T];
    W[(int64_t)r * T] = acc / S[(int64_t)(r * s + r) * T];
  }
  for (int r = s - 1; r >= 0; --r) {
    double acc = W[(int64_t)r * T];
    for (int j = r + 1; j < s; ++j) acc -= S[(int64_t)(j * s + r) * T] * W[(int64_t)j * T];
    W[(int64_t)r * T] = acc / S[(int64_t)(r * s + r) * T];
  }
}
__device__ bool chol_solve_strided(double* S, double* W, int s, int64_t T) {
  if (!chol_factor_strided(S, s, T)) return false;
  chol_subst_strided(S, W, s, T);
  return true;
}

// FP64 per-(candidate, point) solve: cholesky_solve_in_place
// (linalg.rs:123-203) on the assembled K_SS of vecchia.rs:302-320.
// OWN_EXP: covariances with the table-driven FP64 exp (the re-solve of
// flagged systems); the FP64 build keeps the library exp.
template <int D, bool OWN_EXP, bool REML = false>
__global__ void vecchia_fp64_kernel(VArgs a, const int64_t* list, int64_t nlist, double* scratch,
                                    int64_t T, int32_t* cand_status, Exp64Table et_g) {
  __shared__ Exp64Table et;
  if (OWN_EXP) {
    for (int q = threadIdx.x; q < 64; q += blockDim.x) {
      et.hi[q] = et_g.hi[q];
      et.lo[q] = et_g.lo[q];
    }
    if (threadIdx.x == 0) {
      et.l1 = et_g.l1;
      et.l2 = et_g.l2;
      et.inv = et_g.inv;
    }
    __syncthreads();
  }
  auto cov = [&](const DevModel& md, const double* h) {
    return OWN_EXP ? cov_fp64x<D>(md, h, et) : cov_fp64<D>(md, h);
  };
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (tid >= T) return;
  const int M = a.m;
  double* S = scratch + tid;
  double* W = scratch + (int64_t)M * M * T + tid;
  double* K0 = W + (int64_t)M * T;
  for (int64_t it = tid; it < nlist; it += T) {
    const int64_t span = a.k1 - a.k0;
    const int64_t code = list ? list[it] : (it / span) * a.n + a.k0 + it % span;
    const int c = (int)(code / a.n);
    const int64_t k = code % a.n;
    const DevModel& mdl = a.models[c];
    const int64_t i = a.order[k];
    const int s = a.cnt[k];
    const double zi = REML ? a.v[i] : a.v[i] - a.mean;
    const double sill = mdl.c0;
    double* rc = REML ? a.rec + code * (2 + a.p) : nullptr;
    if (s == 0) {
      if (REML) {
        rc[0] = sill;
        rc[1] = zi;
        for (int q = 0; q < a.p; ++q) rc[2 + q] = a.basis[(int64_t)q * a.n + i];
      } else {
        a.terms[code] = -0.5 * (kLn2Pi + log(sill) + zi * zi / sill);
      }
      continue;
    }
    const int32_t* nbk = a.nb + k * (int64_t)M;
    double pi[3] = {a.x[i], a.y[i], D == 3 ? a.z[i] : 0.0};
    for (int aa = 0; aa < s; ++aa) {
      const int ja = nbk[aa];
      double h[3] = {pi[0] - a.x[ja], pi[1] - a.y[ja], D == 3 ? pi[2] - a.z[ja] : 0.0};
      const double kv = cov(mdl, h);
      W[(int64_t)aa * T] = kv;
      K0[(int64_t)aa * T] = kv;
      for (int bb = aa; bb < s; ++bb) {
        const int jb = nbk[bb];
        double g[3] = {a.x[ja] - a.x[jb], a.y[ja] - a.y[jb], D == 3 ? a.z[ja] - a.z[jb] : 0.0};
        const double cv = cov(mdl, g);
        S[(int64_t)(aa * s + bb) * T] = cv;
        S[(int64_t)(bb * s + aa) * T] = cv;
      }
    }
    if (!chol_solve_strided(S, W, s, T)) {
      atomicExch(&cand_status[c], (int32_t)GS_ERR_SINGULAR_SYSTEM);
      if (REML) rc[0] = __longlong_as_double(0x7ff8000000000000ll);
      else a.terms[code] = __longlong_as_double(0x7ff8000000000000ll);
      continue;
    }
    double mu = 0.0, red = 0.0;
    for (int q = 0; q < s; ++q) mu += W[(int64_t)q * T] * (REML ? a.v[nbk[q]] : a.v[nbk[q]] - a.mean);
    for (int q = 0; q < s; ++q) red += W[(int64_t)q * T] * K0[(int64_t)q * T];
    const double var = fmax(sill - red, 1e-12);
    const double r = zi - mu;
    if (REML) {
      rc[0] = var;
      rc[1] = r;
      for (int col = 0; col < a.p; ++col) {
        double g = 0.0;
        for (int q = 0; q < s; ++q) g += W[(int64_t)q * T] * a.basis[(int64_t)col * a.n + nbk[q]];
        rc[2 + col] = a.basis[(int64_t)col * a.n + i] - g;
      }
    } else {
      a.terms[code] = -0.5 * (kLn2Pi + log(var) + r * r / var);
    }
  }
}

// REML's sums over the points from the records (var, r, g): row y = c * W + w
// of the output sums ln var (w = 0), r^2 / var (1), g_f r / var (2 .. 1 + p)
// and g_f g_g / var (f <= g, row-packed); the same fixed-order tree as
// reduce_terms.
__global__ void reduce_reml(const double* rec, int64_t n, int p, int64_t chunk, int64_t y0,
                            const uint8_t* exclude, double* partial) {
  __shared__ double sh[256];
  const int W = 2 + p + p * (p + 1) / 2;
  const int64_t y = y0 + blockIdx.y;
  const int c = (int)(y / W), w = (int)(y % W);
  int r1 = 0, r2 = 0;  // record fields multiplied: 1 = r, 2 + f = g_f
  if (w == 1) {
    r1 = r2 = 1;
  } else if (w >= 2 && w < 2 + p) {
    r1 = 2 + (w - 2);
    r2 = 1;
  } else if (w >= 2 + p) {
    int e = w - 2 - p, f = 0;
    while (e >= p - f) {
      e -= p - f;
      ++f;
    }
    r1 = 2 + f;
    r2 = 2 + f + e;
  }
  const int64_t lo = blockIdx.x * chunk;
  const int64_t hi = min(n, lo + chunk);
  double acc = 0.0;
  for (int64_t q = lo + threadIdx.x; q < hi; q += blockDim.x) {
    if (exclude && exclude[q]) continue;
    const double* rc = rec + ((int64_t)c * n + q) * (2 + p);
    acc += w == 0 ? log(rc[0]) : rc[r1] * rc[r2] / rc[0];
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s2 = blockDim.x / 2; s2 > 0; s2 >>= 1) {
    if ((int)threadIdx.x < s2) sh[threadIdx.x] += sh[threadIdx.x + s2];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[y * gridDim.x + blockIdx.x] = sh[0];
}


// Fixed-order reduction: block b sums terms [k0 + b*chunk, k0 + (b+1)*chunk)
// of one candidate (positions below k1) in a fixed tree; the partials are
// added in block order.
__global__ void reduce_terms(const double* terms, int64_t n, int64_t k0, int64_t k1, int64_t chunk,
                             double* partial) {
  __shared__ double sh[256];
  const int c = blockIdx.y;
  const int64_t lo = k0 + blockIdx.x * chunk;
  const int64_t hi = min(k1, lo + chunk);
  double acc = 0.0;
  for (int64_t q = lo + threadIdx.x; q < hi; q += blockDim.x) acc += terms[(int64_t)c * n + q];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(int64_t)c * gridDim.x + blockIdx.x] = sh[0];
}

__global__ void reduce_partials(const double* partial, int nblk, int ncand, double* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncand) return;
  double s = 0.0;
  for (int b = 0; b < nblk; ++b) s += partial[(int64_t)c * nblk + b];
  out[c] = s;
}

// ---------------------------------------- grouped likelihood (Guinness) --
// loglik_with_blocks (vecchia.rs:613-668) in FP64, one warp per (block,
// candidate): the joint covariance of a block's set V (sill on the diagonal,
// sill - gamma off it) bordered by nr data rows, LDL^T over V (the
// reference's Cholesky test: pivot > 1e-12 sill).  For a member t,
// Cholesky's L_tt^2 is the pivot d_t and a data row's forward-solved value
// is a_t / sqrt(d_t), a_t = that row's entry after t's elimination, so the
// likelihood's terms are
//     term_t = -1/2 (ln 2 pi + ln d_t + a_t^2 / d_t)     (one row: z - mean)
// and REML (vecchia.rs:1366-1457; rows: z, then the trend basis columns)
// sums, per block, ln d_t, a_z^2 / d_t, a_f a_z / d_t and a_f a_g / d_t.
// Singleton blocks stand for the ungrouped REML (vecchia.rs:1278-1345),
// whose member variance is max(d, 1e-12) rather than a pivot test.
// Trailing updates use the flattened pair table of the kriging re-solve
// (the system embedded at the bottom right of a Vmax frame).
struct GroupArgs {
  const int64_t* off;
  const int32_t* vid;
  const int32_t* slen;
  int64_t nblocks;      // blocks evaluated (the list's length when blist is set)
  const int64_t* blist; // the blocks to evaluate, or null for all
  int vmax;             // frame size: the largest set + the data rows
  int nr;               // data rows: 1, or 1 + p for REML
  const double* basis;  // REML: p x n trend basis, column-major; else null
  int clamp_member;     // singleton blocks of the ungrouped REML
};

__host__ __device__ inline size_t group_warp_doubles(int vmax) {
  return (size_t)vmax * (vmax + 1) / 2 + 2 * (size_t)vmax;
}

__host__ __device__ inline int reml_sums(int p) { return 2 + p + p * (p + 1) / 2; }

template <int D, bool REML>
__global__ void vecchia_group_kernel(VArgs a, GroupArgs g, int wpb, int32_t* cstat,
                                     Exp64Table et_g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ Exp64Table et;  // the table-driven FP64 exp of the covariances
  for (int q = threadIdx.x; q < 64; q += blockDim.x) {
    et.hi[q] = et_g.hi[q];
    et.lo[q] = et_g.lo[q];
  }
  if (threadIdx.x == 0) {
    et.l1 = et_g.l1;
    et.l2 = et_g.l2;
    et.inv = et_g.inv;
  }
  const int Vmax = g.vmax;
  uint32_t* ptab = reinterpret_cast<uint32_t*>(smem_raw);
  const size_t ptab_bytes = (((size_t)Vmax * (Vmax - 1) / 2) * 4 + 15) & ~(size_t)15;
  for (int j = 1; j < Vmax; ++j) {
    const int off = ((Vmax - 1 - j) * (Vmax - j)) >> 1;
    for (int i = j + threadIdx.x; i < Vmax; i += blockDim.x)
      ptab[off + i - j] = ((uint32_t)pk(i, j) << 16) | ((uint32_t)i << 8) | (uint32_t)j;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* A = reinterpret_cast<double*>(smem_raw + ptab_bytes) + (size_t)warp * group_warp_doubles(Vmax);
  double* lsc = A + (size_t)Vmax * (Vmax + 1) / 2;
  double* lun = lsc + Vmax;
  const int nr = g.nr;
  const int p = nr - 1;
  const int64_t items = (int64_t)a.ncand * g.nblocks;
  const int64_t nw = (int64_t)gridDim.x * wpb;
  const double* xs[3] = {a.x, a.y, a.z};
  for (int64_t it = (int64_t)blockIdx.x * wpb + warp; it < items; it += nw) {
    const int c = (int)(it / g.nblocks);
    const int64_t bi = it % g.nblocks;  // output slot
    const int64_t b = g.blist ? g.blist[bi] : bi;
    const DevModel& mdl = a.models[c];
    const int32_t* ids = g.vid + g.off[b];
    const int vn = (int)(g.off[b + 1] - g.off[b]);
    const int sl = g.slen[b];
    const int M = vn + nr;
    const int o = Vmax - M;
    const int iz = o + vn;  // first data row
    for (int e = lane; e < (vn * (vn - 1)) / 2 + vn; e += 32) {
      // (r, q), q <= r < vn, packed order
      int r = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
      while ((r * (r + 1)) / 2 > e) --r;
      while (((r + 1) * (r + 2)) / 2 <= e) ++r;
      const int q = e - (r * (r + 1)) / 2;
      double v = mdl.c0;
      if (q != r) {
        double h[3];
#pragma unroll
        for (int d = 0; d < D; ++d) h[d] = xs[d][ids[q]] - xs[d][ids[r]];
        v = cov_fp64x<D>(mdl, h, et);
      }
      A[pk(o + r, o + q)] = v;
    }
    for (int e = lane; e < nr * vn; e += 32) {
      const int row = e / vn, q = e - row * vn;
      double v;
      if (REML)
        v = row == 0 ? a.v[ids[q]] : g.basis[(int64_t)(row - 1) * a.n + ids[q]];
      else
        v = a.v[ids[q]] - a.mean;
      A[pk(iz + row, o + q)] = v;
    }
    for (int e = lane; e < (nr * (nr + 1)) / 2; e += 32) {
      int r = 0;
      while (((r + 1) * (r + 2)) / 2 <= e) ++r;
      A[pk(iz + r, iz + e - (r * (r + 1)) / 2)] = 0.0;
    }
    __syncwarp();
    const double tol = 1e-12 * fmax(mdl.c0, 2.2250738585072014e-308);
    // pivots lie in [1e-12 c0, c0] (or at the 1e-12 clamp): scaled by a power
    // of two near 1 / c0 they are in FP32's range for the reciprocal's seed
    const double sc = ldexp(1.0, -ilogb(fmax(mdl.c0, 1e-300)));
    bool ok = true;
    for (int k = o; k < iz; ++k) {
      double dk = A[pk(k, k)];
      if (g.clamp_member && k >= o + sl) {
        dk = fmax(dk, 1e-12);
      } else if (!(dk > tol)) {
        ok = false;
        break;
      }
      const double r = (g.clamp_member && k >= o + sl) ? 1.0 / dk : rcp_fp64(dk, sc, true);
      for (int i = k + 1 + lane; i < Vmax; i += 32) {
        const double v = A[pk(i, k)];
        lun[i] = v;
        lsc[i] = v * r;
      }
      __syncwarp();
      const int T = ((Vmax - 1 - k) * (Vmax - k)) >> 1;
      for (int e = lane; e < T; e += 32) {
        const uint32_t en = ptab[e];
        const int pe = (int)(en >> 16), i = (int)((en >> 8) & 255u), j = (int)(en & 255u);
        A[pe] = fma(-lsc[i], lun[j], A[pe]);
      }
      __syncwarp();
    }
    if (!REML) {
      if (lane == 0) {
        double sum = __longlong_as_double(0x7ff8000000000000ll);
        if (ok) {
          sum = 0.0;
          for (int t = sl; t < vn; ++t) {
            const double dt = A[pk(o + t, o + t)];
            const double at = A[pk(iz, o + t)];
            sum += -0.5 * (kLn2Pi + log(dt) + at * at / dt);
          }
        } else {
          atomicExch(&cstat[c], (int32_t)GS_ERR_SINGULAR_SYSTEM);
        }
        a.terms[(int64_t)c * g.nblocks + bi] = sum;
      }
    } else {
      // sums: [0] ln d, [1] a_z^2 / d, [2, 2 + p) a_f a_z / d, then a_f a_g / d
      // over f <= g, row-packed
      const int W = reml_sums(p);
      if (!ok && lane == 0) atomicExch(&cstat[c], (int32_t)GS_ERR_SINGULAR_SYSTEM);
      for (int w = lane; w < W; w += 32) {
        int r1 = 0, r2 = 0;  // data rows multiplied (w >= 1)
        if (w >= 2 && w < 2 + p) {
          r1 = 1 + (w - 2);
        } else if (w >= 2 + p) {
          int e = w - 2 - p, f = 0;
          while (e >= p - f) {
            e -= p - f;
            ++f;
          }
          r1 = 1 + f;
          r2 = 1 + f + e;
        }
        double sum = __longlong_as_double(0x7ff8000000000000ll);
        if (ok) {
          sum = 0.0;
          for (int t = sl; t < vn; ++t) {
            double dt = A[pk(o + t, o + t)];
            if (g.clamp_member) dt = fmax(dt, 1e-12);
            sum += w == 0 ? log(dt) : A[pk(iz + r1, o + t)] * A[pk(iz + r2, o + t)] / dt;
          }
        }
        a.terms[((int64_t)c * W + w) * g.nblocks + bi] = sum;
      }
    }
    __syncwarp();
  }
}

ExpTable g_vtab;
Exp64Table g_vet;
DfConsts g_vkc;
std::once_flag g_vonce;

void ensure_vtables() {
  std::call_once(g_vonce, [] {
    df_consts_host(&g_vtab, &g_vkc);
    exp64_table_host(&g_vet);
  });
}

int reject_vecchia_model(const gs_model& m, int dim) {
  GS_TRY(validate_model(m));
  if (has_power(m))
    return fail(GS_ERR_INVALID_PARAMETER,
                "Vecchia needs a valid covariance function and cannot use the unbounded Power model");
  for (int k = 0; k < m.n_structures; ++k)
    if (m.s[k].kind == GS_KIND_CIRCULAR && dim > 2)
      return fail(GS_ERR_INVALID_PARAMETER, "Circular is not a valid covariance in 3 dimensions");
  return GS_OK;
}

}  // namespace

// Evaluates ncand candidates on a plan; ll[c] and status[c] per candidate.
__global__ void exclude_terms_kernel(double* terms, int64_t n, int64_t ncand,
                                     const uint8_t* exclude) {
  const int64_t total = n * ncand;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x)
    if (exclude[i % n]) terms[i] = 0.0;
}

// REML (basis set, p columns; conditioning sets of at most 32 points, mixed
// precision): instead of log-likelihoods, reml_sums receives per candidate
// the reml_sums(p) sums of the ungrouped REML (ll is left NaN).
// Systems of the last mixed likelihood evaluation on this host thread that
// were accepted at the double-float floor / refined with FP64 residuals.
static thread_local int64_t g_vtiers[2] = {0, 0};

int vecchia_eval(const gs_vecchia_plan* P, int64_t ncand, const gs_model* models, double* ll,
                 int32_t* status, int precision, cudaStream_t s, const uint8_t* exclude,
                 const double* basis, int p, double* reml_sums, int64_t k0, int64_t k1) {
  NvtxRange nvtx_range("gs.vecchia_loglik");
  const gs_pointset* ps = P->ps;
  const int dim = ps->dim;
  const int64_t n = P->n;
  const int M = (int)P->m;
  if (k1 < 0) k1 = n;
  if (k0 < 0 || k1 > n || k0 > k1)
    return fail(GS_ERR_INVALID_PARAMETER, "point range [" + std::to_string(k0) + ", " +
                                              std::to_string(k1) + ") outside the plan's " +
                                              std::to_string(n) + " points");
  const bool partial_range = k0 != 0 || k1 != n;
  if (partial_range && basis)
    return fail(GS_ERR_INVALID_PARAMETER, "REML sums cover the whole plan");
  const int64_t span = k1 - k0;
  ensure_vtables();
  std::vector<DevModel> dms(std::max<int64_t>(ncand, 1));
  std::vector<int> valid(ncand, 0);
  bool all_iso = true;
  for (int64_t c = 0; c < ncand; ++c) {
    status[c] = GS_OK;
    ll[c] = NAN;
    int rc = reject_vecchia_model(models[c], dim);
    if (!rc) rc = make_dev_model(models[c], dim, &dms[c], true);
    if (rc) {
      status[c] = rc;
      dms[c] = DevModel{};
      dms[c].ns = 0;
      dms[c].c0 = 1.0;
      dms[c].c0_df = df_from_double(1.0);
      continue;
    }
    valid[c] = 1;
    for (int k = 0; k < models[c].n_structures; ++k)
      if (models[c].s[k].has_anis) all_iso = false;
  }
  if (ncand == 0) return GS_OK;
  if (span == 0) {  // an empty point range sums to zero
    for (int64_t c = 0; c < ncand; ++c)
      if (valid[c]) ll[c] = 0.0;
    return GS_OK;
  }
  DevBuf dmod, terms, flag, partial, out, cstat;
  GS_TRY(dmod.alloc(sizeof(DevModel) * ncand, s));
  GS_CUDA(cudaMemcpyAsync(dmod.ptr, dms.data(), sizeof(DevModel) * ncand, cudaMemcpyHostToDevice, s));
  const bool reml = basis != nullptr;
  const int LW = 2 + p;
  DevBuf rec;
  if (reml) GS_TRY(rec.alloc((size_t)ncand * n * LW * 8, s));
  else GS_TRY(terms.alloc((size_t)ncand * n * 8, s));
  GS_TRY(flag.alloc((size_t)ncand * n, s));
  // positions outside a partial range are never written: no flagged systems there
  if (partial_range) GS_CUDA(cudaMemsetAsync(flag.ptr, 0, (size_t)ncand * n, s));
  GS_TRY(cstat.alloc((size_t)ncand * 4, s));
  GS_CUDA(cudaMemsetAsync(cstat.ptr, 0, ncand * 4, s));
  DevBuf tiers;
  GS_TRY(tiers.alloc(2 * sizeof(unsigned long long), s));
  GS_CUDA(cudaMemsetAsync(tiers.ptr, 0, 2 * sizeof(unsigned long long), s));
  g_vtiers[0] = g_vtiers[1] = 0;
  VArgs a{};
  a.dim = dim;
  a.n = n;
  a.k0 = k0;
  a.k1 = k1;
  a.m = M;
  a.ncand = (int)ncand;
  a.iso_shared = all_iso ? 1 : 0;
  a.x = ps->d_x;
  a.y = ps->d_y;
  a.z = ps->d_z;
  a.v = ps->d_v;
  a.mean = P->mean;
  a.cdf = (const df*)ps->d_cdf;
  a.vdf = (const df*)ps->d_vdf;
  a.mean_df = df_from_double(P->mean);
  a.order = P->d_order;
  a.nb = P->d_nb;
  a.cnt = P->d_cnt;
  a.models = (const DevModel*)dmod.ptr;
  a.terms = (double*)terms.ptr;
  a.flag = (uint8_t*)flag.ptr;
  a.basis = basis;
  a.p = p;
  a.rec = (double*)rec.ptr;
  a.tiers = (unsigned long long*)tiers.ptr;
  int64_t nfl = 0;
  DevBuf list;
  const bool mixed = precision != GS_PREC_FP64 && M <= GS_MIXED_MAX_NEIGHBORS;
  if (reml && !(mixed && M <= kWarpN))
    return fail(GS_ERR_INVALID_PARAMETER, "mixed REML needs conditioning sets of at most 32");
  cudaEvent_t ev[4];
  for (int e = 0; e < 4; ++e) GS_CUDA(cudaEventCreate(&ev[e]));
  struct EvGuard {
    cudaEvent_t* e;
    ~EvGuard() {
      for (int q = 0; q < 4; ++q) cudaEventDestroy(e[q]);
    }
  } ev_guard{ev};
  GS_CUDA(cudaEventRecord(ev[0], s));
  if (mixed) {
    const int sms = sm_count();
    if (M <= kWarpN) {
      const size_t smem = vecchia_warp_layout(std::max(M, 1), dim, reml ? LW : 2).total * kVWarps;
      auto kern = reml ? (dim == 2 ? vecchia_warp_kernel<2, true> : vecchia_warp_kernel<3, true>)
                       : (dim == 2 ? vecchia_warp_kernel<2, false> : vecchia_warp_kernel<3, false>);
      GS_TRY(allow_dynamic_smem((const void*)kern, smem));
      int per_sm = 0;
      GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * kVWarps, smem));
      per_sm = std::max(per_sm, 1);
      const int blocks =
          (int)std::min<int64_t>((span + kVWarps - 1) / kVWarps, (int64_t)sms * per_sm);
      kern<<<blocks, 32 * kVWarps, smem, s>>>(a, g_vtab, g_vkc, g_vet);
    } else {
      const VLayout lay = vecchia_layout(std::max(M, 1), dim);
      const size_t smem = lay.total;
      const int tiles = lay.nbr * (lay.nbr + 1) / 2;
      const int block = std::min(256, std::max(64, ((tiles + 31) / 32) * 32));
      auto kern = dim == 2 ? vecchia_loglik_kernel<2, 256> : vecchia_loglik_kernel<3, 256>;
      GS_TRY(allow_dynamic_smem((const void*)kern, smem));
      int per_sm = 0;
      GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem));
      per_sm = std::max(per_sm, 1);
      const int blocks = (int)std::min<int64_t>(span, (int64_t)sms * per_sm);
      kern<<<blocks, block, smem, s>>>(a, g_vtab, g_vkc);
    }
    GS_CUDA(cudaGetLastError());
    count_launch(1);
    GS_CUDA(cudaEventRecord(ev[1], s));
    // compact flagged (candidate, point) pairs
    DevBuf nsel, tmp;
    GS_TRY(nsel.alloc(8, s));
    GS_TRY(list.alloc((size_t)ncand * n * 8, s));
    size_t tb = 0;
    GS_CUDA(cub::DeviceSelect::Flagged(nullptr, tb, thrust::counting_iterator<int64_t>(0),
                                       (uint8_t*)flag.ptr, (int64_t*)list.ptr, (int64_t*)nsel.ptr,
                                       (int64_t)(ncand * n), s));
    GS_TRY(tmp.alloc(tb, s));
    GS_CUDA(cub::DeviceSelect::Flagged(tmp.ptr, tb, thrust::counting_iterator<int64_t>(0),
                                       (uint8_t*)flag.ptr, (int64_t*)list.ptr, (int64_t*)nsel.ptr,
                                       (int64_t)(ncand * n), s));
    unsigned long long ht[2] = {0, 0};
    GS_CUDA(cudaMemcpyAsync(&nfl, nsel.ptr, 8, cudaMemcpyDeviceToHost, s));
    GS_CUDA(cudaMemcpyAsync(ht, tiers.ptr, sizeof(ht), cudaMemcpyDeviceToHost, s));
    GS_CUDA(cudaStreamSynchronize(s));
    g_vtiers[0] = (int64_t)ht[0];
    g_vtiers[1] = (int64_t)ht[1];
  }
  if (!mixed) GS_CUDA(cudaEventRecord(ev[1], s));
  GS_CUDA(cudaEventRecord(ev[2], s));
  if (!mixed || nfl > 0) {
    const int64_t work = mixed ? nfl : ncand * span;
    const int64_t per = ((int64_t)M * M + 2 * (int64_t)M) * 8;
    // 512 threads per SM: measured fastest (the strided scratch then stays
    // mostly in L2; more threads spill it to HBM)
    int64_t T = std::min<int64_t>(std::max<int64_t>(((int64_t)1 << 31) / std::max<int64_t>(per, 1), 128), (int64_t)sm_count() * 512);
    T = std::min<int64_t>(T, ((work + 127) / 128) * 128);
    T = std::max<int64_t>(T, 128);
    DevBuf scratch;
    GS_TRY(scratch.alloc((size_t)T * per, s));
    const int blocks = (int)((T + 127) / 128);
    const int64_t* lp = mixed ? (const int64_t*)list.ptr : nullptr;
    double* sp = (double*)scratch.ptr;
    int32_t* cs = (int32_t*)cstat.ptr;
    if (reml && dim == 2)
      vecchia_fp64_kernel<2, true, true><<<blocks, 128, 0, s>>>(a, lp, work, sp, T, cs, g_vet);
    else if (reml)
      vecchia_fp64_kernel<3, true, true><<<blocks, 128, 0, s>>>(a, lp, work, sp, T, cs, g_vet);
    else if (dim == 2 && mixed)
      vecchia_fp64_kernel<2, true><<<blocks, 128, 0, s>>>(a, lp, work, sp, T, cs, g_vet);
    else if (dim == 2)
      vecchia_fp64_kernel<2, false><<<blocks, 128, 0, s>>>(a, lp, work, sp, T, cs, g_vet);
    else if (mixed)
      vecchia_fp64_kernel<3, true><<<blocks, 128, 0, s>>>(a, lp, work, sp, T, cs, g_vet);
    else
      vecchia_fp64_kernel<3, false><<<blocks, 128, 0, s>>>(a, lp, work, sp, T, cs, g_vet);
    GS_CUDA(cudaGetLastError());
    count_launch(1);
  }
  GS_CUDA(cudaEventRecord(ev[3], s));
  if (reml) {
    const int W = 2 + p + p * (p + 1) / 2;
    const int64_t rows = ncand * W;
    const int64_t chunk = 8192;
    const int nblk = (int)((n + chunk - 1) / chunk);
    GS_TRY(partial.alloc((size_t)nblk * rows * 8, s));
    GS_TRY(out.alloc((size_t)rows * 8, s));
    int launches = 1;
    for (int64_t y0 = 0; y0 < rows; y0 += 65535, ++launches)
      reduce_reml<<<dim3(nblk, (unsigned)std::min<int64_t>(65535, rows - y0)), 256, 0, s>>>(
          (const double*)rec.ptr, n, p, chunk, y0, exclude, (double*)partial.ptr);
    reduce_partials<<<(int)((rows + 127) / 128), 128, 0, s>>>((double*)partial.ptr, nblk, (int)rows,
                                                              (double*)out.ptr);
    GS_CUDA(cudaGetLastError());
    count_launch(launches);
    std::vector<int32_t> hst(ncand);
    GS_CUDA(cudaMemcpyAsync(reml_sums, out.ptr, rows * 8, cudaMemcpyDeviceToHost, s));
    GS_CUDA(cudaMemcpyAsync(hst.data(), cstat.ptr, ncand * 4, cudaMemcpyDeviceToHost, s));
    GS_CUDA(cudaStreamSynchronize(s));
    for (int64_t c = 0; c < ncand; ++c)
      if (valid[c] && hst[c] != 0) status[c] = hst[c];
    return GS_OK;
  }
  if (exclude) {
    exclude_terms_kernel<<<sm_count() * 8, 256, 0, s>>>((double*)terms.ptr, n, ncand, exclude);
    GS_CUDA(cudaGetLastError());
    count_launch(1);
  }
  const int64_t chunk = 8192;
  const int nblk = (int)((span + chunk - 1) / chunk);
  GS_TRY(partial.alloc((size_t)nblk * ncand * 8, s));
  GS_TRY(out.alloc((size_t)ncand * 8, s));
  reduce_terms<<<dim3(nblk, (unsigned)ncand), 256, 0, s>>>((double*)terms.ptr, n, k0, k1, chunk,
                                                           (double*)partial.ptr);
  reduce_partials<<<(int)((ncand + 127) / 128), 128, 0, s>>>((double*)partial.ptr, nblk, (int)ncand, (double*)out.ptr);
  GS_CUDA(cudaGetLastError());
  count_launch(2);
  std::vector<double> hll(ncand);
  std::vector<int32_t> hst(ncand);
  GS_CUDA(cudaMemcpyAsync(hll.data(), out.ptr, ncand * 8, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaMemcpyAsync(hst.data(), cstat.ptr, ncand * 4, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaStreamSynchronize(s));
  {
    float a01 = 0, a23 = 0, a03 = 0;
    cudaEventElapsedTime(&a01, ev[0], ev[1]);
    cudaEventElapsedTime(&a23, ev[2], ev[3]);
    cudaEventElapsedTime(&a03, ev[0], ev[3]);
    const double ms4[4] = {0.0, mixed ? (double)a01 : 0.0, (double)a23, (double)a03};
    set_last_timings(ms4, mixed ? nfl : ncand * span);
  }
  for (int64_t c = 0; c < ncand; ++c) {
    if (!valid[c]) continue;
    if (hst[c] != 0) {
      status[c] = hst[c];
      ll[c] = NAN;
    } else {
      ll[c] = hll[c];
    }
  }
  return GS_OK;
}

int64_t vecchia_plan_points(const gs_vecchia_plan* P) { return P->n; }

// ---------------------------------------------- log-likelihood gradient --
// loglik_grad_inner (vecchia.rs:428-530) for single-structure isotropic
// models of the closed-form kinds (g_and_dg, vecchia.rs:353-389): the
// log-likelihood and its derivatives in (nugget, psill, range), per point
// and candidate, reduced per candidate in the same fixed order as the
// log-likelihood.  With w = K^{-1} k the derivative of each conditional
// follows from dw = K^{-1} (dk - dK w) on the same factorisation.
namespace {

// rho = 1 - g and dg/dd at d (df), branch free.
__device__ __forceinline__ void rho_dg_df(int kind, df d, const ExpTable& tab, const DfConsts& k,
                                          df& rho, df& dg) {
  switch (kind) {
    case GS_KIND_SPHERICAL: {
      const bool inside = !(d.hi > 1.0f || (d.hi == 1.0f && d.lo >= 0.0f));
      rho = rho_sph_df(d);
      // 1.5 (1 - d^2); scaling by 1.5 is not exact in FP32, so it goes through df_mul_f
      const df v = df_mul_f(df_add_f(df_neg(df_sqr(d)), 1.0f), 1.5f);
      dg = inside ? v : df_make(0.0f, 0.0f);
      break;
    }
    case GS_KIND_EXPONENTIAL:
      rho = df_expneg(d, tab, k);
      dg = rho;
      break;
    case GS_KIND_GAUSSIAN: {
      rho = df_expneg(df_sqr(d), tab, k);
      const df twod = df_make(2.0f * d.hi, 2.0f * d.lo);
      dg = df_mul(twod, rho);
      break;
    }
    case GS_KIND_MATERN15: {
      const df sq = df_mul(d, df_make(k.s3h, k.s3l));
      const df e = df_expneg(sq, tab, k);
      rho = df_mul(df_add_f(sq, 1.0f), e);
      dg = df_mul(df_mul_f(d, 3.0f), e);
      break;
    }
    default: {  // GS_KIND_MATERN25: dg = 5 d (1 + s) / 3 e
      const df sq = df_mul(d, df_make(k.s5h, k.s5l));
      const df e = df_expneg(sq, tab, k);
      rho = rho_mat25_df(d, tab, k);
      const df num = df_mul(df_mul_f(d, 5.0f), df_add_f(sq, 1.0f));
      const float q = num.hi * (1.0f / 3.0f);
      const df q3 = two_prod(q, 3.0f);
      const float rq = (num.hi - q3.hi - q3.lo + num.lo) * (1.0f / 3.0f);
      dg = df_mul(fast_two_sum(q, rq), e);
      break;
    }
  }
}

// Per-warp shared-memory layout of vecchia_grad_kernel.
struct VGLayout {
  size_t off_a, off_dp, off_dr, off_h, off_v, off_h0, off_z, off_b, off_bp, off_br, off_wv, off_rhs,
      off_row, off_vec, off_xd, total;
};

__host__ __device__ inline VGLayout vecchia_grad_layout(int m, int dim) {
  VGLayout L;
  const int np = m * (m + 1) / 2;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t r = o;
    o += (bytes + 15) & ~(size_t)15;
    return r;
  };
  L.off_a = take((size_t)np * sizeof(df));
  L.off_dp = take((size_t)np * sizeof(df));
  L.off_dr = take((size_t)np * sizeof(df));
  L.off_h = take((size_t)np * sizeof(df));
  L.off_v = take((size_t)dim * m * sizeof(df));
  L.off_h0 = take((size_t)m * sizeof(df));
  L.off_z = take((size_t)m * sizeof(df));
  L.off_b = take((size_t)m * sizeof(df));
  L.off_bp = take((size_t)m * sizeof(df));
  L.off_br = take((size_t)m * sizeof(df));
  L.off_wv = take((size_t)m * sizeof(df));
  L.off_rhs = take((size_t)m * sizeof(df));
  L.off_row = take(kWarpRowFloats * sizeof(float));
  L.off_vec = take(kWarpN * sizeof(float));
  L.off_xd = take(kWarpN * sizeof(df));
  L.total = o;
  return L;
}

// terms: (4 x ncand) x n -- log term, then d/dnugget, d/dpsill, d/drange.
template <int D>
__global__ void __launch_bounds__(32 * kVWarps) vecchia_grad_kernel(VArgs a, ExpTable tab_g,
                                                                   DfConsts kc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ ExpTable tab;
  for (int i = threadIdx.x; i < 256; i += blockDim.x) tab.v[i] = tab_g.v[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int M = a.m;
  const int64_t NC = (int64_t)a.ncand * a.n;
  const VGLayout lay = vecchia_grad_layout(M, D);
  unsigned char* base = smem_raw + (size_t)wib * lay.total;
  df* A = reinterpret_cast<df*>(base + lay.off_a);
  df* DP = reinterpret_cast<df*>(base + lay.off_dp);
  df* DR = reinterpret_cast<df*>(base + lay.off_dr);
  df* H = reinterpret_cast<df*>(base + lay.off_h);
  df* V = reinterpret_cast<df*>(base + lay.off_v);
  df* H0 = reinterpret_cast<df*>(base + lay.off_h0);
  df* ZV = reinterpret_cast<df*>(base + lay.off_z);
  df* B = reinterpret_cast<df*>(base + lay.off_b);
  df* BP = reinterpret_cast<df*>(base + lay.off_bp);
  df* BR = reinterpret_cast<df*>(base + lay.off_br);
  df* WV = reinterpret_cast<df*>(base + lay.off_wv);
  df* RHS = reinterpret_cast<df*>(base + lay.off_rhs);
  WarpScratch W;
  W.row = reinterpret_cast<float*>(base + lay.off_row);
  W.vec = reinterpret_cast<float*>(base + lay.off_vec);
  W.xd = reinterpret_cast<df*>(base + lay.off_xd);
  const int64_t nwarps = (int64_t)gridDim.x * kVWarps;
  for (int64_t k = (int64_t)blockIdx.x * kVWarps + wib; k < a.n; k += nwarps) {
    const int64_t i = a.order[k];
    const int s = a.cnt[k];
    const df zi = df_sub(a.vdf[i], a.mean_df);
    if (s == 0) {
      // first point: N(0, sill); only nugget and psill move the sill
      const double z = df_to_double(zi);
      for (int c = lane; c < a.ncand; c += 32) {
        const double var = a.models[c].c0;
        const int64_t at = (int64_t)c * a.n + k;
        a.terms[at] = -0.5 * (kLn2Pi + log(var) + z * z / var);
        const double common = -0.5 / var + 0.5 * z * z / (var * var);
        a.terms[NC + at] = common;
        a.terms[2 * NC + at] = common;
        a.terms[3 * NC + at] = 0.0;
        a.flag[at] = 0;
      }
      continue;
    }
    __syncwarp();
    if (lane < s) {
      const int j = a.nb[k * (int64_t)M + lane];
#pragma unroll
      for (int d = 0; d < D; ++d)
        V[d * M + lane] = df_sub(a.cdf[(int64_t)d * a.n + j], a.cdf[(int64_t)d * a.n + i]);
      ZV[lane] = df_sub(a.vdf[j], a.mean_df);
    }
    __syncwarp();
    if (lane < s) H0[lane] = norm_origin<D>(V, M, 0, lane);
    for_pairs2(s, lane, 32, [&](int i0, int j0, int i1, int j1, bool two) {
      const df h0 = norm_pair<D>(V, M, 0, i0, j0);
      const df h1 = norm_pair<D>(V, M, 0, i1, j1);
      H[pk(i0, j0)] = h0;
      if (two) H[pk(i1, j1)] = h1;
    });
    __syncwarp();
    for (int c = 0; c < a.ncand; ++c) {
      const DevModel& mdl = a.models[c];
      const DevStruct& st = mdl.s[0];
      const int64_t at = (int64_t)c * a.n + k;
      // covariances and their psill / range derivatives
      auto entry = [&](df h, df& cv, df& dp, df& dr) {
        const df d = df_mul(h, st.inv_range_df);
        df rho, dg;
        rho_dg_df(st.kind, d, tab, kc, rho, dg);
        cv = df_mul(st.sill_df, rho);
        dp = rho;
        dr = df_mul(df_mul(st.sill_df, dg), df_mul(d, st.inv_range_df));
      };
      if (lane < s) {
        entry(H0[lane], B[lane], BP[lane], BR[lane]);
        A[pk(lane, lane)] = mdl.c0_df;
        DP[pk(lane, lane)] = df_make(1.0f, 0.0f);
        DR[pk(lane, lane)] = df_make(0.0f, 0.0f);
      }
      for_pairs2(s, lane, 32, [&](int i0, int j0, int i1, int j1, bool two) {
        df c0, p0, r0;
        entry(H[pk(i0, j0)], c0, p0, r0);
        A[pk(i0, j0)] = c0;
        DP[pk(i0, j0)] = p0;
        DR[pk(i0, j0)] = r0;
        if (two) {
          df c1, p1, r1;
          entry(H[pk(i1, j1)], c1, p1, r1);
          A[pk(i1, j1)] = c1;
          DP[pk(i1, j1)] = p1;
          DR[pk(i1, j1)] = r1;
        }
      });
      __syncwarp();
      // one factorisation, four right-hand sides: the row stays in registers
      RegisterRow row;
      row.load([&](int e) { return A[e]; }, s, lane);
      WarpFactor f;
      bool ok = warp_factor(row, s, lane, f, W) && warp_refine(f, row, B, s, lane, W);
      if (!ok) {
        if (lane == 0) a.flag[at] = 1;
        __syncwarp();
        continue;
      }
      const df w = lane < s ? W.xd[lane] : df_make(0.0f, 0.0f);
      if (lane < s) WV[lane] = w;
      df mu = warp_sum_df(lane < s ? df_mul(w, ZV[lane]) : df_make(0.0f, 0.0f));
      df red = warp_sum_df(lane < s ? df_mul(w, B[lane]) : df_make(0.0f, 0.0f));
      const df rawv = df_sub(mdl.c0_df, red);
      const double raw_var = df_to_double(rawv);
      const double var = fmax(raw_var, 1e-12);
      const bool clamped = raw_var <= 1e-12;
      const double r = df_to_double(df_sub(zi, mu));
      double g3[3];
      for (int prm = 0; prm < 3 && ok; ++prm) {
        __syncwarp();
        // right-hand side: -w (nugget), dk - dK w (psill, range)
        if (lane < s) {
          df rhs = df_neg(w);
          if (prm > 0) {
            const df* DK = prm == 1 ? DP : DR;
            df acc = prm == 1 ? BP[lane] : BR[lane];
            for (int b = 0; b < s; ++b)
              acc = df_sub(acc, df_mul(DK[lane >= b ? pk(lane, b) : pk(b, lane)], WV[b]));
            rhs = acc;
          }
          RHS[lane] = rhs;
        }
        __syncwarp();
        ok = warp_refine(f, row, RHS, s, lane, W);
        if (!ok) break;
        const df dw = lane < s ? W.xd[lane] : df_make(0.0f, 0.0f);
        const df dmu = warp_sum_df(lane < s ? df_mul(dw, ZV[lane]) : df_make(0.0f, 0.0f));
        df dred = lane < s ? df_mul(dw, B[lane]) : df_make(0.0f, 0.0f);
        if (prm > 0 && lane < s) dred = df_add(dred, df_mul(w, prm == 1 ? BP[lane] : BR[lane]));
        dred = warp_sum_df(dred);
        const double dsill = prm < 2 ? 1.0 : 0.0;
        const double dvar = clamped ? 0.0 : dsill - df_to_double(dred);
        const double dm = df_to_double(dmu);
        g3[prm] = -0.5 * dvar / var + r * dm / var + 0.5 * r * r / (var * var) * dvar;
      }
      if (!ok) {
        if (lane == 0) a.flag[at] = 1;
        __syncwarp();
        continue;
      }
      if (lane == 0) {
        a.terms[at] = -0.5 * (kLn2Pi + log(var) + r * r / var);
        a.terms[NC + at] = g3[0];
        a.terms[2 * NC + at] = g3[1];
        a.terms[3 * NC + at] = g3[2];
        a.flag[at] = 0;
      }
      __syncwarp();
    }
  }
}

__device__ __forceinline__ void g_and_dg_fp64(int kind, double d, double& g, double& dg) {
  switch (kind) {
    case GS_KIND_SPHERICAL:
      if (d >= 1.0) {
        g = 1.0;
        dg = 0.0;
      } else {
        g = 1.5 * d - 0.5 * d * d * d;
        dg = 1.5 - 1.5 * d * d;
      }
      break;
    case GS_KIND_EXPONENTIAL: {
      const double e = exp(-d);
      g = 1.0 - e;
      dg = e;
      break;
    }
    case GS_KIND_GAUSSIAN: {
      const double e = exp(-(d * d));
      g = 1.0 - e;
      dg = 2.0 * d * e;
      break;
    }
    case GS_KIND_MATERN15: {
      const double sq = 1.7320508075688772 * d;
      const double e = exp(-sq);
      g = 1.0 - (1.0 + sq) * e;
      dg = 3.0 * d * e;
      break;
    }
    default: {
      const double sq = 2.23606797749979 * d;
      const double e = exp(-sq);
      g = 1.0 - (1.0 + sq + sq * sq / 3.0) * e;
      dg = 5.0 * d * (1.0 + sq) / 3.0 * e;
      break;
    }
  }
}

template <int D>
__device__ __forceinline__ double vg_dist(const VArgs& a, int64_t p, int64_t q) {
  double s2 = 0.0;
  const double* c[3] = {a.x, a.y, a.z};
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const double v = c[d][p] - c[d][q];
    s2 += v * v;
  }
  return sqrt(s2);
}

// One thread per flagged (candidate, point): loglik_grad_inner's per-point
// body in FP64 (vecchia.rs:463-527).  Scratch per thread: K (s x s), then
// k, dk_psill, dk_range, w, dw.
template <int D>
__global__ void vecchia_grad_fp64_kernel(VArgs a, const int64_t* list, int64_t nlist,
                                         double* scratch, int64_t T, int32_t* cand_status) {
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (tid >= T) return;
  const int M = a.m;
  const int64_t NC = (int64_t)a.ncand * a.n;
  double* S = scratch + tid;
  double* KI = scratch + (int64_t)M * M * T + tid;
  double* KP = KI + (int64_t)M * T;
  double* KR = KP + (int64_t)M * T;
  double* Wv = KR + (int64_t)M * T;
  double* DW = Wv + (int64_t)M * T;
  for (int64_t it = tid; it < nlist; it += T) {
    const int64_t code = list ? list[it] : it;
    const int c = (int)(code / a.n);
    const int64_t k = code % a.n;
    const DevModel& mdl = a.models[c];
    const int kind = mdl.s[0].kind;
    const double psill = mdl.s[0].sill, nugget = mdl.nugget, sill = mdl.c0;
    const double range = 1.0 / mdl.s[0].inv_range;
    const int64_t i = a.order[k];
    const int s = a.cnt[k];
    const double zi = a.v[i] - a.mean;
    if (s == 0) {
      a.terms[code] = -0.5 * (kLn2Pi + log(sill) + zi * zi / sill);
      const double common = -0.5 / sill + 0.5 * zi * zi / (sill * sill);
      a.terms[NC + code] = common;
      a.terms[2 * NC + code] = common;
      a.terms[3 * NC + code] = 0.0;
      continue;
    }
    const int32_t* nbk = a.nb + k * (int64_t)M;
    for (int p = 0; p < s; ++p) {
      const double h = vg_dist<D>(a, i, nbk[p]);
      double g, dg;
      g_and_dg_fp64(kind, h / range, g, dg);
      KI[(int64_t)p * T] = sill - (nugget + psill * g);
      KP[(int64_t)p * T] = 1.0 - g;
      KR[(int64_t)p * T] = psill * dg * h / (range * range);
      S[(int64_t)(p * s + p) * T] = sill;
      for (int q = p + 1; q < s; ++q) {
        const double hq = vg_dist<D>(a, nbk[p], nbk[q]);
        double gq, dgq;
        g_and_dg_fp64(kind, hq / range, gq, dgq);
        const double cv = sill - (nugget + psill * gq);
        S[(int64_t)(p * s + q) * T] = cv;
        S[(int64_t)(q * s + p) * T] = cv;
      }
    }
    if (!chol_factor_strided(S, s, T)) {
      atomicExch(&cand_status[c], (int32_t)GS_ERR_SINGULAR_SYSTEM);
      for (int q = 0; q < 4; ++q) a.terms[q * NC + code] = __longlong_as_double(0x7ff8000000000000ll);
      continue;
    }
    for (int p = 0; p < s; ++p) Wv[(int64_t)p * T] = KI[(int64_t)p * T];
    chol_subst_strided(S, Wv, s, T);
    double mu = 0.0, red = 0.0;
    for (int p = 0; p < s; ++p) mu += Wv[(int64_t)p * T] * (a.v[nbk[p]] - a.mean);
    for (int p = 0; p < s; ++p) red += Wv[(int64_t)p * T] * KI[(int64_t)p * T];
    const double raw_var = sill - red;
    const double var = fmax(raw_var, 1e-12);
    const bool clamped = raw_var <= 1e-12;
    const double r = zi - mu;
    a.terms[code] = -0.5 * (kLn2Pi + log(var) + r * r / var);
    for (int prm = 0; prm < 3; ++prm) {
      // rhs = dk - dK w (dK rebuilt from the distances), or -w for the nugget
      for (int p = 0; p < s; ++p) {
        double rhs;
        if (prm == 0) {
          rhs = -Wv[(int64_t)p * T];
        } else {
          double acc = 0.0;
          for (int q = 0; q < s; ++q) {
            double dk;
            if (q == p) {
              dk = prm == 1 ? 1.0 : 0.0;
            } else {
              const double hq = vg_dist<D>(a, nbk[p], nbk[q]);
              double gq, dgq;
              g_and_dg_fp64(kind, hq / range, gq, dgq);
              dk = prm == 1 ? 1.0 - gq : psill * dgq * hq / (range * range);
            }
            acc += dk * Wv[(int64_t)q * T];
          }
          rhs = (prm == 1 ? KP[(int64_t)p * T] : KR[(int64_t)p * T]) - acc;
        }
        DW[(int64_t)p * T] = rhs;
      }
      chol_subst_strided(S, DW, s, T);
      double dmu = 0.0, d1 = 0.0, d2 = 0.0;
      for (int p = 0; p < s; ++p) dmu += DW[(int64_t)p * T] * (a.v[nbk[p]] - a.mean);
      for (int p = 0; p < s; ++p) d1 += DW[(int64_t)p * T] * KI[(int64_t)p * T];
      if (prm > 0)
        for (int p = 0; p < s; ++p)
          d2 += Wv[(int64_t)p * T] * (prm == 1 ? KP[(int64_t)p * T] : KR[(int64_t)p * T]);
      const double dsill = prm < 2 ? 1.0 : 0.0;
      const double dvar = clamped ? 0.0 : dsill - (d1 + d2);
      a.terms[(1 + prm) * NC + code] =
          -0.5 * dvar / var + r * dmu / var + 0.5 * r * r / (var * var) * dvar;
    }
  }
}

}  // namespace

// Single-structure isotropic models of the closed-form kinds only.
int reject_grad_model(const gs_model& m, int dim) {
  GS_TRY(reject_vecchia_model(m, dim));
  if (m.n_structures != 1 || m.s[0].has_anis)
    return fail(GS_ERR_INVALID_PARAMETER,
                "the log-likelihood gradient needs a single isotropic structure");
  const int k = m.s[0].kind;
  if (k != GS_KIND_SPHERICAL && k != GS_KIND_EXPONENTIAL && k != GS_KIND_GAUSSIAN &&
      k != GS_KIND_MATERN15 && k != GS_KIND_MATERN25)
    return fail(GS_ERR_INVALID_PARAMETER, "no closed-form range derivative for this kind");
  return GS_OK;
}

// Log-likelihood and gradient of ncand candidates on a plan.
// guinness_blocks (vecchia.rs:570-602) and each block's joint set
// (vecchia.rs:628-641) on the host, with per-point marks instead of the
// reference's list searches (the same sets, in the same order).
static int build_groups(const gs_vecchia_plan* P, int64_t gsize, gs_vecchia_plan::Groups* out) {
  const int64_t n = P->n, M = P->m;
  std::vector<int32_t> nb((size_t)n * M), cnt(n);
  GS_CUDA(cudaMemcpy(nb.data(), P->d_nb, nb.size() * 4, cudaMemcpyDeviceToHost));
  GS_CUDA(cudaMemcpy(cnt.data(), P->d_cnt, cnt.size() * 4, cudaMemcpyDeviceToHost));
  const std::vector<int64_t>& order = P->order;
  std::vector<int64_t> mark_v(n, -1), mark_b(n, -1);
  std::vector<std::pair<int64_t, int64_t>> blocks;
  int64_t stamp = 0;
  for (int64_t k0 = 0; k0 < n;) {
    ++stamp;
    for (int a = 0; a < cnt[k0]; ++a) mark_v[nb[k0 * M + a]] = stamp;
    mark_b[order[k0]] = stamp;
    int64_t k1 = k0 + 1;
    while (k1 < n && (k1 - k0) < gsize) {
      const int c = cnt[k1];
      const int m = std::max(c, 1);
      int fresh = 0;
      for (int a = 0; a < c; ++a) {
        const int32_t j = nb[k1 * M + a];
        if (mark_v[j] != stamp && mark_b[j] != stamp) ++fresh;
      }
      if ((double)fresh > 0.34 * (double)m) break;
      for (int a = 0; a < c; ++a) {
        const int32_t j = nb[k1 * M + a];
        if (mark_v[j] != stamp && mark_b[j] != stamp) mark_v[j] = stamp;
      }
      mark_b[order[k1]] = stamp;
      ++k1;
    }
    blocks.emplace_back(k0, k1);
    k0 = k1;
  }
  std::vector<int64_t> off(blocks.size() + 1, 0);
  std::vector<int32_t> vid, slen(blocks.size());
  std::vector<int64_t> mark_m(n, -1), mark_s(n, -1);
  int vmax = 0;
  for (size_t b = 0; b < blocks.size(); ++b) {
    const int64_t k0 = blocks[b].first, k1 = blocks[b].second;
    const int64_t st = (int64_t)b;
    for (int64_t k = k0; k < k1; ++k) mark_m[order[k]] = st;
    const size_t start = vid.size();
    for (int64_t k = k0; k < k1; ++k)
      for (int a = 0; a < cnt[k]; ++a) {
        const int32_t j = nb[k * M + a];
        if (mark_m[j] != st && mark_s[j] != st) {
          mark_s[j] = st;
          vid.push_back(j);
        }
      }
    slen[b] = (int32_t)(vid.size() - start);
    for (int64_t k = k0; k < k1; ++k) vid.push_back((int32_t)order[k]);
    off[b + 1] = (int64_t)vid.size();
    vmax = std::max(vmax, (int)(vid.size() - start));
  }
  out->nblocks = (int64_t)blocks.size();
  out->vmax = vmax;
  std::vector<int64_t> multi;
  std::vector<uint8_t> in_multi(n, 0);
  for (size_t b = 0; b < blocks.size(); ++b) {
    if (blocks[b].second - blocks[b].first < 2) continue;
    multi.push_back((int64_t)b);
    out->vmax_multi = std::max(out->vmax_multi, (int)(off[b + 1] - off[b]));
    for (int64_t k = blocks[b].first; k < blocks[b].second; ++k) in_multi[k] = 1;
  }
  out->nmulti = (int64_t)multi.size();
  if (dev_malloc((void**)&out->d_off, off.size() * 8) != cudaSuccess ||
      dev_malloc((void**)&out->d_vid, std::max<size_t>(vid.size(), 1) * 4) != cudaSuccess ||
      dev_malloc((void**)&out->d_slen, slen.size() * 4) != cudaSuccess)
    return fail(GS_ERR_OUT_OF_MEMORY, "grouped plan allocation failed");
  GS_CUDA(cudaMemcpy(out->d_off, off.data(), off.size() * 8, cudaMemcpyHostToDevice));
  GS_CUDA(cudaMemcpy(out->d_vid, vid.data(), vid.size() * 4, cudaMemcpyHostToDevice));
  GS_CUDA(cudaMemcpy(out->d_slen, slen.data(), slen.size() * 4, cudaMemcpyHostToDevice));
  if (dev_malloc((void**)&out->d_multi, std::max<size_t>(multi.size(), 1) * 8) != cudaSuccess ||
      dev_malloc((void**)&out->d_in_multi, (size_t)n) != cudaSuccess)
    return fail(GS_ERR_OUT_OF_MEMORY, "grouped plan allocation failed");
  if (!multi.empty())
    GS_CUDA(cudaMemcpy(out->d_multi, multi.data(), multi.size() * 8, cudaMemcpyHostToDevice));
  GS_CUDA(cudaMemcpy(out->d_in_multi, in_multi.data(), (size_t)n, cudaMemcpyHostToDevice));
  return GS_OK;
}

// The blocks of one group size, built on first use and kept on the plan.
int plan_groups(const gs_vecchia_plan* P, int64_t gsize, gs_vecchia_plan::Groups* G) {
  std::lock_guard<std::mutex> lk(P->groups_mu);
  auto it = P->groups.find(gsize);
  if (it == P->groups.end()) {
    gs_vecchia_plan::Groups fresh;
    const int rc = build_groups(P, gsize, &fresh);
    if (rc) {
      cudaFree(fresh.d_off);
      cudaFree(fresh.d_vid);
      cudaFree(fresh.d_slen);
      cudaFree(fresh.d_multi);
      cudaFree(fresh.d_in_multi);
      return rc;
    }
    it = P->groups.emplace(gsize, fresh).first;
  }
  *G = it->second;
  return GS_OK;
}

// One launch of vecchia_group_kernel over every (candidate, block) and the
// fixed-order reduction over blocks: per candidate the log-likelihood
// (nr = 1) or the reml_sums(nr - 1) REML sums, into sums[c * per + w].
// status[c] / valid[c] as in vecchia_eval.
int eval_blocks(const gs_vecchia_plan* P, int64_t ncand, const gs_model* models,
                const gs_vecchia_plan::Groups& G, int nr, const double* d_basis, bool clamp,
                std::vector<double>& sums, int32_t* status, std::vector<int>& valid,
                cudaStream_t s, bool multi_only = false) {
  const gs_pointset* ps = P->ps;
  const int dim = ps->dim;
  const bool reml = d_basis != nullptr;
  const int per = reml ? reml_sums(nr - 1) : 1;
  std::vector<DevModel> dms(std::max<int64_t>(ncand, 1));
  valid.assign(ncand, 0);
  sums.assign((size_t)ncand * per, NAN);
  for (int64_t c = 0; c < ncand; ++c) {
    status[c] = GS_OK;
    int rc = reject_vecchia_model(models[c], dim);
    if (!rc) rc = make_dev_model(models[c], dim, &dms[c], true);
    if (rc) {
      status[c] = rc;
      dms[c] = DevModel{};
      dms[c].c0 = 1.0;
      continue;
    }
    valid[c] = 1;
  }
  if (ncand == 0) return GS_OK;
  const int64_t nbl = multi_only ? G.nmulti : G.nblocks;
  if (nbl == 0) {  // nothing to evaluate: every valid candidate's sums are zero
    for (int64_t c = 0; c < ncand; ++c)
      if (valid[c])
        for (int w = 0; w < per; ++w) sums[(size_t)c * per + w] = 0.0;
    return GS_OK;
  }
  const int frame = (multi_only ? G.vmax_multi : G.vmax) + nr;
  const size_t ptab_bytes = (((size_t)frame * (frame - 1) / 2) * 4 + 15) & ~(size_t)15;
  const size_t per_warp = group_warp_doubles(frame) * 8;
  const int sms = sm_count();
  int dev = 0, per_sm = 0, smem_max = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  smem_max -= 2048;  // the kernel's static shared memory (the exp table)
  if (frame > 255 || ptab_bytes + per_warp > (size_t)smem_max)
    return fail(GS_ERR_INVALID_PARAMETER,
                "a grouped conditioning set of " + std::to_string(G.vmax) + " points with " +
                    std::to_string(nr) + " data rows exceeds the CUDA path's shared-memory frame");
  const int wpb = (int)std::max<size_t>(
      1, std::min<size_t>(4, (std::min<size_t>(smem_max, 200 * 1024) - ptab_bytes) / per_warp));
  const size_t smem = ptab_bytes + wpb * per_warp;
  DevBuf dmod, terms, partial, out, cstat;
  GS_TRY(dmod.alloc(sizeof(DevModel) * ncand, s));
  GS_CUDA(cudaMemcpyAsync(dmod.ptr, dms.data(), sizeof(DevModel) * ncand, cudaMemcpyHostToDevice, s));
  const int64_t rows = ncand * per;
  GS_TRY(terms.alloc((size_t)rows * nbl * 8, s));
  GS_TRY(cstat.alloc((size_t)ncand * 4, s));
  GS_CUDA(cudaMemsetAsync(cstat.ptr, 0, ncand * 4, s));
  VArgs a{};
  a.dim = dim;
  a.n = P->n;
  a.k0 = 0;
  a.k1 = P->n;
  a.m = (int)P->m;
  a.ncand = (int)ncand;
  a.x = ps->d_x;
  a.y = ps->d_y;
  a.z = ps->d_z;
  a.v = ps->d_v;
  a.mean = P->mean;
  a.models = (const DevModel*)dmod.ptr;
  a.terms = (double*)terms.ptr;
  GroupArgs g{G.d_off, G.d_vid, G.d_slen, nbl, multi_only ? G.d_multi : nullptr, frame, nr,
              d_basis, clamp ? 1 : 0};
  auto kern = reml ? (dim == 2 ? vecchia_group_kernel<2, true> : vecchia_group_kernel<3, true>)
                   : (dim == 2 ? vecchia_group_kernel<2, false> : vecchia_group_kernel<3, false>);
  GS_TRY(allow_dynamic_smem((const void*)kern, smem));
  GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * wpb, smem));
  const int64_t items = ncand * nbl;
  const int blocks = (int)std::max<int64_t>(
      1, std::min<int64_t>((items + wpb - 1) / wpb, (int64_t)sms * std::max(per_sm, 1)));
  ensure_vtables();
  kern<<<blocks, 32 * wpb, smem, s>>>(a, g, wpb, (int32_t*)cstat.ptr, g_vet);
  GS_CUDA(cudaGetLastError());
  const int64_t chunk = 8192;
  const int nblk = (int)((nbl + chunk - 1) / chunk);
  GS_TRY(partial.alloc((size_t)nblk * rows * 8, s));
  GS_TRY(out.alloc((size_t)rows * 8, s));
  int launches = 1;
  for (int64_t r0 = 0; r0 < rows; r0 += 65535) {
    const int64_t nr_ = std::min<int64_t>(65535, rows - r0);
    reduce_terms<<<dim3(nblk, (unsigned)nr_), 256, 0, s>>>(
        (double*)terms.ptr + r0 * nbl, nbl, 0, nbl, chunk, (double*)partial.ptr + r0 * nblk);
    ++launches;
  }
  reduce_partials<<<(int)((rows + 127) / 128), 128, 0, s>>>((double*)partial.ptr, nblk, (int)rows,
                                                            (double*)out.ptr);
  GS_CUDA(cudaGetLastError());
  count_launch(launches + 1);
  std::vector<double> hout(rows);
  std::vector<int32_t> hst(ncand);
  GS_CUDA(cudaMemcpyAsync(hout.data(), out.ptr, rows * 8, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaMemcpyAsync(hst.data(), cstat.ptr, ncand * 4, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaStreamSynchronize(s));
  for (int64_t c = 0; c < ncand; ++c) {
    if (!valid[c]) continue;
    if (hst[c] != 0) {
      status[c] = hst[c];
      continue;
    }
    for (int w = 0; w < per; ++w) sums[c * per + w] = hout[c * per + w];
  }
  return GS_OK;
}

int vecchia_eval_grouped(const gs_vecchia_plan* P, int64_t ncand, const gs_model* models,
                         int64_t gsize, double* ll, int32_t* status, cudaStream_t s) {
  NvtxRange nvtx_range("gs.vecchia_loglik_grouped");
  if (gsize <= 1) return vecchia_eval(P, ncand, models, ll, status, GS_PREC_MIXED, s);
  gs_vecchia_plan::Groups G;
  GS_TRY(plan_groups(P, gsize, &G));
  // A one-member block's term is the ungrouped term of its point (its joint
  // set is the point's conditioning set): those go through the mixed
  // ungrouped path, which leaves out the positions of larger blocks; the
  // larger blocks run on the FP64 block kernel.
  GS_TRY(vecchia_eval(P, ncand, models, ll, status, GS_PREC_MIXED, s,
                      G.nmulti ? G.d_in_multi : nullptr));
  if (G.nmulti == 0) return GS_OK;
  std::vector<double> sums;
  std::vector<int> valid;
  std::vector<int32_t> st2(ncand);
  GS_TRY(eval_blocks(P, ncand, models, G, 1, nullptr, false, sums, st2.data(), valid, s, true));
  for (int64_t c = 0; c < ncand; ++c) {
    if (status[c] == 0 && st2[c] != 0) status[c] = st2[c];
    ll[c] = (status[c] == 0) ? ll[c] + sums[c] : NAN;
  }
  return GS_OK;
}

// The GLS step of reml_loglik_with_plan (vecchia.rs:1347-1356): A = F'S^-1F
// and c = F'S^-1z from the sums, LU with partial pivoting (lu_factor's
// pivot test: the largest candidate below 1e-12 max|A| is singular), then
//     ll = -1/2 ((n - p) ln 2 pi + ln det S + ln |det A| + z'S^-1z - c'beta).
int gls_finish(int64_t n, int p, const double* sums, double* ll) {
  std::vector<double> A((size_t)p * p), c(p);
  int w = 2 + p;
  for (int f = 0; f < p; ++f) {
    c[f] = sums[2 + f];
    for (int g = f; g < p; ++g, ++w) A[(size_t)f * p + g] = A[(size_t)g * p + f] = sums[w];
  }
  double scale = 2.2250738585072014e-308;
  for (double v : A) scale = std::fmax(scale, std::fabs(v));
  std::vector<int> piv(p);
  for (int k = 0; k < p; ++k) {
    int best = k;
    double mx = std::fabs(A[(size_t)k * p + k]);
    for (int i = k + 1; i < p; ++i)
      if (std::fabs(A[(size_t)i * p + k]) > mx) {
        mx = std::fabs(A[(size_t)i * p + k]);
        best = i;
      }
    if (!(mx >= 1e-12 * scale)) return GS_ERR_SINGULAR_SYSTEM;
    piv[k] = best;
    if (best != k)
      for (int j = 0; j < p; ++j) std::swap(A[(size_t)k * p + j], A[(size_t)best * p + j]);
    for (int i = k + 1; i < p; ++i) {
      const double f = A[(size_t)i * p + k] / A[(size_t)k * p + k];
      A[(size_t)i * p + k] = f;
      if (f != 0.0)
        for (int j = k + 1; j < p; ++j) A[(size_t)i * p + j] -= f * A[(size_t)k * p + j];
    }
  }
  std::vector<double> beta = c;
  for (int k = 0; k < p; ++k) std::swap(beta[k], beta[piv[k]]);
  for (int i = 0; i < p; ++i)
    for (int j = 0; j < i; ++j) beta[i] -= A[(size_t)i * p + j] * beta[j];
  for (int i = p - 1; i >= 0; --i) {
    for (int j = i + 1; j < p; ++j) beta[i] -= A[(size_t)i * p + j] * beta[j];
    beta[i] /= A[(size_t)i * p + i];
  }
  double ln_det_a = 0.0, cb = 0.0;
  for (int i = 0; i < p; ++i) {
    ln_det_a += std::log(std::fabs(A[(size_t)i * p + i]));
    cb += c[i] * beta[i];
  }
  *ll = -0.5 * ((double)(n - p) * kLn2Pi + sums[0] + ln_det_a + (sums[1] - cb));
  return GS_OK;
}

// Vecchia REML log-likelihoods of ncand candidates with the trend basis
// d_basis (p x n on the device, column-major): reml_loglik_with_plan
// (gsize <= 1, as singleton blocks) or reml_loglik_with_blocks.
int vecchia_eval_reml(const gs_vecchia_plan* P, int64_t ncand, const gs_model* models,
                      int64_t gsize, const double* d_basis, int p, double* ll, int32_t* status,
                      cudaStream_t s) {
  NvtxRange nvtx_range("gs.vecchia_reml");
  const int per_m = reml_sums(p);
  if (P->m <= kWarpN) {
    // the ungrouped REML through the mixed warp kernel (the conditioning
    // solve of the likelihood, plus the basis rows' residuals); grouped:
    // one-member blocks the same way (their sums are their points'), the
    // larger blocks on the FP64 block kernel
    gs_vecchia_plan::Groups G;
    if (gsize > 1) GS_TRY(plan_groups(P, gsize, &G));
    std::vector<double> sums((size_t)std::max<int64_t>(ncand, 1) * per_m, NAN);
    GS_TRY(vecchia_eval(P, ncand, models, ll, status, GS_PREC_MIXED, s,
                        G.nmulti ? G.d_in_multi : nullptr, d_basis, p, sums.data()));
    if (G.nmulti) {
      std::vector<double> sums2;
      std::vector<int> valid;
      std::vector<int32_t> st2(ncand);
      GS_TRY(eval_blocks(P, ncand, models, G, 1 + p, d_basis, false, sums2, st2.data(), valid, s,
                         true));
      for (int64_t c = 0; c < ncand; ++c) {
        if (status[c] == 0 && st2[c] != 0) status[c] = st2[c];
        for (int w = 0; w < per_m; ++w) sums[(size_t)c * per_m + w] += sums2[(size_t)c * per_m + w];
      }
    }
    for (int64_t c = 0; c < ncand; ++c) {
      ll[c] = NAN;
      if (status[c] != 0) continue;
      const int rc = gls_finish(P->n, p, &sums[(size_t)c * per_m], &ll[c]);
      if (rc) status[c] = rc;
    }
    return GS_OK;
  }
  gs_vecchia_plan::Groups G;
  GS_TRY(plan_groups(P, std::max<int64_t>(gsize, 1), &G));
  std::vector<double> sums;
  std::vector<int> valid;
  GS_TRY(eval_blocks(P, ncand, models, G, 1 + p, d_basis, gsize <= 1, sums, status, valid, s));
  const int per = reml_sums(p);
  for (int64_t c = 0; c < ncand; ++c) {
    ll[c] = NAN;
    if (!valid[c] || status[c] != 0) continue;
    const int rc = gls_finish(P->n, p, &sums[(size_t)c * per], &ll[c]);
    if (rc) status[c] = rc;
  }
  return GS_OK;
}

int vecchia_eval_grad(const gs_vecchia_plan* P, int64_t ncand, const gs_model* models, double* ll,
                      double* grad, int32_t* status, int precision, cudaStream_t s) {
  NvtxRange nvtx_range("gs.vecchia_grad");
  const gs_pointset* ps = P->ps;
  const int dim = ps->dim;
  const int64_t n = P->n;
  const int M = (int)P->m;
  ensure_vtables();
  std::vector<DevModel> dms(std::max<int64_t>(ncand, 1));
  for (int64_t c = 0; c < ncand; ++c) {
    status[c] = GS_OK;
    ll[c] = NAN;
    for (int q = 0; q < 3; ++q) grad[c * 3 + q] = NAN;
    int rc = reject_grad_model(models[c], dim);
    if (!rc) rc = make_dev_model(models[c], dim, &dms[c], true);
    if (rc) {
      // a harmless stand-in the kernels can evaluate; its results are dropped
      status[c] = rc;
      gs_model stand{};
      stand.nugget = 0.1;
      stand.n_structures = 1;
      stand.s[0].kind = GS_KIND_EXPONENTIAL;
      stand.s[0].sill = 1.0;
      stand.s[0].range = 1.0;
      make_dev_model(stand, dim, &dms[c], true);
    }
  }
  if (ncand == 0) return GS_OK;
  const int64_t NC = ncand * n;
  DevBuf dmod, terms, flag, partial, out, cstat, list;
  GS_TRY(dmod.alloc(sizeof(DevModel) * ncand, s));
  GS_CUDA(cudaMemcpyAsync(dmod.ptr, dms.data(), sizeof(DevModel) * ncand, cudaMemcpyHostToDevice, s));
  GS_TRY(terms.alloc((size_t)4 * NC * 8, s));
  GS_TRY(flag.alloc((size_t)NC, s));
  GS_TRY(cstat.alloc((size_t)ncand * 4, s));
  GS_CUDA(cudaMemsetAsync(cstat.ptr, 0, ncand * 4, s));
  VArgs a{};
  a.dim = dim;
  a.n = n;
  a.k0 = 0;
  a.k1 = n;
  a.m = M;
  a.ncand = (int)ncand;
  a.iso_shared = 1;
  a.x = ps->d_x;
  a.y = ps->d_y;
  a.z = ps->d_z;
  a.v = ps->d_v;
  a.mean = P->mean;
  a.cdf = (const df*)ps->d_cdf;
  a.vdf = (const df*)ps->d_vdf;
  a.mean_df = df_from_double(P->mean);
  a.order = P->d_order;
  a.nb = P->d_nb;
  a.cnt = P->d_cnt;
  a.models = (const DevModel*)dmod.ptr;
  a.terms = (double*)terms.ptr;
  a.flag = (uint8_t*)flag.ptr;
  int64_t nfl = 0;
  const bool mixed = precision != GS_PREC_FP64 && M <= kWarpN;
  if (mixed) {
    const int sms = sm_count();
    const size_t smem = vecchia_grad_layout(std::max(M, 1), dim).total * kVWarps;
    auto kern = dim == 2 ? vecchia_grad_kernel<2> : vecchia_grad_kernel<3>;
    GS_TRY(allow_dynamic_smem((const void*)kern, smem));
    int per_sm = 0;
    GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * kVWarps, smem));
    per_sm = std::max(per_sm, 1);
    const int blocks = (int)std::min<int64_t>((n + kVWarps - 1) / kVWarps, (int64_t)sms * per_sm);
    kern<<<blocks, 32 * kVWarps, smem, s>>>(a, g_vtab, g_vkc);
    GS_CUDA(cudaGetLastError());
    count_launch(1);
    DevBuf nsel, tmp;
    GS_TRY(nsel.alloc(8, s));
    GS_TRY(list.alloc((size_t)NC * 8, s));
    size_t tb = 0;
    GS_CUDA(cub::DeviceSelect::Flagged(nullptr, tb, thrust::counting_iterator<int64_t>(0),
                                       (uint8_t*)flag.ptr, (int64_t*)list.ptr, (int64_t*)nsel.ptr,
                                       NC, s));
    GS_TRY(tmp.alloc(tb, s));
    GS_CUDA(cub::DeviceSelect::Flagged(tmp.ptr, tb, thrust::counting_iterator<int64_t>(0),
                                       (uint8_t*)flag.ptr, (int64_t*)list.ptr, (int64_t*)nsel.ptr,
                                       NC, s));
    GS_CUDA(cudaMemcpyAsync(&nfl, nsel.ptr, 8, cudaMemcpyDeviceToHost, s));
    GS_CUDA(cudaStreamSynchronize(s));
  }
  if (!mixed || nfl > 0) {
    const int64_t work = mixed ? nfl : NC;
    const int64_t per = ((int64_t)M * M + 5 * (int64_t)M) * 8;
    // 512 threads per SM: measured fastest (the strided scratch then stays
    // mostly in L2; more threads spill it to HBM)
    int64_t T = std::min<int64_t>(std::max<int64_t>(((int64_t)1 << 31) / std::max<int64_t>(per, 1), 128), (int64_t)sm_count() * 512);
    T = std::min<int64_t>(T, ((work + 127) / 128) * 128);
    T = std::max<int64_t>(T, 128);
    DevBuf scratch;
    GS_TRY(scratch.alloc((size_t)T * per, s));
    const int blocks = (int)((T + 127) / 128);
    if (dim == 2)
      vecchia_grad_fp64_kernel<2><<<blocks, 128, 0, s>>>(a, mixed ? (const int64_t*)list.ptr : nullptr,
                                                         work, (double*)scratch.ptr, T, (int32_t*)cstat.ptr);
    else
      vecchia_grad_fp64_kernel<3><<<blocks, 128, 0, s>>>(a, mixed ? (const int64_t*)list.ptr : nullptr,
                                                         work, (double*)scratch.ptr, T, (int32_t*)cstat.ptr);
    GS_CUDA(cudaGetLastError());
    count_launch(1);
  }
  const int64_t chunk = 8192;
  const int nblk = (int)((n + chunk - 1) / chunk);
  GS_TRY(partial.alloc((size_t)nblk * 4 * ncand * 8, s));
  GS_TRY(out.alloc((size_t)4 * ncand * 8, s));
  reduce_terms<<<dim3(nblk, (unsigned)(4 * ncand)), 256, 0, s>>>((double*)terms.ptr, n, 0, n, chunk,
                                                                  (double*)partial.ptr);
  reduce_partials<<<(int)((4 * ncand + 127) / 128), 128, 0, s>>>((double*)partial.ptr, nblk,
                                                                 (int)(4 * ncand), (double*)out.ptr);
  GS_CUDA(cudaGetLastError());
  count_launch(2);
  std::vector<double> hout(4 * ncand);
  std::vector<int32_t> hst(ncand);
  GS_CUDA(cudaMemcpyAsync(hout.data(), out.ptr, 4 * ncand * 8, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaMemcpyAsync(hst.data(), cstat.ptr, ncand * 4, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaStreamSynchronize(s));
  for (int64_t c = 0; c < ncand; ++c) {
    if (status[c] != GS_OK) continue;
    if (hst[c] != GS_OK) {
      status[c] = hst[c];
      continue;
    }
    ll[c] = hout[c];
    for (int q = 0; q < 3; ++q) grad[c * 3 + q] = hout[(1 + q) * ncand + c];
  }
  return GS_OK;
}

// vecchia_plan (vecchia.rs:232-282).
int plan_create(const gs_pointset* ps, int64_t m, const int64_t* order, gs_vecchia_plan** out) {
  NvtxRange nvtx_range("gs.vecchia_plan");
  *out = nullptr;
  const int64_t n = ps->n;
  const int dim = ps->dim;
  if (n < 2) return fail(GS_ERR_INSUFFICIENT_DATA, "Vecchia requires at least 2 points");
  if (m <= 0) return fail(GS_ERR_INVALID_PARAMETER, "conditioning size m must be at least 1");
  if (ps->has_dup)
    return fail(GS_ERR_DUPLICATE_POINTS, "duplicate data points: indices " + std::to_string(ps->dup_i) +
                                             " and " + std::to_string(ps->dup_j) +
                                             " share the same coordinates");
  auto* P = new gs_vecchia_plan();
  P->ps = ps;
  P->n = n;
  P->m = std::min<int64_t>(m, n - 1);
  P->order.resize(n);
  if (order) {
    std::vector<char> seen(n, 0);
    for (int64_t k = 0; k < n; ++k) {
      if (order[k] < 0 || order[k] >= n || seen[order[k]]) {
        delete P;
        return fail(GS_ERR_INVALID_PARAMETER, "order must be a permutation of 0..n-1");
      }
      seen[order[k]] = 1;
      P->order[k] = order[k];
    }
  } else {
    maxmin_order(ps->host, dim, n, P->order.data());
  }
  double sum = 0.0;
  for (int64_t i = 0; i < n; ++i) sum += ps->values[i];
  P->mean = sum / (double)n;
  int rc = cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking) == cudaSuccess
               ? GS_OK
               : fail(GS_ERR_CUDA, "stream creation failed");
  cudaStream_t s = P->stream;
  const int M = (int)P->m;
  if (!rc && (dev_malloc((void**)&P->d_order, n * 8) != cudaSuccess ||
              dev_malloc((void**)&P->d_nb, (size_t)n * M * 4) != cudaSuccess ||
              dev_malloc((void**)&P->d_cnt, n * 4) != cudaSuccess))
    rc = fail(GS_ERR_OUT_OF_MEMORY, "plan allocation failed");
  if (!rc) {
    DevBuf ox, oy, oz;
    rc = ox.alloc(n * 8, s);
    if (!rc) rc = oy.alloc(n * 8, s);
    if (!rc && dim == 3) rc = oz.alloc(n * 8, s);
    if (!rc) {
      cudaMemcpyAsync(P->d_order, P->order.data(), n * 8, cudaMemcpyHostToDevice, s);
      const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 32);
      gather_by_order<<<blocks, 256, 0, s>>>(n, P->d_order, ps->d_x, ps->d_y, ps->d_z,
                                            (double*)ox.ptr, (double*)oy.ptr,
                                            dim == 3 ? (double*)oz.ptr : nullptr);
      Grid g;
      rc = grid_build_ranked(&g, dim, n, (double*)ox.ptr, (double*)oy.ptr, (double*)oz.ptr,
                             dim == 2 ? 2.0 : 3.0, s);
      if (!rc) {
        SearchFrame f;
        std::memset(&f, 0, sizeof(f));
        SearchParams sp{};
        sp.k = M;
        sp.kout = M;
        sp.ranked = 1;
        sp.rank0 = 0;
        sp.brute_below = 2048;
        sp.px = (double*)ox.ptr;
        sp.py = (double*)oy.ptr;
        sp.pz = (double*)oz.ptr;
        rc = search_launch(g, f, sp, n, (double*)ox.ptr, (double*)oy.ptr, (double*)oz.ptr, P->d_nb,
                           P->d_cnt, s);
      }
      if (!rc) {
        positions_to_ids<<<(int)std::min<int64_t>((n * M + 255) / 256, (int64_t)sm_count() * 64), 256, 0, s>>>(
            n * M, P->d_order, P->d_nb);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
          rc = fail(GS_ERR_CUDA, "plan kernels failed");
      }
    }
  }
  if (rc) {
    delete P;
    return rc;
  }
  *out = P;
  return GS_OK;
}

// ------------------------------------------------------ joint prediction --
// vecchia_predict (vecchia.rs:748-866).  The conditioning store holds the
// data (store index i = data index) followed by the targets in max-min
// processing order (store index n + k for position k).  Target k conditions
// on its m nearest store points of smaller index -- the ranked device search,
// ties by store index like the reference's incremental BucketGrid.  A target
// depends only on the targets in its conditioning set, so the targets are
// solved level by level: level 0 conditions on data alone, level L on
// targets of lower levels.  Per level, one warp per target solves its
// conditional system (double-float assembly, FP32 inverse, refinement; the
// reference's FP64 Cholesky for systems the refinement cannot certify) and
// writes its weights, conditional mean and innovation variance; then one warp
// per target merges the innovation rows of its conditioning targets.

struct VPArgs {
  int64_t n;            // data points
  int64_t ns;           // store size n + nt
  int kout;             // neighbour slots per target
  const int32_t* nb;    // nt x kout store indices, nearest first
  const int32_t* cnt;
  const df* cdf;        // store coordinates as df, [dim][ns]
  const double* sx;
  const double* sy;
  const double* sz;
  double* smean64;      // conditional means: data z_i, then targets
  df* smean_df;
  double* w64;          // nt x kout conditioning weights
  double* d64;          // innovation variances
  uint8_t* flag;        // 1: solve in FP64
  const int64_t* list;  // the level's targets
  int64_t nlist;
  int32_t* err;         // GS_ERR_SINGULAR_SYSTEM after an FP64 Cholesky failure
};

constexpr int kVPWarps = 4;

// Store coordinates as double-float and the data's centred values.
__global__ void vp_store_kernel(int dim, int64_t n, int64_t ns, const double* sx, const double* sy,
                                const double* sz, const double* v, double mean, df* cdf,
                                double* smean64, df* smean_df) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < ns;
       j += (int64_t)gridDim.x * blockDim.x) {
    cdf[j] = df_from_double(sx[j]);
    cdf[ns + j] = df_from_double(sy[j]);
    if (dim == 3) cdf[2 * ns + j] = df_from_double(sz[j]);
    if (j < n) {
      const double z = v[j] - mean;
      smean64[j] = z;
      smean_df[j] = df_from_double(z);
    }
  }
}

// One warp per target of a level (conditioning sets of at most 32 points).
template <int D>
__global__ void __launch_bounds__(32 * kVPWarps) vp_solve_kernel(VPArgs a, DevModel m, ExpTable tab_g,
                                                                DfConsts kc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ ExpTable tab;
  for (int q = threadIdx.x; q < 256; q += blockDim.x) tab.v[q] = tab_g.v[q];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int M = a.kout;
  const VWLayout lay = vecchia_warp_layout(M, D);
  unsigned char* base = smem_raw + (size_t)wib * lay.total;
  df* A = reinterpret_cast<df*>(base + lay.off_a);
  df* V = reinterpret_cast<df*>(base + lay.off_v);
  df* B = reinterpret_cast<df*>(base + lay.off_b);
  WarpScratch W;
  W.row = reinterpret_cast<float*>(base + lay.off_row);
  W.vec = reinterpret_cast<float*>(base + lay.off_vec);
  W.xd = reinterpret_cast<df*>(base + lay.off_xd);
  const Frames fr = frames_of(m);
  const double* sc[3] = {a.sx, a.sy, a.sz};
  for (int64_t it = (int64_t)blockIdx.x * kVPWarps + wib; it < a.nlist;
       it += (int64_t)gridDim.x * kVPWarps) {
    const int64_t k = a.list[it];
    const int s = a.cnt[k];
    const int32_t* nbk = a.nb + k * (int64_t)M;
    const int64_t tix = a.n + k;
    __syncwarp();
    if (s == 0) {
      if (lane == 0) {
        a.smean64[tix] = 0.0;
        a.smean_df[tix] = df_make(0.0f, 0.0f);
        a.d64[k] = m.c0;
        a.flag[k] = 0;
      }
      continue;
    }
    if (lane < s) {
      const int j = nbk[lane];
      df ud[3];
      bool zero = true;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        ud[d] = df_sub(a.cdf[(int64_t)d * a.ns + j], a.cdf[(int64_t)d * a.ns + tix]);
        zero = zero && same_double(sc[d][j], sc[d][tix]);
      }
      frame_coords<D>(m, fr, ud, V, M, lane);
      B[lane] = zero ? m.c0_df : cov_origin<D>(m, fr, V, M, lane, tab, kc);
      A[pk(lane, lane)] = m.c0_df;
    }
    __syncwarp();
    for_pairs2(s, lane, 32, [&](int i0, int j0, int i1, int j1, bool two) {
      df c0, c1;
      cov_pair2<D>(m, fr, V, M, i0, j0, i1, j1, tab, kc, c0, c1);
      A[pk(i0, j0)] = c0;
      if (two) A[pk(i1, j1)] = c1;
    });
    __syncwarp();
    const bool ok = warp_solve(A, B, s, lane, W);
    if (!ok) {
      if (lane == 0) a.flag[k] = 1;
      __syncwarp();
      continue;
    }
    const df w = lane < s ? W.xd[lane] : df_make(0.0f, 0.0f);
    df mu = lane < s ? df_mul(w, a.smean_df[nbk[lane]]) : df_make(0.0f, 0.0f);
    df red = lane < s ? df_mul(w, B[lane]) : df_make(0.0f, 0.0f);
    mu = warp_sum_df(mu);
    red = warp_sum_df(red);
    if (lane < s) a.w64[k * (int64_t)M + lane] = df_to_double(w);
    if (lane == 0) {
      a.smean64[tix] = df_to_double(mu);
      a.smean_df[tix] = mu;
      a.d64[k] = fmax(df_to_double(df_sub(m.c0_df, red)), 0.0);
      a.flag[k] = 0;
    }
    __syncwarp();
  }
}

// One thread per target of a level in FP64, the reference's algorithm:
// K_SS and k_i from c0 - gamma (vecchia.rs:808-817), cholesky_solve_in_place,
// mu and d in conditioning order.  all = 0: only flagged targets.
template <int D>
__global__ void vp_fp64_kernel(VPArgs a, DevModel m, double* scratch, int64_t T, int all) {
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (tid >= T) return;
  const int M = a.kout;
  double* S = scratch + tid;
  double* W = scratch + (int64_t)M * M * T + tid;
  double* K0 = W + (int64_t)M * T;
  for (int64_t it = tid; it < a.nlist; it += T) {
    const int64_t k = a.list[it];
    if (!all && !a.flag[k]) continue;
    const int s = a.cnt[k];
    const int64_t tix = a.n + k;
    if (s == 0) {
      a.smean64[tix] = 0.0;
      a.smean_df[tix] = df_make(0.0f, 0.0f);
      a.d64[k] = m.c0;
      a.flag[k] = 0;
      continue;
    }
    const int32_t* nbk = a.nb + k * (int64_t)M;
    const double pt[3] = {a.sx[tix], a.sy[tix], D == 3 ? a.sz[tix] : 0.0};
    for (int aa = 0; aa < s; ++aa) {
      const int ja = nbk[aa];
      const double h[3] = {pt[0] - a.sx[ja], pt[1] - a.sy[ja], D == 3 ? pt[2] - a.sz[ja] : 0.0};
      const double kv = cov_fp64<D>(m, h);
      W[(int64_t)aa * T] = kv;
      K0[(int64_t)aa * T] = kv;
      for (int bb = aa; bb < s; ++bb) {
        const int jb = nbk[bb];
        const double g[3] = {a.sx[ja] - a.sx[jb], a.sy[ja] - a.sy[jb],
                             D == 3 ? a.sz[ja] - a.sz[jb] : 0.0};
        const double cv = cov_fp64<D>(m, g);
        S[(int64_t)(aa * s + bb) * T] = cv;
        S[(int64_t)(bb * s + aa) * T] = cv;
      }
    }
    if (!chol_solve_strided(S, W, s, T)) {
      atomicExch(a.err, (int32_t)GS_ERR_SINGULAR_SYSTEM);
      a.flag[k] = 0;
      continue;
    }
    double mu = 0.0, red = 0.0;
    for (int q = 0; q < s; ++q) mu += W[(int64_t)q * T] * a.smean64[nbk[q]];
    for (int q = 0; q < s; ++q) red += W[(int64_t)q * T] * K0[(int64_t)q * T];
    for (int q = 0; q < s; ++q) a.w64[k * (int64_t)M + q] = W[(int64_t)q * T];
    a.smean64[tix] = mu;
    a.smean_df[tix] = df_from_double(mu);
    a.d64[k] = fmax(m.c0 - red, 0.0);
    a.flag[k] = 0;
  }
}

// Upper bound of each merged innovation row: 1 + the parents' row lengths.
__global__ void vp_bound_kernel(const int64_t* list, int64_t nlist, int64_t n, int kout,
                                const int32_t* nb, const int32_t* cnt, const int32_t* row_len,
                                int64_t* bound) {
  for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < nlist;
       it += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = list[it];
    int64_t b = 1;
    for (int q = 0; q < cnt[k]; ++q) {
      const int j = nb[k * (int64_t)kout + q];
      if (j >= n) b += row_len[j - n];
    }
    bound[it] = b;
  }
}

__device__ __forceinline__ int warp_min_i(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Innovation rows (vecchia.rs:830-849): one warp per target; lane l follows
// the rows of conditioning points l, l + 32, ... (rows are sorted by
// innovation id); every step takes the smallest pending id, sums w_q * coef
// over the rows holding it, keeps the sum when |sum| > tol, and finally
// appends the target's own innovation sqrt(d).  var = sum of the squared
// kept coefficients in id order.
constexpr int kVPParentsPerLane = (GS_MAX_SYSTEM + 31) / 32;

__global__ void vp_merge_kernel(const int64_t* list, int64_t nlist, int64_t n, int kout,
                                const int32_t* nb, const int32_t* cnt, const double* w64,
                                const double* d64, const int64_t* off, int64_t base,
                                int64_t* row_off, int32_t* row_len, int32_t* pool_i,
                                double* pool_c, double* var64, double tol) {
  constexpr int PL = kVPParentsPerLane;
  const int lane = threadIdx.x & 31;
  const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t it = wid; it < nlist; it += nw) {
    const int64_t k = list[it];
    const int s = cnt[k];
    int64_t poff[PL];
    int plen[PL], cur[PL];
    double w[PL];
#pragma unroll
    for (int u = 0; u < PL; ++u) {
      poff[u] = 0;
      plen[u] = 0;
      cur[u] = 0;
      w[u] = 0.0;
      const int q = lane + 32 * u;
      if (q < s) {
        const int j = nb[k * (int64_t)kout + q];
        if (j >= n) {
          poff[u] = row_off[j - n];
          plen[u] = row_len[j - n];
          w[u] = w64[k * (int64_t)kout + q];
        }
      }
    }
    const int64_t out = base + off[it];
    int count = 0;
    double var = 0.0;
    while (true) {
      int head = 0x7fffffff;
#pragma unroll
      for (int u = 0; u < PL; ++u)
        if (cur[u] < plen[u]) head = min(head, pool_i[poff[u] + cur[u]]);
      const int mn = warp_min_i(head);
      if (mn == 0x7fffffff) break;
      double contrib = 0.0;
#pragma unroll
      for (int u = 0; u < PL; ++u) {
        if (cur[u] < plen[u] && pool_i[poff[u] + cur[u]] == mn) {
          contrib += w[u] * pool_c[poff[u] + cur[u]];
          ++cur[u];
        }
      }
      const double acc = warp_sum_d(contrib);
      if (fabs(acc) > tol) {
        if (lane == 0) {
          pool_i[out + count] = mn;
          pool_c[out + count] = acc;
        }
        ++count;
        var += acc * acc;
      }
    }
    const double own = sqrt(d64[k]);
    if (lane == 0) {
      pool_i[out + count] = (int)k;
      pool_c[out + count] = own;
      row_off[k] = out;
      row_len[k] = count + 1;
      var64[k] = var + own * own;
    }
  }
}

int vecchia_predict_impl(const gs_pointset* ps, const gs_model* model, int64_t nt, const double* tx,
                         const double* ty, const double* tz, int64_t m, double* value,
                         double* variance) {
  NvtxRange nvtx_range("gs.vecchia_predict");
  const int dim = ps->dim;
  GS_TRY(reject_vecchia_model(*model, dim));
  DevModel dm;
  GS_TRY(make_dev_model(*model, dim, &dm, true));
  if (m <= 0) return fail(GS_ERR_INVALID_PARAMETER, "conditioning size m must be at least 1");
  if (nt == 0) return GS_OK;
  if (ps->has_dup)
    return fail(GS_ERR_DUPLICATE_POINTS, "duplicate data points: indices " + std::to_string(ps->dup_i) +
                                             " and " + std::to_string(ps->dup_j) +
                                             " share the same coordinates");
  const int64_t n = ps->n;
  const int64_t ns = n + nt;
  const int kout = (int)std::min<int64_t>(m, ns - 1);
  if (kout > GS_MAX_SYSTEM)
    return fail(GS_ERR_INVALID_PARAMETER, "the CUDA path conditions on at most " +
                                              std::to_string(GS_MAX_SYSTEM) + " points");
  ensure_vtables();
  double sum = 0.0;
  for (int64_t i = 0; i < n; ++i) sum += ps->values[i];
  const double mean = sum / (double)n;
  // targets in max-min order (vecchia.rs:792)
  std::vector<double> tp((size_t)nt * dim);
  for (int64_t i = 0; i < nt; ++i) {
    tp[i * dim] = tx[i];
    tp[i * dim + 1] = ty[i];
    if (dim == 3) tp[i * dim + 2] = tz[i];
  }
  std::vector<int64_t> order(nt);
  maxmin_order(tp, dim, nt, order.data());
  std::vector<double> ox(nt), oy(nt), oz(dim == 3 ? nt : 0);
  for (int64_t k = 0; k < nt; ++k) {
    ox[k] = tx[order[k]];
    oy[k] = ty[order[k]];
    if (dim == 3) oz[k] = tz[order[k]];
  }
  cudaStream_t s = nullptr;
  GS_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  } guard{s};
  DevBuf sx, sy, sz, cdf, sm64, smdf, nb, cnt, w64, d64, var64, flag, roff, rlen, err, list, bound,
      offs, scan_tmp, pool_i, pool_c;
  GS_TRY(sx.alloc(ns * 8, s));
  GS_TRY(sy.alloc(ns * 8, s));
  if (dim == 3) GS_TRY(sz.alloc(ns * 8, s));
  GS_CUDA(cudaMemcpyAsync(sx.ptr, ps->d_x, n * 8, cudaMemcpyDeviceToDevice, s));
  GS_CUDA(cudaMemcpyAsync(sy.ptr, ps->d_y, n * 8, cudaMemcpyDeviceToDevice, s));
  if (dim == 3) GS_CUDA(cudaMemcpyAsync(sz.ptr, ps->d_z, n * 8, cudaMemcpyDeviceToDevice, s));
  GS_CUDA(cudaMemcpyAsync((double*)sx.ptr + n, ox.data(), nt * 8, cudaMemcpyHostToDevice, s));
  GS_CUDA(cudaMemcpyAsync((double*)sy.ptr + n, oy.data(), nt * 8, cudaMemcpyHostToDevice, s));
  if (dim == 3)
    GS_CUDA(cudaMemcpyAsync((double*)sz.ptr + n, oz.data(), nt * 8, cudaMemcpyHostToDevice, s));
  GS_TRY(cdf.alloc((size_t)dim * ns * sizeof(df), s));
  GS_TRY(sm64.alloc(ns * 8, s));
  GS_TRY(smdf.alloc(ns * sizeof(df), s));
  vp_store_kernel<<<(int)std::min<int64_t>((ns + 255) / 256, (int64_t)sm_count() * 32), 256, 0, s>>>(
      dim, n, ns, (double*)sx.ptr, (double*)sy.ptr, (double*)sz.ptr, ps->d_v, mean, (df*)cdf.ptr,
      (double*)sm64.ptr, (df*)smdf.ptr);
  GS_CUDA(cudaGetLastError());
  count_launch(1);
  // conditioning sets: ranked search over the store (rank = store index)
  GS_TRY(nb.alloc((size_t)nt * kout * 4, s));
  GS_TRY(cnt.alloc(nt * 4, s));
  {
    Grid g;
    GS_TRY(grid_build_ranked(&g, dim, ns, (double*)sx.ptr, (double*)sy.ptr, (double*)sz.ptr,
                             dim == 2 ? 2.0 : 3.0, s));
    SearchFrame f;
    std::memset(&f, 0, sizeof(f));
    SearchParams sp{};
    sp.k = kout;
    sp.kout = kout;
    sp.ranked = 1;
    sp.rank0 = n;
    sp.brute_below = 2048;
    sp.px = (double*)sx.ptr;
    sp.py = (double*)sy.ptr;
    sp.pz = (double*)sz.ptr;
    GS_TRY(search_launch(g, f, sp, nt, (double*)sx.ptr + n, (double*)sy.ptr + n,
                         dim == 3 ? (double*)sz.ptr + n : nullptr, (int32_t*)nb.ptr,
                         (int32_t*)cnt.ptr, s));
  }
  // dependency levels (host): level k = 1 + the highest level among its
  // conditioning targets, 0 when it conditions on data alone
  std::vector<int32_t> hnb((size_t)nt * kout), hcnt(nt);
  GS_CUDA(cudaMemcpyAsync(hnb.data(), nb.ptr, (size_t)nt * kout * 4, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaMemcpyAsync(hcnt.data(), cnt.ptr, nt * 4, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaStreamSynchronize(s));
  std::vector<int32_t> level(nt, 0);
  int nlev = 0;
  for (int64_t k = 0; k < nt; ++k) {
    int lv = 0;
    for (int q = 0; q < hcnt[k]; ++q) {
      const int64_t j = hnb[(size_t)k * kout + q];
      if (j >= n) lv = std::max(lv, level[j - n] + 1);
    }
    level[k] = lv;
    nlev = std::max(nlev, lv + 1);
  }
  std::vector<int64_t> lstart(nlev + 1, 0), hlist(nt);
  for (int64_t k = 0; k < nt; ++k) ++lstart[level[k] + 1];
  for (int l = 0; l < nlev; ++l) lstart[l + 1] += lstart[l];
  {
    std::vector<int64_t> fill(lstart.begin(), lstart.end() - 1);
    for (int64_t k = 0; k < nt; ++k) hlist[fill[level[k]]++] = k;
  }
  GS_TRY(list.alloc(nt * 8, s));
  GS_CUDA(cudaMemcpyAsync(list.ptr, hlist.data(), nt * 8, cudaMemcpyHostToDevice, s));
  GS_TRY(w64.alloc((size_t)nt * kout * 8, s));
  GS_TRY(d64.alloc(nt * 8, s));
  GS_TRY(var64.alloc(nt * 8, s));
  GS_TRY(flag.alloc(nt, s));
  GS_TRY(roff.alloc(nt * 8, s));
  GS_TRY(rlen.alloc(nt * 4, s));
  GS_TRY(err.alloc(4, s));
  GS_TRY(bound.alloc(nt * 8, s));
  GS_TRY(offs.alloc(nt * 8, s));
  GS_CUDA(cudaMemsetAsync(err.ptr, 0, 4, s));
  GS_CUDA(cudaMemsetAsync(flag.ptr, 1, nt, s));
  size_t scan_bytes = 0;
  GS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (int64_t*)nullptr, (int64_t*)nullptr,
                                        (int64_t)nt, s));
  GS_TRY(scan_tmp.alloc(scan_bytes, s));
  int64_t cap = std::max<int64_t>(nt * 8, 1024), used = 0;
  GS_TRY(pool_i.alloc(cap * 4, s));
  GS_TRY(pool_c.alloc(cap * 8, s));
  VPArgs a{};
  a.n = n;
  a.ns = ns;
  a.kout = kout;
  a.nb = (const int32_t*)nb.ptr;
  a.cnt = (const int32_t*)cnt.ptr;
  a.cdf = (const df*)cdf.ptr;
  a.sx = (const double*)sx.ptr;
  a.sy = (const double*)sy.ptr;
  a.sz = (const double*)sz.ptr;
  a.smean64 = (double*)sm64.ptr;
  a.smean_df = (df*)smdf.ptr;
  a.w64 = (double*)w64.ptr;
  a.d64 = (double*)d64.ptr;
  a.flag = (uint8_t*)flag.ptr;
  a.err = (int32_t*)err.ptr;
  const int sms = sm_count();
  const bool mixed = kout <= kWarpN;
  size_t vsmem = 0;
  if (mixed) {
    vsmem = vecchia_warp_layout(kout, dim).total * kVPWarps;
    auto kern = dim == 2 ? vp_solve_kernel<2> : vp_solve_kernel<3>;
    GS_TRY(allow_dynamic_smem((const void*)kern, vsmem));
  }
  // FP64 slabs: up to 2 GiB, at least one block of threads
  const int64_t per = ((int64_t)kout * kout + 2 * (int64_t)kout) * 8;
  int64_t T = std::min<int64_t>(std::max<int64_t>(((int64_t)1 << 31) / per, 128), (int64_t)sm_count() * 1024);
  T = std::max<int64_t>((T / 128) * 128, 128);
  DevBuf slab;
  GS_TRY(slab.alloc((size_t)T * per, s));
  const double tol = 1e-8 * std::sqrt(dm.c0);
  for (int l = 0; l < nlev; ++l) {
    const int64_t l0 = lstart[l], ln = lstart[l + 1] - l0;
    a.list = (const int64_t*)list.ptr + l0;
    a.nlist = ln;
    if (mixed) {
      const int blocks = (int)std::min<int64_t>((ln + kVPWarps - 1) / kVPWarps, (int64_t)sms * 8);
      if (dim == 2) vp_solve_kernel<2><<<blocks, 32 * kVPWarps, vsmem, s>>>(a, dm, g_vtab, g_vkc);
      else vp_solve_kernel<3><<<blocks, 32 * kVPWarps, vsmem, s>>>(a, dm, g_vtab, g_vkc);
      GS_CUDA(cudaGetLastError());
      count_launch(1);
    }
    {
      const int64_t Tl = std::min<int64_t>(T, ((ln + 127) / 128) * 128);
      const int blocks = (int)((Tl + 127) / 128);
      if (dim == 2) vp_fp64_kernel<2><<<blocks, 128, 0, s>>>(a, dm, (double*)slab.ptr, Tl, mixed ? 0 : 1);
      else vp_fp64_kernel<3><<<blocks, 128, 0, s>>>(a, dm, (double*)slab.ptr, Tl, mixed ? 0 : 1);
      GS_CUDA(cudaGetLastError());
      count_launch(1);
    }
    const int gb = (int)std::min<int64_t>((ln + 255) / 256, (int64_t)sm_count() * 32);
    vp_bound_kernel<<<gb, 256, 0, s>>>(a.list, ln, n, kout, a.nb, a.cnt, (const int32_t*)rlen.ptr,
                                      (int64_t*)bound.ptr);
    GS_CUDA(cudaGetLastError());
    size_t b = scan_bytes;
    GS_CUDA(cub::DeviceScan::ExclusiveSum(scan_tmp.ptr, b, (int64_t*)bound.ptr, (int64_t*)offs.ptr,
                                          ln, s));
    count_launch(2);
    int64_t last[2] = {0, 0};
    GS_CUDA(cudaMemcpyAsync(&last[0], (int64_t*)offs.ptr + ln - 1, 8, cudaMemcpyDeviceToHost, s));
    GS_CUDA(cudaMemcpyAsync(&last[1], (int64_t*)bound.ptr + ln - 1, 8, cudaMemcpyDeviceToHost, s));
    GS_CUDA(cudaStreamSynchronize(s));
    const int64_t need = used + last[0] + last[1];
    if (need > cap) {
      const int64_t ncap = std::max<int64_t>(need, cap * 2);
      DevBuf ni, nc;
      GS_TRY(ni.alloc(ncap * 4, s));
      GS_TRY(nc.alloc(ncap * 8, s));
      if (used > 0) {
        GS_CUDA(cudaMemcpyAsync(ni.ptr, pool_i.ptr, used * 4, cudaMemcpyDeviceToDevice, s));
        GS_CUDA(cudaMemcpyAsync(nc.ptr, pool_c.ptr, used * 8, cudaMemcpyDeviceToDevice, s));
      }
      std::swap(ni.ptr, pool_i.ptr);
      std::swap(ni.bytes, pool_i.bytes);
      std::swap(nc.ptr, pool_c.ptr);
      std::swap(nc.bytes, pool_c.bytes);
      cap = ncap;
    }
    const int mb = (int)std::min<int64_t>((ln * 32 + 255) / 256, (int64_t)sm_count() * 32);
    vp_merge_kernel<<<mb, 256, 0, s>>>(a.list, ln, n, kout, a.nb, a.cnt, a.w64, a.d64,
                                       (const int64_t*)offs.ptr, used, (int64_t*)roff.ptr,
                                       (int32_t*)rlen.ptr, (int32_t*)pool_i.ptr,
                                       (double*)pool_c.ptr, (double*)var64.ptr, tol);
    GS_CUDA(cudaGetLastError());
    count_launch(1);
    used = need;
  }
  int32_t herr = 0;
  std::vector<double> hmu(nt), hvar(nt);
  GS_CUDA(cudaMemcpyAsync(&herr, err.ptr, 4, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaMemcpyAsync(hmu.data(), (double*)sm64.ptr + n, nt * 8, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaMemcpyAsync(hvar.data(), var64.ptr, nt * 8, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaStreamSynchronize(s));
  if (herr)
    return fail(GS_ERR_SINGULAR_SYSTEM,
                "non-positive Cholesky pivot in a Vecchia prediction conditioning system");
  for (int64_t k = 0; k < nt; ++k) {
    value[order[k]] = mean + hmu[k];
    variance[order[k]] = hvar[k];
  }
  return GS_OK;
}

}  // namespace gs

using namespace gs;

extern "C" {

int gs_maxmin_order(int dim, int64_t n, const double* x, const double* y, const double* z,
                    int64_t* order) {
  if (dim != 2 && dim != 3) return fail(GS_ERR_DIMENSION_MISMATCH, "dim must be 2 or 3");
  std::vector<double> pts(n * dim);
  for (int64_t i = 0; i < n; ++i) {
    pts[i * dim] = x[i];
    pts[i * dim + 1] = y[i];
    if (dim == 3) pts[i * dim + 2] = z[i];
  }
  maxmin_order(pts, dim, n, order);
  return GS_OK;
}

int gs_vecchia_plan_create(const gs_pointset* ps, int64_t m, const int64_t* order,
                           gs_vecchia_plan** out) {
  if (!ps) return fail(GS_ERR_INVALID_PARAMETER, "null point set");
  return plan_create(ps, m, order, out);
}

int gs_vecchia_plan_get(const gs_vecchia_plan* P, int64_t* order, int64_t* neighbours,
                        int32_t* count) {
  const int64_t n = P->n;
  const int M = (int)P->m;
  std::vector<int32_t> nb((size_t)n * M), cnt(n);
  GS_CUDA(cudaMemcpy(nb.data(), P->d_nb, (size_t)n * M * 4, cudaMemcpyDeviceToHost));
  GS_CUDA(cudaMemcpy(cnt.data(), P->d_cnt, n * 4, cudaMemcpyDeviceToHost));
  for (int64_t k = 0; k < n; ++k) {
    if (order) order[k] = P->order[k];
    if (count) count[k] = cnt[k];
    if (neighbours)
      for (int a = 0; a < M; ++a) neighbours[k * M + a] = a < cnt[k] ? nb[k * M + a] : -1;
  }
  return GS_OK;
}

void gs_vecchia_plan_destroy(gs_vecchia_plan* P) { delete P; }

int gs_vecchia_loglik_batch(const gs_vecchia_plan* P, int64_t ncand, const gs_model* models,
                            double* loglik, int32_t* status, int precision, void* stream) {
  if (!P) return fail(GS_ERR_INVALID_PARAMETER, "null plan");
  cudaStream_t s = stream ? (cudaStream_t)stream : P->stream;
  return vecchia_eval(P, ncand, models, loglik, status, precision, s);
}

int gs_vecchia_loglik_batch_range(const gs_vecchia_plan* P, int64_t lo, int64_t hi, int64_t ncand,
                                  const gs_model* models, double* loglik, int32_t* status,
                                  int precision, void* stream) {
  if (!P) return fail(GS_ERR_INVALID_PARAMETER, "null plan");
  if (lo < 0 || hi < lo || hi > P->n)
    return fail(GS_ERR_INVALID_PARAMETER, "point range [" + std::to_string(lo) + ", " +
                                              std::to_string(hi) + ") outside the plan's " +
                                              std::to_string(P->n) + " points");
  cudaStream_t s = stream ? (cudaStream_t)stream : P->stream;
  return vecchia_eval(P, ncand, models, loglik, status, precision, s, nullptr, nullptr, 0, nullptr,
                      lo, hi);
}

int gs_vecchia_loglik_grouped_batch(const gs_vecchia_plan* P, int64_t ncand,
                                    const gs_model* models, int64_t group_size, double* loglik,
                                    int32_t* status, void* stream) {
  if (!P) return fail(GS_ERR_INVALID_PARAMETER, "null plan");
  cudaStream_t s = stream ? (cudaStream_t)stream : P->stream;
  return vecchia_eval_grouped(P, ncand, models, group_size, loglik, status, s);
}

// vecchia_loglik (vecchia.rs:874-884).
int gs_vecchia_loglik(const gs_pointset* ps, const gs_model* model, int64_t m,
                      const int64_t* order, double* loglik) {
  if (!ps) return fail(GS_ERR_INVALID_PARAMETER, "null point set");
  GS_TRY(reject_vecchia_model(*model, ps->dim));
  gs_vecchia_plan* P = nullptr;
  GS_TRY(plan_create(ps, m, order, &P));
  int32_t st = 0;
  int rc = vecchia_eval(P, 1, model, loglik, &st, GS_PREC_MIXED, P->stream);
  delete P;
  if (rc) return rc;
  if (st) return fail(st, "singular conditioning system");
  return GS_OK;
}

// mle_fit_with_plan (vecchia.rs:952-1081) with every start's simplex
// advanced in lock step so each round's evaluations form one batch.
}  // extern "C"

namespace gs {
namespace {

int check_fit_kind(const gs_pointset* ps, int32_t kind) {
  if (!ps) return fail(GS_ERR_INVALID_PARAMETER, "null point set");
  if (kind == GS_KIND_POWER)
    return fail(GS_ERR_INVALID_PARAMETER,
                "Vecchia needs a valid covariance function and cannot use the unbounded Power model");
  if (kind == GS_KIND_CIRCULAR && ps->dim > 2)
    return fail(GS_ERR_INVALID_PARAMETER, "Circular is not a valid covariance in 3 dimensions");
  if (kind < 0 || kind > GS_KIND_MATERN25)
    return fail(GS_ERR_INVALID_PARAMETER,
                "the CUDA path fits spherical, exponential, gaussian, matern15 and matern25");
  return GS_OK;
}

// Initial scales of mle_fit_with_plan (vecchia.rs:958-980): sample variance,
// domain extent, range0 = extent / 3 and the range regulariser's bound.
struct FitSetup {
  double var0, range0, range_max;
};

FitSetup fit_setup(const gs_pointset* ps, double mean) {
  const int64_t n = ps->n;
  const int dim = ps->dim;
  double sq = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    double t = ps->values[i] - mean;
    sq += t * t;
  }
  FitSetup f;
  f.var0 = std::fmax(sq / (double)n, 1e-12);
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = 0; i < n; ++i)
    for (int d = 0; d < dim; ++d) {
      lo[d] = std::fmin(lo[d], ps->host[i * dim + d]);
      hi[d] = std::fmax(hi[d], ps->host[i * dim + d]);
    }
  double e2 = 0.0;
  for (int d = 0; d < dim; ++d) {
    double t = hi[d] - lo[d];
    e2 += t * t;
  }
  const double extent = std::sqrt(e2);
  f.range0 = std::fmax(extent / 3.0, 1e-9);
  f.range_max = 10.0 * extent;
  return f;
}

// x = (sqrt nugget, ln psill, ln range) -> a single-structure model.
gs_model model_from_x(int32_t kind, const std::vector<double>& x) {
  gs_model mdl;
  std::memset(&mdl, 0, sizeof(mdl));
  mdl.nugget = x[0] * x[0];
  mdl.n_structures = 1;
  mdl.s[0].kind = kind;
  mdl.s[0].sill = std::exp(x[1]);
  mdl.s[0].range = std::exp(x[2]);
  mdl.s[0].ratio = mdl.s[0].ratio_z = 1.0;
  return mdl;
}

double range_reg(double range, double range_max) {
  if (range > range_max) {
    double t = (range - range_max) / range_max;
    return t * t;
  }
  return 0.0;
}

// The objective of mle_fit_with_plan (vecchia.rs:1001-1016) for a batch of
// points: -loglik + 1e6 reg(range), 1e12 for a rejected candidate.
int batch_objective(const gs_vecchia_plan* P, int32_t kind, double range_max,
                    const std::vector<std::vector<double>>& xs, std::vector<double>& f) {
  std::vector<gs_model> batch;
  for (const auto& x : xs) batch.push_back(model_from_x(kind, x));
  std::vector<double> ll(batch.size());
  std::vector<int32_t> sts(batch.size());
  GS_TRY(vecchia_eval(P, (int64_t)batch.size(), batch.data(), ll.data(), sts.data(), GS_PREC_MIXED,
                      P->stream));
  f.resize(batch.size());
  for (size_t b = 0; b < batch.size(); ++b)
    f[b] = (sts[b] == 0 && std::isfinite(ll[b]))
               ? -ll[b] + 1e6 * range_reg(batch[b].s[0].range, range_max)
               : 1e12;
  return GS_OK;
}

// objective_grad of mle_fit_with_plan (vecchia.rs:1039-1061) for a batch.
int batch_gradient(const gs_vecchia_plan* P, int32_t kind, double range_max,
                   const std::vector<std::vector<double>>& xs, std::vector<std::vector<double>>& g) {
  std::vector<gs_model> batch;
  for (const auto& x : xs) batch.push_back(model_from_x(kind, x));
  std::vector<double> ll(batch.size()), gr(3 * batch.size());
  std::vector<int32_t> sts(batch.size());
  GS_TRY(vecchia_eval_grad(P, (int64_t)batch.size(), batch.data(), ll.data(), gr.data(), sts.data(),
                           GS_PREC_MIXED, P->stream));
  g.assign(batch.size(), std::vector<double>(3, 0.0));
  for (size_t b = 0; b < batch.size(); ++b) {
    if (sts[b] != 0) continue;  // singular: no meaningful direction
    const auto& x = xs[b];
    const double psill = batch[b].s[0].sill, range = batch[b].s[0].range;
    g[b] = {-gr[3 * b] * 2.0 * x[0], -gr[3 * b + 1] * psill, -gr[3 * b + 2] * range};
    if (range > range_max) {
      const double dreg = 2.0 * (range - range_max) / (range_max * range_max);
      g[b][2] += 1e6 * dreg * range;
    }
  }
  return GS_OK;
}

int finish_fit(int32_t kind, const std::pair<std::vector<double>, double>& best,
               gs_model* out_model, double* out_loglik, double* out_x) {
  if (best.second >= 1e12)
    return fail(GS_ERR_SINGULAR_SYSTEM,
                "Vecchia MLE did not converge to a feasible fit: every starting point stayed on a "
                "singular/degenerate covariance");
  const auto& xb = best.first;
  if (out_x)
    for (int i = 0; i < 3; ++i) out_x[i] = xb[i];
  if (out_model) {
    *out_model = model_from_x(kind, xb);
    GS_TRY(validate_model(*out_model));
  }
  if (out_loglik) *out_loglik = -best.second;
  return GS_OK;
}

// Nelder-Mead multistart (optim.rs:106-123) with every start's simplex
// advanced in lock step: each round's pending points of all starts are one
// batch of `objective` (xs -> f).
// Batched objective launches of this thread's last lock-step Nelder-Mead fit.
thread_local int64_t g_fit_rounds = 0;

template <class Obj>
int nm_lockstep(const std::vector<std::vector<double>>& starts, double step, int64_t max_iter,
                Obj objective, std::pair<std::vector<double>, double>* best, int64_t* n_evals) {
  std::vector<NelderMead> runs;
  for (const auto& x0 : starts) runs.emplace_back(x0, step, max_iter);
  int64_t evals = 0;
  g_fit_rounds = 0;
  for (int guard = 0; guard < 1000000; ++guard) {
    std::vector<std::vector<double>> xs;
    std::vector<size_t> owner;
    for (size_t r = 0; r < runs.size(); ++r) {
      if (runs[r].done()) continue;
      for (const auto& x : runs[r].pending()) {
        xs.push_back(x);
        owner.push_back(r);
      }
    }
    if (xs.empty()) break;
    std::vector<double> fv;
    GS_TRY(objective(xs, fv));
    evals += (int64_t)xs.size();
    ++g_fit_rounds;
    std::vector<std::vector<double>> fvals(runs.size());
    for (size_t b = 0; b < xs.size(); ++b) fvals[owner[b]].push_back(fv[b]);
    for (size_t r = 0; r < runs.size(); ++r)
      if (!fvals[r].empty()) runs[r].supply(fvals[r]);
  }
  if (n_evals) *n_evals = evals;
  *best = multistart_best(runs);
  return GS_OK;
}

// The reference's three starts (vecchia.rs:1018-1023, 1636-1640).
std::vector<std::vector<double>> reference_starts(const FitSetup& fs) {
  const double lr0 = std::log(fs.range0);
  std::vector<std::vector<double>> st;
  for (double f : {0.3, 1.0, 3.0})
    st.push_back({std::sqrt(0.1 * fs.var0), std::log(0.9 * fs.var0), lr0 + std::log(f)});
  return st;
}

// -loglik + 1e6 reg(range), 1e12 for a rejected candidate, from a batch of
// log-likelihoods and statuses.
void to_objective(int32_t kind, double range_max, const std::vector<std::vector<double>>& xs,
                  const std::vector<double>& ll, const std::vector<int32_t>& st,
                  std::vector<double>& f) {
  f.resize(xs.size());
  for (size_t b = 0; b < xs.size(); ++b)
    f[b] = (st[b] == 0 && std::isfinite(ll[b]))
               ? -ll[b] + 1e6 * range_reg(std::exp(xs[b][2]), range_max)
               : 1e12;
}

// poly_basis (vecchia.rs:1181-1233): monomials of total degree <= degree
// (the first dimension's exponent varying slowest) of the coordinates
// centred and divided by their standard deviation (floored at 1e-12);
// column-major p x n.
std::vector<double> poly_basis_host(const gs_pointset* ps, int degree, int* p_out) {
  const int64_t n = ps->n;
  const int dim = ps->dim;
  double mean[3] = {0, 0, 0}, scale[3] = {1, 1, 1};
  for (int64_t i = 0; i < n; ++i)
    for (int d = 0; d < dim; ++d) mean[d] += ps->host[i * dim + d] / (double)n;
  for (int d = 0; d < dim; ++d) {
    double var = 0.0;
    for (int64_t i = 0; i < n; ++i) {
      const double t = ps->host[i * dim + d] - mean[d];
      var += t * t;
    }
    scale[d] = std::fmax(std::sqrt(var / (double)n), 1e-12);
  }
  std::vector<std::array<int, 3>> exps;
  std::array<int, 3> cur{0, 0, 0};
  std::function<void(int, int)> rec = [&](int d, int rem) {
    if (d == dim) {
      exps.push_back(cur);
      return;
    }
    for (int e = 0; e <= rem; ++e) {
      cur[d] = e;
      rec(d + 1, rem - e);
    }
    cur[d] = 0;
  };
  rec(0, degree);
  const int p = (int)exps.size();
  std::vector<double> f((size_t)p * n);
  for (int64_t i = 0; i < n; ++i) {
    double cs[3];
    for (int d = 0; d < dim; ++d) cs[d] = (ps->host[i * dim + d] - mean[d]) / scale[d];
    for (int col = 0; col < p; ++col) {
      double v = 1.0;
      for (int d = 0; d < dim; ++d)
        for (int e = 0; e < exps[col][d]; ++e) v *= cs[d];
      f[(size_t)col * n + i] = v;
    }
  }
  *p_out = p;
  return f;
}

// standardized_drift_basis (vecchia.rs:1246-1272): an intercept, then each
// covariate centred and divided by its standard deviation (floored at
// 1e-12); column-major (1 + ncov) x n.
std::vector<double> drift_basis_host(const double* drift, int64_t n, int64_t ncov) {
  std::vector<double> f((size_t)(ncov + 1) * n);
  for (int64_t i = 0; i < n; ++i) f[i] = 1.0;
  for (int64_t k = 0; k < ncov; ++k) {
    double mean = 0.0, var = 0.0;
    for (int64_t i = 0; i < n; ++i) mean += drift[i * ncov + k] / (double)n;
    for (int64_t i = 0; i < n; ++i) {
      const double t = drift[i * ncov + k] - mean;
      var += t * t;
    }
    const double sd = std::fmax(std::sqrt(var / (double)n), 1e-12);
    for (int64_t i = 0; i < n; ++i) f[(size_t)(k + 1) * n + i] = (drift[i * ncov + k] - mean) / sd;
  }
  return f;
}

// The trend basis of vecchia_reml (drift == null: poly_basis of degree) or
// vecchia_reml_drift, with the reference's checks (vecchia.rs:1508-1526).
int make_basis(const gs_pointset* ps, int32_t degree, const double* drift, int64_t n_rows,
               int64_t ncov, std::vector<double>* basis, int* p) {
  if (drift) {
    if (n_rows != ps->n)
      return fail(GS_ERR_DIMENSION_MISMATCH, std::to_string(n_rows) + " drift rows vs " +
                                                 std::to_string(ps->n) + " data points");
    if (ncov <= 0)
      return fail(GS_ERR_INVALID_PARAMETER, "external-drift REML needs at least one covariate column");
    *basis = drift_basis_host(drift, ps->n, ncov);
    *p = (int)(ncov + 1);
  } else {
    if (degree < 0 || degree > 255) return fail(GS_ERR_INVALID_PARAMETER, "drift degree out of range");
    *basis = poly_basis_host(ps, degree, p);
  }
  return GS_OK;
}

// reml_fit_with_basis (vecchia.rs:1572-1644) and the grouped path of
// mle_fit_with_plan (vecchia.rs:983, 1001-1016, 1063-1064): Nelder-Mead
// from the reference's three starts, step 0.3, 2000 iterations.
int fit_nm(const gs_pointset* ps, int32_t kind, int64_t m, const int64_t* order, int64_t gsize,
           const std::vector<double>* basis, int p, gs_model* out_model, double* out_loglik,
           double* out_x, int64_t* n_evals) {
  NvtxRange nvtx_range("gs.fit_nelder_mead");
  gs_vecchia_plan* P = nullptr;
  GS_TRY(plan_create(ps, m, order, &P));
  std::unique_ptr<gs_vecchia_plan> own(P);
  if (basis && ps->n <= p + 1)
    return fail(GS_ERR_INSUFFICIENT_DATA, "REML with " + std::to_string(p) +
                                              " trend terms needs more than " +
                                              std::to_string(p + 1) + " points");
  const FitSetup fs = fit_setup(ps, P->mean);
  DevBuf dbasis;
  if (basis) {
    GS_TRY(dbasis.alloc(basis->size() * 8, P->stream));
    GS_CUDA(cudaMemcpyAsync(dbasis.ptr, basis->data(), basis->size() * 8, cudaMemcpyHostToDevice,
                            P->stream));
  }
  auto objective = [&](const std::vector<std::vector<double>>& xs,
                       std::vector<double>& f) -> int {
    std::vector<gs_model> batch;
    for (const auto& x : xs) batch.push_back(model_from_x(kind, x));
    std::vector<double> ll(batch.size());
    std::vector<int32_t> st(batch.size());
    if (basis)
      GS_TRY(vecchia_eval_reml(P, (int64_t)batch.size(), batch.data(), gsize,
                               (const double*)dbasis.ptr, p, ll.data(), st.data(), P->stream));
    else
      GS_TRY(vecchia_eval_grouped(P, (int64_t)batch.size(), batch.data(), gsize, ll.data(),
                                  st.data(), P->stream));
    to_objective(kind, fs.range_max, xs, ll, st, f);
    return GS_OK;
  };
  std::pair<std::vector<double>, double> best;
  GS_TRY(nm_lockstep(reference_starts(fs), 0.3, 2000, objective, &best, n_evals));
  return finish_fit(kind, best, out_model, out_loglik, out_x);
}

}  // namespace
}  // namespace gs

extern "C" {

int64_t gs_last_fit_rounds(void) { return g_fit_rounds; }

void gs_last_vecchia_tiers(int64_t* out2) {
  if (!out2) return;
  out2[0] = g_vtiers[0];
  out2[1] = g_vtiers[1];
}

int gs_vecchia_mle(const gs_pointset* ps, int32_t kind, int64_t m, const int64_t* order,
                   gs_model* out_model, double* out_loglik, double* out_x, int64_t* n_evals) {
  GS_TRY(check_fit_kind(ps, kind));
  gs_vecchia_plan* P = nullptr;
  GS_TRY(plan_create(ps, m, order, &P));
  const FitSetup fs = fit_setup(ps, P->mean);
  // the reference's three starts (vecchia.rs:1018-1023) and 200 iterations
  const double lr0 = std::log(fs.range0);
  std::vector<Bfgs> runs;
  for (double f : {0.3, 1.0, 3.0})
    runs.emplace_back(std::vector<double>{std::sqrt(0.1 * fs.var0), std::log(0.9 * fs.var0),
                                          lr0 + std::log(f)},
                      200);
  int64_t evals = 0;
  int rc = GS_OK;
  for (int guard = 0; guard < 100000 && !rc; ++guard) {
    std::vector<std::vector<double>> fx, gx;
    std::vector<size_t> fo, go;
    for (size_t r = 0; r < runs.size(); ++r) {
      if (runs[r].done()) continue;
      if (runs[r].wants_gradient()) {
        gx.push_back(runs[r].pending_x());
        go.push_back(r);
      } else {
        fx.push_back(runs[r].pending_x());
        fo.push_back(r);
      }
    }
    if (fx.empty() && gx.empty()) break;
    std::vector<double> fv;
    std::vector<std::vector<double>> gv;
    if (!fx.empty()) rc = batch_objective(P, kind, fs.range_max, fx, fv);
    if (!rc && !gx.empty()) rc = batch_gradient(P, kind, fs.range_max, gx, gv);
    if (rc) break;
    evals += (int64_t)(fx.size() + gx.size());
    for (size_t b = 0; b < fo.size(); ++b) runs[fo[b]].supply_f(fv[b]);
    for (size_t b = 0; b < go.size(); ++b) runs[go[b]].supply_g(gv[b]);
  }
  delete P;
  if (rc) return rc;
  if (n_evals) *n_evals = evals;
  return finish_fit(kind, bfgs_multistart_best(runs), out_model, out_loglik, out_x);
}

int gs_vecchia_mle_nm(const gs_pointset* ps, int32_t kind, int64_t m, const int64_t* order,
                      int64_t nstarts, const double* starts, double step, int64_t max_iter,
                      gs_model* out_model, double* out_loglik, double* out_x, int64_t* n_evals) {
  GS_TRY(check_fit_kind(ps, kind));
  gs_vecchia_plan* P = nullptr;
  GS_TRY(plan_create(ps, m, order, &P));
  const FitSetup fs = fit_setup(ps, P->mean);
  std::vector<std::vector<double>> st;
  if (starts) {
    for (int64_t q = 0; q < nstarts; ++q) st.push_back({starts[q * 3], starts[q * 3 + 1], starts[q * 3 + 2]});
  } else {
    const double lr0 = std::log(fs.range0);
    if (nstarts <= 3) {
      for (double f : {0.3, 1.0, 3.0})
        st.push_back({std::sqrt(0.1 * fs.var0), std::log(0.9 * fs.var0), lr0 + std::log(f)});
    } else {
      // a deterministic spread over range and nugget share
      for (int64_t q = 0; q < nstarts; ++q) {
        const double fr = std::pow(10.0, -1.0 + 2.0 * (double)(q % 4) / 3.0);
        const double nugf = 0.05 + 0.15 * (double)((q / 4) % 4);
        st.push_back({std::sqrt(nugf * fs.var0), std::log((1.0 - nugf) * fs.var0), lr0 + std::log(fr)});
      }
    }
  }
  if (st.empty()) {
    delete P;
    return fail(GS_ERR_INVALID_PARAMETER, "at least one start is required");
  }
  std::pair<std::vector<double>, double> best;
  const int rc = nm_lockstep(
      st, step, max_iter,
      [&](const std::vector<std::vector<double>>& xs, std::vector<double>& fv) {
        return batch_objective(P, kind, fs.range_max, xs, fv);
      },
      &best, n_evals);
  delete P;
  if (rc) return rc;
  return finish_fit(kind, best, out_model, out_loglik, out_x);
}

// vecchia_mle_grouped (vecchia.rs:939-950): group_size <= 1 is vecchia_mle.
int gs_vecchia_mle_grouped(const gs_pointset* ps, int32_t kind, int64_t m, const int64_t* order,
                           int64_t group_size, gs_model* out_model, double* out_loglik,
                           double* out_x, int64_t* n_evals) {
  if (group_size <= 1)
    return gs_vecchia_mle(ps, kind, m, order, out_model, out_loglik, out_x, n_evals);
  GS_TRY(check_fit_kind(ps, kind));
  return fit_nm(ps, kind, m, order, group_size, nullptr, 0, out_model, out_loglik, out_x, n_evals);
}

// vecchia_reml / vecchia_reml_grouped (vecchia.rs:1460-1493).
int gs_vecchia_reml(const gs_pointset* ps, int32_t kind, int64_t m, int32_t drift_degree,
                    const int64_t* order, int64_t group_size, gs_model* out_model,
                    double* out_loglik, double* out_x, int64_t* n_evals) {
  GS_TRY(check_fit_kind(ps, kind));
  std::vector<double> basis;
  int p = 0;
  GS_TRY(make_basis(ps, drift_degree, nullptr, 0, 0, &basis, &p));
  return fit_nm(ps, kind, m, order, group_size, &basis, p, out_model, out_loglik, out_x, n_evals);
}

// vecchia_reml_drift / vecchia_reml_drift_grouped (vecchia.rs:1500-1568):
// drift is n_rows x ncov, row-major.
int gs_vecchia_reml_drift(const gs_pointset* ps, int32_t kind, int64_t m, const double* drift,
                          int64_t n_rows, int64_t ncov, const int64_t* order, int64_t group_size,
                          gs_model* out_model, double* out_loglik, double* out_x,
                          int64_t* n_evals) {
  GS_TRY(check_fit_kind(ps, kind));
  if (!drift && n_rows > 0 && ncov > 0) return fail(GS_ERR_INVALID_PARAMETER, "null drift");
  std::vector<double> basis;
  int p = 0;
  static const double kNone = 0.0;
  GS_TRY(make_basis(ps, 0, drift ? drift : &kNone, n_rows, ncov, &basis, &p));
  return fit_nm(ps, kind, m, order, group_size, &basis, p, out_model, out_loglik, out_x, n_evals);
}

// REML log-likelihoods of ncand candidates on a plan (reml_loglik_with_plan
// for group_size <= 1, reml_loglik_with_blocks otherwise) with the trend
// basis of vecchia_reml (drift null: polynomial of drift_degree) or of
// vecchia_reml_drift (drift: n x ncov covariates, row-major).
int gs_vecchia_reml_loglik_batch(const gs_vecchia_plan* P, int64_t ncand, const gs_model* models,
                                 int32_t drift_degree, const double* drift, int64_t ncov,
                                 int64_t group_size, double* loglik, int32_t* status,
                                 void* stream) {
  if (!P) return fail(GS_ERR_INVALID_PARAMETER, "null plan");
  if (ncand < 0) return fail(GS_ERR_INVALID_PARAMETER, "negative candidate count");
  if (ncand > 0 && (!models || !loglik || !status))
    return fail(GS_ERR_INVALID_PARAMETER, "null model or output buffer");
  cudaStream_t s = stream ? (cudaStream_t)stream : P->stream;
  std::vector<double> basis;
  int p = 0;
  GS_TRY(make_basis(P->ps, drift_degree, drift, drift ? P->n : 0, ncov, &basis, &p));
  DevBuf dbasis;
  GS_TRY(dbasis.alloc(basis.size() * 8, s));
  GS_CUDA(cudaMemcpyAsync(dbasis.ptr, basis.data(), basis.size() * 8, cudaMemcpyHostToDevice, s));
  return vecchia_eval_reml(P, ncand, models, group_size, (const double*)dbasis.ptr, p, loglik,
                           status, s);
}

int gs_vecchia_loglik_grad_batch(const gs_vecchia_plan* plan, int64_t ncand, const gs_model* models,
                                 double* loglik, double* grad, int32_t* status, int precision,
                                 void* stream) {
  if (!plan) return fail(GS_ERR_INVALID_PARAMETER, "null plan");
  if (ncand < 0) return fail(GS_ERR_INVALID_PARAMETER, "negative candidate count");
  if (ncand > 0 && (!models || !loglik || !grad || !status))
    return fail(GS_ERR_INVALID_PARAMETER, "null model or output buffer");
  cudaStream_t s = stream ? (cudaStream_t)stream : plan->stream;
  return vecchia_eval_grad(plan, ncand, models, loglik, grad, status, precision, s);
}

int gs_nelder_mead_multistart(gs_objective_fn f, void* ctx, int64_t n, int64_t nstarts,
                              const double* starts, double step, int64_t max_iter, double* x_out,
                              double* f_out) {
  if (nstarts <= 0) return fail(GS_ERR_INVALID_PARAMETER, "starts must be non-empty");
  std::vector<NelderMead> runs;
  for (int64_t q = 0; q < nstarts; ++q)
    runs.emplace_back(std::vector<double>(starts + q * n, starts + (q + 1) * n), step, max_iter);
  for (;;) {
    bool any = false;
    for (auto& r : runs) {
      if (r.done()) continue;
      any = true;
      std::vector<double> fv;
      for (const auto& x : r.pending()) fv.push_back(f(x.data(), n, ctx));
      r.supply(fv);
    }
    if (!any) break;
  }
  auto best = multistart_best(runs);
  for (int64_t i = 0; i < n; ++i) x_out[i] = best.first[i];
  *f_out = best.second;
  return GS_OK;
}

}  // extern "C"

extern "C" int gs_vecchia_predict(const gs_pointset* ps, const gs_model* model, int64_t nt,
                                  const double* tx, const double* ty, const double* tz, int64_t m,
                                  double* value, double* variance) {
  if (!ps || !model) return gs::fail(GS_ERR_INVALID_PARAMETER, "null point set or model");
  if (nt < 0) return gs::fail(GS_ERR_INVALID_PARAMETER, "negative target count");
  if (nt > 0 && (!tx || !ty || (ps->dim == 3 && !tz) || !value || !variance))
    return gs::fail(GS_ERR_INVALID_PARAMETER, "null target or output buffer");
  GS_TRY(gs::ensure_device());
  return gs::vecchia_predict_impl(ps, model, nt, tx, ty, tz, m, value, variance);
}
