// gs_api.cu -- the C ABI (include/geostat_gb300.h): handles, validation in
// the reference's order, and the host orchestration of the device kernels.
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <atomic>
#include <mutex>
#include <map>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "gs_common.cuh"
#include "gs_host.h"
#include "gs_internal.h"
#include "gs_kriging_handle.h"
#include "gs_krige.cuh"
#include "gs_search.cuh"

namespace gs {

// ------------------------------------------------------------ utilities --
static std::once_flag g_pool_once;

int ensure_device() {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0)
    return fail(GS_ERR_CUDA, std::string("no CUDA device available: ") + cudaGetErrorString(e));
  std::call_once(g_pool_once, [] {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t thr = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
  });
  return GS_OK;
}

int allow_dynamic_smem(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::unordered_map<uint64_t, size_t> limit;  // (device, function) -> bytes
  int dev = 0;
  GS_CUDA(cudaGetDevice(&dev));
  const uint64_t key = ((uint64_t)(uintptr_t)func) ^ ((uint64_t)dev << 56);
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = limit[key];
  if (bytes > cur) {
    GS_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cur = bytes;
  }
  return GS_OK;
}

static std::atomic<int64_t> g_launches{0};
static std::atomic<int64_t> g_device_allocs{0};
// Stream-ordered allocations still to be refused (a host-side fake of an
// exhausted device, for failure tests; 0 in normal use).
static std::atomic<int64_t> g_refuse_allocs{0};

void count_launch(int n) { g_launches += n; }

int sm_count() {
  constexpr int kMaxDev = 64;
  static std::atomic<int> cache[kMaxDev];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return 1;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v > 0) return v;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
    return 1;  // grid-stride loops stay correct on any grid
  cache[dev].store(v, std::memory_order_relaxed);
  return v;
}

cudaError_t dev_malloc(void** p, size_t bytes) {
  ++g_device_allocs;
  return cudaMalloc(p, bytes);
}

int DevBuf::alloc(size_t b, cudaStream_t s) {
  release();
  stream = s;
  bytes = b;
  ++g_device_allocs;
  int64_t left = g_refuse_allocs.load();
  while (left > 0 && !g_refuse_allocs.compare_exchange_weak(left, left - 1)) {
  }
  if (left > 0) {
    bytes = 0;
    return cuda_fail(cudaErrorMemoryAllocation, "cudaMallocAsync (refused on request)", __FILE__,
                     __LINE__);
  }
  GS_CUDA(cudaMallocAsync(&ptr, std::max<size_t>(b, 16), s));
  return GS_OK;
}
void DevBuf::release() {
  if (ptr) cudaFreeAsync(ptr, stream);
  ptr = nullptr;
  bytes = 0;
}
DevBuf::~DevBuf() { release(); }

static thread_local double g_timings[4] = {0, 0, 0, 0};
static thread_local int64_t g_fallbacks = 0;
static thread_local int64_t g_lu_resolves = 0;

void set_last_timings(const double* ms4, int64_t fallbacks) {
  for (int i = 0; i < 4; ++i) g_timings[i] = ms4[i];
  g_fallbacks = fallbacks;
  g_lu_resolves = 0;
}

}  // namespace gs

using namespace gs;

// ============================================================== C ABI ====
gs_pointset::~gs_pointset() {
  cudaFree(d_x);
  cudaFree(d_y);
  cudaFree(d_z);
  cudaFree(d_v);
  cudaFree(d_cdf);
  cudaFree(d_vdf);
}

namespace {

// Splits FP64 coordinates and values into double-float copies (once per set).
__global__ void split_df_kernel(int dim, int64_t n, const double* x, const double* y,
                                const double* z, const double* v, gs::df* cdf, gs::df* vdf) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    cdf[i] = gs::df_from_double(x[i]);
    cdf[n + i] = gs::df_from_double(y[i]);
    if (dim == 3) cdf[2 * n + i] = gs::df_from_double(z[i]);
    vdf[i] = gs::df_from_double(v[i]);
  }
}

}  // namespace


extern "C" {

const char* gs_last_error(void) { return gs::last_error(); }
int gs_abi_version(void) { return GS_ABI_VERSION; }

int64_t gs_launch_count(void) { return g_launches.load(); }
int64_t gs_debug_device_allocations(void) { return g_device_allocs.load(); }
int gs_debug_refuse_allocations(int64_t count) {
  if (count < 0) return fail(GS_ERR_INVALID_PARAMETER, "negative count");
  g_refuse_allocs.store(count);
  return GS_OK;
}

int gs_last_timings(double* ms4) {
  for (int i = 0; i < 4; ++i) ms4[i] = g_timings[i];
  return GS_OK;
}

int64_t gs_last_fallbacks(void) { return g_fallbacks; }
int64_t gs_last_lu_resolves(void) { return g_lu_resolves; }

// data.rs:15-83 (+ duplicate_coord_pair, data.rs:384-397).
int gs_pointset_create(int dim, int64_t n, const double* x, const double* y, const double* z,
                       const double* values, gs_pointset** out) {
  *out = nullptr;
  if (dim != 2 && dim != 3) return fail(GS_ERR_DIMENSION_MISMATCH, "dim must be 2 or 3");
  if (n <= 0) return fail(GS_ERR_INSUFFICIENT_DATA, "no points provided");
  if (n > 0x7fffffffll) return fail(GS_ERR_INVALID_PARAMETER, "at most 2^31-1 points");
  for (int64_t i = 0; i < n; ++i) {
    if (!std::isfinite(x[i]) || !std::isfinite(y[i]) || (dim == 3 && !std::isfinite(z[i])))
      return fail(GS_ERR_INVALID_PARAMETER, "non-finite coordinate");
  }
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(values[i])) return fail(GS_ERR_INVALID_PARAMETER, "non-finite value");
  GS_TRY(ensure_device());
  auto* ps = new gs_pointset();
  ps->dim = dim;
  ps->n = n;
  ps->host.resize(n * dim);
  for (int64_t i = 0; i < n; ++i) {
    ps->host[i * dim] = x[i];
    ps->host[i * dim + 1] = y[i];
    if (dim == 3) ps->host[i * dim + 2] = z[i];
  }
  ps->values.assign(values, values + n);
  // first pair with bitwise-identical coordinates, -0.0 normalised
  {
    struct H {
      size_t operator()(const std::array<uint64_t, 3>& k) const {
        uint64_t h = 1469598103934665603ull;
        for (uint64_t v : k) h = (h ^ v) * 1099511628211ull;
        return (size_t)h;
      }
    };
    std::unordered_map<std::array<uint64_t, 3>, int64_t, H> seen;
    seen.reserve(n);
    for (int64_t i = 0; i < n; ++i) {
      std::array<uint64_t, 3> key = {0, 0, 0};
      for (int d = 0; d < dim; ++d) {
        double v = ps->host[i * dim + d] + 0.0;
        std::memcpy(&key[d], &v, 8);
      }
      auto it = seen.find(key);
      if (it != seen.end()) {
        ps->has_dup = true;
        ps->dup_i = it->second;
        ps->dup_j = i;
        break;
      }
      seen.emplace(key, i);
    }
  }
  auto up = [&](double** d, const double* h) -> int {
    GS_CUDA(dev_malloc((void**)d, n * sizeof(double)));
    GS_CUDA(cudaMemcpy(*d, h, n * sizeof(double), cudaMemcpyHostToDevice));
    return GS_OK;
  };
  int rc = up(&ps->d_x, x);
  if (!rc) rc = up(&ps->d_y, y);
  if (!rc && dim == 3) rc = up(&ps->d_z, z);
  if (!rc) rc = up(&ps->d_v, values);
  if (!rc) {
    if (dev_malloc((void**)&ps->d_cdf, (size_t)dim * n * sizeof(df)) != cudaSuccess ||
        dev_malloc((void**)&ps->d_vdf, (size_t)n * sizeof(df)) != cudaSuccess) {
      rc = fail(GS_ERR_OUT_OF_MEMORY, "point set allocation failed");
    } else {
      split_df_kernel<<<(int)std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 32), 256>>>(
          dim, n, ps->d_x, ps->d_y, ps->d_z, ps->d_v, (df*)ps->d_cdf, (df*)ps->d_vdf);
      if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess)
        rc = fail(GS_ERR_CUDA, "point set split failed");
    }
  }
  if (rc) {
    delete ps;
    return rc;
  }
  *out = ps;
  return GS_OK;
}

void gs_pointset_destroy(gs_pointset* ps) { delete ps; }

int gs_pointset_duplicate_pair(const gs_pointset* ps, int64_t* i, int64_t* j) {
  if (!ps->has_dup) return 0;
  *i = ps->dup_i;
  *j = ps->dup_j;
  return 1;
}

}  // extern "C"

namespace {

// KrigingMethod::n_drift (kriging.rs:46-60).
int n_drift(const gs_kcfg& c, int dim) {
  switch (c.method) {
    case GS_SIMPLE:
      return 0;
    case GS_ORDINARY:
      return 1;
    case GS_UNIVERSAL:
      if (c.uk_degree == 1) return 1 + dim;
      if (c.uk_degree == 2) return 1 + dim + dim * (dim + 1) / 2;
      return 0;
    case GS_EXTERNAL_DRIFT:
      return 1 + (int)c.ked_nvars;
  }
  return 0;
}

bool valid_in_dim(const gs_model& m, int dim) {
  for (int k = 0; k < m.n_structures; ++k)
    if (m.s[k].kind == GS_KIND_CIRCULAR && dim > 2) return false;
  return true;
}

// Kriging::build and the three constructors (kriging.rs:166-408).
}  // namespace
namespace {

// Global neighbourhoods larger than the mixed solver's systems are factored
// once at build (kriging.rs:396-406); up to this many unknowns (2 GiB).
constexpr int kGlobalLuMax = 16384;

int kriging_create(const gs_pointset* ps, const gs_model* model, const gs_kcfg* cfg, int ctor,
                   const double* drift, const double* errors, gs_kriging** out) {
  NvtxRange nvtx_range("gs.kriging_build");
  *out = nullptr;
  if (!ps || !model || !cfg) return fail(GS_ERR_INVALID_PARAMETER, "null argument");
  GS_TRY(validate_model(*model));
  const int dim = ps->dim;
  const int64_t n = ps->n;
  if (ctor == 0) {
    if (cfg->method == GS_EXTERNAL_DRIFT)
      return fail(GS_ERR_INVALID_PARAMETER,
                  "external drift kriging requires Kriging::with_external_drift");
  } else if (ctor == 2) {
    if (cfg->method == GS_EXTERNAL_DRIFT)
      return fail(GS_ERR_INVALID_PARAMETER, "measurement error with external drift is not supported yet");
    if (has_power(*model))
      return fail(GS_ERR_INVALID_PARAMETER,
                  "measurement error with Power (IRF-0) models is not supported yet");
    for (int64_t i = 0; i < n; ++i)
      if (!(std::isfinite(errors[i]) && errors[i] >= 0.0))
        return fail(GS_ERR_INVALID_PARAMETER,
                    "measurement-error variances must be finite and non-negative");
  } else {
    if (cfg->method != GS_EXTERNAL_DRIFT)
      return fail(GS_ERR_INVALID_PARAMETER, "with_external_drift requires KrigingMethod::ExternalDrift");
    if (cfg->ked_nvars <= 0)
      return fail(GS_ERR_INVALID_PARAMETER, "external drift requires at least one covariate");
    for (int64_t i = 0; i < n * cfg->ked_nvars; ++i)
      if (!std::isfinite(drift[i]))
        return fail(GS_ERR_INVALID_PARAMETER,
                    "non-finite drift value at data point " + std::to_string(i / cfg->ked_nvars));
  }
  if (cfg->method < GS_SIMPLE || cfg->method > GS_EXTERNAL_DRIFT)
    return fail(GS_ERR_INVALID_PARAMETER, "unknown kriging method");
  if (cfg->method == GS_UNIVERSAL && !(cfg->uk_degree >= 1 && cfg->uk_degree <= 2))
    return fail(GS_ERR_INVALID_PARAMETER, "universal kriging drift degree must be 1 or 2, got " +
                                              std::to_string(cfg->uk_degree));
  if (has_power(*model) && cfg->method == GS_SIMPLE)
    return fail(GS_ERR_INVALID_PARAMETER,
                "Power (unbounded) models have no covariance function, so simple kriging cannot "
                "use them");
  if (!valid_in_dim(*model, dim))
    return fail(GS_ERR_INVALID_PARAMETER, "this model is not a valid covariance in 3 dimensions");
  if (cfg->has_search_radius && !(cfg->search_radius > 0.0))
    return fail(GS_ERR_INVALID_PARAMETER, "search radius must be positive");
  if (cfg->has_anisotropic_search)
    GS_TRY(validate_anisotropy(cfg->search_azimuth_deg, cfg->search_ratio, cfg->search_ratio_z,
                               cfg->search_dip_deg, cfg->search_rake_deg));
  if (cfg->max_neighbors == 0) return fail(GS_ERR_INVALID_PARAMETER, "max_neighbors must be at least 1");
  if (ps->has_dup)
    return fail(GS_ERR_DUPLICATE_POINTS, "duplicate data points: indices " +
                                             std::to_string(ps->dup_i) + " and " +
                                             std::to_string(ps->dup_j) +
                                             " share the same coordinates");
  if (cfg->max_per_octant == 0) return fail(GS_ERR_INVALID_PARAMETER, "max_per_octant must be at least 1");
  if (cfg->min_neighbors >= 0) {
    if (cfg->min_neighbors == 0) return fail(GS_ERR_INVALID_PARAMETER, "min_neighbors must be at least 1");
    if (cfg->min_neighbors > n)
      return fail(GS_ERR_INSUFFICIENT_DATA, "min_neighbors (" + std::to_string(cfg->min_neighbors) +
                                                ") exceeds the number of data points (" +
                                                std::to_string(n) + ")");
    if (cfg->max_neighbors >= 0 && cfg->min_neighbors > cfg->max_neighbors)
      return fail(GS_ERR_INVALID_PARAMETER, "min_neighbors exceeds max_neighbors");
  }
  // GPU-path limits (kinds, drift terms)
  auto* k = new gs_kriging();
  if (cudaGetDevice(&k->device) != cudaSuccess) k->device = 0;
  int rc = make_dev_model(*model, dim, &k->dm, true);
  if (rc) {
    delete k;
    return rc;
  }
  k->ps = ps;
  k->cfg = *cfg;
  k->model = *model;
  k->p = n_drift(*cfg, dim);
  if (k->p > GS_MIXED_MAX_DRIFT || (cfg->method == GS_EXTERNAL_DRIFT && cfg->ked_nvars > GS_MAX_KED_VARS)) {
    delete k;
    return fail(GS_ERR_INVALID_PARAMETER, "at most 8 external-drift covariates on the CUDA path");
  }
  k->nv = cfg->method == GS_EXTERNAL_DRIFT ? (int)cfg->ked_nvars : 0;
  // bbox centre / scale (kriging.rs:340-347)
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = 0; i < n; ++i)
    for (int d = 0; d < dim; ++d) {
      mn[d] = std::fmin(mn[d], ps->host[i * dim + d]);
      mx[d] = std::fmax(mx[d], ps->host[i * dim + d]);
    }
  double spread = 0.0;
  for (int d = 0; d < dim; ++d) {
    k->center[d] = 0.5 * (mn[d] + mx[d]);
    spread = std::fmax(spread, mx[d] - mn[d]);
  }
  k->scale = std::fmax(0.5 * spread, 2.2250738585072014e-308);
  if (ctor == 1) {
    const int nv = k->nv;
    for (int c = 0; c < nv; ++c) {
      double s = 0.0;
      for (int64_t i = 0; i < n; ++i) s += drift[i * nv + c];
      double mean = s / (double)n;
      double v = 0.0;
      for (int64_t i = 0; i < n; ++i) {
        double t = drift[i * nv + c] - mean;
        v += t * t;
      }
      v = v / (double)n;
      k->dmean[c] = mean;
      k->dscale[c] = std::fmax(std::sqrt(v), 2.2250738585072014e-308);
    }
  }
  rc = cudaStreamCreateWithFlags(&k->stream, cudaStreamNonBlocking) == cudaSuccess ? GS_OK : fail(GS_ERR_CUDA, "stream creation failed");
  if (!rc && ctor == 1) {
    if (dev_malloc((void**)&k->d_drift, n * k->nv * sizeof(double)) != cudaSuccess ||
        cudaMemcpy(k->d_drift, drift, n * k->nv * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
      rc = fail(GS_ERR_CUDA, "drift upload failed");
  }
  if (!rc && ctor == 2) {
    if (dev_malloc((void**)&k->d_err, n * sizeof(double)) != cudaSuccess ||
        cudaMemcpy(k->d_err, errors, n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
      rc = fail(GS_ERR_CUDA, "measurement-error upload failed");
  }
  // drift basis of every data point (fill_basis, kriging.rs:410-439) and the
  // measurement errors, as double-float device arrays for the mixed kernel
  if (!rc && k->p > 0) {
    const int p = k->p;
    std::vector<df> basis((size_t)p * n);
    for (int64_t i = 0; i < n; ++i) {
      const double* pi = &ps->host[i * dim];
      double xn[3] = {0, 0, 0};
      for (int d = 0; d < dim; ++d) xn[d] = (pi[d] - k->center[d]) / k->scale;
      for (int q = 0; q < p; ++q) {
        double f = 0.0;
        if (q == 0) f = 1.0;
        else if (cfg->method == GS_EXTERNAL_DRIFT)
          f = (drift[i * k->nv + (q - 1)] - k->dmean[q - 1]) / k->dscale[q - 1];
        else if (q <= dim) f = xn[q - 1];
        else {
          int idx = 1 + dim;
          for (int u = 0; u < dim; ++u)
            for (int v = u; v < dim; ++v) {
              if (idx == q) f = xn[u] * xn[v];
              ++idx;
            }
        }
        basis[(size_t)q * n + i] = df_from_double(f);
      }
    }
    if (dev_malloc((void**)&k->d_basis_df, basis.size() * sizeof(df)) != cudaSuccess ||
        cudaMemcpy(k->d_basis_df, basis.data(), basis.size() * sizeof(df),
                   cudaMemcpyHostToDevice) != cudaSuccess)
      rc = fail(GS_ERR_OUT_OF_MEMORY, "drift basis upload failed");
  }
  if (!rc && ctor == 2) {
    std::vector<df> e(n);
    for (int64_t i = 0; i < n; ++i) e[i] = df_from_double(errors[i]);
    if (dev_malloc((void**)&k->d_err_df, n * sizeof(df)) != cudaSuccess ||
        cudaMemcpy(k->d_err_df, e.data(), n * sizeof(df), cudaMemcpyHostToDevice) != cudaSuccess)
      rc = fail(GS_ERR_OUT_OF_MEMORY, "measurement-error upload failed");
  }
  k->use_tree = cfg->max_neighbors >= 0 || cfg->has_search_radius || cfg->max_per_octant >= 0;
  if (!rc && k->use_tree) {
    SearchFrame& f = k->frame;
    std::memset(&f, 0, sizeof(f));
    if (cfg->has_anisotropic_search) {
      f.aniso = 1;
      f.ratio = cfg->search_ratio;
      if (dim == 2) {
        double a = cfg->search_azimuth_deg * (3.14159265358979323846 / 180.0);
        f.s = std::sin(a);
        f.c = std::cos(a);
      } else {
        rotation_3d(cfg->search_azimuth_deg, cfg->search_ratio, cfg->search_ratio_z,
                    cfg->search_dip_deg, cfg->search_rake_deg, f.rot);
      }
    }
    double ppc = dim == 2 ? 3.0 : 4.0;
    rc = grid_build(&k->grid, dim, n, ps->d_x, ps->d_y, ps->d_z, f, ppc, k->stream);
  }
  if (!rc && !k->use_tree && n > GS_MIXED_MAX_NEIGHBORS && n >= k->p) {
    const int64_t N = n + k->p;
    if (N > kGlobalLuMax) {
      rc = fail(GS_ERR_INVALID_PARAMETER,
                "global neighbourhood of " + std::to_string(N) + " unknowns exceeds " +
                    std::to_string(kGlobalLuMax) + " on the CUDA path; set max_neighbors");
    } else if (dev_malloc((void**)&k->d_lu, (size_t)N * N * 8) != cudaSuccess ||
               dev_malloc((void**)&k->d_perm, (size_t)N * 4) != cudaSuccess) {
      rc = fail(GS_ERR_OUT_OF_MEMORY, "global system allocation failed");
    } else {
      DevBuf piv;
      int state = 0;
      rc = piv.alloc((size_t)N * 4, k->stream);
      if (!rc)
        rc = global_factor(gs::base_args(k), k->dm, (int)N, k->d_lu, (int32_t*)piv.ptr, &state,
                           k->stream);
      if (!rc) {
        // Lu::solve's row swaps applied in order, as one permutation
        std::vector<int32_t> pv(N), perm(N);
        if (cudaMemcpy(pv.data(), piv.ptr, N * 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
          rc = fail(GS_ERR_CUDA, "pivot download failed");
        } else {
          for (int64_t i = 0; i < N; ++i) perm[i] = (int32_t)i;
          if (state == 1)
            for (int64_t kk = 0; kk < N; ++kk) std::swap(perm[kk], perm[pv[kk]]);
          if (cudaMemcpy(k->d_perm, perm.data(), N * 4, cudaMemcpyHostToDevice) != cudaSuccess)
            rc = fail(GS_ERR_CUDA, "permutation upload failed");
        }
        k->lu_n = (int)N;
        k->lu_state = state;
      }
    }
  }
  if (rc) {
    delete k;
    return rc;
  }
  *out = k;
  return GS_OK;
}

// Global neighbourhood in cross-validation: target c0 + t (a data point)
// conditions on every point with another label, in index order.
__global__ void excl_rows_kernel(int64_t nt, int64_t c0, int n, const int32_t* label, int kout,
                                 int32_t* nb, int32_t* nbc) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t own = label[c0 + t];
    int32_t* row = nb + t * (int64_t)kout;
    int c = 0;
    for (int j = 0; j < n && c < kout; ++j)
      if (label[j] != own) row[c++] = j;
    nbc[t] = c;
  }
}

__global__ void iota_rows_kernel(int64_t nt, int n, int32_t* nb, int32_t* nbc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nt * n;
       i += (int64_t)gridDim.x * blockDim.x) {
    nb[i] = (int32_t)(i % n);
    if (i % n == 0) nbc[i / n] = n;
  }
}

struct PhaseTimer {
  cudaEvent_t ev[4];
  bool ok = false;
  explicit PhaseTimer(cudaStream_t s) {
    ok = true;
    for (int i = 0; i < 4; ++i) ok = ok && cudaEventCreate(&ev[i]) == cudaSuccess;
    (void)s;
  }
  ~PhaseTimer() {
    for (int i = 0; i < 4; ++i) cudaEventDestroy(ev[i]);
  }
};

}  // namespace

namespace gs {

// Targets whose neighbour count is at most / above a threshold (binning).
struct NbLe {
  const int32_t* nbc;
  int thr;
  __host__ __device__ bool operator()(int64_t t) const { return nbc[t] <= thr; }
};
struct NbGt {
  const int32_t* nbc;
  int thr;
  __host__ __device__ bool operator()(int64_t t) const { return nbc[t] > thr; }
};

// Calls with at least this many targets are autotuned (per size class).
constexpr int64_t kTuneMinTargets = 65536;
// Targets of the first chunk the candidates are timed on.
constexpr int64_t kTuneSample = 131072;
// Warps of the FP64 LDL^T re-solve (slot-covariance scratch, 16.6 KB each).
int64_t chol_scratch_warps() { return (int64_t)sm_count() * 16; }
// Leading targets of each chunk whose FP32 failure rate routes the rest.
constexpr int64_t kRouteSample = 16384;

// Calls large enough to fill the GPU share one tuned shape per predictor
// (the best run length depends on the systems, not on how many there are);
// smaller calls use the default.
int size_class(int64_t nt) { return nt >= kTuneMinTargets ? 1 : 0; }

// Shapes tuned by earlier predictors, keyed by what decides the best launch
// shape: device, dimension, neighbour slots, drift terms, nested structures,
// binning, cross-validation exclusion and size class.  A predictor whose
// first call of a size class finds its key here starts from that shape
// instead of timing the candidates again (repeated cross-validation or
// tuning calls build a new predictor each time).
struct TuneKey {
  int device, dim, kout, p, ns, binnable, excl, cls;
  bool operator<(const TuneKey& o) const {
    return std::tie(device, dim, kout, p, ns, binnable, excl, cls) <
           std::tie(o.device, o.dim, o.kout, o.p, o.ns, o.binnable, o.excl, o.cls);
  }
};
std::mutex g_tuned_mu;
std::map<TuneKey, Tiles> g_tuned;

// Launch shape without measurement: the longest run that still gives every
// SM a few blocks.
Tiles default_tiles(int64_t nt, bool binnable) {
  Tiles t;
  t.bins = binnable ? 1 : 0;
  t.run = 64;
  while (t.run > 8 && (nt + t.run - 1) / t.run < (int64_t)sm_count() * 4) t.run >>= 1;
  return t;
}

KrigeArgs base_args(const gs_kriging* k) {
  const gs_pointset* ps = k->ps;
  const gs_kcfg& c = k->cfg;
  KrigeArgs a{};
  a.dim = ps->dim;
  a.method = (int)c.method;
  a.p = k->p;
  a.nv = k->nv;
  a.uk_degree = (int)c.uk_degree;
  a.min_nb = c.min_neighbors >= 0 ? (int)c.min_neighbors : 1;
  a.sk_mean = c.sk_mean;
  for (int d = 0; d < 3; ++d) a.center[d] = k->center[d];
  a.scale = k->scale;
  for (int v = 0; v < GS_MAX_KED_VARS; ++v) {
    a.dmean[v] = k->dmean[v];
    a.dscale[v] = k->dscale[v];
  }
  a.x = ps->d_x;
  a.y = ps->d_y;
  a.z = ps->d_z;
  a.val = ps->d_v;
  a.meas_err = k->d_err;
  a.drift = k->d_drift;
  a.cdf = (const df*)ps->d_cdf;
  a.vdf = (const df*)ps->d_vdf;
  a.basis_df = k->d_basis_df;
  a.err_df = k->d_err_df;
  a.n = ps->n;
  return a;
}

// Search + solves for targets already on the device.  timed: phase timings,
// FP64 re-solve count and a final synchronisation; otherwise the whole pass
// is only enqueued on `stream` (no host synchronisation: it can be captured
// into a CUDA graph).
// Block kriging: the shared discretisation offsets (noff x dim, device) and
// the within-block covariance (device); the pass then runs the FP64 kernel.
struct BlockSpec {
  const double* off;
  int noff;
  const double* cbb;
};

// The factored global system's matrix-product form, prepared on first use by
// a mixed-precision call of at least N / 4 targets (N solves with the
// factors: about 2 N^3 FP64 FMAs, so a predictor used only at FP64, or only
// for a few targets at a time, never pays for it).  Without device memory
// for it, mixed-precision calls take the per-target solves.
static int ensure_global_gemm(const gs_kriging* k) {
  std::lock_guard<std::mutex> lk(k->gemm_mu);
  if (k->gemm_state != 0) return GS_OK;
  const int N = k->lu_n;
  const size_t nn = (size_t)N * N;
  auto unavailable = [&]() {
    cudaGetLastError();  // clear the failed allocation
    cudaFree(k->d_rh);
    cudaFree(k->d_rl);
    cudaFree(k->d_lambda);
    cudaFree(k->d_arow);
    k->d_rh = k->d_rl = nullptr;
    k->d_lambda = k->d_arow = nullptr;
    k->gemm_state = 2;
    return GS_OK;
  };
  if (dev_malloc((void**)&k->d_rh, nn * 4) != cudaSuccess ||
      dev_malloc((void**)&k->d_rl, nn * 4) != cudaSuccess ||
      dev_malloc((void**)&k->d_lambda, (size_t)N * 8) != cudaSuccess ||
      dev_malloc((void**)&k->d_arow, (size_t)N * 8) != cudaSuccess)
    return unavailable();
  const int rc = global_gemm_prepare(base_args(k), N, k->d_lu, k->d_perm, k->d_rh, k->d_rl,
                                     k->d_lambda, k->d_arow, k->stream);
  if (rc == GS_ERR_OUT_OF_MEMORY) return unavailable();  // its temporary buffers did not fit
  if (rc) return rc;
  k->gemm_state = 1;
  return GS_OK;
}

int predict_pass(const gs_kriging* k, int64_t nt, const double* tx, const double* ty,
                 const double* tz, const double* tdrift, double* value, double* variance,
                 double* lagrange, uint8_t* status, int precision, cudaStream_t stream, bool timed,
                 const int32_t* excl_labels = nullptr, const BlockSpec* blk = nullptr) {
  NvtxRange nvtx_range("gs.predict_pass");
  if (nt == 0) return GS_OK;
  const gs_pointset* ps = k->ps;
  const gs_kcfg& c = k->cfg;
  const int dim = ps->dim;
  const int64_t n = ps->n;
  const int p = k->p;
  // neighbourhood geometry
  SearchParams sp{};
  int kout;
  const int64_t navail = excl_labels ? n - 1 : n;  // cross-validation: at most n - 1 others
  if (!k->use_tree && k->lu_state != 0 && !excl_labels && !blk) {
    kout = (int)n;  // the factored global path below
  } else if (!k->use_tree) {
    if (navail + p > GS_MAX_SYSTEM)
      return fail(GS_ERR_INVALID_PARAMETER,
                  "global neighbourhood of " + std::to_string(navail) +
                      " points exceeds the CUDA path's system limit; set max_neighbors");
    kout = (int)navail;
  } else if (c.max_per_octant >= 0) {
    const int NB = 1 << dim;
    int per = (int)std::min<int64_t>(c.max_per_octant, n);
    sp.octant = 1;
    sp.k = per;
    kout = NB * per;
    if (c.max_neighbors >= 0) kout = (int)std::min<int64_t>(kout, c.max_neighbors);
  } else if (c.max_neighbors >= 0) {
    sp.k = (int)std::min<int64_t>(c.max_neighbors, n);
    kout = sp.k;
  } else {
    sp.unbounded = 1;
    sp.k = (int)std::min<int64_t>(n, GS_MAX_SYSTEM - p);
    kout = sp.k;
  }
  const bool global_lu = !k->use_tree && k->lu_state != 0 && !excl_labels && !blk;
  if (!global_lu && kout + p > GS_MAX_SYSTEM)
    return fail(GS_ERR_INVALID_PARAMETER, "neighbourhood plus drift terms exceed " +
                                              std::to_string(GS_MAX_SYSTEM) + " on the CUDA path");
  sp.kout = kout;
  sp.excl_label = excl_labels;
  sp.has_radius = c.has_search_radius ? 1 : 0;
  sp.r2 = c.has_search_radius ? c.search_radius * c.search_radius : 0.0;
  const int nmax_all = kout + p;

  KrigeArgs a = base_args(k);
  a.kout = kout;
  if (blk) {
    a.boff = blk->off;
    a.nboff = blk->noff;
    a.cbb = blk->cbb;
  }

  // global neighbourhood factored at build: per-target solves only
  if (global_lu) {
    const int N = k->lu_n;
    const int64_t warps = std::max<int64_t>(
        1, std::min<int64_t>((int64_t)sm_count() * 32, ((int64_t)512 << 20) / (16 * (int64_t)N)));
    DevBuf scratch;
    // the form is prepared by the first mixed call of at least N / 4 targets
    // (its 2 N^3 FMAs are then at most four times the call's per-target
    // solves, 2 N^2 each); smaller calls before it take the per-target solves
    if (precision != GS_PREC_FP64 && k->lu_state == 1 && 4 * nt >= N)
      GS_TRY(ensure_global_gemm(k));
    const bool gemm = precision != GS_PREC_FP64 && k->lu_state == 1 && k->gemm_state == 1;
    if (!gemm) GS_TRY(scratch.alloc((size_t)warps * 2 * N * 8, stream));
    KrigeArgs g = a;
    g.tx = tx;
    g.ty = ty;
    g.tz = tz;
    g.tdrift = tdrift;
    g.out_v = value;
    g.out_var = variance;
    g.out_lag = lagrange;
    g.out_st = status;
    g.ntl = nt;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (timed) {
      GS_CUDA(cudaEventCreate(&e0));
      GS_CUDA(cudaEventCreate(&e1));
      GS_CUDA(cudaEventRecord(e0, stream));
    }
    if (gemm) {
      GS_TRY(global_gemm_launch(g, k->dm, N, k->d_rh, k->d_rl, k->d_lambda, k->d_arow, stream));
    } else {
      GS_TRY(global_solve_launch(g, k->dm, N, k->d_lu, k->d_perm, k->lu_state,
                                 (double*)scratch.ptr, warps, stream));
    }
    if (!timed) return GS_OK;
    GS_CUDA(cudaEventRecord(e1, stream));
    GS_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    g_timings[0] = 0;
    g_timings[1] = 0;
    g_timings[2] = ms;
    g_timings[3] = ms;
    g_fallbacks = nt;
    g_lu_resolves = 0;
    return GS_OK;
  }

  // chunking keeps the neighbour lists within a fixed budget (4 GiB: a
  // 4.19 M-target grid with 64 neighbours is one chunk)
  const int64_t chunk = std::max<int64_t>(1024, std::min<int64_t>(nt, (int64_t)(4ll << 30) / (4ll * kout + 16)));
  const int64_t nchunks = (nt + chunk - 1) / chunk;
  // uneven neighbourhoods (octant, radius) are binned by system size: the
  // small systems run on the 32-thread kernel, the rest on the 64-thread one
  const bool mixed = precision != GS_PREC_FP64 && !blk;
  const bool binnable = mixed && kout > 32 && kout <= GS_MIXED_MAX_NEIGHBORS &&
                        (sp.octant || sp.has_radius || sp.unbounded);
  // launch shape: pinned, tuned earlier for this size class, tuned now on
  // the first chunk (timed calls only), or the default
  Tiles tiles = default_tiles(nt, binnable);
  bool tune_now = false;
  const TuneKey tkey{k->device, dim, kout, p, k->dm.ns, binnable ? 1 : 0, excl_labels ? 1 : 0,
                     size_class(nt)};
  if (mixed) {
    std::lock_guard<std::mutex> lk(k->tiles_mu);
    auto it = k->tiles.find(size_class(nt));
    if (k->pinned.run > 0) {
      tiles = k->pinned;
    } else if (it != k->tiles.end()) {
      tiles = it->second;
    } else {
      std::lock_guard<std::mutex> gl(g_tuned_mu);
      auto g = g_tuned.find(tkey);
      if (g != g_tuned.end()) {
        tiles = g->second;
        k->tiles[size_class(nt)] = tiles;
      } else {
        tune_now = timed && nt >= kTuneMinTargets;
      }
    }
  }
  const bool binned = binnable;
  DevBuf nb, nbc, flag, tlist, nsel, tmp, bins, counts;
  GS_TRY(nb.alloc((size_t)chunk * kout * 4, stream));
  GS_TRY(nbc.alloc((size_t)chunk * 4, stream));
  GS_TRY(flag.alloc((size_t)chunk, stream));
  GS_TRY(tlist.alloc((size_t)chunk * 8, stream));
  GS_TRY(nsel.alloc(32, stream));
  GS_TRY(counts.alloc((size_t)nchunks * 16, stream));
  size_t sel_bytes = 0, bin_bytes = 0;
  GS_CUDA(cub::DeviceSelect::Flagged(nullptr, sel_bytes, thrust::counting_iterator<int64_t>(0),
                                     (uint8_t*)nullptr, (int64_t*)nullptr, (int64_t*)nullptr,
                                     (int64_t)chunk, stream));
  if (binned) {
    GS_CUDA(cub::DeviceSelect::If(nullptr, bin_bytes, thrust::counting_iterator<int64_t>(0),
                                  (int64_t*)nullptr, (int64_t*)nullptr, (int64_t)chunk,
                                  NbLe{nullptr, 32}, stream));
    GS_TRY(bins.alloc((size_t)chunk * 2 * 8 + 16, stream));
  }
  GS_TRY(tmp.alloc(std::max(sel_bytes, bin_bytes), stream));
  // FP64 scratch (plain build or re-solve)
  const int64_t budget = (int64_t)2 << 30;
  const int64_t fthreads = fp64_threads_for(nmax_all, budget);
  DevBuf scratch, cscratch;
  GS_TRY(scratch.alloc((size_t)fp64_scratch_doubles(nmax_all, fthreads) * 8, stream));
  // slot scratch for at most one warp per target of a chunk
  const int64_t cwarps = std::min<int64_t>(chol_scratch_warps(), (chunk + 3) / 4 * 4);
  if (mixed) GS_TRY(cscratch.alloc((size_t)chol_scratch_doubles(cwarps) * 8, stream));

  cudaEvent_t ev[6] = {};
  if (timed)
    for (int i = 0; i < 6; ++i) GS_CUDA(cudaEventCreate(&ev[i]));
  auto mark = [&](int i) -> int {
    if (timed) GS_CUDA(cudaEventRecord(ev[i], stream));
    return GS_OK;
  };
  float t_search = 0, t_mixed = 0, t_fp64 = 0;
  GS_TRY(mark(0));
  int rc = GS_OK;
  for (int64_t ci = 0; ci < nchunks && !rc; ++ci) {
    const int64_t c0 = ci * chunk;
    const int64_t cn = std::min(chunk, nt - c0);
    const double* ctx = tx + c0;
    const double* cty = ty + c0;
    const double* ctz = dim == 3 ? tz + c0 : nullptr;
    int32_t* dnb = (int32_t*)nb.ptr;
    int32_t* dnbc = (int32_t*)nbc.ptr;
    GS_TRY(mark(1));
    if (k->use_tree) {
      SearchParams spc = sp;
      if (excl_labels) spc.target_label = excl_labels + c0;  // targets are the data points
      rc = search_launch(k->grid, k->frame, spc, cn, ctx, cty, ctz, dnb, dnbc, stream);
    } else if (excl_labels) {
      excl_rows_kernel<<<(int)std::min<int64_t>((cn + 127) / 128, (int64_t)sm_count() * 64), 128, 0, stream>>>(
          cn, c0, (int)n, excl_labels, kout, dnb, dnbc);
      rc = cudaGetLastError() == cudaSuccess ? GS_OK : fail(GS_ERR_CUDA, "launch failed");
    } else {
      iota_rows_kernel<<<(int)std::min<int64_t>((cn * kout + 255) / 256, (int64_t)sm_count() * 64), 256, 0, stream>>>(
          cn, kout, dnb, dnbc);
      rc = cudaGetLastError() == cudaSuccess ? GS_OK : fail(GS_ERR_CUDA, "launch failed");
    }
    if (rc) break;
    GS_TRY(mark(2));
    KrigeArgs ca = a;
    ca.tx = ctx;
    ca.ty = cty;
    ca.tz = ctz;
    ca.tdrift = tdrift ? tdrift + c0 * k->nv : nullptr;
    ca.nb = dnb;
    ca.nbc = dnbc;
    ca.out_v = value + c0;
    ca.out_var = variance + c0;
    ca.out_lag = lagrange ? lagrange + c0 : nullptr;
    ca.out_st = status + c0;
    if (!mixed) {
      ca.nmax = nmax_all;
      ca.tlist = nullptr;
      ca.ntl = cn;
      GS_TRY(mark(3));
      rc = krige_fp64_launch(ca, k->dm, (double*)scratch.ptr, fthreads, stream);
      if (rc) break;
      GS_TRY(mark(4));
    } else {
      ca.nmax = std::min(nmax_all, GS_MIXED_MAX_NEIGHBORS + p);
      ca.tlist = nullptr;
      // mixed solves of the chunk's first `count` targets with shape t
      // mixed solves of the chunk's targets [b0, b0 + count) with shape t
      // (per-target arrays offset to b0); route: the FP64 routing switch
      auto solve_mixed = [&](int64_t b0, int64_t count, const Tiles& t, const int* route) -> int {
        KrigeArgs sa = ca;
        sa.tx += b0;
        sa.ty += b0;
        if (sa.tz) sa.tz += b0;
        if (sa.tdrift) sa.tdrift += b0 * k->nv;
        sa.nb += b0 * kout;
        sa.nbc += b0;
        sa.out_v += b0;
        sa.out_var += b0;
        if (sa.out_lag) sa.out_lag += b0;
        sa.out_st += b0;
        sa.ntl = count;
        sa.run = t.run;
        sa.spc = t.spc;
        sa.route_fp64 = route;
        uint8_t* fl = (uint8_t*)flag.ptr + b0;
        if (!(binned && t.bins)) return krige_mixed_launch(sa, k->dm, fl, 0, stream);
        int64_t* lists = (int64_t*)bins.ptr;
        int64_t* cnts = lists + 2 * chunk;
        size_t b = bin_bytes;
        GS_CUDA(cub::DeviceSelect::If(tmp.ptr, b, thrust::counting_iterator<int64_t>(0), lists,
                                      cnts, count, NbLe{sa.nbc, 32}, stream));
        b = bin_bytes;
        GS_CUDA(cub::DeviceSelect::If(tmp.ptr, b, thrust::counting_iterator<int64_t>(0),
                                      lists + chunk, cnts + 1, count, NbGt{sa.nbc, 32}, stream));
        sa.tlist = lists;
        sa.ntl_dev = cnts;
        GS_TRY(krige_mixed_launch(sa, k->dm, fl, 32, stream));
        sa.tlist = lists + chunk;
        sa.ntl_dev = cnts + 1;
        return krige_mixed_launch(sa, k->dm, fl, 64, stream);
      };
      if (tune_now && ci == 0) {
        // autotuner over run length, warps per system (binning) and systems
        // per block: candidates are run once untimed (module loading), then
        // timed on the same sample.  Stage 1 times every run length and
        // binning at one system per block, stage 2 the winner at two systems
        // per block; the fastest shape serves this size class.
        const int64_t ns = std::min(cn, kTuneSample);
        auto time_shapes = [&](const std::vector<Tiles>& cand, std::vector<float>& ms) -> int {
          std::vector<cudaEvent_t> te(cand.size() + 1);
          for (auto& e : te) GS_CUDA(cudaEventCreate(&e));
          int r = GS_OK;
          for (int pass = 0; pass < 2 && !r; ++pass) {
            for (size_t c = 0; c < cand.size() && !r; ++c) {
              if (pass == 1 && c == 0 && cudaEventRecord(te[0], stream) != cudaSuccess)
                r = fail(GS_ERR_CUDA, "event record failed");
              if (!r) r = solve_mixed(0, ns, cand[c], nullptr);
              if (!r && pass == 1 && cudaEventRecord(te[c + 1], stream) != cudaSuccess)
                r = fail(GS_ERR_CUDA, "event record failed");
            }
          }
          if (!r && cudaEventSynchronize(te.back()) != cudaSuccess)
            r = fail(GS_ERR_CUDA, "event synchronisation failed");
          ms.assign(cand.size(), 0.0f);
          if (!r)
            for (size_t c = 0; c < cand.size(); ++c) cudaEventElapsedTime(&ms[c], te[c], te[c + 1]);
          for (auto& e : te) cudaEventDestroy(e);
          return r;
        };
        std::vector<Tiles> cand;
        for (int run : {16, 32, 64, 128})
          for (int bn = 0; bn <= (binned ? 1 : 0); ++bn) cand.push_back(Tiles{run, bn, 1});
        std::vector<float> ms;
        rc = time_shapes(cand, ms);
        if (!rc) {
          size_t best = 0;
          for (size_t c = 1; c < cand.size(); ++c)
            if (ms[c] < ms[best]) best = c;
          tiles = cand[best];
          std::vector<float> ms2;
          const std::vector<Tiles> cand2{Tiles{tiles.run, tiles.bins, 2}};
          rc = time_shapes(cand2, ms2);
          if (!rc && ms2[0] < ms[best]) tiles = cand2[0];
        }
        if (!rc) {
          std::lock_guard<std::mutex> lk(k->tiles_mu);
          k->tiles[size_class(nt)] = tiles;
          std::lock_guard<std::mutex> gl(g_tuned_mu);
          g_tuned[tkey] = tiles;
        }
        if (rc) break;
      }
      // the first kRouteSample targets decide (on the device) whether the
      // rest of the chunk goes straight to the FP64 re-solve
      const int64_t nprobe = std::min(cn, kRouteSample);
      int* route = (int*)((int64_t*)nsel.ptr + 2);
      rc = solve_mixed(0, nprobe, tiles, nullptr);
      if (!rc && cn > nprobe) {
        rc = route_launch((const uint8_t*)flag.ptr, nprobe, route, stream);
        if (!rc) rc = solve_mixed(nprobe, cn - nprobe, tiles, route);
      }
      ca.ntl = cn;
      if (rc) break;
      GS_TRY(mark(3));
      // systems the refinement could not certify: FP64 re-solve over the
      // flagged list, its length read on the device (no host round trip);
      // first the bordered LDL^T kernel, then the partial-pivoting LU for
      // what it leaves flagged
      int64_t* nsel2 = (int64_t*)nsel.ptr + 1;
      size_t b = sel_bytes;
      GS_CUDA(cub::DeviceSelect::Flagged(tmp.ptr, b, thrust::counting_iterator<int64_t>(0),
                                         (uint8_t*)flag.ptr, (int64_t*)tlist.ptr,
                                         (int64_t*)nsel.ptr, cn, stream));
      GS_CUDA(cudaMemcpyAsync((int64_t*)counts.ptr + ci, nsel.ptr, 8, cudaMemcpyDeviceToDevice,
                              stream));
      ca.nmax = nmax_all;
      ca.tlist = (const int64_t*)tlist.ptr;
      ca.ntl = cn;
      ca.ntl_dev = (const int64_t*)nsel.ptr;
      rc = krige_chol_launch(ca, k->dm, (uint8_t*)flag.ptr, (double*)cscratch.ptr, cwarps, stream);
      if (rc) break;
      b = sel_bytes;
      GS_CUDA(cub::DeviceSelect::Flagged(tmp.ptr, b, thrust::counting_iterator<int64_t>(0),
                                         (uint8_t*)flag.ptr, (int64_t*)tlist.ptr, nsel2, cn,
                                         stream));
      GS_CUDA(cudaMemcpyAsync((int64_t*)counts.ptr + nchunks + ci, nsel2, 8,
                              cudaMemcpyDeviceToDevice, stream));
      ca.ntl_dev = nsel2;
      rc = krige_fp64_launch(ca, k->dm, (double*)scratch.ptr, fthreads, stream);
      if (rc) break;
      GS_TRY(mark(4));
    }
    if (timed) {
      GS_CUDA(cudaEventSynchronize(ev[4]));
      float ms = 0;
      cudaEventElapsedTime(&ms, ev[1], ev[2]);
      t_search += ms;
      if (!mixed) {
        cudaEventElapsedTime(&ms, ev[3], ev[4]);
        t_fp64 += ms;
      } else {
        cudaEventElapsedTime(&ms, ev[2], ev[3]);
        t_mixed += ms;
        cudaEventElapsedTime(&ms, ev[3], ev[4]);
        t_fp64 += ms;
      }
    }
  }
  if (!timed) return rc;  // enqueued only: the caller synchronises
  GS_TRY(mark(5));
  GS_CUDA(cudaEventSynchronize(ev[5]));
  float tot = 0;
  cudaEventElapsedTime(&tot, ev[0], ev[5]);
  for (int i = 0; i < 6; ++i) cudaEventDestroy(ev[i]);
  int64_t n_resolved = nt, n_lu = nt;
  if (mixed) {
    std::vector<int64_t> hc(2 * nchunks, 0);
    GS_CUDA(cudaMemcpyAsync(hc.data(), counts.ptr, nchunks * 16, cudaMemcpyDeviceToHost, stream));
    GS_CUDA(cudaStreamSynchronize(stream));
    n_resolved = n_lu = 0;
    for (int64_t c = 0; c < nchunks; ++c) {
      n_resolved += hc[c];
      n_lu += hc[nchunks + c];
    }
  }
  g_lu_resolves = n_lu;
  g_timings[0] = t_search;
  g_timings[1] = t_mixed;
  g_timings[2] = t_fp64;
  g_timings[3] = tot;
  g_fallbacks = n_resolved;
  if (rc) return rc;
  GS_CUDA(cudaStreamSynchronize(stream));
  return GS_OK;
}

int predict_device(const gs_kriging* k, int64_t nt, const double* tx, const double* ty,
                   const double* tz, const double* tdrift, double* value, double* variance,
                   double* lagrange, uint8_t* status, int precision, cudaStream_t stream) {
  return predict_pass(k, nt, tx, ty, tz, tdrift, value, variance, lagrange, status, precision,
                      stream, true);
}

}  // namespace gs

extern "C" {

int gs_kriging_new(const gs_pointset* ps, const gs_model* model, const gs_kcfg* cfg,
                   gs_kriging** out) {
  return kriging_create(ps, model, cfg, 0, nullptr, nullptr, out);
}
int gs_kriging_with_external_drift(const gs_pointset* ps, const gs_model* model,
                                   const gs_kcfg* cfg, const double* drift, gs_kriging** out) {
  return kriging_create(ps, model, cfg, 1, drift, nullptr, out);
}
int gs_kriging_with_measurement_error(const gs_pointset* ps, const gs_model* model,
                                      const gs_kcfg* cfg, const double* errors,
                                      gs_kriging** out) {
  return kriging_create(ps, model, cfg, 2, nullptr, errors, out);
}
void gs_kriging_destroy(gs_kriging* k) { delete k; }

int gs_kriging_predict_many_device(const gs_kriging* k, int64_t nt, const double* tx,
                                   const double* ty, const double* tz, const double* tdrift,
                                   double* value, double* variance, double* lagrange,
                                   uint8_t* status, int precision, void* stream) {
  if (!k) return fail(GS_ERR_INVALID_PARAMETER, "null predictor");
  if (k->cfg.method == GS_EXTERNAL_DRIFT && !tdrift)
    return fail(GS_ERR_INVALID_PARAMETER, "external drift kriging requires predict_with_drift");
  if (k->cfg.method != GS_EXTERNAL_DRIFT && tdrift)
    return fail(GS_ERR_INVALID_PARAMETER, "predict_with_drift requires KrigingMethod::ExternalDrift");
  cudaStream_t s = stream ? (cudaStream_t)stream : k->stream;
  return predict_device(k, nt, tx, ty, tz, tdrift, value, variance, lagrange, status, precision, s);
}

int gs_kriging_set_tiles(gs_kriging* k, int run, int bins, int systems_per_block) {
  if (!k) return fail(GS_ERR_INVALID_PARAMETER, "null predictor");
  if (run != 0 && (run < 1 || run > 1024 || (run & (run - 1))))
    return fail(GS_ERR_INVALID_PARAMETER, "run must be 0 or a power of two in [1, 1024]");
  if (bins != 0 && bins != 1) return fail(GS_ERR_INVALID_PARAMETER, "bins must be 0 or 1");
  if (systems_per_block != 1 && systems_per_block != 2)
    return fail(GS_ERR_INVALID_PARAMETER, "systems per block must be 1 or 2");
  std::lock_guard<std::mutex> lk(k->tiles_mu);
  k->pinned = gs::Tiles{run, bins, systems_per_block};
  return GS_OK;
}

// validation.rs:136-153 fold_assignment: a seeded shuffle of 0..n-1 (rng.rs
// shuffle), position j of the shuffled order goes to fold j mod k.
static void fold_assignment(int64_t n, int64_t k, uint64_t seed, std::vector<int32_t>& fold_of) {
  std::vector<int64_t> order(n);
  for (int64_t i = 0; i < n; ++i) order[i] = i;
  gs::Xoshiro r(seed);
  for (int64_t i = n - 1; i >= 1; --i) {
    const int64_t j = (int64_t)(r.next() % (uint64_t)(i + 1));
    std::swap(order[i], order[j]);
  }
  fold_of.assign(n, 0);
  for (int64_t j = 0; j < n; ++j) fold_of[order[j]] = (int32_t)(j % k);
}

}  // extern "C"
static int cv_with_labels(const gs_kriging* k, const std::vector<int32_t>& label,
                          double* predicted, double* variance, uint8_t* status, int precision);
extern "C" {

int gs_kriging_cross_validate(const gs_kriging* k, int64_t nfolds, uint64_t seed, double* predicted,
                              double* variance, uint8_t* status, int precision) {
  NvtxRange nvtx_range("gs.cross_validate");
  if (!k || !predicted || !variance) return fail(GS_ERR_INVALID_PARAMETER, "null argument");
  const gs_pointset* ps = k->ps;
  const int64_t n = ps->n;
  if (n < 3)
    return fail(GS_ERR_INSUFFICIENT_DATA, nfolds == 0
                                              ? "leave-one-out cross-validation requires at least 3 points"
                                              : "cross-validation requires at least 3 points");
  if (nfolds != 0 && !(nfolds >= 2 && nfolds <= n))
    return fail(GS_ERR_INVALID_PARAMETER, "k-fold requires 2 <= k <= n (k=" + std::to_string(nfolds) +
                                              ", n=" + std::to_string(n) + ")");
  std::vector<int32_t> label(n);
  if (nfolds == 0) {
    for (int64_t i = 0; i < n; ++i) label[i] = (int32_t)i;
  } else {
    fold_assignment(n, nfolds, seed, label);
  }
  return cv_with_labels(k, label, predicted, variance, status, precision);
}

// validation.rs:298-328 spatial_block_assignment: a regular grid of
// blocks_per_dim[d] cells over the bounding box, dimension 0 fastest.
static void spatial_block_assignment(const gs_pointset* ps, const int64_t* bpd,
                                     std::vector<int32_t>& label) {
  const int dim = ps->dim;
  const int64_t n = ps->n;
  double lo[3], hi[3];
  for (int d = 0; d < dim; ++d) lo[d] = hi[d] = ps->host[d];
  for (int64_t i = 0; i < n; ++i)
    for (int d = 0; d < dim; ++d) {
      lo[d] = std::fmin(lo[d], ps->host[i * dim + d]);
      hi[d] = std::fmax(hi[d], ps->host[i * dim + d]);
    }
  for (int64_t i = 0; i < n; ++i) {
    int64_t idx = 0, stride = 1;
    for (int d = 0; d < dim; ++d) {
      const double span = std::fmax(hi[d] - lo[d], 2.2250738585072014e-308);
      const double frac = std::fmin(std::fmax((ps->host[i * dim + d] - lo[d]) / span, 0.0),
                                    1.0 - 1e-12);
      const int64_t bd = std::min<int64_t>((int64_t)(frac * (double)bpd[d]), bpd[d] - 1);
      idx += bd * stride;
      stride *= bpd[d];
    }
    label[i] = (int32_t)idx;
  }
}

// validation.rs:348-374 block_cv.
int gs_kriging_block_cv(const gs_kriging* k, const int64_t* blocks_per_dim, double* predicted,
                        double* variance, uint8_t* status, int precision) {
  if (!k || !blocks_per_dim || !predicted || !variance)
    return fail(GS_ERR_INVALID_PARAMETER, "null argument");
  const gs_pointset* ps = k->ps;
  const int64_t n = ps->n;
  if (n < 3) return fail(GS_ERR_INSUFFICIENT_DATA, "cross-validation requires at least 3 points");
  double nblocks = 1.0;
  for (int d = 0; d < ps->dim; ++d) {
    if (blocks_per_dim[d] <= 0)
      return fail(GS_ERR_INVALID_PARAMETER, "blocks_per_dim entries must be at least 1");
    nblocks *= (double)blocks_per_dim[d];
  }
  if (nblocks < 2.0) return fail(GS_ERR_INVALID_PARAMETER, "block CV requires at least 2 blocks total");
  if (nblocks > 2147483647.0) return fail(GS_ERR_INVALID_PARAMETER, "too many blocks");
  std::vector<int32_t> label(n);
  spatial_block_assignment(ps, blocks_per_dim, label);
  return cv_with_labels(k, label, predicted, variance, status, precision);
}

}  // extern "C"

// cv_with_folds (validation.rs:219-265) as one prediction pass over the data
// points, each excluding the data points of its own label.
static int cv_with_labels(const gs_kriging* k, const std::vector<int32_t>& label,
                          double* predicted, double* variance, uint8_t* status, int precision) {
  const gs_pointset* ps = k->ps;
  const int64_t n = ps->n;
  cudaStream_t s = k->stream;
  gs::DevBuf dl, dv, dvar, dst;
  GS_TRY(dl.alloc((size_t)n * 4, s));
  GS_TRY(dv.alloc((size_t)n * 8, s));
  GS_TRY(dvar.alloc((size_t)n * 8, s));
  GS_TRY(dst.alloc((size_t)n, s));
  GS_CUDA(cudaMemcpyAsync(dl.ptr, label.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s));
  GS_TRY(gs::predict_pass(k, n, ps->d_x, ps->d_y, ps->dim == 3 ? ps->d_z : nullptr,
                          k->cfg.method == GS_EXTERNAL_DRIFT ? k->d_drift : nullptr,
                          (double*)dv.ptr, (double*)dvar.ptr, nullptr, (uint8_t*)dst.ptr, precision,
                          s, true, (const int32_t*)dl.ptr));
  std::vector<uint8_t> st(n);
  GS_CUDA(cudaMemcpyAsync(predicted, dv.ptr, (size_t)n * 8, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaMemcpyAsync(variance, dvar.ptr, (size_t)n * 8, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaMemcpyAsync(st.data(), dst.ptr, (size_t)n, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaStreamSynchronize(s));
  if (status) std::memcpy(status, st.data(), (size_t)n);
  // the reference stops at a point whose prediction fails (Kriging::predict)
  for (int64_t i = 0; i < n; ++i) {
    const int code = st[i] & 0x3f;
    if (code == GS_ST_OK) continue;
    const std::string at = "cross-validation at point " + std::to_string(i) + ": ";
    if (code == GS_ST_NO_NEIGHBORS) return fail(GS_ERR_NO_NEIGHBORS, at + "not enough neighbours");
    if (code == GS_ST_INSUFFICIENT_DATA)
      return fail(GS_ERR_INSUFFICIENT_DATA, at + "fewer neighbours than drift terms");
    if (code == GS_ST_SINGULAR) return fail(GS_ERR_SINGULAR_SYSTEM, at + "singular kriging system");
    return fail(GS_ERR_INVALID_PARAMETER, at + "neighbourhood beyond the CUDA path's system limit");
  }
  return GS_OK;
}

extern "C" {

int gs_kriging_tiles(const gs_kriging* k, int64_t nt, int* run, int* bins,
                     int* systems_per_block, int* tuned) {
  if (!k || !run || !bins || !systems_per_block || !tuned)
    return fail(GS_ERR_INVALID_PARAMETER, "null argument");
  std::lock_guard<std::mutex> lk(k->tiles_mu);
  auto it = k->tiles.find(gs::size_class(nt));
  gs::Tiles t = gs::default_tiles(nt, true);
  *tuned = 0;
  if (k->pinned.run > 0) {
    t = k->pinned;
    *tuned = 2;
  } else if (it != k->tiles.end()) {
    t = it->second;
    *tuned = 1;
  }
  *run = t.run;
  *bins = t.bins;
  *systems_per_block = t.spc;
  return GS_OK;
}

int gs_kriging_predict_many_async(const gs_kriging* k, int64_t nt, const double* tx,
                                  const double* ty, const double* tz, const double* tdrift,
                                  double* value, double* variance, double* lagrange,
                                  uint8_t* status, int precision, void* stream) {
  if (!k) return fail(GS_ERR_INVALID_PARAMETER, "null predictor");
  if (k->cfg.method == GS_EXTERNAL_DRIFT && !tdrift)
    return fail(GS_ERR_INVALID_PARAMETER, "external drift kriging requires predict_with_drift");
  if (k->cfg.method != GS_EXTERNAL_DRIFT && tdrift)
    return fail(GS_ERR_INVALID_PARAMETER, "predict_with_drift requires KrigingMethod::ExternalDrift");
  if (nt == 0) return GS_OK;
  cudaStream_t s = stream ? (cudaStream_t)stream : k->stream;
  return predict_pass(k, nt, tx, ty, tz, tdrift, value, variance, lagrange, status, precision, s,
                      false);
}

int gs_kriging_predict_many(const gs_kriging* k, int64_t nt, const double* tx, const double* ty,
                            const double* tz, const double* tdrift, double* value,
                            double* variance, double* lagrange, uint8_t* status, int precision,
                            void* stream) {
  if (!k) return fail(GS_ERR_INVALID_PARAMETER, "null predictor");
  if (k->cfg.method == GS_EXTERNAL_DRIFT && !tdrift)
    return fail(GS_ERR_INVALID_PARAMETER, "external drift kriging requires predict_with_drift");
  if (k->cfg.method != GS_EXTERNAL_DRIFT && tdrift)
    return fail(GS_ERR_INVALID_PARAMETER, "predict_with_drift requires KrigingMethod::ExternalDrift");
  if (nt == 0) return GS_OK;
  cudaStream_t s = stream ? (cudaStream_t)stream : k->stream;
  const int dim = k->ps->dim;
  const int nv = k->nv;
  DevBuf dx, dy, dz, dd, dv, dvar, dlag, dst;
  GS_TRY(dx.alloc(nt * 8, s));
  GS_TRY(dy.alloc(nt * 8, s));
  if (dim == 3) GS_TRY(dz.alloc(nt * 8, s));
  if (tdrift) GS_TRY(dd.alloc(nt * nv * 8, s));
  GS_TRY(dv.alloc(nt * 8, s));
  GS_TRY(dvar.alloc(nt * 8, s));
  if (lagrange) GS_TRY(dlag.alloc(nt * 8, s));
  GS_TRY(dst.alloc(nt, s));
  GS_CUDA(cudaMemcpyAsync(dx.ptr, tx, nt * 8, cudaMemcpyHostToDevice, s));
  GS_CUDA(cudaMemcpyAsync(dy.ptr, ty, nt * 8, cudaMemcpyHostToDevice, s));
  if (dim == 3) GS_CUDA(cudaMemcpyAsync(dz.ptr, tz, nt * 8, cudaMemcpyHostToDevice, s));
  if (tdrift) GS_CUDA(cudaMemcpyAsync(dd.ptr, tdrift, nt * nv * 8, cudaMemcpyHostToDevice, s));
  GS_TRY(predict_device(k, nt, (double*)dx.ptr, (double*)dy.ptr, (double*)dz.ptr,
                        (double*)dd.ptr, (double*)dv.ptr, (double*)dvar.ptr,
                        lagrange ? (double*)dlag.ptr : nullptr, (uint8_t*)dst.ptr, precision, s));
  GS_CUDA(cudaMemcpyAsync(value, dv.ptr, nt * 8, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaMemcpyAsync(variance, dvar.ptr, nt * 8, cudaMemcpyDeviceToHost, s));
  if (lagrange) GS_CUDA(cudaMemcpyAsync(lagrange, dlag.ptr, nt * 8, cudaMemcpyDeviceToHost, s));
  if (status) GS_CUDA(cudaMemcpyAsync(status, dst.ptr, nt, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaStreamSynchronize(s));
  return GS_OK;
}

int gs_kriging_predict_grid(const gs_kriging* k, const double* bbox_min, const double* bbox_max,
                            const int64_t* ncell, double* value, double* variance,
                            uint8_t* status, int precision, void* stream) {
  if (!k) return fail(GS_ERR_INVALID_PARAMETER, "null predictor");
  if (k->cfg.method == GS_EXTERNAL_DRIFT)
    return fail(GS_ERR_INVALID_PARAMETER, "external drift kriging requires predict_with_drift");
  const int dim = k->ps->dim;
  double step[3] = {0, 0, 0};
  int64_t total = 1;
  for (int d = 0; d < dim; ++d) {
    if (ncell[d] == 0) return fail(GS_ERR_INVALID_PARAMETER, "grid must have at least one cell per axis");
    if (!(bbox_max[d] > bbox_min[d])) return fail(GS_ERR_INVALID_PARAMETER, "degenerate bbox");
    step[d] = (bbox_max[d] - bbox_min[d]) / (double)ncell[d];
    total *= ncell[d];
  }
  cudaStream_t s = stream ? (cudaStream_t)stream : k->stream;
  DevBuf dx, dy, dz, dv, dvar, dst;
  GS_TRY(dx.alloc(total * 8, s));
  GS_TRY(dy.alloc(total * 8, s));
  if (dim == 3) GS_TRY(dz.alloc(total * 8, s));
  GS_TRY(dv.alloc(total * 8, s));
  GS_TRY(dvar.alloc(total * 8, s));
  GS_TRY(dst.alloc(total, s));
  GS_TRY(grid_centers_launch(dim, bbox_min, step, ncell, (double*)dx.ptr, (double*)dy.ptr,
                             (double*)dz.ptr, s));
  GS_TRY(predict_device(k, total, (double*)dx.ptr, (double*)dy.ptr, (double*)dz.ptr, nullptr,
                        (double*)dv.ptr, (double*)dvar.ptr, nullptr, (uint8_t*)dst.ptr, precision, s));
  GS_CUDA(cudaMemcpyAsync(value, dv.ptr, total * 8, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaMemcpyAsync(variance, dvar.ptr, total * 8, cudaMemcpyDeviceToHost, s));
  if (status) GS_CUDA(cudaMemcpyAsync(status, dst.ptr, total, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaStreamSynchronize(s));
  return GS_OK;
}

// block_offsets (kriging.rs:815-838): an n[0] x n[1] grid of cell centres
// covering a block of `size`, centred on the origin, x fastest.
int gs_block_offsets(const double* size, const int64_t* ndisc, double* out) {
  if (!size || !ndisc || !out) return fail(GS_ERR_INVALID_PARAMETER, "null argument");
  if (ndisc[0] <= 0 || ndisc[1] <= 0)
    return fail(GS_ERR_INVALID_PARAMETER, "block discretization needs at least 1 point per axis");
  if (!(size[0] > 0.0) || !(size[1] > 0.0))
    return fail(GS_ERR_INVALID_PARAMETER, "block size must be positive");
  int64_t q = 0;
  for (int64_t iy = 0; iy < ndisc[1]; ++iy)
    for (int64_t ix = 0; ix < ndisc[0]; ++ix, ++q) {
      out[2 * q] = (((double)ix + 0.5) / (double)ndisc[0] - 0.5) * size[0];
      out[2 * q + 1] = (((double)iy + 0.5) / (double)ndisc[1] - 0.5) * size[1];
    }
  return GS_OK;
}

}  // extern "C"

namespace gs {

// predict_block's checks (kriging.rs:678-700), in its order.
static int check_block(const gs_kriging* k, int64_t noff) {
  if (k->cfg.method != GS_SIMPLE && k->cfg.method != GS_ORDINARY)
    return fail(GS_ERR_INVALID_PARAMETER, "block kriging supports simple and ordinary kriging only");
  if (has_power(k->model))
    return fail(GS_ERR_INVALID_PARAMETER,
                "block kriging with a Power model is not supported (needs a block-averaged "
                "semivariogram)");
  if (noff <= 0) return fail(GS_ERR_INVALID_PARAMETER, "block discretization needs at least one point");
  if (noff > (1 << 20)) return fail(GS_ERR_INVALID_PARAMETER, "block discretization too large");
  return GS_OK;
}

// Blocks centred at (cx, cy, cz) (device), offsets on the host: C(B,B) once,
// then one FP64 prediction pass with block right-hand sides.
static int block_pass(const gs_kriging* k, int64_t nb, const double* cx, const double* cy,
               const double* cz, const double* offsets, int64_t noff, double* value,
               double* variance, double* lagrange, uint8_t* status, cudaStream_t s) {
  const int dim = k->ps->dim;
  DevBuf doff, dcbb;
  GS_TRY(doff.alloc((size_t)noff * dim * 8, s));
  GS_TRY(dcbb.alloc(8, s));
  GS_CUDA(cudaMemcpyAsync(doff.ptr, offsets, (size_t)noff * dim * 8, cudaMemcpyHostToDevice, s));
  GS_TRY(block_cbb_launch(dim, k->dm, (const double*)doff.ptr, (int)noff, k->model.nugget,
                          (double*)dcbb.ptr, s));
  BlockSpec blk{(const double*)doff.ptr, (int)noff, (const double*)dcbb.ptr};
  return predict_pass(k, nb, cx, cy, cz, nullptr, value, variance, lagrange, status, GS_PREC_FP64,
                      s, true, nullptr, &blk);
}

}  // namespace gs

extern "C" {

// Kriging::predict_block (kriging.rs:674-779) for nb blocks sharing one
// discretisation (offsets: noff x dim, host); host buffers.  Per-block
// failures (no neighbours, singular) are NaN with their status.
int gs_kriging_predict_block(const gs_kriging* k, int64_t nb, const double* cx, const double* cy,
                             const double* cz, const double* offsets, int64_t noff, double* value,
                             double* variance, double* lagrange, uint8_t* status, void* stream) {
  if (!k) return fail(GS_ERR_INVALID_PARAMETER, "null predictor");
  GS_TRY(check_block(k, noff));
  if (!offsets) return fail(GS_ERR_INVALID_PARAMETER, "null offsets");
  if (nb == 0) return GS_OK;
  const int dim = k->ps->dim;
  if (!cx || !cy || (dim == 3 && !cz) || !value || !variance)
    return fail(GS_ERR_INVALID_PARAMETER, "null centre or output buffer");
  cudaStream_t s = stream ? (cudaStream_t)stream : k->stream;
  DevBuf dx, dy, dz, dv, dvar, dlag, dst;
  GS_TRY(dx.alloc(nb * 8, s));
  GS_TRY(dy.alloc(nb * 8, s));
  if (dim == 3) GS_TRY(dz.alloc(nb * 8, s));
  GS_TRY(dv.alloc(nb * 8, s));
  GS_TRY(dvar.alloc(nb * 8, s));
  if (lagrange) GS_TRY(dlag.alloc(nb * 8, s));
  GS_TRY(dst.alloc(nb, s));
  GS_CUDA(cudaMemcpyAsync(dx.ptr, cx, nb * 8, cudaMemcpyHostToDevice, s));
  GS_CUDA(cudaMemcpyAsync(dy.ptr, cy, nb * 8, cudaMemcpyHostToDevice, s));
  if (dim == 3) GS_CUDA(cudaMemcpyAsync(dz.ptr, cz, nb * 8, cudaMemcpyHostToDevice, s));
  GS_TRY(block_pass(k, nb, (double*)dx.ptr, (double*)dy.ptr, (double*)dz.ptr, offsets, noff,
                    (double*)dv.ptr, (double*)dvar.ptr, lagrange ? (double*)dlag.ptr : nullptr,
                    (uint8_t*)dst.ptr, s));
  GS_CUDA(cudaMemcpyAsync(value, dv.ptr, nb * 8, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaMemcpyAsync(variance, dvar.ptr, nb * 8, cudaMemcpyDeviceToHost, s));
  if (lagrange) GS_CUDA(cudaMemcpyAsync(lagrange, dlag.ptr, nb * 8, cudaMemcpyDeviceToHost, s));
  if (status) GS_CUDA(cudaMemcpyAsync(status, dst.ptr, nb, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaStreamSynchronize(s));
  return GS_OK;
}

// Kriging::predict_block_grid (kriging.rs:787-805), 2-D: blocks of
// block_size at every cell centre, discretised by block_offsets(block_size,
// discr).  A method or model predict_block rejects gives NaN at every cell
// (the reference's unwrap_or(NAN_ESTIMATE)) with status
// GS_ST_INVALID_PARAMETER.
int gs_kriging_predict_block_grid(const gs_kriging* k, const double* bbox_min,
                                  const double* bbox_max, const int64_t* ncell,
                                  const double* block_size, const int64_t* discr, double* value,
                                  double* variance, uint8_t* status, void* stream) {
  if (!k) return fail(GS_ERR_INVALID_PARAMETER, "null predictor");
  if (k->ps->dim != 2) return fail(GS_ERR_INVALID_PARAMETER, "block grids are 2-D");
  std::vector<double> off;
  if (discr && discr[0] > 0 && discr[1] > 0 && discr[0] * discr[1] <= (1 << 20))
    off.resize((size_t)(discr[0] * discr[1]) * 2);
  else if (discr && (discr[0] <= 0 || discr[1] <= 0))
    return fail(GS_ERR_INVALID_PARAMETER, "block discretization needs at least 1 point per axis");
  else
    return fail(GS_ERR_INVALID_PARAMETER, "block discretization too large");
  GS_TRY(gs_block_offsets(block_size, discr, off.data()));
  double step[3] = {0, 0, 0};
  int64_t total = 1;
  for (int d = 0; d < 2; ++d) {
    if (ncell[d] == 0) return fail(GS_ERR_INVALID_PARAMETER, "grid must have at least one cell per axis");
    if (!(bbox_max[d] > bbox_min[d])) return fail(GS_ERR_INVALID_PARAMETER, "degenerate bbox");
    step[d] = (bbox_max[d] - bbox_min[d]) / (double)ncell[d];
    total *= ncell[d];
  }
  if (check_block(k, (int64_t)off.size() / 2) != GS_OK) {
    for (int64_t i = 0; i < total; ++i) value[i] = variance[i] = NAN;
    if (status) std::memset(status, GS_ST_INVALID_PARAMETER, (size_t)total);
    return GS_OK;
  }
  cudaStream_t s = stream ? (cudaStream_t)stream : k->stream;
  DevBuf dx, dy, dv, dvar, dst;
  GS_TRY(dx.alloc(total * 8, s));
  GS_TRY(dy.alloc(total * 8, s));
  GS_TRY(dv.alloc(total * 8, s));
  GS_TRY(dvar.alloc(total * 8, s));
  GS_TRY(dst.alloc(total, s));
  GS_TRY(grid_centers_launch(2, bbox_min, step, ncell, (double*)dx.ptr, (double*)dy.ptr, nullptr, s));
  GS_TRY(block_pass(k, total, (double*)dx.ptr, (double*)dy.ptr, nullptr, off.data(),
                    (int64_t)off.size() / 2, (double*)dv.ptr, (double*)dvar.ptr, nullptr,
                    (uint8_t*)dst.ptr, s));
  GS_CUDA(cudaMemcpyAsync(value, dv.ptr, total * 8, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaMemcpyAsync(variance, dvar.ptr, total * 8, cudaMemcpyDeviceToHost, s));
  if (status) GS_CUDA(cudaMemcpyAsync(status, dst.ptr, total, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaStreamSynchronize(s));
  return GS_OK;
}

int gs_kriging_neighbors(const gs_kriging* k, int64_t nt, const double* tx, const double* ty,
                         const double* tz, int64_t kcap, int32_t* idx, int32_t* count,
                         void* stream) {
  if (!k) return fail(GS_ERR_INVALID_PARAMETER, "null predictor");
  if (nt == 0) return GS_OK;
  const gs_kcfg& c = k->cfg;
  const int dim = k->ps->dim;
  const int64_t n = k->ps->n;
  cudaStream_t s = stream ? (cudaStream_t)stream : k->stream;
  if (!k->use_tree) {
    for (int64_t t = 0; t < nt; ++t) {
      for (int64_t j = 0; j < kcap; ++j) idx[t * kcap + j] = j < n ? (int32_t)j : -1;
      if (count) count[t] = (int32_t)n;
    }
    return GS_OK;
  }
  SearchParams sp{};
  int kout;
  if (c.max_per_octant >= 0) {
    int per = (int)std::min<int64_t>(c.max_per_octant, n);
    sp.octant = 1;
    sp.k = per;
    kout = (1 << dim) * per;
    if (c.max_neighbors >= 0) kout = (int)std::min<int64_t>(kout, c.max_neighbors);
  } else if (c.max_neighbors >= 0) {
    sp.k = (int)std::min<int64_t>(c.max_neighbors, n);
    kout = sp.k;
  } else {
    sp.unbounded = 1;
    sp.k = (int)std::min<int64_t>(n, GS_MAX_SYSTEM);
    kout = sp.k;
  }
  sp.kout = kout;
  sp.has_radius = c.has_search_radius ? 1 : 0;
  sp.r2 = c.has_search_radius ? c.search_radius * c.search_radius : 0.0;
  DevBuf dx, dy, dz, dnb, dnbc;
  GS_TRY(dx.alloc(nt * 8, s));
  GS_TRY(dy.alloc(nt * 8, s));
  if (dim == 3) GS_TRY(dz.alloc(nt * 8, s));
  GS_TRY(dnb.alloc((size_t)nt * kout * 4, s));
  GS_TRY(dnbc.alloc(nt * 4, s));
  GS_CUDA(cudaMemcpyAsync(dx.ptr, tx, nt * 8, cudaMemcpyHostToDevice, s));
  GS_CUDA(cudaMemcpyAsync(dy.ptr, ty, nt * 8, cudaMemcpyHostToDevice, s));
  if (dim == 3) GS_CUDA(cudaMemcpyAsync(dz.ptr, tz, nt * 8, cudaMemcpyHostToDevice, s));
  GS_TRY(search_launch(k->grid, k->frame, sp, nt, (double*)dx.ptr, (double*)dy.ptr,
                       (double*)dz.ptr, (int32_t*)dnb.ptr, (int32_t*)dnbc.ptr, s));
  std::vector<int32_t> h((size_t)nt * kout), hc(nt);
  GS_CUDA(cudaMemcpyAsync(h.data(), dnb.ptr, (size_t)nt * kout * 4, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaMemcpyAsync(hc.data(), dnbc.ptr, nt * 4, cudaMemcpyDeviceToHost, s));
  GS_CUDA(cudaStreamSynchronize(s));
  for (int64_t t = 0; t < nt; ++t) {
    for (int64_t j = 0; j < kcap; ++j) idx[t * kcap + j] = j < kout ? h[t * kout + j] : -1;
    if (count) count[t] = hc[t];
  }
  return GS_OK;
}

void gs_rng_uniform(uint64_t seed, int64_t count, double* out) {
  Xoshiro r(seed);
  for (int64_t i = 0; i < count; ++i) out[i] = r.uniform();
}
void gs_rng_normal(uint64_t seed, int64_t count, double* out) {
  Xoshiro r(seed);
  for (int64_t i = 0; i < count; ++i) out[i] = r.normal();
}

}  // extern "C"
