// gs_noalloc.cu -- FP64 kriging prediction that allocates no device memory.
//
// Who needs it: callers that may not allocate device memory while they
// predict.  A service that reserves all of its device memory once at start-up
// and must never grow afterwards; a host application that runs its own
// allocator over the whole device and gives this library no share of it; a
// latency-bound loop that cannot afford the implicit synchronisation an
// allocation may bring.  The generic entry points allocate neighbour lists,
// flags and FP64 scratch from the stream-ordered pool on every call, which
// these callers cannot accept.
//
// How: the neighbour lists, neighbour counts and the per-thread FP64 scratch
// of the plain FP64 solve (krige_fp64_kernel) live in one statically sized
// device array of this file, g_noalloc_scratch.  Its address is looked up once
// per device (cudaGetSymbolAddress, with that device current) and then passed
// to the kernels as an ordinary pointer.  A call therefore allocates nothing;
// the first call on a device does that set-up (which also makes the driver
// load this file's device code) and should come before any section in which
// the caller cannot afford set-up work.  A call runs on the device the
// predictor was built on: it makes that device current for its duration and
// restores the caller's current device afterwards.
//
// Limits: at most GS_NOALLOC_MAX_TARGETS targets per call; the FP64 scratch
// gets what the neighbour lists leave of GS_NOALLOC_SCRATCH_BYTES, so larger
// systems run on fewer threads (never fewer than needed for correctness).
//
// Sharing: every call on one device uses the same array.  Calls ordered on one
// stream are safe; calls whose work can overlap in time (different streams, or
// host threads that do not order their calls) race on the array and their
// results are undefined.  Each device has its own copy of the array.
//
// Nothing in the array needs to start at zero: the search writes every
// neighbour slot and count of the call's targets before the solve reads them,
// and every system initialises its own scratch slab before use.
#include <algorithm>
#include <mutex>
#include <string>

#include "gs_common.cuh"
#include "gs_internal.h"
#include "gs_kriging_handle.h"
#include "gs_krige.cuh"
#include "gs_search.cuh"

namespace gs {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[GS_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};

// Address of device dev's copy of g_noalloc_scratch (set up on first use;
// dev must be the current device).
int noalloc_scratch(int dev, void** out) {
  if (dev < 0 || dev >= kMaxDevices)
    return fail(GS_ERR_INVALID_PARAMETER, "device ordinal beyond the allocation-free path's table");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(GS_ERR_CUDA, std::string("allocation-free scratch set-up failed: ") +
                                   cudaGetErrorString(e));
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return GS_OK;
}

// Makes `dev` the calling thread's current device for one call and puts the
// previous one back afterwards.
struct DeviceGuard {
  int prev = -1;
  int enter(int dev) {
    GS_CUDA(cudaGetDevice(&prev));
    if (prev != dev) GS_CUDA(cudaSetDevice(dev));
    return GS_OK;
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

// Global neighbourhood: every data point is a neighbour of every target.
__global__ void noalloc_all_rows(int64_t nt, int n, int32_t* nb, int32_t* nbc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nt * n;
       i += (int64_t)gridDim.x * blockDim.x) {
    nb[i] = (int32_t)(i % n);
    if (i % n == 0) nbc[i / n] = n;
  }
}

// Neighbourhood geometry of a predictor (the same rules as the generic path:
// global, octant, k nearest or radius-only).
int noalloc_geometry(const gs_kriging* k, SearchParams* sp, int* kout) {
  const gs_kcfg& c = k->cfg;
  const int64_t n = k->ps->n;
  const int dim = k->ps->dim;
  const int p = k->p;
  *sp = SearchParams{};
  if (!k->use_tree) {
    if (n + p > GS_MAX_SYSTEM)
      return fail(GS_ERR_INVALID_PARAMETER,
                  "global neighbourhood of " + std::to_string(n) +
                      " points exceeds the CUDA path's system limit; set max_neighbors");
    *kout = (int)n;
  } else if (c.max_per_octant >= 0) {
    const int per = (int)std::min<int64_t>(c.max_per_octant, n);
    sp->octant = 1;
    sp->k = per;
    *kout = (1 << dim) * per;
    if (c.max_neighbors >= 0) *kout = (int)std::min<int64_t>(*kout, c.max_neighbors);
  } else if (c.max_neighbors >= 0) {
    sp->k = (int)std::min<int64_t>(c.max_neighbors, n);
    *kout = sp->k;
  } else {
    sp->unbounded = 1;
    sp->k = (int)std::min<int64_t>(n, GS_MAX_SYSTEM - p);
    *kout = sp->k;
  }
  if (*kout + p > GS_MAX_SYSTEM)
    return fail(GS_ERR_INVALID_PARAMETER, "neighbourhood plus drift terms exceed " +
                                              std::to_string(GS_MAX_SYSTEM) + " on the CUDA path");
  sp->kout = *kout;
  sp->has_radius = c.has_search_radius ? 1 : 0;
  sp->r2 = c.has_search_radius ? c.search_radius * c.search_radius : 0.0;
  return GS_OK;
}

}  // namespace
}  // namespace gs

using namespace gs;

extern "C" int gs_kriging_predict_fp64_noalloc(const gs_kriging* k, int64_t nt, const double* tx,
                                               const double* ty, const double* tz,
                                               const double* tdrift, double* value,
                                               double* variance, double* lagrange,
                                               uint8_t* status, void* stream) {
  if (!k) return fail(GS_ERR_INVALID_PARAMETER, "null predictor");
  if (nt < 0) return fail(GS_ERR_INVALID_PARAMETER, "negative target count");
  if (nt > GS_NOALLOC_MAX_TARGETS)
    return fail(GS_ERR_INVALID_PARAMETER,
                "allocation-free prediction takes at most " +
                    std::to_string(GS_NOALLOC_MAX_TARGETS) + " targets per call (got " +
                    std::to_string(nt) + "); split the batch");
  if (k->cfg.method == GS_EXTERNAL_DRIFT && !tdrift)
    return fail(GS_ERR_INVALID_PARAMETER, "external drift kriging requires predict_with_drift");
  if (k->cfg.method != GS_EXTERNAL_DRIFT && tdrift)
    return fail(GS_ERR_INVALID_PARAMETER, "predict_with_drift requires KrigingMethod::ExternalDrift");
  cudaStream_t s = stream ? (cudaStream_t)stream : k->stream;
  // the predictor's device: its data, its stream and its copy of the array
  DeviceGuard guard;
  GS_TRY(guard.enter(k->device));
  const gs_pointset* ps = k->ps;
  const int dim = ps->dim;
  SearchParams sp;
  int kout = 0;
  GS_TRY(noalloc_geometry(k, &sp, &kout));
  void* base = nullptr;
  GS_TRY(noalloc_scratch(k->device, &base));
  if (nt == 0) return GS_OK;
  // carve the array: neighbour lists, counts, then the FP64 slabs
  const int nmax = kout + k->p;
  const size_t nb_bytes = ((size_t)nt * kout * 4 + 255) & ~(size_t)255;
  const size_t nbc_bytes = ((size_t)nt * 4 + 255) & ~(size_t)255;
  const size_t per_thread = (size_t)fp64_scratch_doubles(nmax, 1) * 8;
  if (nb_bytes + nbc_bytes + per_thread > (size_t)GS_NOALLOC_SCRATCH_BYTES)
    return fail(GS_ERR_INVALID_PARAMETER,
                "neighbourhood of " + std::to_string(kout) + " points for " + std::to_string(nt) +
                    " targets does not fit the " + std::to_string(GS_NOALLOC_SCRATCH_BYTES) +
                    "-byte allocation-free scratch; split the batch");
  unsigned char* b = (unsigned char*)base;
  int32_t* dnb = (int32_t*)b;
  int32_t* dnbc = (int32_t*)(b + nb_bytes);
  double* slab = (double*)(b + nb_bytes + nbc_bytes);
  const int64_t threads =
      (int64_t)(((size_t)GS_NOALLOC_SCRATCH_BYTES - nb_bytes - nbc_bytes) / per_thread);

  if (k->use_tree) {
    GS_TRY(search_launch(k->grid, k->frame, sp, nt, tx, ty, dim == 3 ? tz : nullptr, dnb, dnbc, s));
  } else {
    const int64_t cap = (int64_t)sm_count() * 64;
    noalloc_all_rows<<<(int)std::min<int64_t>((nt * kout + 255) / 256, cap), 256, 0, s>>>(
        nt, kout, dnb, dnbc);
    GS_CUDA(cudaGetLastError());
    count_launch(1);
  }
  // the predictor's arguments as the generic path builds them, then this call's
  KrigeArgs a = base_args(k);
  a.kout = kout;
  a.nmax = nmax;
  a.tx = tx;
  a.ty = ty;
  a.tz = dim == 3 ? tz : nullptr;
  a.tdrift = tdrift;
  a.nb = dnb;
  a.nbc = dnbc;
  a.out_v = value;
  a.out_var = variance;
  a.out_lag = lagrange;
  a.out_st = status;
  a.tlist = nullptr;
  a.ntl = nt;
  return krige_fp64_launch(a, k->dm, slab, threads, s);
}
