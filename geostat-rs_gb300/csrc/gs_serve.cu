// gs_serve.cu -- a continuous-batching request loop over resident data sets.
//
// Data sets stay resident in device memory as built predictors (gs_kriging:
// points, bucket grid, model) and Vecchia plans.  Callers submit prediction
// and log-likelihood requests from any thread; executor threads, each with
// its own CUDA stream, take a pending request as soon as device memory admits
// it, coalesce every other pending request of the same data set and kind into
// the same launch (targets concatenated, likelihood candidates batched), run
// it, and scatter the results back.  Requests that arrive while others are on
// the device join the next batch an executor forms, so the device keeps
// working on mixed requests of very different sizes; batches of different
// executors overlap on their streams.
//
// Size-aware admission: predictions of at least kLargeTargets targets are
// large.  Executor 0 is the large lane: it serves large requests in arrival
// order, one batch at a time, and small ones when no large request waits.
// The other executors serve small requests only, in arrival order, so a small
// request never waits behind a large one.  (With one executor, it serves the
// oldest request of either size.)
//
// Admission by free device memory: a batch starts once its device bytes fit
// both the caller's budget and the device's current headroom (free memory
// plus what the stream-ordered pool holds unused), less a reserve.  A request
// that could never fit the budget is refused at submission; pending requests
// can be cancelled.
//
// A prediction's result does not depend on which requests it was batched
// with beyond the order of roundings (each target's system is solved on its
// own); a likelihood is computed per candidate in a fixed order and is
// bit-identical alone or in a batch.
#include <algorithm>
#include <chrono>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gs_common.cuh"
#include "gs_host.h"
#include "gs_internal.h"
#include "gs_kriging_handle.h"
#include "gs_vecchia.h"

namespace gs {
namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t id = 0;
  int kind = 0;  // 0: prediction, 1: log-likelihood
  int32_t dataset = 0;
  int64_t nt = 0;
  const double* tx = nullptr;
  const double* ty = nullptr;
  const double* tz = nullptr;
  double* value = nullptr;
  double* variance = nullptr;
  uint8_t* status = nullptr;
  gs_model model{};
  double* loglik = nullptr;
  int32_t* lstatus = nullptr;
  int64_t bytes = 0;
  Clock::time_point submitted, finished;
  int rc = GS_OK;
  std::string err;  // the failing call's message (worker thread)
  bool done = false;
  bool large = false;
};

struct Dataset {
  const gs_kriging* k = nullptr;
  const gs_vecchia_plan* plan = nullptr;
};

// Largest coalesced batches: targets per prediction launch, candidates per
// likelihood launch.
constexpr int64_t kMaxBatchTargets = (int64_t)1 << 22;
constexpr int64_t kMaxBatchCandidates = 64;
// Predictions of at least this many targets go to the large lane.
constexpr int64_t kLargeTargets = (int64_t)1 << 17;
// Device memory kept free of admitted batches (other allocations of the
// process, the driver's own needs).
constexpr int64_t kHeadroomReserve = (int64_t)512 << 20;

}  // namespace
}  // namespace gs

struct gs_server {
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<gs::Request*> pending_small, pending_large;
  std::unordered_map<int64_t, std::unique_ptr<gs::Request>> requests;
  std::vector<gs::Dataset> datasets;
  int64_t budget = 0;
  int64_t in_use = 0;
  int64_t next_id = 1;
  int64_t batches = 0;
  std::atomic<int> precision{GS_PREC_MIXED};
  bool stop = false;
  int device = 0;
  int executors = 1;
  std::vector<std::thread> workers;
  std::vector<double> latencies_ms;
  int64_t cancelled = 0;
};

namespace gs {
namespace {

// Device bytes a request needs while it runs (inputs, outputs, neighbour
// lists, flags; likelihood terms and flags per point).
int64_t request_bytes(const gs_server* S, const Request& r) {
  if (r.kind == 0) {
    const gs_kriging* k = S->datasets[r.dataset].k;
    const int64_t kout = k->cfg.max_neighbors > 0 ? k->cfg.max_neighbors : GS_MAX_SYSTEM;
    // + the FP64 re-solve's slot scratch (up to 40.5 MB)
    return r.nt * (3 * 8 + 8 + 8 + 8 + 1 + 4 * kout + 4 + 1 + 8) + (1 << 20) +
           std::min<int64_t>(r.nt * 16640, (int64_t)sm_count() * 16 * 16640);
  }
  return vecchia_plan_points(S->datasets[r.dataset].plan) * 9 + (1 << 20);
}

int run_predictions(gs_server* S, const std::vector<Request*>& batch, cudaStream_t s) {
  const gs_kriging* k = S->datasets[batch[0]->dataset].k;
  const int dim = k->ps->dim;
  int64_t nt = 0;
  for (Request* r : batch) nt += r->nt;
  DevBuf x, y, z, v, var, st;
  GS_TRY(x.alloc(nt * 8, s));
  GS_TRY(y.alloc(nt * 8, s));
  if (dim == 3) GS_TRY(z.alloc(nt * 8, s));
  GS_TRY(v.alloc(nt * 8, s));
  GS_TRY(var.alloc(nt * 8, s));
  GS_TRY(st.alloc(nt, s));
  int64_t off = 0;
  for (Request* r : batch) {
    GS_CUDA(cudaMemcpyAsync((double*)x.ptr + off, r->tx, r->nt * 8, cudaMemcpyHostToDevice, s));
    GS_CUDA(cudaMemcpyAsync((double*)y.ptr + off, r->ty, r->nt * 8, cudaMemcpyHostToDevice, s));
    if (dim == 3)
      GS_CUDA(cudaMemcpyAsync((double*)z.ptr + off, r->tz, r->nt * 8, cudaMemcpyHostToDevice, s));
    off += r->nt;
  }
  GS_TRY(predict_device(k, nt, (double*)x.ptr, (double*)y.ptr, (double*)z.ptr, nullptr,
                        (double*)v.ptr, (double*)var.ptr, nullptr, (uint8_t*)st.ptr,
                        S->precision.load(), s));
  off = 0;
  for (Request* r : batch) {
    GS_CUDA(cudaMemcpyAsync(r->value, (double*)v.ptr + off, r->nt * 8, cudaMemcpyDeviceToHost, s));
    GS_CUDA(cudaMemcpyAsync(r->variance, (double*)var.ptr + off, r->nt * 8, cudaMemcpyDeviceToHost,
                            s));
    if (r->status)
      GS_CUDA(cudaMemcpyAsync(r->status, (uint8_t*)st.ptr + off, r->nt, cudaMemcpyDeviceToHost, s));
    off += r->nt;
  }
  GS_CUDA(cudaStreamSynchronize(s));
  return GS_OK;
}

int run_logliks(gs_server* S, const std::vector<Request*>& batch, cudaStream_t s) {
  const gs_vecchia_plan* plan = S->datasets[batch[0]->dataset].plan;
  std::vector<gs_model> models;
  for (Request* r : batch) models.push_back(r->model);
  std::vector<double> ll(models.size());
  std::vector<int32_t> st(models.size());
  GS_TRY(vecchia_eval(plan, (int64_t)models.size(), models.data(), ll.data(), st.data(),
                      S->precision.load(), s));
  for (size_t i = 0; i < batch.size(); ++i) {
    *batch[i]->loglik = ll[i];
    if (batch[i]->lstatus) *batch[i]->lstatus = st[i];
  }
  return GS_OK;
}

// Device memory a new batch may still take: the device's free memory plus
// what the stream-ordered pool holds unused, less the reserve (read outside
// the server lock).
int64_t device_headroom() {
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return INT64_MAX;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaMemPool_t pool;
  uint64_t reserved = 0, used = 0;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved);
    cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used);
  }
  const int64_t pooled = reserved > used ? (int64_t)(reserved - used) : 0;
  return (int64_t)free_b + pooled - kHeadroomReserve;
}

// The queue executor `lane` serves next (null: nothing it may take).
std::deque<Request*>* pick_queue(gs_server* S, int lane) {
  if (S->executors == 1) {
    if (S->pending_small.empty()) return S->pending_large.empty() ? nullptr : &S->pending_large;
    if (S->pending_large.empty()) return &S->pending_small;
    return S->pending_large.front()->id < S->pending_small.front()->id ? &S->pending_large
                                                                       : &S->pending_small;
  }
  if (lane == 0 && !S->pending_large.empty()) return &S->pending_large;
  return S->pending_small.empty() ? nullptr : &S->pending_small;
}

void worker_loop(gs_server* S, int lane) {
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) s = nullptr;
  int64_t headroom = device_headroom();
  for (;;) {
    std::vector<Request*> batch;
    int64_t bytes = 0;
    {
      std::unique_lock<std::mutex> lock(S->mu);
      std::deque<Request*>* q = nullptr;
      S->cv_work.wait(lock, [&] {
        if (S->stop) return true;
        q = pick_queue(S, lane);
        if (!q) return false;
        // admission by memory: the batch's bytes within the budget and
        // within the device's headroom at the last reading (a request alone
        // on an idle server always fits: submission refused larger ones)
        const int64_t need = q->front()->bytes;
        return S->in_use == 0 || (S->in_use + need <= S->budget && need <= headroom);
      });
      if (S->stop && S->pending_small.empty() && S->pending_large.empty()) break;
      if (!q) continue;
      Request* head = q->front();
      q->pop_front();
      batch.push_back(head);
      bytes = head->bytes;
      int64_t units = head->kind == 0 ? head->nt : 1;
      const int64_t cap = head->kind == 0 ? kMaxBatchTargets : kMaxBatchCandidates;
      for (auto it = q->begin(); it != q->end();) {
        Request* r = *it;
        const int64_t u = r->kind == 0 ? r->nt : 1;
        if (r->dataset == head->dataset && r->kind == head->kind && units + u <= cap &&
            S->in_use + bytes + r->bytes <= S->budget && bytes + r->bytes <= headroom) {
          batch.push_back(r);
          bytes += r->bytes;
          units += u;
          it = q->erase(it);
        } else {
          ++it;
        }
      }
      S->in_use += bytes;
      ++S->batches;
    }
    int rc = s ? (batch[0]->kind == 0 ? run_predictions(S, batch, s) : run_logliks(S, batch, s))
               : fail(GS_ERR_CUDA, "stream creation failed");
    const std::string err = rc ? std::string(last_error()) : std::string();
    headroom = device_headroom();
    {
      std::lock_guard<std::mutex> lock(S->mu);
      S->in_use -= bytes;
      const auto now = Clock::now();
      for (Request* r : batch) {
        r->rc = rc;
        r->err = err;
        r->done = true;
        r->finished = now;
        S->latencies_ms.push_back(
            std::chrono::duration<double, std::milli>(r->finished - r->submitted).count());
      }
    }
    S->cv_done.notify_all();
    S->cv_work.notify_all();
  }
  if (s) cudaStreamDestroy(s);
}

int submit(gs_server* S, std::unique_ptr<Request> r, int64_t* request_id) {
  if (r->dataset < 0 || r->dataset >= (int32_t)S->datasets.size())
    return fail(GS_ERR_INVALID_PARAMETER, "unknown data set");
  const Dataset& d = S->datasets[r->dataset];
  if ((r->kind == 0 && !d.k) || (r->kind == 1 && !d.plan))
    return fail(GS_ERR_INVALID_PARAMETER, "the data set does not serve this kind of request");
  r->bytes = request_bytes(S, *r);
  if (r->bytes > S->budget)
    return fail(GS_ERR_OUT_OF_MEMORY,
                "request needs " + std::to_string(r->bytes) + " bytes of device memory, more than "
                "the server's budget of " + std::to_string(S->budget) + "; split it");
  r->large = r->kind == 0 && r->nt >= kLargeTargets;
  r->submitted = Clock::now();
  {
    std::lock_guard<std::mutex> lock(S->mu);
    r->id = S->next_id++;
    *request_id = r->id;
    (r->large ? S->pending_large : S->pending_small).push_back(r.get());
    S->requests[r->id] = std::move(r);
  }
  S->cv_work.notify_all();
  return GS_OK;
}

}  // namespace
}  // namespace gs

using namespace gs;

extern "C" {

int gs_server_create(int64_t mem_budget_bytes, int32_t executors, gs_server** out) {
  if (!out) return fail(GS_ERR_INVALID_PARAMETER, "null output handle");
  *out = nullptr;
  if (mem_budget_bytes <= 0 || executors <= 0 || executors > 16)
    return fail(GS_ERR_INVALID_PARAMETER, "memory budget must be positive and executors in 1..16");
  GS_TRY(ensure_device());
  auto* S = new gs_server();
  S->budget = mem_budget_bytes;
  S->executors = executors;
  int dev = 0;
  cudaGetDevice(&dev);
  S->device = dev;
  for (int i = 0; i < executors; ++i)
    S->workers.emplace_back([S, dev, i] {
      cudaSetDevice(dev);
      worker_loop(S, i);
    });
  *out = S;
  return GS_OK;
}

int gs_server_add_kriging(gs_server* S, const gs_kriging* k, int32_t* dataset) {
  if (!S || !k || !dataset) return fail(GS_ERR_INVALID_PARAMETER, "null argument");
  if (k->cfg.method == GS_EXTERNAL_DRIFT)
    return fail(GS_ERR_INVALID_PARAMETER, "external-drift predictors need per-target covariates");
  std::lock_guard<std::mutex> lock(S->mu);
  Dataset d;
  d.k = k;
  S->datasets.push_back(d);
  *dataset = (int32_t)S->datasets.size() - 1;
  return GS_OK;
}

int gs_server_add_vecchia(gs_server* S, const gs_vecchia_plan* plan, int32_t* dataset) {
  if (!S || !plan || !dataset) return fail(GS_ERR_INVALID_PARAMETER, "null argument");
  std::lock_guard<std::mutex> lock(S->mu);
  Dataset d;
  d.plan = plan;
  S->datasets.push_back(d);
  *dataset = (int32_t)S->datasets.size() - 1;
  return GS_OK;
}

int gs_server_submit_predict(gs_server* S, int32_t dataset, int64_t nt, const double* tx,
                             const double* ty, const double* tz, double* value, double* variance,
                             uint8_t* status, int64_t* request_id) {
  NvtxRange nvtx_range("gs.server_submit_predict");
  if (!S || !request_id) return fail(GS_ERR_INVALID_PARAMETER, "null argument");
  if (nt <= 0 || !tx || !ty || !value || !variance)
    return fail(GS_ERR_INVALID_PARAMETER, "a prediction request needs targets and outputs");
  auto r = std::make_unique<Request>();
  r->kind = 0;
  r->dataset = dataset;
  r->nt = nt;
  r->tx = tx;
  r->ty = ty;
  r->tz = tz;
  r->value = value;
  r->variance = variance;
  r->status = status;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    if (dataset >= 0 && dataset < (int32_t)S->datasets.size() && S->datasets[dataset].k &&
        S->datasets[dataset].k->ps->dim == 3 && !tz)
      return fail(GS_ERR_INVALID_PARAMETER, "3-D data set: tz is required");
  }
  return submit(S, std::move(r), request_id);
}

int gs_server_submit_loglik(gs_server* S, int32_t dataset, const gs_model* model, double* loglik,
                            int32_t* status, int64_t* request_id) {
  NvtxRange nvtx_range("gs.server_submit_loglik");
  if (!S || !model || !loglik || !request_id) return fail(GS_ERR_INVALID_PARAMETER, "null argument");
  auto r = std::make_unique<Request>();
  r->kind = 1;
  r->dataset = dataset;
  r->model = *model;
  r->loglik = loglik;
  r->lstatus = status;
  return submit(S, std::move(r), request_id);
}

int gs_server_set_precision(gs_server* s, int precision) {
  if (!s) return gs::fail(GS_ERR_INVALID_PARAMETER, "null server");
  if (precision != GS_PREC_MIXED && precision != GS_PREC_FP64)
    return gs::fail(GS_ERR_INVALID_PARAMETER, "unknown precision");
  s->precision.store(precision);
  return GS_OK;
}

int gs_server_cancel(gs_server* S, int64_t request_id) {
  if (!S) return fail(GS_ERR_INVALID_PARAMETER, "null server");
  {
    std::lock_guard<std::mutex> lock(S->mu);
    auto it = S->requests.find(request_id);
    if (it == S->requests.end()) return fail(GS_ERR_INVALID_PARAMETER, "unknown request");
    Request* r = it->second.get();
    bool found = false;
    for (auto* q : {&S->pending_small, &S->pending_large}) {
      auto pos = std::find(q->begin(), q->end(), r);
      if (pos != q->end()) {
        q->erase(pos);
        found = true;
        break;
      }
    }
    if (!found)
      return fail(GS_ERR_INVALID_PARAMETER,
                  r->done ? "request already finished" : "request already running");
    r->rc = GS_ERR_CANCELLED;
    r->err = "cancelled before it started";
    r->done = true;
    r->finished = Clock::now();
    ++S->cancelled;
  }
  S->cv_done.notify_all();
  S->cv_work.notify_all();
  return GS_OK;
}

int gs_server_wait(gs_server* S, int64_t request_id, double* latency_ms) {
  if (!S) return fail(GS_ERR_INVALID_PARAMETER, "null server");
  std::unique_lock<std::mutex> lock(S->mu);
  auto it = S->requests.find(request_id);
  if (it == S->requests.end()) return fail(GS_ERR_INVALID_PARAMETER, "unknown request");
  Request* r = it->second.get();
  S->cv_done.wait(lock, [&] { return r->done; });
  if (latency_ms)
    *latency_ms = std::chrono::duration<double, std::milli>(r->finished - r->submitted).count();
  const int rc = r->rc;
  const std::string err = r->err;
  S->requests.erase(it);
  if (rc) return fail(rc, "request failed: " + err);
  return GS_OK;
}

int gs_server_stats(gs_server* S, double* p50_ms, double* p99_ms, int64_t* completed,
                    int64_t* batches) {
  if (!S) return fail(GS_ERR_INVALID_PARAMETER, "null server");
  std::lock_guard<std::mutex> lock(S->mu);
  std::vector<double> l = S->latencies_ms;
  if (completed) *completed = (int64_t)l.size();
  if (batches) *batches = S->batches;
  auto pct = [&](double q) {
    if (l.empty()) return 0.0;
    const size_t i = std::min(l.size() - 1, (size_t)(q * (double)(l.size() - 1) + 0.5));
    std::nth_element(l.begin(), l.begin() + i, l.end());
    return l[i];
  };
  if (p50_ms) *p50_ms = pct(0.50);
  if (p99_ms) *p99_ms = pct(0.99);
  return GS_OK;
}

void gs_server_destroy(gs_server* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  for (auto& t : S->workers) t.join();
  delete S;
}

}  // extern "C"
