// gs_internal.h -- small host helpers shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stddef.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace gs {

// Records `msg` as this thread's last error (gs_last_error) and returns code.
int fail(int code, const std::string& msg);

// Counts kernels this library launched (reported by gs_launch_count).
void count_launch(int n);

// Streaming multiprocessors of the current device, queried once per device
// (grid caps and scratch sizes scale with it).
int sm_count();

// cudaMalloc that the library's device-allocation counter sees
// (gs_debug_device_allocations); DevBuf::alloc counts its allocations too.
cudaError_t dev_malloc(void** p, size_t bytes);

// Initialises the device (and keeps the stream-ordered memory pool from
// returning memory to the driver between calls).
int ensure_device();

// Records the phase timings (ms: search, mixed solve, FP64 re-solve, whole
// call) and the number of FP64 re-solved systems of this thread's last call.
void set_last_timings(const double* ms4, int64_t fallbacks);

// Allows launches of `func` with `bytes` of dynamic shared memory on the
// current device.  The per-function limit is process-wide state, so it is
// only ever raised (under a lock): a thread launching with a smaller size
// can never invalidate another thread's larger launch.
int allow_dynamic_smem(const void* func, size_t bytes);

// NVTX range over a scope of host code (visible in Nsight timelines; costs a
// few nanoseconds when no tool is attached).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// Stream-ordered device allocation released at scope exit.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  int alloc(size_t b, cudaStream_t s);
  void release();
  ~DevBuf();
};

}  // namespace gs

// Device-resident point set behind the opaque gs_pointset handle.
struct gs_pointset {
  int dim = 2;
  int64_t n = 0;
  std::vector<double> host;  // n x dim, row-major
  std::vector<double> values;
  double* d_x = nullptr;
  double* d_y = nullptr;
  double* d_z = nullptr;
  double* d_v = nullptr;
  void* d_cdf = nullptr;  // gs::df[dim][n]: coordinates as double-float, axis-major
  void* d_vdf = nullptr;  // gs::df[n]: values as double-float
  bool has_dup = false;
  int64_t dup_i = 0, dup_j = 0;
  ~gs_pointset();
};
