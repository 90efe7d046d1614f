// gs_probe.cu -- measurement helpers for the benchmark and the tests (not part
// of the drop-in library): CUDA-core FMA throughput (the roofline denominator
// of the per-system kernels, which run on the FP32 pipe with a little FP64)
// and the FP64 re-solve kernels' table-driven exp(-x) for accuracy checks.
#include <algorithm>
#include <atomic>

#include "gs_common.cuh"
#include "gs_internal.h"
#include "gs_workload.h"

namespace gs {

namespace {

// Eight independent FMA chains per thread; the result is stored so the
// chains cannot be removed.
template <class T>
__global__ void fma_probe(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// The same with packed FP32x2 FMAs (two lanes per instruction).
__global__ void fma2_probe(float2* out, int iters, float2 a, float2 b) {
  const float s = (float)threadIdx.x;
  float2 x0 = make_float2(s, s + 0.5f), x1 = make_float2(s + 1.0f, s + 1.5f);
  float2 x2 = make_float2(s + 2.0f, s + 2.5f), x3 = make_float2(s + 3.0f, s + 3.5f);
  float2 x4 = make_float2(s + 4.0f, s + 4.5f), x5 = make_float2(s + 5.0f, s + 5.5f);
  float2 x6 = make_float2(s + 6.0f, s + 6.5f), x7 = make_float2(s + 7.0f, s + 7.5f);
  for (int i = 0; i < iters; ++i) {
    x0 = __ffma2_rn(x0, a, b); x1 = __ffma2_rn(x1, a, b); x2 = __ffma2_rn(x2, a, b);
    x3 = __ffma2_rn(x3, a, b); x4 = __ffma2_rn(x4, a, b); x5 = __ffma2_rn(x5, a, b);
    x6 = __ffma2_rn(x6, a, b); x7 = __ffma2_rn(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] =
      make_float2(x0.x + x1.x + x2.x + x3.x + x4.x + x5.x + x6.x + x7.x,
                  x0.y + x1.y + x2.y + x3.y + x4.y + x5.y + x6.y + x7.y);
}

template <class T>
void launch_probe(T* out, int blocks, int threads, int iters) {
  fma_probe<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
}
template <>
void launch_probe<float2>(float2* out, int blocks, int threads, int iters) {
  fma2_probe<<<blocks, threads>>>(out, iters, make_float2(0.999999f, 0.999999f),
                                  make_float2(1e-7f, 1e-7f));
}

template <class T>
int probe(double* tflops, int iters, int lanes) {
  const int threads = 256, blocks = sm_count() * 8;
  T* out = nullptr;
  GS_CUDA(cudaMalloc(&out, sizeof(T) * threads * blocks));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0);
    launch_probe<T>(out, blocks, threads, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0) best = std::min(best, ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaError_t err = cudaGetLastError();
  cudaFree(out);
  if (err != cudaSuccess) return cuda_fail(err, "fma probe", __FILE__, __LINE__);
  const double flops = 2.0 * 8.0 * lanes * (double)iters * threads * blocks;
  *tflops = flops / (best * 1e-3) / 1e12;
  return GS_OK;
}

__global__ void expneg_probe(int64_t n, const double* x, double* out, Exp64Table et) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = expneg_fp64(x[i], et);
}

}  // namespace
}  // namespace gs

extern "C" int gs_probe_expneg(int64_t n, const double* x, double* out) {
  if (n < 0 || (n > 0 && (!x || !out))) return gs::fail(GS_ERR_INVALID_PARAMETER, "bad arguments");
  if (n == 0) return GS_OK;
  GS_TRY(gs::ensure_device());
  gs::Exp64Table et;
  gs::exp64_table_host(&et);
  gs::DevBuf dx, dout;
  GS_TRY(dx.alloc((size_t)n * 8, nullptr));
  GS_TRY(dout.alloc((size_t)n * 8, nullptr));
  GS_CUDA(cudaMemcpy(dx.ptr, x, (size_t)n * 8, cudaMemcpyHostToDevice));
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)gs::sm_count() * 8);
  gs::expneg_probe<<<blocks, 256>>>(n, (const double*)dx.ptr, (double*)dout.ptr, et);
  GS_CUDA(cudaGetLastError());
  GS_CUDA(cudaMemcpy(out, dout.ptr, (size_t)n * 8, cudaMemcpyDeviceToHost));
  return GS_OK;
}

extern "C" int gs_probe_fma_tflops(int precision, double* tflops) {
  GS_TRY(gs::ensure_device());
  if (precision == GS_PREC_FP64) return gs::probe<double>(tflops, 1 << 13, 1);
  if (precision == 2) return gs::probe<float2>(tflops, 1 << 16, 2);
  return gs::probe<float>(tflops, 1 << 16, 1);
}

