// gs_synth.cu -- seeded synthetic Gaussian fields for the benchmark and the
// tests (not part of the drop-in library).
//
// A random-Fourier-feature field (Rahimi & Recht 2007): for each structure,
// sqrt(2 sill / F) * sum_f cos(w_f . (R x) + phi_f) with w_f drawn from the
// structure's spectral density (Matern nu = 1/2, 3/2, 5/2: a multivariate
// Student-t with 2 nu degrees of freedom scaled by sqrt(2 nu)/range;
// Gaussian: N(0, 2/range^2); spherical: the exponential density at the same
// practical range), plus iid N(0, nugget) noise.  Frequencies, phases and
// noise come from the xoshiro256++ stream of crates/geostat-core/src/rng.rs.
#include <cmath>
#include <vector>

#include "gs_common.cuh"
#include "gs_host.h"
#include "gs_internal.h"
#include "gs_workload.h"

namespace gs {
namespace {

__global__ void rff_kernel(int dim, int64_t n, const double* x, const double* y, const double* z,
                           int nf, const double* w, const double* phi, double amp, double* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double p0 = x[i], p1 = y[i], p2 = dim == 3 ? z[i] : 0.0;
    double acc = 0.0;
    for (int f = 0; f < nf; ++f) {
      double ph = w[f * 3] * p0 + w[f * 3 + 1] * p1 + w[f * 3 + 2] * p2 + phi[f];
      // reduce the phase in FP64, evaluate the cosine in FP32
      double r = ph - 6.283185307179586 * rint(ph * 0.15915494309189535);
      acc += (double)cosf((float)r);
    }
    out[i] += amp * acc;
  }
}

}  // namespace
}  // namespace gs

using namespace gs;

extern "C" int gs_synth_rff_field(int dim, int64_t n, const double* x, const double* y,
                                  const double* z, const gs_model* model, int64_t n_features,
                                  uint64_t seed, double* out) {
  if (dim != 2 && dim != 3) return fail(GS_ERR_DIMENSION_MISMATCH, "dim must be 2 or 3");
  GS_TRY(validate_model(*model));
  GS_TRY(ensure_device());
  Xoshiro rng(seed);
  std::vector<double> host(n, 0.0);
  if (model->nugget > 0.0) {
    double sd = std::sqrt(model->nugget);
    for (int64_t i = 0; i < n; ++i) host[i] = sd * rng.normal();
  }
  double *dx = nullptr, *dy = nullptr, *dz = nullptr, *dout = nullptr, *dw = nullptr, *dphi = nullptr;
  auto cleanup = [&] {
    cudaFree(dx); cudaFree(dy); cudaFree(dz); cudaFree(dout); cudaFree(dw); cudaFree(dphi);
  };
  const int64_t F = std::max<int64_t>(n_features, 1);
  if (cudaMalloc(&dx, n * 8) || cudaMalloc(&dy, n * 8) || (dim == 3 && cudaMalloc(&dz, n * 8)) ||
      cudaMalloc(&dout, n * 8) || cudaMalloc(&dw, F * 3 * 8) || cudaMalloc(&dphi, F * 8)) {
    cleanup();
    return fail(GS_ERR_OUT_OF_MEMORY, "device allocation failed");
  }
  cudaMemcpy(dx, x, n * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(dy, y, n * 8, cudaMemcpyHostToDevice);
  if (dim == 3) cudaMemcpy(dz, z, n * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(dout, host.data(), n * 8, cudaMemcpyHostToDevice);
  for (int s = 0; s < model->n_structures; ++s) {
    const gs_structure& st = model->s[s];
    double rot[9];
    rotation_matrix(st, dim, rot);
    if (!st.has_anis) {
      for (int i = 0; i < 9; ++i) rot[i] = (i % 4 == 0) ? 1.0 : 0.0;
    }
    std::vector<double> w(F * 3, 0.0), phi(F);
    for (int64_t f = 0; f < F; ++f) {
      double g[3] = {rng.normal(), rng.normal(), dim == 3 ? rng.normal() : 0.0};
      double scale;
      int dof = 0;
      double kappa = 1.0 / st.range;
      switch (st.kind) {
        case GS_KIND_GAUSSIAN: dof = 0; kappa = std::sqrt(2.0) / st.range; break;
        case GS_KIND_MATERN15: dof = 3; kappa = std::sqrt(3.0) / st.range; break;
        case GS_KIND_MATERN25: dof = 5; kappa = std::sqrt(5.0) / st.range; break;
        case GS_KIND_SPHERICAL: dof = 1; kappa = 3.0 / st.range; break;
        default: dof = 1; kappa = 1.0 / st.range; break;
      }
      if (dof == 0) {
        scale = kappa;
      } else {
        double chi = 0.0;
        for (int q = 0; q < dof; ++q) {
          double v = rng.normal();
          chi += v * v;
        }
        scale = kappa / std::sqrt(std::max(chi, 1e-300));
      }
      // phase = w_iso . (R x) = (R^T w_iso) . x
      double wi[3] = {g[0] * scale, g[1] * scale, g[2] * scale};
      for (int c = 0; c < 3; ++c) {
        double acc = 0.0;
        for (int r = 0; r < dim; ++r) acc += rot[r * 3 + c] * wi[r];
        w[f * 3 + c] = c < dim ? acc : 0.0;
      }
      phi[f] = 6.283185307179586 * rng.uniform();
    }
    cudaMemcpy(dw, w.data(), F * 3 * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dphi, phi.data(), F * 8, cudaMemcpyHostToDevice);
    double amp = std::sqrt(2.0 * st.sill / (double)F);
    rff_kernel<<<(int)std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 32), 256>>>(dim, n, dx, dy, dz, (int)F, dw, dphi, amp, dout);
  }
  cudaError_t e = cudaMemcpy(out, dout, n * 8, cudaMemcpyDeviceToHost);
  cleanup();
  if (e != cudaSuccess) return cuda_fail(e, "rff field", __FILE__, __LINE__);
  return GS_OK;
}
