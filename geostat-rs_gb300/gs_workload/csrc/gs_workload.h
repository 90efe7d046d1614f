/* gs_workload.h -- C ABI of libgeostat_workload.so: the seeded synthetic
 * workloads and measurement probes used by the benchmark and the tests.
 * It is not part of the drop-in library (include/geostat_gb300.h); it links
 * against libgeostat_gb300.so for the model validation, the xoshiro256++
 * stream and the device helpers. */
#ifndef GS_WORKLOAD_H
#define GS_WORKLOAD_H

#include <stdint.h>

#include "geostat_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Random-Fourier-feature Gaussian field at n points (host coordinates and
 * output): kind of each structure picks the spectral family (exponential,
 * gaussian, matern15, matern25; spherical uses the exponential family at the
 * same practical range), plus iid N(0, nugget) noise; frequencies, phases and
 * noise come from the xoshiro256++ stream of crates/geostat-core/src/rng.rs. */
int gs_synth_rff_field(int dim, int64_t n, const double* x, const double* y, const double* z,
                       const gs_model* model, int64_t n_features, uint64_t seed, double* out);

/* Sustained CUDA-core FMA throughput in TFLOP/s for FP32 (precision 0), FP64
 * (1) or packed FP32x2 FMAs (2): the roofline denominator of the per-system
 * kernels. */
int gs_probe_fma_tflops(int precision, double* tflops);

/* exp(-x) for x >= 0 as the FP64 re-solve kernels compute it (table-driven
 * exp on the device; 0 for x >= 708), for accuracy checks. */
int gs_probe_expneg(int64_t n, const double* x, double* out);

#ifdef __cplusplus
}
#endif
#endif
