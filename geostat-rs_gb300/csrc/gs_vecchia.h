// gs_vecchia.h -- Vecchia entry points shared with other translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/geostat_gb300.h"

namespace gs {
// Log-likelihood of ncand candidate models on a plan (one batched launch);
// ll[c] and status[c] per candidate; synchronises `s` before returning.
// exclude (device, per ordered position, or null): positions whose terms
// are left out of the sums.
// REML (basis set: p x n trend basis on the device; conditioning sets of at
// most 32 points): reml_sums receives per candidate the ungrouped REML's
// sums instead of log-likelihoods.
// [k0, k1): the ordered positions whose terms are evaluated and summed
// (k1 < 0: the whole plan); REML always covers the whole plan.
int vecchia_eval(const gs_vecchia_plan* P, int64_t ncand, const gs_model* models, double* ll,
                 int32_t* status, int precision, cudaStream_t s,
                 const uint8_t* exclude = nullptr, const double* basis = nullptr, int p = 0,
                 double* reml_sums = nullptr, int64_t k0 = 0, int64_t k1 = -1);
// Points of the plan's data set.
int64_t vecchia_plan_points(const gs_vecchia_plan* P);
}  // namespace gs
