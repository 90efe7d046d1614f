// gs_search.cu -- device bucket grid (K1) and warp-per-target neighbour
// search (K2).
//
// The search returns exactly the set the reference's kd-tree returns
// (crates/geostat-core/src/search.rs:57-99 via kriging.rs:441-490): the k
// smallest (squared distance, index) pairs within the radius, in that order.
// Squared distances are formed exactly as the reference does --
// ((0 + dx0^2) + dx1^2) + dx2^2 with dx = point - target, every operation
// separately rounded -- so the comparisons see bit-identical values.  The
// kd-tree keeps the first-visited candidate when the k-th and (k+1)-th tie
// exactly; this search keeps the smaller index.  The two agree whenever no
// such boundary tie exists (the oracle counts them).
//
// Octant search (kriging.rs:462-489) keeps, per 2^D sector around the
// target, the per_octant smallest (d2, index) candidates, merges the sectors
// in (d2, index) order and truncates to max_neighbors -- the same selection
// as the reference's distance-ordered walk over all candidates.
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gs_internal.h"
#include "gs_search.cuh"

namespace gs {

namespace {

constexpr unsigned kFull = 0xffffffffu;

// search_point (kriging.rs:16-21) with the reference's operation order.
template <int D>
__device__ __forceinline__ void to_search_frame(const SearchFrame& f, const double* p, double* q) {
  if (!f.aniso) {
#pragma unroll
    for (int d = 0; d < D; ++d) q[d] = p[d];
    return;
  }
  if (D == 2) {
    // out[0] = dh0*s + dh1*c ; out[1] = (dh0*c - dh1*s) / ratio
    q[0] = __dadd_rn(__dmul_rn(p[0], f.s), __dmul_rn(p[1], f.c));
    q[1] = __ddiv_rn(__dsub_rn(__dmul_rn(p[0], f.c), __dmul_rn(p[1], f.s)), f.ratio);
  } else {
#pragma unroll
    for (int r = 0; r < 3; ++r)
      q[r] = __dadd_rn(__dadd_rn(__dmul_rn(f.rot[r * 3 + 0], p[0]), __dmul_rn(f.rot[r * 3 + 1], p[1])),
                       __dmul_rn(f.rot[r * 3 + 2], p[2]));
  }
}

template <int D>
__global__ void transform_kernel(SearchFrame f, int64_t n, const double* x, const double* y,
                                 const double* z, double* ox, double* oy, double* oz) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double p[3] = {x[i], y[i], D == 3 ? z[i] : 0.0};
    double q[3];
    to_search_frame<D>(f, p, q);
    ox[i] = q[0];
    oy[i] = q[1];
    if (D == 3) oz[i] = q[2];
  }
}

__device__ __forceinline__ int clamp_cell(double v, int n) {
  double c = floor(v);
  if (!(c >= 0.0)) return 0;  // also NaN
  if (c >= (double)(n - 1)) return n - 1;
  return (int)c;
}

template <int D>
__global__ void cell_id_kernel(GridDev g, int64_t n, const double* x, const double* y,
                               const double* z, uint32_t* keys, uint32_t* vals) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int cx = clamp_cell((x[i] - g.origin[0]) * g.inv_cell, g.n[0]);
    int cy = clamp_cell((y[i] - g.origin[1]) * g.inv_cell, g.n[1]);
    int cz = D == 3 ? clamp_cell((z[i] - g.origin[2]) * g.inv_cell, g.n[2]) : 0;
    keys[i] = (uint32_t)(cx + g.n[0] * (cy + g.n[1] * cz));
    vals[i] = (uint32_t)i;
  }
}

template <int D>
__global__ void gather_kernel(int64_t n, const uint32_t* perm, const double* x, const double* y,
                              const double* z, double* sx, double* sy, double* sz,
                              uint32_t* sidx, GridDev g, float* f) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t p = perm[i];
    sx[i] = x[p];
    sy[i] = y[p];
    if (D == 3) sz[i] = z[p];
    sidx[i] = p;
    f[i] = (float)(x[p] - g.origin[0]);
    f[n + i] = (float)(y[p] - g.origin[1]);
    if (D == 3) f[2 * n + i] = (float)(z[p] - g.origin[2]);
  }
}

__global__ void cell_start_kernel(int64_t ncells, int64_t n, const uint32_t* keys,
                                  uint32_t* cstart) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c <= ncells;
       c += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = n;  // first position with key >= c
    while (lo < hi) {
      int64_t mid = (lo + hi) >> 1;
      if ((int64_t)keys[mid] < c) lo = mid + 1;
      else hi = mid;
    }
    cstart[c] = (uint32_t)lo;
  }
}

// Offset of the s-th cell on the surface of the Chebyshev shell of radius r.
template <int D>
__device__ __forceinline__ void shell_offset(int r, int s, int* o) {
  if (r == 0) {
    o[0] = o[1] = o[2] = 0;
    return;
  }
  const int w = 2 * r + 1, wi = 2 * r - 1;
  if (D == 2) {
    if (s < w) {
      o[0] = -r + s;
      o[1] = -r;
    } else if (s < 2 * w) {
      o[0] = -r + (s - w);
      o[1] = r;
    } else {
      int rem = s - 2 * w;
      o[0] = (rem / wi) ? r : -r;
      o[1] = -r + 1 + rem % wi;
    }
    o[2] = 0;
  } else {
    const int fz = w * w, fy = w * wi;
    if (s < 2 * fz) {
      int q = s % fz;
      o[0] = -r + q % w;
      o[1] = -r + q / w;
      o[2] = (s / fz) ? r : -r;
    } else if (s < 2 * fz + 2 * fy) {
      int rem = s - 2 * fz;
      int q = rem % fy;
      o[0] = -r + q % w;
      o[2] = -r + 1 + q / w;
      o[1] = (rem / fy) ? r : -r;
    } else {
      int rem = s - 2 * fz - 2 * fy;
      int fx = wi * wi;
      int q = rem % fx;
      o[1] = -r + 1 + q % wi;
      o[2] = -r + 1 + q / wi;
      o[0] = (rem / fx) ? r : -r;
    }
  }
}

// Rings whose cell offsets the search reads from a table (built once per
// block) instead of deriving them with integer divisions: rings 0..4 in 3-D
// (9^3 cells), 0..8 in 2-D (17^2 cells).  Offset (o0, o1, o2) is packed as
// (o0 + 128) | (o1 + 128) << 8 | (o2 + 128) << 16; ring r starts at entry
// (2r - 1)^D.
template <int D>
struct ShellTab {
  static constexpr int kRings = D == 3 ? 4 : 8;
  static constexpr int kEntries = D == 3 ? 729 : 289;
};
template <int D>
__device__ __forceinline__ int shell_start(int r) {
  const int w = 2 * r - 1;
  return r == 0 ? 0 : (D == 3 ? w * w * w : w * w);
}

template <int D>
__device__ __forceinline__ int shell_size(int r) {
  if (r == 0) return 1;
  return D == 2 ? 8 * r : 24 * r * r + 2;
}

// FP32 bound for the prefilter: every candidate whose exact squared distance
// is <= T has an FP32 squared distance (from origin-relative FP32
// coordinates) <= the returned value.  delta bounds the per-axis FP32
// coordinate error (both roundings); the FP32 sum adds a relative 4 ulp.
// Every term is positive and every operation rounds up, so the FP32 result
// is an upper bound of the exact expression (no FP64 arithmetic).
__device__ __forceinline__ float prefilter_bound(double T, float delta, int D) {
  const float inf = __int_as_float(0x7f800000);
  if (!(T < 1e300)) return inf;
  const float t = __double2float_ru(T);
  const float st = __fsqrt_ru(t);
  const float sd = __fmul_ru(st, delta);
  float b = __fmul_ru(t, 1.0f + 1.0f / 1048576.0f);
  b = __fadd_ru(b, __fmul_ru(2.0f * (float)D * (1.0f + 2.4e-7f), sd));
  b = __fadd_ru(b, __fmul_ru((float)D, __fmul_ru(delta, delta)));
  return __fmul_ru(b, 1.0f + 1e-6f);
}

// Per-target set-up of the search (FP64 frame coordinates, cell, FP32
// prefilter coordinates and bounds), computed for a warp's group of targets
// one lane per target and read by the whole warp when it reaches the target.
struct TargetSetup {
  double q[3];
  int tc[3];
  float qf[3];
  float delta, r2f;
  int pad[2];
};
// Targets per warp group (the lanes that compute set-ups side by side).
constexpr int kSearchGroup = 32;

// Shared memory of one warp of knn_kernel: NB buffers of capb (d2, idx)
// entries, then NB thresholds, counts and dirty flags, the cached prefilter
// bound, a queue of 64 prefilter survivors and the group's target set-ups.
// Used by both the kernel and its launch.
__host__ __device__ inline size_t knn_setup_offset(int NB, int capb) {
  return ((size_t)NB * capb * 12 + (size_t)NB * 16 + 16 + 64 * sizeof(uint32_t) + 15) & ~(size_t)15;
}
__host__ __device__ inline size_t knn_per_warp(int NB, int capb) {
  return knn_setup_offset(NB, capb) + kSearchGroup * sizeof(TargetSetup);
}

// Squared distances are never negative (and never -0: they are sums of
// squares), so the IEEE bit pattern of a squared distance, read as an
// unsigned integer, orders exactly like the value; +inf is the largest key.
// The search compares these keys on the integer pipes: an FP64 compare costs
// as much issue time as dozens of integer instructions on this GPU.
typedef unsigned long long dkey;
constexpr dkey kInfKey = 0x7ff0000000000000ull;

__device__ __forceinline__ dkey d2key(double d2) { return (dkey)__double_as_longlong(d2); }

// True when a >= b for doubles given a - b (IEEE: a - b is +/-0 only when
// a == b, and its sign is that of a - b otherwise).
__device__ __forceinline__ bool diff_nonneg(double diff) {
  const dkey u = (dkey)__double_as_longlong(diff);
  return (u >> 63) == 0 || (u << 1) == 0;
}

// Lane 0: refreshes the cached prefilter bound after a threshold changed.
template <int NB>
__device__ __forceinline__ void refresh_bound(const dkey* thr, float* tfs, float delta, int D,
                                              float r2f) {
  dkey tmax = thr[0];
#pragma unroll
  for (int b = 1; b < NB; ++b) tmax = tmax > thr[b] ? tmax : thr[b];
  tfs[0] = fminf(prefilter_bound(__longlong_as_double((long long)tmax), delta, D), r2f);
}

// Warp-wide bitonic sort of cap (power of two) entries by (d2, idx), keys as
// in d2key.
__device__ __noinline__ void warp_sort(dkey* key, uint32_t* id, int n_valid, int cap, int lane) {
  for (int i = n_valid + lane; i < cap; i += 32) {
    key[i] = kInfKey;
    id[i] = 0xffffffffu;
  }
  __syncwarp();
  for (int size = 2; size <= cap; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = lane; i < (cap >> 1); i += 32) {
        const int a = 2 * stride * (i / stride) + (i % stride);
        const int b = a + stride;
        const bool up = (a & size) == 0;
        const dkey ka = key[a], kb = key[b];
        const uint32_t ia = id[a], ib = id[b];
        const bool gt = (ka > kb) || (ka == kb && ia > ib);
        if (gt == up) {
          key[a] = kb;
          key[b] = ka;
          id[a] = ib;
          id[b] = ia;
        }
      }
      __syncwarp();
    }
  }
}

// Blocks per SM the compiler plans registers for, measured on GB300: eight
// for the single-buffer search (64 registers, a few values spilled: 9 %
// faster than the 80-96 registers the compiler takes unbounded; ten and
// twelve were slower again), four for the octant search (18 % faster than
// unbounded, six slower).
constexpr int kKnnBlocksPerSm = 8;
constexpr int kKnnOctantBlocksPerSm = 4;

template <int D, bool OCT, bool RANKED>
__global__ void __launch_bounds__(128, OCT ? kKnnOctantBlocksPerSm : kKnnBlocksPerSm)
    knn_kernel(GridDev g, SearchFrame fr, SearchParams p, int64_t nt, int gs, const double* tx,
               const double* ty, const double* tz, int32_t* nb, int32_t* nbc) {
  constexpr int NB = OCT ? (1 << D) : 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const int capb = p.capb;
  const size_t per_warp = knn_per_warp(NB, capb);
  unsigned char* base = smem_raw + (size_t)wib * per_warp;
  dkey* bd2 = reinterpret_cast<dkey*>(base);
  uint32_t* bid = reinterpret_cast<uint32_t*>(bd2 + NB * capb);
  dkey* thr = reinterpret_cast<dkey*>(bid + NB * capb);
  int* cnt = reinterpret_cast<int*>(thr + NB);
  int* dirty = cnt + NB;
  float* tfs = reinterpret_cast<float*>(dirty + NB);  // cached prefilter bound
  uint32_t* sq = reinterpret_cast<uint32_t*>(tfs + 4);  // prefilter survivors (64)
  TargetSetup* tset = reinterpret_cast<TargetSetup*>(base + knn_setup_offset(NB, capb));
  __shared__ uint32_t shell_tab[ShellTab<D>::kEntries];
  for (int r = 0; r <= ShellTab<D>::kRings; ++r) {
    const int S = shell_size<D>(r), s0 = shell_start<D>(r);
    for (int q = threadIdx.x; q < S; q += blockDim.x) {
      int o[3];
      shell_offset<D>(r, q, o);
      shell_tab[s0 + q] = (uint32_t)(o[0] + 128) | ((uint32_t)(o[1] + 128) << 8) |
                          ((uint32_t)(o[2] + 128) << 16);
    }
  }
  __syncthreads();
  const double kInf = __longlong_as_double(0x7ff0000000000000ll);
  const double r2 = p.has_radius ? p.r2 : kInf;
  const dkey r2k = d2key(r2);
  const int kb = p.k;

  // A warp takes gs consecutive targets at a time; their FP64 set-up runs one
  // lane per target (the same operations a lane-redundant set-up would do,
  // at 1/gs of the FP64 issue).
  for (int64_t g0 = ((int64_t)blockIdx.x * wpb + wib) * gs; g0 < nt;
       g0 += (int64_t)gridDim.x * wpb * gs) {
  const int gn = (int)min((int64_t)gs, nt - g0);
  __syncwarp();
  if (lane < gn) {
    const int64_t t = g0 + lane;
    const double pt[3] = {tx[t], ty[t], D == 3 ? tz[t] : 0.0};
    TargetSetup& su = tset[lane];
    to_search_frame<D>(fr, pt, su.q);
    float delta = 0.0f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      su.tc[d] = 0;
      su.qf[d] = 0.0f;
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
      su.tc[d] = clamp_cell((su.q[d] - g.origin[d]) * g.inv_cell, g.n[d]);
      // prefilter: FP32 target coordinates and the per-axis error bound
      const double rel = su.q[d] - g.origin[d];
      su.qf[d] = (float)rel;
      // (extent + |rel|) * 2^-23, rounded up
      const float mag = __fadd_ru(g.extf[d], __double2float_ru(fabs(rel)));
      delta = fmaxf(delta, __fadd_ru(mag * (1.0f / 8388608.0f), 1e-30f));
    }
    su.delta = delta;
    su.r2f = prefilter_bound(r2, delta, D);
  }
  __syncwarp();
  for (int j = 0; j < gn; ++j) {
    const int64_t t = g0 + j;
    const TargetSetup& su = tset[j];
    const double q[3] = {su.q[0], su.q[1], D == 3 ? su.q[2] : 0.0};
    const int tc[3] = {su.tc[0], su.tc[1], su.tc[2]};
    const float qf[3] = {su.qf[0], su.qf[1], su.qf[2]};
    const float delta = su.delta;
    const float r2f = su.r2f;
    int maxring = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) maxring = max(maxring, max(tc[d], g.n[d] - 1 - tc[d]));
    int octmax[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      int m = 0;
      if (OCT) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
          int ext = ((b >> d) & 1) ? (g.n[d] - 1 - tc[d]) : tc[d];
          m = max(m, max(ext, 1));
        }
      } else {
        m = maxring;
      }
      octmax[b] = m;
    }
    if (lane < NB) {
      thr[lane] = kInfKey;
      cnt[lane] = 0;
      dirty[lane] = 0;
    }
    if (lane == 0) tfs[0] = r2f;
    __syncwarp();
    long long inrad = 0;
    const int64_t qrank = RANKED ? p.rank0 + t : 0;
    const int32_t tlabel = p.excl_label ? p.target_label[t] : 0;
    if (RANKED && qrank <= p.brute_below) {
      // early ranks: scan the whole (short) prefix of the store
      for (int64_t rb = 0; rb < qrank; rb += 32) {
        const int64_t r = rb + lane;
        const bool valid = r < qrank;
        double d2 = kInf;
        if (valid) {
          const double dx = __dsub_rn(p.px[r], q[0]);
          const double dy = __dsub_rn(p.py[r], q[1]);
          d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
          if (D == 3) {
            const double dz = __dsub_rn(p.pz[r], q[2]);
            d2 = __dadd_rn(d2, __dmul_rn(dz, dz));
          }
        }
        const dkey k2 = d2key(d2);
        bool want = valid && k2 <= r2k && k2 <= thr[0];
        unsigned m = __ballot_sync(kFull, want);
        if (!m) continue;
        if (cnt[0] + __popc(m) > capb) {
          warp_sort(bd2, bid, cnt[0], capb, lane);
          if (lane == 0) {
            cnt[0] = min(cnt[0], kb);
            if (cnt[0] >= kb) thr[0] = bd2[kb - 1];
          }
          __syncwarp();
          want = want && k2 <= thr[0];
          m = __ballot_sync(kFull, want);
        }
        if (want) {
          int slot = cnt[0] + __popc(m & ((1u << lane) - 1u));
          bd2[slot] = k2;
          bid[slot] = (uint32_t)r;
        }
        __syncwarp();
        if (lane == 0) {
          cnt[0] += __popc(m);
          dirty[0] = 1;
        }
        __syncwarp();
      }
      maxring = -1;  // skip the ring walk
    }

    // Exact squared distance in the reference's operation order and insertion
    // into the candidate buffers, for one batch of prefilter survivors
    // (called by the whole warp).
    auto process = [&](uint32_t pi, bool valid) {
      double d2 = kInf;
      uint32_t oid = 0;
      int ob = 0;
      if (valid) {
        const double px = g.sx[pi], py = g.sy[pi];
        const double dx = __dsub_rn(px, q[0]);
        const double dy = __dsub_rn(py, q[1]);
        d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
        if (OCT) ob = (diff_nonneg(dx) ? 1 : 0) | (diff_nonneg(dy) ? 2 : 0);
        if (D == 3) {
          const double pz = g.sz[pi];
          const double dz = __dsub_rn(pz, q[2]);
          d2 = __dadd_rn(d2, __dmul_rn(dz, dz));
          if (OCT) ob |= (diff_nonneg(dz) ? 4 : 0);
        }
        oid = g.sidx[pi];
      }
      const dkey k2 = d2key(d2);
      const bool inr = valid && k2 <= r2k && (!RANKED || (int64_t)oid < qrank) &&
                       !(p.excl_label && p.excl_label[oid] == tlabel);
      if (p.unbounded) inrad += __popc(__ballot_sync(kFull, inr));
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        bool want = inr && (ob == b) && k2 <= thr[b];
        unsigned m = __ballot_sync(kFull, want);
        if (!m) continue;
        if (cnt[b] + __popc(m) > capb) {
          warp_sort(bd2 + b * capb, bid + b * capb, cnt[b], capb, lane);
          if (lane == 0) {
            cnt[b] = min(cnt[b], kb);
            if (cnt[b] >= kb) thr[b] = bd2[b * capb + kb - 1];
            dirty[b] = 0;
            refresh_bound<NB>(thr, tfs, delta, D, r2f);
          }
          __syncwarp();
          want = want && k2 <= thr[b];
          m = __ballot_sync(kFull, want);
        }
        if (want) {
          int slot = cnt[b] + __popc(m & ((1u << lane) - 1u));
          bd2[b * capb + slot] = k2;
          bid[b * capb + slot] = oid;
        }
        __syncwarp();
        if (lane == 0) {
          cnt[b] += __popc(m);
          dirty[b] = 1;
        }
        __syncwarp();
      }
    };
    int qn = 0;  // queued survivors (warp-uniform)

    for (int ring = 0; ring <= maxring; ++ring) {
      // lower bound of the distance to any point of this ring, in FP32
      // rounded down (with a 2^-20 relative margin for the cell placement)
      const float rmin = __fmul_rd(__fmul_rd((float)max(ring - 1, 0), g.cellf_lo),
                                   1.0f - 1.0f / 1048576.0f);
      const dkey rmin2k = d2key((double)__fmul_rd(rmin, rmin));
      unsigned active = 0;
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        bool done = (rmin2k > r2k) || (cnt[b] >= kb && rmin2k > thr[b]) || (ring > octmax[b]);
        if (!done) active |= 1u << b;
      }
      if (!active) break;
      const int S = shell_size<D>(ring);
      for (int sbase = 0; sbase < S; sbase += 32) {
        int s = sbase + lane;
        int ccount = 0;
        uint32_t cst = 0;
        if (s < S) {
          int o[3];
          if (ring <= ShellTab<D>::kRings) {
            const uint32_t v = shell_tab[shell_start<D>(ring) + s];
            o[0] = (int)(v & 0xffu) - 128;
            o[1] = (int)((v >> 8) & 0xffu) - 128;
            o[2] = (int)((v >> 16) & 0xffu) - 128;
          } else {
            shell_offset<D>(ring, s, o);
          }
          int c[3] = {tc[0] + o[0], tc[1] + o[1], tc[2] + o[2]};
          bool ok = true;
#pragma unroll
          for (int d = 0; d < D; ++d) ok = ok && c[d] >= 0 && c[d] < g.n[d];
          if (OCT && ok) {
            // sectors a cell can hold (conservative by one cell for rounding)
            unsigned mask = (1u << NB) - 1u;
#pragma unroll
            for (int d = 0; d < D; ++d) {
              unsigned hi_side = 0, lo_side = 0;
#pragma unroll
              for (int b = 0; b < NB; ++b) {
                if ((b >> d) & 1) hi_side |= 1u << b;
                else lo_side |= 1u << b;
              }
              if (o[d] >= 2) mask &= hi_side;
              else if (o[d] <= -2) mask &= lo_side;
            }
            ok = (mask & active) != 0;
          }
          if (ok) {
            int64_t cid = c[0] + (int64_t)g.n[0] * (c[1] + (int64_t)g.n[1] * c[2]);
            cst = g.cstart[cid];
            ccount = (int)(g.cstart[cid + 1] - cst);
          }
        }
        int incl = ccount;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          int v = __shfl_up_sync(kFull, incl, off);
          if (lane >= off) incl += v;
        }
        const int tot = __shfl_sync(kFull, incl, 31);
        const int excl = incl - ccount;
        for (int pbase = 0; pbase < tot; pbase += 32) {
          const int my = pbase + lane;
          int pos = 0;
#pragma unroll
          for (int st = 16; st > 0; st >>= 1) {
            int v = __shfl_sync(kFull, incl, pos + st - 1);
            if (v <= my) pos += st;
          }
          const int src = pos & 31;
          const uint32_t sst = __shfl_sync(kFull, cst, src);
          const int sex = __shfl_sync(kFull, excl, src);
          bool valid = my < tot;
          const uint32_t pi = sst + (uint32_t)(my - sex);
          if (valid) {
            // FP32 prefilter against the loosest live threshold
            const float tf = tfs[0];
            float e = g.fx[pi] - qf[0];
            float d2f = e * e;
            e = g.fy[pi] - qf[1];
            d2f = fmaf(e, e, d2f);
            if (D == 3) {
              e = g.fz[pi] - qf[2];
              d2f = fmaf(e, e, d2f);
            }
            valid = d2f <= tf;
          }
          // queue the survivors; exact distances run on full batches of 32
          const unsigned m = __ballot_sync(kFull, valid);
          if (valid) sq[qn + __popc(m & ((1u << lane) - 1u))] = pi;
          qn += __popc(m);
          __syncwarp();
          if (qn >= 32) {
            const uint32_t bpi = sq[lane];
            __syncwarp();
            if (lane < qn - 32) sq[lane] = sq[32 + lane];
            qn -= 32;
            __syncwarp();
            process(bpi, true);
          }
        }
      }
      if (qn > 0) {  // the ring's last survivors
        const bool v = lane < qn;
        const uint32_t bpi = v ? sq[lane] : 0u;
        qn = 0;
        __syncwarp();
        process(bpi, v);
      }
      // ring end: settle thresholds of buffers that reached k
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        if (dirty[b] && cnt[b] >= kb) {
          warp_sort(bd2 + b * capb, bid + b * capb, cnt[b], capb, lane);
          if (lane == 0) {
            cnt[b] = kb;
            thr[b] = bd2[b * capb + kb - 1];
            dirty[b] = 0;
            refresh_bound<NB>(thr, tfs, delta, D, r2f);
          }
          __syncwarp();
        }
      }
    }
    // final ordering
    int total = 0;
    if (!OCT) {
      warp_sort(bd2, bid, cnt[0], capb, lane);
      total = min(cnt[0], kb);
    } else {
      for (int b = 0; b < NB; ++b) {
        if (dirty[b]) warp_sort(bd2 + b * capb, bid + b * capb, cnt[b], capb, lane);
        int c = min(cnt[b], kb);
        total += c;
        for (int i = c + lane; i < capb; i += 32) {
          bd2[b * capb + i] = kInfKey;
          bid[b * capb + i] = 0xffffffffu;
        }
      }
      __syncwarp();
      warp_sort(bd2, bid, NB * capb, NB * capb, lane);
    }
    const int kout = p.kout;
    const int outn = min(total, kout);
    for (int jj = lane; jj < kout; jj += 32) nb[t * kout + jj] = jj < outn ? (int32_t)bid[jj] : -1;
    if (lane == 0) {
      bool overflow = p.unbounded && inrad > (long long)kout;
      nbc[t] = overflow ? -1 : outn;
    }
    __syncwarp();
  }
  }
}

inline unsigned ceil_pow2(unsigned v) {
  unsigned p = 1;
  while (p < v) p <<= 1;
  return p;
}

template <class T>
int dalloc(T** p, size_t count) {
  GS_CUDA(dev_malloc((void**)p, std::max<size_t>(count, 1) * sizeof(T)));
  return GS_OK;
}

}  // namespace

Grid::~Grid() {
  cudaFree(d_sx);
  cudaFree(d_sy);
  cudaFree(d_sz);
  cudaFree(d_sidx);
  cudaFree(d_cstart);
  cudaFree(d_f);
}

int grid_build(Grid* g, int dim, int64_t n, const double* x, const double* y, const double* z,
               const SearchFrame& frame, double points_per_cell, cudaStream_t stream) {
  NvtxRange nvtx_range("gs.grid_build");
  if (n <= 0 || n > 0xfffffff0ll) return fail(GS_ERR_INVALID_PARAMETER, "point count out of range");
  g->dim = dim;
  g->n = n;
  double *tx = nullptr, *ty = nullptr, *tz = nullptr;
  GS_TRY(dalloc(&tx, n));
  GS_TRY(dalloc(&ty, n));
  if (dim == 3) GS_TRY(dalloc(&tz, n));
  const int threads = 256;
  const int blocks = (int)std::min<int64_t>((n + threads - 1) / threads, (int64_t)sm_count() * 32);
  if (dim == 2) transform_kernel<2><<<blocks, threads, 0, stream>>>(frame, n, x, y, z, tx, ty, tz);
  else transform_kernel<3><<<blocks, threads, 0, stream>>>(frame, n, x, y, z, tx, ty, tz);
  GS_CUDA(cudaGetLastError());

  // bounding box of the search-frame coordinates
  double* d_red = nullptr;
  GS_TRY(dalloc(&d_red, 6));
  void* tmp = nullptr;
  size_t tmp_bytes = 0;
  GS_CUDA(cub::DeviceReduce::Min(tmp, tmp_bytes, tx, d_red, (int)n, stream));
  size_t need = tmp_bytes;
  GS_CUDA(cub::DeviceReduce::Max(nullptr, tmp_bytes, tx, d_red, (int)n, stream));
  need = std::max(need, tmp_bytes);
  GS_CUDA(dev_malloc((void**)&tmp, need));
  const double* axes[3] = {tx, ty, tz};
  for (int d = 0; d < dim; ++d) {
    tmp_bytes = need;
    GS_CUDA(cub::DeviceReduce::Min(tmp, tmp_bytes, axes[d], d_red + d, (int)n, stream));
    tmp_bytes = need;
    GS_CUDA(cub::DeviceReduce::Max(tmp, tmp_bytes, axes[d], d_red + 3 + d, (int)n, stream));
  }
  double h_red[6] = {0, 0, 0, 0, 0, 0};
  GS_CUDA(cudaMemcpyAsync(h_red, d_red, 6 * sizeof(double), cudaMemcpyDeviceToHost, stream));
  GS_CUDA(cudaStreamSynchronize(stream));
  cudaFree(tmp);
  cudaFree(d_red);

  // cell size: about points_per_cell points per cell over the active axes
  double ext[3] = {0, 0, 0}, maxext = 0.0;
  for (int d = 0; d < dim; ++d) {
    ext[d] = h_red[3 + d] - h_red[d];
    maxext = std::max(maxext, ext[d]);
  }
  double vol = 1.0;
  int act = 0;
  for (int d = 0; d < dim; ++d)
    if (ext[d] > maxext * 1e-9) {
      vol *= ext[d];
      ++act;
    }
  double cell;
  if (act == 0 || !(maxext > 0.0)) {
    cell = 1.0;
  } else {
    cell = std::pow(vol * points_per_cell / (double)n, 1.0 / act);
    if (!(cell > 0.0)) cell = maxext;
  }
  int64_t total = 1;
  int nd[3] = {1, 1, 1};
  for (int guard = 0; guard < 200; ++guard) {
    total = 1;
    for (int d = 0; d < dim; ++d) {
      double c = ext[d] > maxext * 1e-9 ? std::ceil(ext[d] / cell) : 1.0;
      nd[d] = (int)std::max(1.0, std::min(c, 1.0e6));
      total *= nd[d];
    }
    if (total <= 2 * n + 64) break;
    cell *= 1.25;
  }
  GridDev& G = g->dev;
  for (int d = 0; d < 3; ++d) {
    G.origin[d] = d < dim ? h_red[d] : 0.0;
    G.n[d] = nd[d];
  }
  G.cell = cell;
  G.inv_cell = 1.0 / cell;
  G.ncells = total;

  uint32_t *keys = nullptr, *vals = nullptr, *keys2 = nullptr, *vals2 = nullptr;
  GS_TRY(dalloc(&keys, n));
  GS_TRY(dalloc(&vals, n));
  GS_TRY(dalloc(&keys2, n));
  GS_TRY(dalloc(&vals2, n));
  if (dim == 2) cell_id_kernel<2><<<blocks, threads, 0, stream>>>(G, n, tx, ty, tz, keys, vals);
  else cell_id_kernel<3><<<blocks, threads, 0, stream>>>(G, n, tx, ty, tz, keys, vals);
  GS_CUDA(cudaGetLastError());
  int bits = 1;
  while (bits < 32 && ((int64_t)1 << bits) < total) ++bits;
  tmp = nullptr;
  tmp_bytes = 0;
  GS_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys2, vals, vals2, (int)n, 0,
                                          bits, stream));
  GS_CUDA(dev_malloc((void**)&tmp, std::max<size_t>(tmp_bytes, 1)));
  GS_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys2, vals, vals2, (int)n, 0,
                                          bits, stream));
  GS_TRY(dalloc(&g->d_sx, n));
  GS_TRY(dalloc(&g->d_sy, n));
  if (dim == 3) GS_TRY(dalloc(&g->d_sz, n));
  GS_TRY(dalloc(&g->d_sidx, n));
  GS_TRY(dalloc(&g->d_cstart, total + 1));
  GS_TRY(dalloc(&g->d_f, 3 * n));
  for (int d = 0; d < 3; ++d) {
    G.ext[d] = d < dim ? ext[d] : 0.0;
    float f = (float)G.ext[d];
    if ((double)f < G.ext[d]) f = std::nextafter(f, INFINITY);
    G.extf[d] = f;
  }
  {
    float f = (float)G.cell;
    if ((double)f > G.cell) f = std::nextafter(f, -INFINITY);
    G.cellf_lo = f;
  }
  if (dim == 2)
    gather_kernel<2><<<blocks, threads, 0, stream>>>(n, vals2, tx, ty, tz, g->d_sx, g->d_sy,
                                                     g->d_sz, g->d_sidx, G, g->d_f);
  else
    gather_kernel<3><<<blocks, threads, 0, stream>>>(n, vals2, tx, ty, tz, g->d_sx, g->d_sy,
                                                     g->d_sz, g->d_sidx, G, g->d_f);
  GS_CUDA(cudaGetLastError());
  {
    int cb = (int)std::min<int64_t>((total + 1 + threads - 1) / threads, (int64_t)sm_count() * 32);
    cell_start_kernel<<<cb, threads, 0, stream>>>(total, n, keys2, g->d_cstart);
    GS_CUDA(cudaGetLastError());
  }
  GS_CUDA(cudaStreamSynchronize(stream));
  cudaFree(tmp);
  cudaFree(keys);
  cudaFree(vals);
  cudaFree(keys2);
  cudaFree(vals2);
  cudaFree(tx);
  cudaFree(ty);
  cudaFree(tz);
  G.sx = g->d_sx;
  G.sy = g->d_sy;
  G.sz = g->d_sz;
  G.fx = g->d_f;
  G.fy = g->d_f + n;
  G.fz = g->d_f + 2 * n;
  G.sidx = g->d_sidx;
  G.cstart = g->d_cstart;
  return GS_OK;
}

int grid_build_ranked(Grid* g, int dim, int64_t n, const double* x, const double* y,
                      const double* z, double points_per_cell, cudaStream_t stream) {
  NvtxRange nvtx_range("gs.grid_build_ranked");
  SearchFrame f;
  std::memset(&f, 0, sizeof(f));
  return grid_build(g, dim, n, x, y, z, f, points_per_cell, stream);
}

int search_launch(const Grid& g, const SearchFrame& frame, const SearchParams& p0, int64_t nt,
                  const double* tx, const double* ty, const double* tz, int32_t* nb,
                  int32_t* nbc, cudaStream_t stream) {
  NvtxRange nvtx_range("gs.search");
  if (nt == 0) return GS_OK;
  SearchParams p = p0;
  p.capb = (int)ceil_pow2((unsigned)std::max(p.k + 32, 64));
  const int NB = p.octant ? (1 << g.dim) : 1;
  const int wpb = 4;
  const size_t per_warp = knn_per_warp(NB, p.capb);
  size_t smem = per_warp * wpb;
  // 227 KB per block, less the static ring-offset table
  static const size_t kMaxSmem = 227 * 1024 - ShellTab<3>::kEntries * sizeof(uint32_t);
  if (smem > kMaxSmem) return fail(GS_ERR_INVALID_PARAMETER, "neighbourhood too large for the device search");
  // targets per warp group: up to 32 once there are 16 warps' worth of
  // groups per SM, fewer for small batches (latency)
  const int64_t warps_full = (int64_t)sm_count() * 16;
  const int gs = (int)std::min<int64_t>(kSearchGroup, std::max<int64_t>(1, (nt + warps_full - 1) / warps_full));
  const int64_t groups = (nt + gs - 1) / gs;
  int64_t blocks64 = (groups + wpb - 1) / wpb;
  int blocks = (int)std::min<int64_t>(blocks64, (int64_t)sm_count() * 64);
  auto launch = [&](auto kern) -> int {
    GS_TRY(allow_dynamic_smem((const void*)kern, smem));
    kern<<<blocks, wpb * 32, smem, stream>>>(g.dev, frame, p, nt, gs, tx, ty, tz, nb, nbc);
    GS_CUDA(cudaGetLastError());
    count_launch(1);
    return GS_OK;
  };
  if (p.ranked) {
    if (p.octant) return fail(GS_ERR_INVALID_PARAMETER, "ranked octant search is not supported");
    if (g.dim == 2) return launch(knn_kernel<2, false, true>);
    return launch(knn_kernel<3, false, true>);
  }
  if (g.dim == 2) {
    if (p.octant) return launch(knn_kernel<2, true, false>);
    return launch(knn_kernel<2, false, false>);
  }
  if (p.octant) return launch(knn_kernel<3, true, false>);
  return launch(knn_kernel<3, false, false>);
}

}  // namespace gs
