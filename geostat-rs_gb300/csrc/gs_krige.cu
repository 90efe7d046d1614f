// gs_krige.cu -- per-target kriging solves.
//
// K3 (krige_rows_kernel): one system per block of 32 or 64 threads, thread
// i owning neighbour i.  The system (kriging.rs:527-567 build_lhs + the
// right-hand side of predict_inner, kriging.rs:569-612) is assembled in shared
// memory as packed lower-triangular double-float entries.  The FP32 hi parts
// of the covariance block are inverted by a sweep with each thread's row in
// registers; drift terms enter through the Schur complement F^T C^{-1} F
// (the covariance block is positive definite, so no pivoting is needed).  The
// solution is refined with residuals b - A x formed from the double-float
// entries in compensated FP32 (Ogita-Rump-Oishi Dot2) and accumulated in
// double-float; the outputs (kriging.rs:614-643) are double-float sums
// converted to FP64 once.  A system whose refinement does not contract to
// ~1e-13 relative, or whose pivot is too small for FP32, is flagged for the
// FP64 solver.
//
// K3' (krige_fp64_kernel): one system per thread, the reference's own
// algorithm in FP64 -- build_lhs, LU with partial pivoting and its singular
// test (linalg.rs:27-111), the same summation order for the outputs.  Each
// thread's matrix lives in a global scratch slab, interleaved across threads
// so neighbouring threads touch neighbouring addresses.
#include <algorithm>
#include <cmath>
#include <mutex>

#include "gs_internal.h"
#include "gs_krige.cuh"
#include "gs_rows.cuh"
#include "gs_warp.cuh"
#include "gs_solve.cuh"

namespace gs {

namespace {

// Basis function k of fill_basis (kriging.rs:410-439) at point pt, FP64.
template <int D>
__device__ __forceinline__ double basis_at(const KrigeArgs& a, const double* pt,
                                           const double* drow, int k) {
  if (k == 0) return 1.0;
  if (a.method == GS_EXTERNAL_DRIFT) return (drow[k - 1] - a.dmean[k - 1]) / a.dscale[k - 1];
  // universal: normalised coordinates, then their degree-2 monomials
  if (k <= D) return (pt[k - 1] - a.center[k - 1]) / a.scale;
  int idx = 1 + D;
  for (int u = 0; u < D; ++u)
    for (int v = u; v < D; ++v) {
      if (idx == k)
        return ((pt[u] - a.center[u]) / a.scale) * ((pt[v] - a.center[v]) / a.scale);
      ++idx;
    }
  return 0.0;
}

// fill_basis (kriging.rs:410-439) in FP64.
template <int D>
__device__ __forceinline__ void fill_basis(const KrigeArgs& a, const double* pt,
                                           const double* drow, double* out) {
  switch (a.method) {
    case GS_ORDINARY:
      out[0] = 1.0;
      break;
    case GS_UNIVERSAL: {
      double xn[3];
#pragma unroll
      for (int d = 0; d < D; ++d) xn[d] = (pt[d] - a.center[d]) / a.scale;
      out[0] = 1.0;
#pragma unroll
      for (int d = 0; d < D; ++d) out[1 + d] = xn[d];
      if (a.uk_degree == 2) {
        int idx = 1 + D;
#pragma unroll
        for (int u = 0; u < D; ++u)
#pragma unroll
          for (int v = u; v < D; ++v) out[idx++] = xn[u] * xn[v];
      }
      break;
    }
    case GS_EXTERNAL_DRIFT:
      out[0] = 1.0;
      for (int k = 0; k < a.nv; ++k) out[1 + k] = (drow[k] - a.dmean[k]) / a.dscale[k];
      break;
    default:
      break;
  }
}

// Shared-memory layout of one system of krige_rows_kernel (R rows, PC drift
// columns, nf coordinate frames).
struct RowsLayout {
  size_t off_a, off_f, off_v, off_b, off_z, off_x, off_row, off_vec, off_red, off_redd, off_s,
      off_td, off_flag, off_slots, total;
};

// Targets per run: a block solves consecutive targets of its run one after
// another and keeps the matrix entries of the neighbours they share.
constexpr int kRowsRun = 64;

__host__ __device__ inline RowsLayout rows_layout(int R, int PC, int nf, int dim) {
  RowsLayout L;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t r = o;
    o += (bytes + 15) & ~(size_t)15;
    return r;
  };
  const int W = R + PC;
  L.off_a = take((size_t)(R * (R + 1) / 2) * sizeof(df));
  L.off_f = take((size_t)PC * R * sizeof(df));
  L.off_v = take((size_t)nf * dim * R * sizeof(df));
  L.off_b = take((size_t)W * sizeof(df));
  L.off_z = take((size_t)R * sizeof(df));
  L.off_x = take((size_t)R * sizeof(df));
  L.off_row = take((size_t)2 * (W + 4) * sizeof(float));
  L.off_vec = take((size_t)W * sizeof(float));
  L.off_red = take((size_t)2 * (R / 32) * PC * sizeof(float));
  L.off_redd = take((size_t)2 * (R / 32) * 2 * sizeof(df));
  L.off_s = take((size_t)PC * PC * sizeof(float));
  L.off_td = take(8 * sizeof(df));
  L.off_flag = take(16);
  L.off_slots = take((size_t)5 * R * sizeof(int) + 8 * sizeof(unsigned));
  L.total = o;
  return L;
}

// K3: one system per R threads (n <= R neighbours, p <= PC drift terms),
// S systems per block side by side (each with its own part of the shared
// memory, its own runs of targets and its own barriers).  The system [C F; F^T 0] [w; mu] = [c; f] is solved through the
// covariance block: the sweep gives -C^{-1} and G = C^{-1} F in registers,
// S = F^T G (p x p) is inverted in FP32, and a correction for a residual
// (r1, r2) is
//     y = C^{-1} r1,  dmu = S^{-1} (F^T y - r2),  dw = y - G dmu.
// Residuals come from the double-float system (compensated FP32 products),
// the solution is accumulated in double-float, and the outputs are
// double-float sums converted to FP64 once.
//
// Slots: thread s owns slot s, which holds one neighbour (a data point id) or
// nothing.  A block walks a run of consecutive targets; neighbours that the
// next target shares with the previous one keep their slot, so the
// covariances between kept neighbours (target independent) stay in the
// packed matrix, and only pairs with a newly placed neighbour are evaluated.
// Solving in slot order instead of neighbour order changes only the order of
// roundings.
template <int D, int R, int PC, int S>
__global__ void __launch_bounds__(R * S, (R == 64 ? 8 : 16) / S)
    krige_rows_kernel(KrigeArgs a, DevModel m, ExpTable tab_g, DfConsts kc, uint8_t* flag) {
  constexpr int W = R + PC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ ExpTable tab;
  for (int q = threadIdx.x; q < 256; q += R * S) tab.v[q] = tab_g.v[q];
  const int i = rows_tid<R, S>();
  const Frames fr = frames_of(m);
  const RowsLayout L = rows_layout(R, PC, fr.nf, D);
  // this system's part of the block's shared memory
  unsigned char* const sbase = smem_raw + (size_t)rows_sys<R, S>() * L.total;
  df* A = reinterpret_cast<df*>(sbase + L.off_a);     // packed covariance block (slots)
  df* F = reinterpret_cast<df*>(sbase + L.off_f);     // F[q * R + s]: drift q at slot s
  df* V = reinterpret_cast<df*>(sbase + L.off_v);     // frame coordinates (slots)
  df* B = reinterpret_cast<df*>(sbase + L.off_b);     // c (slots), f (R..R+p-1)
  df* Z = reinterpret_cast<df*>(sbase + L.off_z);     // values (slots)
  float* Xh = reinterpret_cast<float*>(sbase + L.off_x);  // -w (hi parts), broadcast
  float* Xl = Xh + R;                                      // -w (lo parts)
  float* rowbuf = reinterpret_cast<float*>(sbase + L.off_row);
  float* vec = reinterpret_cast<float*>(sbase + L.off_vec);
  float* red = reinterpret_cast<float*>(sbase + L.off_red);
  df* redd = reinterpret_cast<df*>(sbase + L.off_redd);
  float* Sinv = reinterpret_cast<float*>(sbase + L.off_s);
  df* TD = reinterpret_cast<df*>(sbase + L.off_td);  // target coordinates, sk mean
  int* sflag = reinterpret_cast<int*>(sbase + L.off_flag);
  int* new_idx = reinterpret_cast<int*>(sbase + L.off_slots);  // this target's neighbours
  int* matched = new_idx + R;     // neighbour already in a slot
  int* umap = matched + R;        // k-th unplaced neighbour
  int* act_list = umap + R;       // occupied slots, ascending (the pivot order)
  int* fresh_list = act_list + R; // newly placed slots, ascending
  unsigned* bal = reinterpret_cast<unsigned*>(fresh_list + R);  // 2 x 4 ballot words
  const double* coord[3] = {a.x, a.y, a.z};
  int slot = 0;
  int my_idx = -1;  // data point in this thread's slot
  __syncthreads();

  const int64_t ntl = a.ntl_dev ? *a.ntl_dev : a.ntl;
  const int run = a.run > 0 ? a.run : kRowsRun;
  const bool route = a.route_fp64 && *a.route_fp64;
  for (int64_t r0 = ((int64_t)blockIdx.x * S + rows_sys<R, S>()) * run; r0 < ntl;
       r0 += (int64_t)gridDim.x * S * run) {
  const int64_t r1 = r0 + run < ntl ? r0 + run : ntl;
  for (int64_t it = r0; it < r1; ++it) {
    const int64_t t = a.tlist ? a.tlist[it] : it;
    const int n = a.nbc[t];
    const int p = a.p;
    uint8_t st = GS_ST_OK;
    if (n < 0) st = GS_ST_CAPACITY;
    else if (n < a.min_nb) st = GS_ST_NO_NEIGHBORS;
    else if (n < p) st = GS_ST_INSUFFICIENT_DATA;
    if (st != GS_ST_OK) {
      if (i == 0) {
        a.out_v[t] = __longlong_as_double(0x7ff8000000000000ll);
        a.out_var[t] = __longlong_as_double(0x7ff8000000000000ll);
        if (a.out_lag) a.out_lag[t] = __longlong_as_double(0x7ff8000000000000ll);
        a.out_st[t] = st;
        flag[t] = 0;
      }
      continue;
    }
    if (n > R || p > PC || route) {
      if (i == 0) flag[t] = 1;
      continue;
    }
    const double tp[3] = {a.tx[t], a.ty[t], D == 3 ? a.tz[t] : 0.0};
    if (i < D) TD[i] = df_from_double(tp[i]);
    if (i == 3) TD[3] = df_from_double(a.sk_mean);
    if (i < p) B[R + i] = df_from_double(basis_at<D>(a, tp, a.tdrift ? a.tdrift + t * a.nv : nullptr, i));
    // --- slots: keep shared neighbours, place new ones in free slots
    if (i < n) new_idx[i] = a.nb[t * (int64_t)a.kout + i];
    matched[i] = 0;
    rows_bar<R, S>();
    int pos = -1;
    if (my_idx >= 0) {
      for (int q = 0; q < n; ++q) pos = new_idx[q] == my_idx ? q : pos;
    }
    const bool keep = pos >= 0;
    if (keep) matched[pos] = 1;
    rows_bar<R, S>();
    unsigned long long m_un, m_free;
    rows_ballot2<R, S>(i < n && !matched[i], !keep, m_un, m_free, bal);
    const int n_un = __popcll(m_un);
    if ((m_un >> i) & 1ull) umap[rank_below(m_un, i)] = i;
    rows_bar<R, S>();
    const int rf = rank_below(m_free, i);
    const bool fresh = !keep && rf < n_un;
    my_idx = keep ? my_idx : (fresh ? new_idx[umap[rf]] : -1);
    const bool act = my_idx >= 0;
    unsigned long long m_act, m_fresh;
    rows_ballot2<R, S>(act, fresh, m_act, m_fresh, bal + 4);
    const int nact = __popcll(m_act);  // == n
    const int nfresh = __popcll(m_fresh);
    if (act) act_list[rank_below(m_act, i)] = i;
    if (fresh) fresh_list[rank_below(m_fresh, i)] = i;
    // --- this slot's point: frames, value, covariance with the target, drift row
    if (act) {
      const int idx = my_idx;
      df ud[3];
      bool zero = true;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        ud[d] = df_sub(a.cdf[(int64_t)d * a.n + idx], TD[d]);
        zero = zero && same_double(coord[d][idx], tp[d]);
      }
      frame_coords<D>(m, fr, ud, V, R, i);
      B[i] = zero ? m.c0_df : cov_origin<D>(m, fr, V, R, i, tab, kc);
      Z[i] = a.vdf[idx];
      A[pk(i, i)] = a.err_df ? df_add(m.c0_df, a.err_df[idx]) : m.c0_df;
#pragma unroll
      for (int q = 0; q < PC; ++q)
        if (q < p) F[q * R + i] = a.basis_df[(int64_t)q * a.n + idx];
    }
    rows_bar<R, S>();
    // --- covariances of pairs with a newly placed point, two at a time.
    // When most slots are new, the whole strict lower triangle over the
    // occupied slots (pair (a, b), b < a, of act_list); otherwise the
    // (new slot, occupied slot) pairs (fresh_list[a], act_list[b]), a pair
    // of two new slots once.  One loop and one call site of the covariance
    // code for both, so the kernel carries a single copy of it.
    {
      const bool full = 2 * nfresh >= nact;
      const int P = full ? ((nact * (nact - 1)) >> 1) : nfresh * nact;
      // advance pair cursor (a, b) by `step` pair numbers
      auto adv = [&](int& pa, int& pb, int step) {
        pb += step;
        if (full) {
          while (pb >= pa && pa < nact) {
            pb -= pa;
            ++pa;
          }
        } else {
          while (pb >= nact) {
            pb -= nact;
            ++pa;
          }
        }
      };
      int a0 = full ? 1 : 0, b0 = 0;
      adv(a0, b0, i);
      for (int q = i; q < P; q += 2 * R) {
        int a1 = a0, b1 = b0;
        adv(a1, b1, R);
        const bool has1 = q + R < P;
        if (!has1) {
          a1 = a0;
          b1 = b0;
        }
        const int s0 = full ? act_list[a0] : fresh_list[a0], u0 = act_list[b0];
        const int s1 = full ? act_list[a1] : fresh_list[a1], u1 = act_list[b1];
        const bool v0 = full || (u0 != s0 && (!((m_fresh >> u0) & 1ull) || u0 < s0));
        const bool v1 = has1 && (full || (u1 != s1 && (!((m_fresh >> u1) & 1ull) || u1 < s1)));
        if (v0 || v1) {
          df e0, e1;
          cov_pair2<D>(m, fr, V, R, s0, u0, s1, u1, tab, kc, e0, e1);
          if (v0) A[s0 >= u0 ? pk(s0, u0) : pk(u0, s0)] = e0;
          if (v1) A[s1 >= u1 ? pk(s1, u1) : pk(u1, s1)] = e1;
        }
        if (has1) {
          a0 = a1;
          b0 = b1;
          adv(a0, b0, R);
        }
      }
    }
    rows_bar<R, S>();
    // --- FP32 rows: covariance block (identity off the occupied slots), drift block
    float4 tr[W / 4];
    auto cov_hi = [&](int j) {
      float v = i == j ? 1.0f : 0.0f;
      if (act && ((m_act >> j) & 1ull)) v = i >= j ? A[pk(i, j)].hi : A[pk(j, i)].hi;
      return v;
    };
#pragma unroll
    for (int q = 0; q < R / 4; ++q)
      tr[q] = make_float4(cov_hi(4 * q), cov_hi(4 * q + 1), cov_hi(4 * q + 2), cov_hi(4 * q + 3));
    float amax = 0.0f;
#pragma unroll
    for (int q = 0; q < R / 4; ++q)
      amax = fmaxf(amax, act ? fmaxf(fmaxf(fabsf(tr[q].x), fabsf(tr[q].y)),
                                     fmaxf(fabsf(tr[q].z), fabsf(tr[q].w)))
                             : 0.0f);
    amax = rows_max<R, S>(amax, red, slot);
    // power-of-two scale sc with sc * max|C| in [0.5, 1): every pivot is then
    // <= 1, so the pivot thread's multiplier 1 - 1/d never cancels.  The
    // covariance rows and the drift columns are both scaled, so the drift
    // block ends as C^{-1} F unscaled; C^{-1} itself comes out divided by sc.
    int ex = 0;
    frexpf(amax, &ex);
    const float sc = ldexpf(1.0f, -ex);
#pragma unroll
    for (int q = 0; q < R / 4; ++q) {
      if (act && ((m_act >> (4 * q)) & 1ull)) tr[q].x *= sc;
      if (act && ((m_act >> (4 * q + 1)) & 1ull)) tr[q].y *= sc;
      if (act && ((m_act >> (4 * q + 2)) & 1ull)) tr[q].z *= sc;
      if (act && ((m_act >> (4 * q + 3)) & 1ull)) tr[q].w *= sc;
    }
    auto drift_hi = [&](int q) { return (act && q < p) ? F[q * R + i].hi * sc : 0.0f; };
#pragma unroll
    for (int q4 = 0; q4 < PC / 4; ++q4)
      tr[R / 4 + q4] = make_float4(drift_hi(4 * q4), drift_hi(4 * q4 + 1), drift_hi(4 * q4 + 2),
                                   drift_hi(4 * q4 + 3));
    // (an empty simple-kriging system has nothing to invert: w = 0)
    bool ok = nact == 0 || (amax > 0.0f && rows_sweep<R, W / 4, S>(tr, act_list, nact, 1e-6f * amax * sc, rowbuf));
    // --- Schur complement S = F^T G and its FP32 inverse (thread 0)
    if (ok && p > 0) {
      for (int q = 0; q < p; ++q) {
        float v[PC];
        const float fq = act ? F[q * R + i].hi : 0.0f;
#pragma unroll
        for (int r = 0; r < PC; ++r) v[r] = fq * row_elt(tr, R + r);
        rows_sum<R, PC, S>(v, red, slot);
        if (i == 0) {
#pragma unroll
          for (int r = 0; r < PC; ++r) Sinv[q * PC + r] = v[r];
        }
      }
      if (i == 0) {
        // Gauss-Jordan without pivoting (S is positive definite for full-rank drift)
        float smax = 0.0f;
        for (int q = 0; q < p; ++q) smax = fmaxf(smax, fabsf(Sinv[q * PC + q]));
        int good = 1;
        for (int k = 0; k < p && good; ++k) {
          const float d = Sinv[k * PC + k];
          if (!(fabsf(d) > 1e-6f * smax)) {
            good = 0;
            break;
          }
          const float inv = 1.0f / d;
          for (int r = 0; r < p; ++r) {
            if (r == k) continue;
            const float lr = Sinv[r * PC + k] * inv;
            for (int c = 0; c < p; ++c)
              if (c != k) Sinv[r * PC + c] -= lr * Sinv[k * PC + c];
            Sinv[r * PC + k] = -lr;
          }
          for (int c = 0; c < p; ++c)
            if (c != k) Sinv[k * PC + c] *= inv;
          Sinv[k * PC + k] = inv;
        }
        sflag[0] = good;
      }
      rows_bar<R, S>();
      ok = sflag[0] != 0;
    }
    if (!ok) {
      if (i == 0) flag[t] = 1;
      rows_bar<R, S>();
      continue;
    }
    // --- correction operator: (r1 in vec[0..R), r2 in vec[R..R+p)) -> (d1, d2)
    auto apply = [&](float& d1, float (&d2)[PC]) {
      const float y = sc * rows_cinv_apply<R, W / 4, S>(tr, vec, act);
      d1 = y;
#pragma unroll
      for (int q = 0; q < PC; ++q) d2[q] = 0.0f;
      if (p > 0) {
        float u[PC];
#pragma unroll
        for (int q = 0; q < PC; ++q) u[q] = (act && q < p) ? F[q * R + i].hi * y : 0.0f;
        rows_sum<R, PC, S>(u, red, slot);
#pragma unroll
        for (int q = 0; q < PC; ++q) u[q] = q < p ? u[q] - vec[R + q] : 0.0f;
#pragma unroll
        for (int q = 0; q < PC; ++q) {
          float s = 0.0f;
#pragma unroll
          for (int r = 0; r < PC; ++r) s = fmaf(q < p && r < p ? Sinv[q * PC + r] : 0.0f, u[r], s);
          d2[q] = s;
        }
        float g = 0.0f;
#pragma unroll
        for (int q = 0; q < PC; ++q) g = fmaf(row_elt(tr, R + q), d2[q], g);
        d1 = act ? y - g : 0.0f;
      }
    };
    // x0 from the hi parts of the right-hand side
    vec[i] = act ? B[i].hi : 0.0f;
    if (i < p) vec[R + i] = B[R + i].hi;
    rows_bar<R, S>();
    float d1, d2[PC];
    apply(d1, d2);
    df x1 = df_make(d1, 0.0f);
    df x2[PC];
#pragma unroll
    for (int q = 0; q < PC; ++q) x2[q] = df_make(d2[q], 0.0f);
    float mx = fabsf(d1);
#pragma unroll
    for (int q = 0; q < PC; ++q) mx = fmaxf(mx, fabsf(d2[q]));
    const float nx = rows_max<R, S>(mx, red, slot);
    float nd_prev = nx;
    bool conv = false;
    for (int sweep = 1; sweep <= kMaxRefineSweeps && !conv; ++sweep) {
      Xh[i] = -x1.hi;
      Xl[i] = -x1.lo;
      rows_bar<R, S>();
      // r1_i = c_i - sum_j A_ij w_j - sum_q F_iq mu_q over occupied slots:
      // compensated products and sums (Dot2), two occupied slots at a time
      // as packed FP32x2 operations (even and odd positions of act_list in
      // the two lanes of the accumulator pair), joined by one error-free sum
      float s = 0.0f, c = 0.0f;
      // acc(sa, ca, a, -x): sa + ca += -a x
      auto acc = [](float& sa, float& ca, df aij, df nxj) {
        const float ph = __fmul_rn(aij.hi, nxj.hi);
        float pe = __fmaf_rn(aij.hi, nxj.hi, -ph);
        pe = __fmaf_rn(aij.hi, nxj.lo, pe);
        pe = __fmaf_rn(aij.lo, nxj.hi, pe);
        const df ts = two_sum(sa, ph);
        sa = ts.hi;
        ca += ts.lo + pe;
      };
      if (act) {
        float2 s2 = make_float2(B[i].hi, 0.0f), c2 = make_float2(B[i].lo, 0.0f);
        int jj = 0;
        for (; jj + 1 < nact; jj += 2) {
          const int j0 = act_list[jj], j1 = act_list[jj + 1];
          const df a0 = A[j0 <= i ? pk(i, j0) : pk(j0, i)];
          const df a1 = A[j1 <= i ? pk(i, j1) : pk(j1, i)];
          const float2 ah = make_float2(a0.hi, a1.hi), al = make_float2(a0.lo, a1.lo);
          const float2 xh = make_float2(Xh[j0], Xh[j1]), xl = make_float2(Xl[j0], Xl[j1]);
          const float2 ph = __fmul2_rn(ah, xh);
          float2 pe = __ffma2_rn(ah, xh, p_neg(ph));
          pe = __ffma2_rn(ah, xl, pe);
          pe = __ffma2_rn(al, xh, pe);
          const dfp ts = p_two_sum(s2, ph);
          s2 = ts.hi;
          c2 = p_add(c2, p_add(ts.lo, pe));
        }
        const df st2 = two_sum(s2.x, s2.y);
        s = st2.hi;
        c = (c2.x + c2.y) + st2.lo;
        if (jj < nact) {
          const int j0 = act_list[jj];
          acc(s, c, A[j0 <= i ? pk(i, j0) : pk(j0, i)], df_make(Xh[j0], Xl[j0]));
        }
#pragma unroll
        for (int q = 0; q < PC; ++q)
          if (q < p) acc(s, c, F[q * R + i], df_neg(x2[q]));
      }
      // r2_q = f_q - sum_i F_iq w_i, as double-float block sums
      float r2[PC];
#pragma unroll
      for (int q = 0; q < PC; ++q) r2[q] = 0.0f;
      for (int q = 0; q < p; ++q) {
        df v[1] = {act ? df_mul(F[q * R + i], x1) : df_make(0.0f, 0.0f)};
        rows_sum_df<R, 1, S>(v, redd, slot);
        const df rq = df_sub(B[R + q], v[0]);
#pragma unroll
        for (int r = 0; r < PC; ++r)
          if (r == q) r2[r] = rq.hi + rq.lo;
      }
      vec[i] = act ? s + c : 0.0f;
      if (i == 0) {
#pragma unroll
        for (int q = 0; q < PC; ++q)
          if (q < p) vec[R + q] = r2[q];
      }
      rows_bar<R, S>();
      apply(d1, d2);
      if (act) x1 = df_add_f(x1, d1);
      mx = fabsf(d1);
#pragma unroll
      for (int q = 0; q < PC; ++q) {
        x2[q] = df_add_f(x2[q], d2[q]);
        mx = fmaxf(mx, fabsf(d2[q]));
      }
      const float nd = rows_max<R, S>(mx, red, slot);
      if (nd <= 1e-15f * nx) conv = true;
      else if (sweep >= 2) {
        const float rho = nd / nd_prev;
        if (rho < 0.5f && rho * nd <= 1e-13f * nx) conv = true;
        else if (!(rho < 0.5f)) break;  // no longer contracting: FP64 re-solve
      }
      nd_prev = nd;
    }
    if (!conv) {
      if (i == 0) flag[t] = 1;
      rows_bar<R, S>();
      continue;
    }
    // --- outputs: double-float sums, FP64 at the end
    // (w . z, w . c) as one packed double-float product and block sum
    dfp op = dp_zero();
    if (act)
      op = dp_mul(dp_splat(x1),
                  dp_pack(a.method == GS_SIMPLE ? df_sub(Z[i], TD[3]) : Z[i], B[i]));
    op = rows_sum_dfp<R, S>(op, redd, slot);
    const df o[2] = {dp_first(op), dp_second(op)};
    if (i == 0) {
      df sr = o[1];
#pragma unroll
      for (int q = 0; q < PC; ++q)
        if (q < p) sr = df_add(sr, df_mul(x2[q], B[R + q]));
      const double val = a.method == GS_SIMPLE ? a.sk_mean + df_to_double(o[0]) : df_to_double(o[0]);
      a.out_v[t] = val;
      a.out_var[t] = fmax(df_to_double(df_sub(m.c0_df, sr)), 0.0);
      if (a.out_lag)
        a.out_lag[t] = a.method == GS_SIMPLE ? __longlong_as_double(0x7ff8000000000000ll)
                                             : df_to_double(x2[0]);
      a.out_st[t] = GS_ST_OK;
      flag[t] = 0;
    }
    rows_bar<R, S>();
  }
  }
}

// ----------------------------------------------- FP64 re-solve (LDL^T) --
// Systems the mixed kernel could not certify are solved here in FP64, one
// system per warp, with the matrix in shared memory.  The covariance block C
// (n x n) is bordered by q = p + 2 rows -- the covariances with the target
// c, the drift columns F and the data values z -- into the symmetric
//     [ C    c    F    z ]
//     [ c'   C(0)           ]
//     [ F'   f    0         ]
//     [ z'   0    0    0    ]
// and n steps of LDL^T elimination leave in the trailing q x q block the
// Schur complements  C(0) - c'C^-1 c,  f - F'C^-1 c,  -F'C^-1 F,  -z'C^-1 c,
// -z'C^-1 F.  With S = F'C^-1 F and g = F'C^-1 c - f the drift weights are
// mu = S^-1 g (the kriging system's Lagrange multipliers), and
//     estimate = z'C^-1 c - z'C^-1 F mu,   variance = C(0) - c'C^-1 c + g'mu,
// the same quantities as solving [C F; F' 0][w; mu] = [c; f] and forming
// w'z and C(0) - w'c - mu'f (kriging.rs:569-644), without the weights.
// Every entry is FP64 as in the reference (cov_fp64, basis_at): with
// condition numbers up to ~1e11 the double-float covariances of the mixed
// kernel (~1e-14 relative) would move estimates and variances by more than
// 1e-9.  The elimination is FP64.
//
// Work split: an n-system is embedded at the bottom right of an Mmax x Mmax
// frame, so the trailing update of pivot k always covers the pairs (i, j),
// k < j <= i < Mmax -- a prefix of one pair table sorted by j descending,
// shared by every system size.  Lanes take consecutive pairs of the prefix.
// A pivot below 1e-11 of the largest diagonal entry (or a Schur complement
// of the drift below 1e-11 of its largest diagonal entry) leaves the system
// flagged for the partial-pivoting LU solver below, which also decides
// singularity exactly as the reference does.
constexpr int kCholWarps = 4;
// Packed slot covariances per warp (global scratch, L2-resident): keeping
// them out of shared memory leaves room for two blocks per SM.
constexpr int kCholSlotDoubles = GS_MIXED_MAX_NEIGHBORS * (GS_MIXED_MAX_NEIGHBORS + 1) / 2;
constexpr double kCholPivotTol = 1e-11;

struct CholLayout {
  size_t off_ptab, off_warp, warp_bytes, off_a, off_cs, off_lsc, off_lun, off_v, off_idx, total;
};

__host__ __device__ inline CholLayout chol_layout(int Mmax, int dim) {
  CholLayout L;
  size_t o = 0, w = 0;
  auto take = [&](size_t& at, size_t bytes) {
    size_t r = at;
    at += (bytes + 15) & ~(size_t)15;
    return r;
  };
  L.off_ptab = take(o, (size_t)(Mmax * (Mmax - 1) / 2) * 4);
  constexpr int NS = GS_MIXED_MAX_NEIGHBORS;
  L.off_a = take(w, (size_t)(Mmax * (Mmax + 1) / 2) * 8);
  L.off_cs = 0;  // the slot covariances live in global scratch (kCholSlotDoubles per warp)
  L.off_lsc = take(w, (size_t)Mmax * 8);
  L.off_lun = take(w, (size_t)Mmax * 8);
  L.off_v = take(w, (size_t)dim * NS * sizeof(double));
  L.off_idx = take(w, (size_t)6 * NS * 4);
  L.warp_bytes = w;
  L.off_warp = take(o, w * kCholWarps);
  L.total = o;
  return L;
}


// Warp-private neighbour slots of the FP64 re-solve kernels: slot s holds
// data point sidx[s] (or -1), its coordinates P[d * NS + s] and, in global
// scratch, the packed FP64 covariances cs between slot points.
struct WarpSlots {
  int* sidx;
  int* newi;  // the target's neighbours
  int* mt;    // neighbour q already in a slot
  int* um;    // k-th unplaced neighbour
  int* act;   // occupied slots, ascending (system row -> slot)
  int* frl;   // newly filled slots, ascending
  double* P;
  double* cs;
};

// Places a target's n neighbours (nbt) in the slots -- neighbours already in
// a slot keep it, new ones fill vacated slots -- and evaluates the FP64
// covariances (kriging.rs:527-567, separations p_i - p_j as in the
// reference) of every pair with a newly placed point.  Afterwards act[0..n)
// lists the occupied slots.  Ends with a warp barrier.
template <int D>
__device__ __forceinline__ void slots_update(const WarpSlots& ws, const KrigeArgs& a,
                                             const DevModel& m, const Exp64Table& et,
                                             const int32_t* nbt, int n, int lane) {
  constexpr int NS = GS_MIXED_MAX_NEIGHBORS;
  const double* coord[3] = {a.x, a.y, a.z};
  // --- slots: kept neighbours stay, new ones fill the vacated slots
  for (int s = lane; s < NS; s += 32) {
    ws.newi[s] = s < n ? nbt[s] : -2;
    ws.mt[s] = 0;
  }
  __syncwarp();
  bool keep[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int id = ws.sidx[lane + 32 * h];
    int pos = -1;
    if (id >= 0)
      for (int u = 0; u < n; ++u) pos = ws.newi[u] == id ? u : pos;
    keep[h] = pos >= 0;
    if (keep[h]) ws.mt[pos] = 1;
  }
  __syncwarp();
  const unsigned un0 = __ballot_sync(0xffffffffu, lane < n && !ws.mt[lane]);
  const unsigned un1 = __ballot_sync(0xffffffffu, lane + 32 < n && !ws.mt[lane + 32]);
  const unsigned fr0 = __ballot_sync(0xffffffffu, !keep[0]);
  const unsigned fr1 = __ballot_sync(0xffffffffu, !keep[1]);
  const unsigned below = (1u << lane) - 1u;
  if ((un0 >> lane) & 1u) ws.um[__popc(un0 & below)] = lane;
  if ((un1 >> lane) & 1u) ws.um[__popc(un0) + __popc(un1 & below)] = lane + 32;
  const int n_un = __popc(un0) + __popc(un1);
  __syncwarp();
  bool fresh[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int s = lane + 32 * h;
    const int rk = h == 0 ? __popc(fr0 & below) : __popc(fr0) + __popc(fr1 & below);
    fresh[h] = !keep[h] && rk < n_un;
    if (fresh[h]) {
      const int id = ws.newi[ws.um[rk]];
      ws.sidx[s] = id;
#pragma unroll
      for (int d = 0; d < D; ++d) ws.P[d * NS + s] = coord[d][id];
      const double dg = m.c0 + (a.meas_err ? a.meas_err[id] : 0.0);
      ws.cs[pk(s, s)] = dg;
    } else if (!keep[h]) {
      ws.sidx[s] = -1;
    }
  }
  const unsigned ac0 = __ballot_sync(0xffffffffu, keep[0] || fresh[0]);
  const unsigned ac1 = __ballot_sync(0xffffffffu, keep[1] || fresh[1]);
  const unsigned fs0 = __ballot_sync(0xffffffffu, fresh[0]);
  const unsigned fs1 = __ballot_sync(0xffffffffu, fresh[1]);
  const unsigned long long mfresh = (unsigned long long)fs0 | ((unsigned long long)fs1 << 32);
  if (keep[0] || fresh[0]) ws.act[__popc(ac0 & below)] = lane;
  if (keep[1] || fresh[1]) ws.act[__popc(ac0) + __popc(ac1 & below)] = lane + 32;
  if (fresh[0]) ws.frl[__popc(fs0 & below)] = lane;
  if (fresh[1]) ws.frl[__popc(fs0) + __popc(fs1 & below)] = lane + 32;
  const int nfresh = __popc(fs0) + __popc(fs1);
  __syncwarp();
  auto put = [&](int e, double v) { ws.cs[e] = v; };
  auto cov_slots = [&](int s0, int u0) {
    double h[3];
#pragma unroll
    for (int d = 0; d < D; ++d) h[d] = ws.P[d * NS + s0] - ws.P[d * NS + u0];
    return cov_fp64x<D>(m, h, et);
  };
  if (2 * nfresh >= n) {
    for_pairs2(n, lane, 32, [&](int i0, int j0, int i1, int j1, bool two) {
      const int s0 = ws.act[i0], u0 = ws.act[j0], s1 = ws.act[i1], u1 = ws.act[j1];
      const double c0 = cov_slots(s0, u0);
      const double c1 = cov_slots(s1, u1);
      put(pk(s0, u0), c0);  // act ascending: s > u
      if (two) put(pk(s1, u1), c1);
    });
  } else {
    const int np = nfresh * n;
    for (int e = lane; e < np; e += 32) {
      const int f = e / n, c = e - f * n;
      const int s0 = ws.frl[f], u0 = ws.act[c];
      if (u0 != s0 && (!((mfresh >> u0) & 1ull) || u0 < s0)) {
        const double cv = cov_slots(s0, u0);
        put(s0 > u0 ? pk(s0, u0) : pk(u0, s0), cv);
      }
    }
  }
  __syncwarp();
}

template <int D>
__global__ void __launch_bounds__(kCholWarps * 32)
    krige_chol_kernel(KrigeArgs a, DevModel m, Exp64Table et_g, uint8_t* flag, int Mmax,
                      double* cs_scratch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ Exp64Table et;
  for (int q = threadIdx.x; q < 64; q += blockDim.x) {
    et.hi[q] = et_g.hi[q];
    et.lo[q] = et_g.lo[q];
  }
  if (threadIdx.x == 0) {
    et.l1 = et_g.l1;
    et.l2 = et_g.l2;
    et.inv = et_g.inv;
  }
  const CholLayout L = chol_layout(Mmax, D);
  // pairs (i, j), 1 <= j <= i < Mmax, j descending: packed index << 16 | i << 8 | j
  uint32_t* ptab = reinterpret_cast<uint32_t*>(smem_raw + L.off_ptab);
  for (int j = 1; j < Mmax; ++j) {
    const int off = ((Mmax - 1 - j) * (Mmax - j)) >> 1;
    for (int i = j + threadIdx.x; i < Mmax; i += blockDim.x)
      ptab[off + i - j] = ((uint32_t)pk(i, j) << 16) | ((uint32_t)i << 8) | (uint32_t)j;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* wb = smem_raw + L.off_warp + (size_t)warp * L.warp_bytes;
  constexpr int NS = GS_MIXED_MAX_NEIGHBORS;
  double* A = reinterpret_cast<double*>(wb + L.off_a);
  // slot covariances, packed (this warp's part of the global scratch)
  double* Cs = cs_scratch + ((int64_t)blockIdx.x * kCholWarps + warp) * kCholSlotDoubles;
  double* lsc = reinterpret_cast<double*>(wb + L.off_lsc);
  double* lun = reinterpret_cast<double*>(wb + L.off_lun);
  double* P = reinterpret_cast<double*>(wb + L.off_v);  // P[d * NS + s]: slot s's coordinates
  int* sidx = reinterpret_cast<int*>(wb + L.off_idx);   // data point in slot s, or -1
  int* newi = sidx + NS;                                 // this target's neighbours
  int* mt = newi + NS;                                   // neighbour q already in a slot
  int* um = mt + NS;                                     // k-th unplaced neighbour
  int* act = um + NS;                                    // system row r -> slot (ascending)
  int* frl = act + NS;                                   // newly filled slots (ascending)
  const WarpSlots ws{sidx, newi, mt, um, act, frl, P, Cs};
  const double* coord[3] = {a.x, a.y, a.z};
  const double kNaN = __longlong_as_double(0x7ff8000000000000ll);
  const int p = a.p;
  const int q = p + 2;
  sidx[lane] = -1;
  sidx[lane + 32] = -1;
  __syncwarp();
  const int64_t ntl = a.ntl_dev ? *a.ntl_dev : a.ntl;
  // each warp walks runs of consecutive list entries: neighbouring targets
  // share most neighbours, whose slots keep their covariances (only pairs
  // with a newly placed point are evaluated)
  const int64_t nwarps = (int64_t)gridDim.x * kCholWarps;
  const int64_t run = ntl >= 64 * nwarps ? 64 : (ntl + nwarps - 1) / nwarps;
  for (int64_t r0 = ((int64_t)blockIdx.x * kCholWarps + warp) * run; r0 < ntl; r0 += nwarps * run) {
  const int64_t r1 = r0 + run < ntl ? r0 + run : ntl;
  for (int64_t it = r0; it < r1; ++it) {
    const int64_t t = a.tlist ? a.tlist[it] : it;
    const int n = a.nbc[t];
    // only systems the mixed kernel flagged arrive; those outside this
    // kernel's bounds stay flagged for the LU solver
    if (n < 1 || n < p || n > NS || p > GS_MIXED_MAX_DRIFT || n + q > Mmax) continue;
    const int o = Mmax - (n + q);  // frame offset of the system
    const int ic = o + n;           // row of c; F at ic + 1 .. ic + p; z at ic + p + 1
    const int iz = ic + p + 1;
    const double tp[3] = {a.tx[t], a.ty[t], D == 3 ? a.tz[t] : 0.0};
    const int32_t* nbt = a.nb + t * (int64_t)a.kout;
    slots_update<D>(ws, a, m, et, nbt, n, lane);
    // --- the system in slot order, embedded at the frame's bottom right
    for (int e = lane; e < (n * (n + 1)) >> 1; e += 32) {
      int r = 0;
      {
        // row of packed entry e: the largest r with r (r + 1) / 2 <= e
        r = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
        while ((r * (r + 1)) >> 1 > e) --r;
        while (((r + 1) * (r + 2)) >> 1 <= e) ++r;
      }
      const int c = e - ((r * (r + 1)) >> 1);
      A[pk(o + r, o + c)] = Cs[pk(act[r], act[c])];
    }
    const double* trow = a.tdrift ? a.tdrift + t * a.nv : nullptr;
    double scale = 0.0;
    for (int r = lane; r < n; r += 32) {
      const int s = act[r];
      const int idx = sidx[s];
      scale = fmax(scale, Cs[pk(s, s)]);
      const double pt[3] = {P[s], P[NS + s], D == 3 ? P[2 * NS + s] : 0.0};
      const double h[3] = {pt[0] - tp[0], pt[1] - tp[1], pt[2] - tp[2]};
      A[pk(ic, o + r)] = cov_fp64x<D>(m, h, et);
      for (int k = 0; k < p; ++k)
        A[pk(ic + 1 + k, o + r)] =
            basis_at<D>(a, pt, a.drift ? a.drift + (int64_t)idx * a.nv : nullptr, k);
      A[pk(iz, o + r)] = a.method == GS_SIMPLE ? a.val[idx] - a.sk_mean : a.val[idx];
    }
    // the border block: C(0), the target's drift bases, zeros
    for (int r = lane; r < q; r += 32) {
      for (int c = 0; c <= r; ++c) {
        double v = 0.0;
        if (r == 0) v = m.c0;
        else if (c == 0 && r <= p) v = basis_at<D>(a, tp, trow, r - 1);
        A[pk(ic + r, ic + c)] = v;
      }
    }
    scale = warp_max_d(scale);
    int ex = 0;
    frexp(scale, &ex);
    const double sc = ldexp(1.0, -ex);
    const bool scaled = !(scale > 1e-20 && scale < 1e20);  // pivots then fit FP32
    const double tol = kCholPivotTol * scale;
    __syncwarp();
    bool ok = true;
    for (int k = o; k < ic; ++k) {
      const double d = A[pk(k, k)];
      if (!(d > tol)) {  // the same value in every lane
        ok = false;
        break;
      }
      const double r = rcp_fp64(d, sc, scaled);
      for (int i = k + 1 + lane; i < Mmax; i += 32) {
        const double v = A[pk(i, k)];
        lun[i] = v;
        lsc[i] = v * r;
      }
      __syncwarp();
      const int T = ((Mmax - 1 - k) * (Mmax - k)) >> 1;
      // pairs are distinct, so four of them are loaded before any store
      int e = lane;
      for (; e + 96 < T; e += 128) {
        uint32_t en[4];
        double av[4], lv[4], uv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) en[u] = ptab[e + 32 * u];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          av[u] = A[en[u] >> 16];
          lv[u] = lsc[(en[u] >> 8) & 255u];
          uv[u] = lun[en[u] & 255u];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) A[en[u] >> 16] = fma(-lv[u], uv[u], av[u]);
      }
      for (; e < T; e += 32) {
        const uint32_t en = ptab[e];
        const int pe = (int)(en >> 16), i = (int)((en >> 8) & 255u), j = (int)(en & 255u);
        A[pe] = fma(-lsc[i], lun[j], A[pe]);
      }
      __syncwarp();
    }
    if (ok && lane == 0) {
      const double Tcc = A[pk(ic, ic)], Tzc = A[pk(iz, ic)];
      double v, var, lag = kNaN;
      if (p == 0) {
        v = a.sk_mean - Tzc;
        var = Tcc;
      } else {
        // S mu = g, S = -T_FF, g = -T_Fc, by LDL^T (p <= GS_MIXED_MAX_DRIFT)
        double S[GS_MIXED_MAX_DRIFT * (GS_MIXED_MAX_DRIFT + 1) / 2], g[GS_MIXED_MAX_DRIFT];
        double smax = 0.0;
        for (int k = 0; k < p; ++k) {
          g[k] = -A[pk(ic + 1 + k, ic)];
          for (int l = 0; l <= k; ++l) S[pk(k, l)] = -A[pk(ic + 1 + k, ic + 1 + l)];
          smax = fmax(smax, fabs(S[pk(k, k)]));
        }
        for (int k = 0; k < p && ok; ++k) {
          const double d = S[pk(k, k)];
          if (!(d > kCholPivotTol * smax)) {
            ok = false;
            break;
          }
          // rows from the bottom up, so column k still holds S's values
          // (not multipliers) when the rows above use them
          for (int i = p - 1; i > k; --i) {
            const double l = S[pk(i, k)] / d;
            for (int j = k + 1; j <= i; ++j) S[pk(i, j)] -= l * S[pk(j, k)];
            g[i] -= l * g[k];
            S[pk(i, k)] = l;
          }
        }
        if (ok) {
          // back substitution with L^T D: mu_k = g_k / d_k - sum_{i>k} l_ik mu_i
          double mu[GS_MIXED_MAX_DRIFT];
          for (int k = p - 1; k >= 0; --k) {
            double s = g[k] / S[pk(k, k)];
            for (int i = k + 1; i < p; ++i) s -= S[pk(i, k)] * mu[i];
            mu[k] = s;
          }
          v = -Tzc;
          var = Tcc;
          for (int k = 0; k < p; ++k) {
            v = fma(A[pk(iz, ic + 1 + k)], mu[k], v);
            var = fma(-A[pk(ic + 1 + k, ic)], mu[k], var);
          }
          lag = mu[0];
        }
      }
      if (ok) {
        a.out_v[t] = v;
        a.out_var[t] = fmax(var, 0.0);
        if (a.out_lag) a.out_lag[t] = lag;
        a.out_st[t] = GS_ST_OK | GS_ST_FP64_RESOLVED;
        flag[t] = 0;
      }
    }
    __syncwarp();
  }
  }
}

// ------------------------------------------------------------- FP64 path --
template <int D>
__global__ void __launch_bounds__(128) krige_fp64_kernel(KrigeArgs a, DevModel m, double* scratch,
                                                         int64_t T) {
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (tid >= T) return;
  const int NMAX = a.nmax;
  // element e of this thread's slab lives at S[e * T]
  double* S = scratch + tid;
  auto AT = [&](int r, int c, int N) -> double& { return S[(int64_t)(r * N + c) * T]; };
  double* Bv = scratch + (int64_t)NMAX * NMAX * T + tid;  // rhs / solution
  double* B0 = Bv + (int64_t)NMAX * T;                     // original rhs
  const double kNaN = __longlong_as_double(0x7ff8000000000000ll);
  const int64_t ntl = a.ntl_dev ? *a.ntl_dev : a.ntl;
  for (int64_t it = tid; it < ntl; it += T) {
    const int64_t t = a.tlist ? a.tlist[it] : it;
    const int n = a.nbc[t];
    const int p = a.p;
    uint8_t st = GS_ST_OK;
    if (n < 0) st = GS_ST_CAPACITY;
    else if (n < a.min_nb) st = GS_ST_NO_NEIGHBORS;
    else if (n < p) st = GS_ST_INSUFFICIENT_DATA;
    else if (n + p > NMAX) st = GS_ST_CAPACITY;
    const uint8_t fb = a.tlist ? GS_ST_FP64_RESOLVED : 0;
    if (st != GS_ST_OK) {
      a.out_v[t] = kNaN;
      a.out_var[t] = kNaN;
      if (a.out_lag) a.out_lag[t] = kNaN;
      a.out_st[t] = st;
      continue;
    }
    const int N = n + p;
    const int32_t* nbt = a.nb + t * (int64_t)a.kout;
    double tp[3] = {a.tx[t], a.ty[t], D == 3 ? a.tz[t] : 0.0};
    // build_lhs (kriging.rs:527-567)
    for (int r = 0; r < N; ++r)
      for (int c = 0; c < N; ++c) AT(r, c, N) = 0.0;
    for (int ii = 0; ii < n; ++ii) {
      const int i = nbt[ii];
      double pi[3] = {a.x[i], a.y[i], D == 3 ? a.z[i] : 0.0};
      AT(ii, ii, N) = m.c0 + (a.meas_err ? a.meas_err[i] : 0.0);
      for (int jj = ii + 1; jj < n; ++jj) {
        const int j = nbt[jj];
        double h[3] = {pi[0] - a.x[j], pi[1] - a.y[j], D == 3 ? pi[2] - a.z[j] : 0.0};
        const double c = cov_fp64<D>(m, h);
        AT(ii, jj, N) = c;
        AT(jj, ii, N) = c;
      }
      if (p > 0) {
        double f[GS_MIXED_MAX_DRIFT];
        fill_basis<D>(a, pi, a.drift ? a.drift + (int64_t)i * a.nv : nullptr, f);
        for (int k = 0; k < p; ++k) {
          AT(ii, n + k, N) = f[k];
          AT(n + k, ii, N) = f[k];
        }
      }
      double bi;
      if (a.nboff > 0) {
        // point-to-block covariance: the mean over the discretisation
        // points centre + offset (kriging.rs:726-735)
        double s = 0.0;
        for (int u = 0; u < a.nboff; ++u) {
          double h[3] = {0.0, 0.0, 0.0};
#pragma unroll
          for (int d = 0; d < D; ++d) h[d] = pi[d] - (tp[d] + a.boff[u * D + d]);
          s += cov_fp64<D>(m, h);
        }
        bi = s / (double)a.nboff;
      } else {
        double h[3] = {pi[0] - tp[0], pi[1] - tp[1], D == 3 ? pi[2] - tp[2] : 0.0};
        bi = cov_fp64<D>(m, h);
      }
      Bv[(int64_t)ii * T] = bi;
      B0[(int64_t)ii * T] = bi;
    }
    if (p > 0) {
      double f[GS_MIXED_MAX_DRIFT];
      fill_basis<D>(a, tp, a.tdrift ? a.tdrift + t * a.nv : nullptr, f);
      for (int k = 0; k < p; ++k) {
        Bv[(int64_t)(n + k) * T] = f[k];
        B0[(int64_t)(n + k) * T] = f[k];
      }
    }
    // lu_factor (linalg.rs:27-76) fused with Lu::solve's row swaps
    double scale = 0.0;
    for (int r = 0; r < N; ++r)
      for (int c = 0; c < N; ++c) scale = fmax(scale, fabs(AT(r, c, N)));
    scale = fmax(scale, 2.2250738585072014e-308);
    bool singular = false;
    for (int k = 0; k < N && !singular; ++k) {
      int pv = k;
      double mx = fabs(AT(k, k, N));
      for (int i = k + 1; i < N; ++i) {
        const double v = fabs(AT(i, k, N));
        if (v > mx) {
          mx = v;
          pv = i;
        }
      }
      if (mx < 1e-12 * scale) {
        singular = true;
        break;
      }
      if (pv != k) {
        for (int c = 0; c < N; ++c) {
          const double tmp = AT(k, c, N);
          AT(k, c, N) = AT(pv, c, N);
          AT(pv, c, N) = tmp;
        }
        const double tb = Bv[(int64_t)k * T];
        Bv[(int64_t)k * T] = Bv[(int64_t)pv * T];
        Bv[(int64_t)pv * T] = tb;
      }
      const double pivot = AT(k, k, N);
      for (int i = k + 1; i < N; ++i) {
        const double f = AT(i, k, N) / pivot;
        AT(i, k, N) = f;
        if (f != 0.0)
          for (int c = k + 1; c < N; ++c) AT(i, c, N) -= f * AT(k, c, N);
      }
    }
    if (singular) {
      a.out_v[t] = kNaN;
      a.out_var[t] = kNaN;
      if (a.out_lag) a.out_lag[t] = kNaN;
      a.out_st[t] = GS_ST_SINGULAR | fb;
      continue;
    }
    for (int i = 0; i < N; ++i) {
      double s = Bv[(int64_t)i * T];
      for (int j = 0; j < i; ++j) s -= AT(i, j, N) * Bv[(int64_t)j * T];
      Bv[(int64_t)i * T] = s;
    }
    for (int i = N - 1; i >= 0; --i) {
      double s = Bv[(int64_t)i * T];
      for (int j = i + 1; j < N; ++j) s -= AT(i, j, N) * Bv[(int64_t)j * T];
      Bv[(int64_t)i * T] = s / AT(i, i, N);
    }
    // outputs (kriging.rs:614-643; blocks: C(B,B) in place of c0, 758-778)
    const double c_self = a.nboff > 0 ? *a.cbb : m.c0;
    double v, var, lag = kNaN;
    if (a.method == GS_SIMPLE) {
      v = a.sk_mean;
      double red = 0.0;
      for (int ii = 0; ii < n; ++ii) {
        const double w = Bv[(int64_t)ii * T];
        v += w * (a.val[nbt[ii]] - a.sk_mean);
        red += w * B0[(int64_t)ii * T];
      }
      var = c_self - red;
    } else {
      v = 0.0;
      for (int ii = 0; ii < n; ++ii) v += Bv[(int64_t)ii * T] * a.val[nbt[ii]];
      double red = 0.0;
      for (int i = 0; i < N; ++i) red += Bv[(int64_t)i * T] * B0[(int64_t)i * T];
      var = c_self - red;
      lag = Bv[(int64_t)n * T];
    }
    a.out_v[t] = v;
    a.out_var[t] = fmax(var, 0.0);
    if (a.out_lag) a.out_lag[t] = lag;
    a.out_st[t] = GS_ST_OK | fb;
  }
}

__global__ void route_kernel(const uint8_t* flag, int64_t n, int* route) {
  __shared__ int part[32];
  int c = 0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) c += flag[i] ? 1 : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t tot = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += part[w];
    *route = 4 * tot > 3 * n ? 1 : 0;
  }
}

// ---------------------------------------------------- global neighbourhood --
// Kriging::build's global system (kriging.rs:396-406): build_lhs over all n
// points, factored once by lu_factor (linalg.rs:27-76) on the device; each
// target then only solves with the factors (Lu::solve, linalg.rs:87-111).

// A[i * N + j], i, j < N = n + p (row-major; both triangles).
template <int D>
__global__ void global_lhs_kernel(KrigeArgs a, DevModel m, int N, double* A) {
  const int64_t total = (int64_t)N * N;
  const int n = (int)a.n, p = a.p;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / N), j = (int)(e % N);
    double v = 0.0;
    if (i < n && j < n) {
      if (i == j) {
        v = m.c0 + (a.meas_err ? a.meas_err[i] : 0.0);
      } else {
        const double h[3] = {a.x[i] - a.x[j], a.y[i] - a.y[j], D == 3 ? a.z[i] - a.z[j] : 0.0};
        v = cov_fp64<D>(m, h);
      }
    } else if (i < n || j < n) {
      const int r = i < n ? i : j, q = (i < n ? j : i) - n;
      const double pt[3] = {a.x[r], a.y[r], D == 3 ? a.z[r] : 0.0};
      if (q < p) v = basis_at<D>(a, pt, a.drift ? a.drift + (int64_t)r * a.nv : nullptr, q);
    }
    A[e] = v;
  }
}

// max |A| as the bits of a non-negative double (they order like the values).
__global__ void absmax_kernel(const double* A, int64_t total, unsigned long long* out) {
  double mx = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x)
    mx = fmax(mx, fabs(A[e]));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(mx));
}

// Step k: pivot = first row i >= k with the largest |A[i, k]|; singular (state
// 2) below tol; the rows are swapped in full.  One block.
__global__ void lu_pivot_kernel(double* A, int N, int k, int32_t* piv, int* state,
                                const unsigned long long* scale_bits) {
  if (*state != 0) return;
  __shared__ double sv[32];
  __shared__ int si[32];
  double best = -1.0;
  int bi = N;
  for (int i = k + threadIdx.x; i < N; i += blockDim.x) {
    const double v = fabs(A[(int64_t)i * N + k]);
    if (v > best) {  // ascending i per thread: the first of equal maxima
      best = v;
      bi = i;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ov > best || (ov == best && oi < bi)) {
      best = ov;
      bi = oi;
    }
  }
  if ((threadIdx.x & 31) == 0) {
    sv[threadIdx.x >> 5] = best;
    si[threadIdx.x >> 5] = bi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      if (sv[w] > best || (sv[w] == best && si[w] < bi)) {
        best = sv[w];
        bi = si[w];
      }
    const double scale = fmax(__longlong_as_double((long long)*scale_bits), 2.2250738585072014e-308);
    piv[k] = bi;
    if (best < 1e-12 * scale) *state = 2;
    si[0] = bi;
  }
  __syncthreads();
  if (*state != 0) return;
  const int pr = si[0];
  if (pr != k)
    for (int c = threadIdx.x; c < N; c += blockDim.x) {
      const double t = A[(int64_t)k * N + c];
      A[(int64_t)k * N + c] = A[(int64_t)pr * N + c];
      A[(int64_t)pr * N + c] = t;
    }
}

// Step k: multipliers f_i = A[i, k] / A[k, k] stored in place (rows > k).
__global__ void lu_scale_kernel(double* A, int N, int k, const int* state) {
  if (*state != 0) return;
  const double pivot = A[(int64_t)k * N + k];
  for (int i = k + 1 + blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    A[(int64_t)i * N + k] = A[(int64_t)i * N + k] / pivot;
}

// Step k: trailing update A[i, c] -= f_i A[k, c] for rows i > k with f_i != 0.
__global__ void lu_update_kernel(double* A, int N, int k, const int* state) {
  if (*state != 0) return;
  const int i = k + 1 + blockIdx.y;
  const double f = A[(int64_t)i * N + k];
  if (f == 0.0) return;
  const double* rk = A + (int64_t)k * N;
  double* ri = A + (int64_t)i * N;
  for (int c = k + 1 + blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x)
    ri[c] -= f * rk[c];
}

// One warp per target: the right-hand side (kriging.rs:580-598), Lu::solve
// with the factors (rows permuted by perm, unit-lower forward and upper back
// substitution), outputs as krige_fp64_kernel.  scratch: 2 N doubles per warp.
template <int D>
__global__ void global_solve_kernel(KrigeArgs a, DevModel m, int N, const double* LU,
                                    const int32_t* perm, int state, double* scratch,
                                    int64_t nwarps_scratch) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  if (w0 >= nwarps_scratch) return;
  double* R = scratch + w0 * 2 * (int64_t)N;  // b in system order
  double* Y = R + N;                            // permuted b, then the solution
  const int n = (int)a.n, p = a.p;
  const double kNaN = __longlong_as_double(0x7ff8000000000000ll);
  for (int64_t t = w0; t < a.ntl; t += nw) {
    uint8_t st = GS_ST_OK;
    if (n < a.min_nb) st = GS_ST_NO_NEIGHBORS;
    else if (n < p) st = GS_ST_INSUFFICIENT_DATA;
    else if (state != 1) st = GS_ST_SINGULAR;
    if (st != GS_ST_OK) {
      if (lane == 0) {
        a.out_v[t] = kNaN;
        a.out_var[t] = kNaN;
        if (a.out_lag) a.out_lag[t] = kNaN;
        a.out_st[t] = st;
      }
      continue;
    }
    const double tp[3] = {a.tx[t], a.ty[t], D == 3 ? a.tz[t] : 0.0};
    const double* trow = a.tdrift ? a.tdrift + t * a.nv : nullptr;
    for (int i = lane; i < N; i += 32) {
      double b;
      if (i < n) {
        const double h[3] = {a.x[i] - tp[0], a.y[i] - tp[1], D == 3 ? a.z[i] - tp[2] : 0.0};
        b = cov_fp64<D>(m, h);
      } else {
        b = basis_at<D>(a, tp, trow, i - n);
      }
      R[i] = b;
    }
    __syncwarp();
    for (int i = lane; i < N; i += 32) Y[i] = R[perm[i]];
    __syncwarp();
    // forward: y_i -= sum_{j < i} L_ij y_j (unit lower)
    for (int i = 1; i < N; ++i) {
      const double* Li = LU + (int64_t)i * N;
      double s = 0.0;
      for (int j = lane; j < i; j += 32) s = fma(Li[j], Y[j], s);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) Y[i] -= s;
      __syncwarp();
    }
    // back: y_i = (y_i - sum_{j > i} U_ij y_j) / U_ii
    for (int i = N - 1; i >= 0; --i) {
      const double* Ui = LU + (int64_t)i * N;
      double s = 0.0;
      for (int j = i + 1 + lane; j < N; j += 32) s = fma(Ui[j], Y[j], s);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) Y[i] = (Y[i] - s) / Ui[i];
      __syncwarp();
    }
    // outputs (kriging.rs:614-643)
    double v = 0.0, red = 0.0;
    if (a.method == GS_SIMPLE) {
      for (int i = lane; i < n; i += 32) {
        v = fma(Y[i], a.val[i] - a.sk_mean, v);
        red = fma(Y[i], R[i], red);
      }
    } else {
      for (int i = lane; i < n; i += 32) v = fma(Y[i], a.val[i], v);
      for (int i = lane; i < N; i += 32) red = fma(Y[i], R[i], red);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v += __shfl_xor_sync(0xffffffffu, v, o);
      red += __shfl_xor_sync(0xffffffffu, red, o);
    }
    if (lane == 0) {
      a.out_v[t] = a.method == GS_SIMPLE ? a.sk_mean + v : v;
      a.out_var[t] = fmax(m.c0 - red, 0.0);
      if (a.out_lag) a.out_lag[t] = a.method == GS_SIMPLE ? kNaN : Y[n];
      a.out_st[t] = GS_ST_OK;
    }
    __syncwarp();
  }
}

// ----------------------------------------- global neighbourhood, GEMM form --
// For a factored global system a predict call's work is one matrix product.
// At build the solves of A x = e_j with the LU factors (one warp per column,
// the substitutions of global_solve_kernel) give R, row j = A^{-1} e_j, so
// x = R^T b for any right-hand side b; R is kept split into FP32 hi / lo
// parts, with lambda = R z (z the data values, or z - mean for simple
// kriging, and 0 on the drift rows) and a = R e_n (the first drift row's
// column).  Per target with right-hand side b (kriging.rs:580-598):
//     estimate  = lambda . b   (+ mean, simple kriging),
//     Lagrange  = a . b,
//     variance  = C(0) - b^T R b,
// the first two as FP64 dot products, the quadratic form through X = R' B
// for a tile of targets, R' the upper triangle of R with its off-diagonal
// entries doubled: a double-float GEMM on the CUDA cores (compensated Dot2
// accumulation in packed FP32x2 arithmetic) whose epilogue forms
// sum_i B_it X_it per row tile; the row tiles' partial sums are added in a
// fixed order.  b^T R b equals b^T x of the reference's solve
// (kriging.rs:614-643: C(0) - w . c - mu . f).

// Column j of A^{-1} for j = w, w + nw, ...: row j of R.
__global__ void global_inverse_kernel(int N, const double* LU, const int32_t* perm, double* R,
                                      double* scratch, int64_t nwarps_scratch) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  if (w0 >= nwarps_scratch) return;
  double* Y = scratch + w0 * (int64_t)N;
  for (int64_t j = w0; j < N; j += nw) {
    for (int i = lane; i < N; i += 32) Y[i] = perm[i] == (int)j ? 1.0 : 0.0;
    __syncwarp();
    for (int i = 1; i < N; ++i) {
      const double* Li = LU + (int64_t)i * N;
      double sum = 0.0;
      for (int q = lane; q < i; q += 32) sum = fma(Li[q], Y[q], sum);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
      if (lane == 0) Y[i] -= sum;
      __syncwarp();
    }
    for (int i = N - 1; i >= 0; --i) {
      const double* Ui = LU + (int64_t)i * N;
      double sum = 0.0;
      for (int q = i + 1 + lane; q < N; q += 32) sum = fma(Ui[q], Y[q], sum);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
      if (lane == 0) Y[i] = (Y[i] - sum) / Ui[i];
      __syncwarp();
    }
    for (int i = lane; i < N; i += 32) R[j * N + i] = Y[i];
    __syncwarp();
  }
}

// lambda = R z (one warp per row), a = R e_n, and R split into hi / lo.
__global__ void global_vectors_kernel(int N, int n, int p, int simple, double mean,
                                      const double* val, const double* R, double* lambda,
                                      double* arow, float* Rh, float* Rl) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = w0; i < N; i += nw) {
    const double* Ri = R + i * N;
    double sum = 0.0;
    for (int j = lane; j < n; j += 32) sum = fma(Ri[j], simple ? val[j] - mean : val[j], sum);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) {
      lambda[i] = sum;
      arow[i] = p > 0 ? Ri[n] : 0.0;
    }
    for (int j = lane; j < N; j += 32) {
      const double r = Ri[j];
      const float h = (float)r;
      Rh[i * N + j] = h;
      Rl[i * N + j] = (float)(r - (double)h);
    }
  }
}

// Right-hand sides of a tile of targets, split: Bh/Bl[i * T + t] (i < N
// system rows, t < T targets of this chunk), with lambda . b and a . b in
// FP64 while b is at hand: a block takes 32 consecutive targets (one per
// lane) and its 8 warps the rows i = w (mod 8); VL[t] = the warps' partial
// sums added in warp order.
template <int D>
__global__ void __launch_bounds__(256) global_rhs_kernel(KrigeArgs a, DevModel m, int N, int64_t T,
                                                        const double* lambda, const double* arow,
                                                        float* Bh, float* Bl, double2* VL) {
  __shared__ double2 part[8][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int n = (int)a.n;
  for (int64_t t0 = (int64_t)blockIdx.x * 32; t0 < T; t0 += (int64_t)gridDim.x * 32) {
    const int64_t t = t0 + lane;
    double v = 0.0, lg = 0.0;
    if (t < T) {
      const double tp[3] = {a.tx[t], a.ty[t], D == 3 ? a.tz[t] : 0.0};
      const double* trow = a.tdrift ? a.tdrift + t * a.nv : nullptr;
      for (int i = w; i < N; i += 8) {
        double b;
        if (i < n) {
          const double h[3] = {a.x[i] - tp[0], a.y[i] - tp[1], D == 3 ? a.z[i] - tp[2] : 0.0};
          b = cov_fp64<D>(m, h);
        } else {
          b = basis_at<D>(a, tp, trow, i - n);
        }
        const float h = (float)b;
        Bh[(int64_t)i * T + t] = h;
        Bl[(int64_t)i * T + t] = (float)(b - (double)h);
        v = fma(lambda[i], b, v);
        lg = fma(arow[i], b, lg);
      }
    }
    part[w][lane] = make_double2(v, lg);
    __syncthreads();
    if (w == 0 && t < T) {
      double2 sum = part[0][lane];
      for (int u = 1; u < 8; ++u) {
        sum.x += part[u][lane].x;
        sum.y += part[u][lane].y;
      }
      VL[t] = sum;
    }
    __syncthreads();
  }
}

// Tiles of the quadratic form: block (bx, by) multiplies rows
// [64 by, 64 by + 64) of R with the targets [64 bx, 64 bx + 64) of B over
// the columns from 64 by on, 16 columns per stage, each thread a 4 x 4 block of X in
// double-float (two FP32x2 accumulator pairs per row, compensated), and
// writes sum_i B_it X_it over its row tile to Q[by * T + t] (hi, lo).  The
// stages are double-buffered in shared memory: the next stage's entries are
// loaded into registers while the current one is multiplied, so one barrier
// per stage and no wait on the loads before the products.
constexpr int kGT = 64;   // rows / targets per tile
constexpr int kGK = 16;   // columns per stage
constexpr int kGE = kGT * kGK / 256;  // entries of each tile a thread stages
__global__ void __launch_bounds__(256, 2) global_quad_kernel(int N, int64_t T, const float* Rh,
                                                            const float* Rl, const float* Bh,
                                                            const float* Bl, df* Q) {
  __shared__ __align__(16) float Ms[2][2][kGK][kGT + 4];  // [stage buffer][hi, lo]
  __shared__ __align__(16) float Bs[2][2][kGK][kGT + 4];
  __shared__ df red[16][kGT];
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  const int64_t i0 = (int64_t)blockIdx.y * kGT, t0 = (int64_t)blockIdx.x * kGT;
  float2 s[4][2], c[4][2];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      s[r][q] = make_float2(0.0f, 0.0f);
      c[r][q] = make_float2(0.0f, 0.0f);
    }
  // R is symmetric up to rounding, so b^T R b = sum_i R_ii b_i^2 +
  // 2 sum_(i<k) R_ik b_i b_k: columns from the diagonal tile on, with the
  // entries left of the diagonal weighted 0 and those right of it 2 (exact
  // scalings) -- half the products of the full form
  float mh[kGE], ml[kGE], bh[kGE], bl[kGE];
  // entries of stage k0 into registers: thread tid holds entries tid + 256 j
  // of the row tile (row r = e / kGK, column kk = e % kGK) and of the target
  // tile (column kk = e / kGT, target tt = e % kGT); zero outside R's upper
  // triangle and outside the matrices
  auto fetch = [&](int k0) {
#pragma unroll
    for (int j = 0; j < kGE; ++j) {
      const int e = tid + 256 * j;
      const int64_t gi = i0 + e / kGK;
      const int gk = k0 + e % kGK;
      const bool in = gi < N && gk < N && gk >= gi;
      mh[j] = in ? Rh[gi * N + gk] : 0.0f;
      ml[j] = in ? Rl[gi * N + gk] : 0.0f;
      const int gkb = k0 + e / kGT;
      const int64_t gt = t0 + e % kGT;
      const bool inb = gkb < N && gt < T;
      bh[j] = inb ? Bh[(int64_t)gkb * T + gt] : 0.0f;
      bl[j] = inb ? Bl[(int64_t)gkb * T + gt] : 0.0f;
    }
  };
  fetch((int)i0);
  int buf = 0;
  for (int k0 = (int)i0; k0 < N; k0 += kGK) {
#pragma unroll
    for (int j = 0; j < kGE; ++j) {
      const int e = tid + 256 * j;
      const int r = e / kGK, kk = e % kGK;
      const float w = k0 + kk == i0 + r ? 1.0f : 2.0f;
      Ms[buf][0][kk][r] = w * mh[j];
      Ms[buf][1][kk][r] = w * ml[j];
      Bs[buf][0][e / kGT][e % kGT] = bh[j];
      Bs[buf][1][e / kGT][e % kGT] = bl[j];
    }
    // a thread stores into this buffer again two stages later, after the
    // next stage's barrier, which every thread reaches only once done here
    __syncthreads();
    if (k0 + kGK < N) fetch(k0 + kGK);
#pragma unroll 4
    for (int kk = 0; kk < kGK; ++kk) {
      const float4 mh4 = *reinterpret_cast<const float4*>(&Ms[buf][0][kk][ty * 4]);
      const float4 ml4 = *reinterpret_cast<const float4*>(&Ms[buf][1][kk][ty * 4]);
      const float4 bh4 = *reinterpret_cast<const float4*>(&Bs[buf][0][kk][tx * 4]);
      const float4 bl4 = *reinterpret_cast<const float4*>(&Bs[buf][1][kk][tx * 4]);
      const float ah[4] = {mh4.x, mh4.y, mh4.z, mh4.w}, al[4] = {ml4.x, ml4.y, ml4.z, ml4.w};
      const float2 bh2[2] = {make_float2(bh4.x, bh4.y), make_float2(bh4.z, bh4.w)};
      const float2 bl2[2] = {make_float2(bl4.x, bl4.y), make_float2(bl4.z, bl4.w)};
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const float2 a2 = make_float2(ah[r], ah[r]), l2 = make_float2(al[r], al[r]);
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const float2 ph = __fmul2_rn(a2, bh2[q]);
          float2 pe = __ffma2_rn(a2, bh2[q], p_neg(ph));
          pe = __ffma2_rn(a2, bl2[q], pe);
          pe = __ffma2_rn(l2, bh2[q], pe);
          const dfp ts = p_two_sum(s[r][q], ph);
          s[r][q] = ts.hi;
          c[r][q] = p_add(c[r][q], p_add(ts.lo, pe));
        }
      }
    }
    buf ^= 1;
  }
  // epilogue: this thread's rows' contribution sum_r B_(i0+4ty+r),t X_r,t
  df part[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) part[u] = df_make(0.0f, 0.0f);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int64_t gi = i0 + ty * 4 + r;
    if (gi >= N) continue;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const df x0 = fast_two_sum(s[r][q].x, c[r][q].x), x1 = fast_two_sum(s[r][q].y, c[r][q].y);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int u = 2 * q + h;
        const int64_t gt = t0 + tx * 4 + u;
        if (gt >= T) continue;
        const df b = df_make(Bh[gi * T + gt], Bl[gi * T + gt]);
        part[u] = df_add(part[u], df_mul(b, h ? x1 : x0));
      }
    }
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) red[ty][tx * 4 + u] = part[u];
  __syncthreads();
  if (tid < kGT) {
    df sum = red[0][tid];
    for (int w = 1; w < 16; ++w) sum = df_add(sum, red[w][tid]);
    const int64_t gt = t0 + tid;
    if (gt < T) Q[blockIdx.y * T + gt] = sum;
  }
}

// Outputs of a tile of targets: one thread per target; the estimate and
// Lagrange multiplier from VL (lambda . b, a . b), the quadratic form from
// the row tiles' partial sums in tile order.
__global__ void global_finish_kernel(KrigeArgs a, DevModel m, int64_t T, int ntiles,
                                     const double2* VL, const df* Q) {
  const int n = (int)a.n, p = a.p;
  const double kNaN = __longlong_as_double(0x7ff8000000000000ll);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < T;
       t += (int64_t)gridDim.x * blockDim.x) {
    uint8_t st = GS_ST_OK;
    if (n < a.min_nb) st = GS_ST_NO_NEIGHBORS;
    else if (n < p) st = GS_ST_INSUFFICIENT_DATA;
    if (st != GS_ST_OK) {
      a.out_v[t] = kNaN;
      a.out_var[t] = kNaN;
      if (a.out_lag) a.out_lag[t] = kNaN;
      a.out_st[t] = st;
      continue;
    }
    const double2 vl = VL[t];
    df q = Q[t];
    for (int r = 1; r < ntiles; ++r) q = df_add(q, Q[(int64_t)r * T + t]);
    a.out_v[t] = a.method == GS_SIMPLE ? a.sk_mean + vl.x : vl.x;
    a.out_var[t] = fmax(m.c0 - df_to_double(q), 0.0);
    if (a.out_lag) a.out_lag[t] = a.method == GS_SIMPLE ? kNaN : vl.y;
    a.out_st[t] = GS_ST_OK;
  }
}

template <int D>
__global__ void grid_centers_kernel(double x0, double y0, double z0, double dx, double dy,
                                    double dz, int64_t nx, int64_t ny, int64_t total, double* x,
                                    double* y, double* z) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ix = i % nx;
    const int64_t iy = (i / nx) % ny;
    const int64_t iz = i / (nx * ny);
    x[i] = x0 + ((double)ix + 0.5) * dx;
    y[i] = y0 + ((double)iy + 0.5) * dy;
    if (D == 3) z[i] = z0 + ((double)iz + 0.5) * dz;
  }
}

}  // namespace

static ExpTable g_tab;
static DfConsts g_kc;
static std::once_flag g_tab_once;

static Exp64Table g_et;

static void ensure_tables() {
  std::call_once(g_tab_once, [] {
    df_consts_host(&g_tab, &g_kc);
    exp64_table_host(&g_et);
  });
}

template <int D, int R, int PC, int S>
static int launch_rows(const KrigeArgs& a, const DevModel& m, uint8_t* flag, int nf,
                       cudaStream_t stream) {
  const RowsLayout lay = rows_layout(R, PC, nf, D);
  const size_t smem = lay.total * S;
  auto kern = krige_rows_kernel<D, R, PC, S>;
  GS_TRY(allow_dynamic_smem((const void*)kern, smem));
  const int sms = sm_count();
  int per_sm = 0;
  GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, R * S, smem));
  per_sm = std::max(per_sm, 1);
  const int run = a.run > 0 ? a.run : kRowsRun;
  const int64_t runs = (a.ntl + run - 1) / run;
  const int blocks = (int)std::max<int64_t>(
      1, std::min<int64_t>((runs + S - 1) / S, (int64_t)sms * per_sm));
  kern<<<blocks, R * S, smem, stream>>>(a, m, g_tab, g_kc, flag);
  GS_CUDA(cudaGetLastError());
  count_launch(1);
  return GS_OK;
}

template <int D, int R, int PC>
static int launch_rows_s(const KrigeArgs& a, const DevModel& m, uint8_t* flag, int nf,
                         cudaStream_t stream) {
  return a.spc == 2 ? launch_rows<D, R, PC, 2>(a, m, flag, nf, stream)
                    : launch_rows<D, R, PC, 1>(a, m, flag, nf, stream);
}

int krige_mixed_launch(const KrigeArgs& a, const DevModel& m, uint8_t* flag, int force_rows,
                       cudaStream_t stream) {
  if (a.ntl == 0) return GS_OK;
  ensure_tables();
  int nf = 1;
  for (int s = 0; s < m.ns; ++s) nf += m.s[s].aniso ? 1 : 0;
  const int nb = a.nmax - a.p;  // neighbour slots
  const bool small = force_rows ? force_rows == 32 : nb <= 32;
  const bool wide = a.p > 4;
  if (a.dim == 2) {
    if (small) return wide ? launch_rows_s<2, 32, 12>(a, m, flag, nf, stream)
                           : launch_rows_s<2, 32, 4>(a, m, flag, nf, stream);
    return wide ? launch_rows_s<2, 64, 12>(a, m, flag, nf, stream)
                : launch_rows_s<2, 64, 4>(a, m, flag, nf, stream);
  }
  if (small) return wide ? launch_rows_s<3, 32, 12>(a, m, flag, nf, stream)
                         : launch_rows_s<3, 32, 4>(a, m, flag, nf, stream);
  return wide ? launch_rows_s<3, 64, 12>(a, m, flag, nf, stream)
              : launch_rows_s<3, 64, 4>(a, m, flag, nf, stream);
}

template <int D>
static int launch_chol(const KrigeArgs& a, const DevModel& m, uint8_t* flag, int Mmax,
                       double* cs_scratch, int64_t scratch_warps, cudaStream_t stream) {
  const CholLayout lay = chol_layout(Mmax, D);
  auto kern = krige_chol_kernel<D>;
  GS_TRY(allow_dynamic_smem((const void*)kern, lay.total));
  const int sms = sm_count();
  int per_sm = 0;
  GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCholWarps * 32, lay.total));
  per_sm = std::max(per_sm, 1);
  const int blocks = (int)std::min<int64_t>(
      std::min<int64_t>((a.ntl + kCholWarps - 1) / kCholWarps, (int64_t)sms * per_sm),
      scratch_warps / kCholWarps);
  if (blocks < 1) return fail(GS_ERR_INVALID_PARAMETER, "re-solve scratch too small");
  kern<<<blocks, kCholWarps * 32, lay.total, stream>>>(a, m, g_et, flag, Mmax, cs_scratch);
  GS_CUDA(cudaGetLastError());
  count_launch(1);
  return GS_OK;
}

int route_launch(const uint8_t* flag, int64_t n, int* route, cudaStream_t stream) {
  route_kernel<<<1, 256, 0, stream>>>(flag, n, route);
  GS_CUDA(cudaGetLastError());
  count_launch(1);
  return GS_OK;
}

int64_t chol_scratch_doubles(int64_t warps) { return warps * kCholSlotDoubles; }

int krige_chol_launch(const KrigeArgs& a, const DevModel& m, uint8_t* flag, double* scratch,
                      int64_t scratch_warps, cudaStream_t stream) {
  if (a.ntl == 0) return GS_OK;
  ensure_tables();
  const int Mmax = std::min(a.kout, GS_MIXED_MAX_NEIGHBORS) + a.p + 2;
  if (a.dim == 2) return launch_chol<2>(a, m, flag, Mmax, scratch, scratch_warps, stream);
  return launch_chol<3>(a, m, flag, Mmax, scratch, scratch_warps, stream);
}

int global_factor(const KrigeArgs& a, const DevModel& m, int N, double* A, int32_t* piv,
                  int* state_out, cudaStream_t stream) {
  NvtxRange nvtx_range("gs.global_factor");
  DevBuf st, sc;
  GS_TRY(st.alloc(sizeof(int), stream));
  GS_TRY(sc.alloc(sizeof(unsigned long long), stream));
  GS_CUDA(cudaMemsetAsync(st.ptr, 0, sizeof(int), stream));
  GS_CUDA(cudaMemsetAsync(sc.ptr, 0, sizeof(unsigned long long), stream));
  const int64_t total = (int64_t)N * N;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)sm_count() * 16);
  if (a.dim == 2) global_lhs_kernel<2><<<blocks, 256, 0, stream>>>(a, m, N, A);
  else global_lhs_kernel<3><<<blocks, 256, 0, stream>>>(a, m, N, A);
  absmax_kernel<<<blocks, 256, 0, stream>>>(A, total, (unsigned long long*)sc.ptr);
  GS_CUDA(cudaGetLastError());
  int* dstate = (int*)st.ptr;
  for (int k = 0; k < N; ++k) {
    lu_pivot_kernel<<<1, 1024, 0, stream>>>(A, N, k, piv, dstate, (const unsigned long long*)sc.ptr);
    const int rows = N - 1 - k;
    if (rows > 0) {
      lu_scale_kernel<<<(rows + 255) / 256, 256, 0, stream>>>(A, N, k, dstate);
      const int cols = N - 1 - k;
      dim3 grid((unsigned)std::min((cols + 127) / 128, 8), (unsigned)rows);
      lu_update_kernel<<<grid, 128, 0, stream>>>(A, N, k, dstate);
    }
  }
  GS_CUDA(cudaGetLastError());
  count_launch(2 + 3 * N);
  int state = 0;
  GS_CUDA(cudaMemcpyAsync(&state, dstate, sizeof(int), cudaMemcpyDeviceToHost, stream));
  GS_CUDA(cudaStreamSynchronize(stream));
  *state_out = state == 0 ? 1 : 2;
  return GS_OK;
}

int global_solve_launch(const KrigeArgs& a, const DevModel& m, int N, const double* LU,
                        const int32_t* perm, int state, double* scratch, int64_t scratch_warps,
                        cudaStream_t stream) {
  if (a.ntl == 0) return GS_OK;
  const int64_t warps = std::min<int64_t>(scratch_warps, a.ntl);
  const int blocks = (int)((warps * 32 + 127) / 128);
  if (a.dim == 2)
    global_solve_kernel<2><<<blocks, 128, 0, stream>>>(a, m, N, LU, perm, state, scratch, warps);
  else
    global_solve_kernel<3><<<blocks, 128, 0, stream>>>(a, m, N, LU, perm, state, scratch, warps);
  GS_CUDA(cudaGetLastError());
  count_launch(1);
  return GS_OK;
}

int global_gemm_prepare(const KrigeArgs& a, int N, const double* LU, const int32_t* perm,
                        float* Rh, float* Rl, double* lambda, double* arow, cudaStream_t stream) {
  NvtxRange nvtx_range("gs.global_gemm_prepare");
  DevBuf R, scratch;
  GS_TRY(R.alloc((size_t)N * N * 8, stream));
  const int64_t warps = std::max<int64_t>(
      1, std::min<int64_t>({(int64_t)sm_count() * 32, (int64_t)N, ((int64_t)512 << 20) / (8 * (int64_t)N)}));
  GS_TRY(scratch.alloc((size_t)warps * N * 8, stream));
  global_inverse_kernel<<<(int)((warps * 32 + 127) / 128), 128, 0, stream>>>(
      N, LU, perm, (double*)R.ptr, (double*)scratch.ptr, warps);
  GS_CUDA(cudaGetLastError());
  const int64_t vw = std::min<int64_t>((int64_t)N, (int64_t)sm_count() * 32);
  global_vectors_kernel<<<(int)((vw * 32 + 127) / 128), 128, 0, stream>>>(
      N, (int)a.n, a.p, a.method == GS_SIMPLE ? 1 : 0, a.sk_mean, a.val, (const double*)R.ptr,
      lambda, arow, Rh, Rl);
  GS_CUDA(cudaGetLastError());
  count_launch(2);
  GS_CUDA(cudaStreamSynchronize(stream));
  return GS_OK;
}

int global_gemm_launch(const KrigeArgs& a, const DevModel& m, int N, const float* Rh,
                       const float* Rl, const double* lambda, const double* arow,
                       cudaStream_t stream) {
  if (a.ntl == 0) return GS_OK;
  // targets per chunk: the split right-hand sides within 1 GiB
  int64_t T = std::min<int64_t>(a.ntl, std::max<int64_t>(kGT, ((int64_t)1 << 30) / (8 * (int64_t)N)));
  const int ntiles = (N + kGT - 1) / kGT;
  DevBuf B, Q;
  GS_TRY(B.alloc((size_t)N * T * 8, stream));
  // Q's row-tile sums, then VL (16-byte aligned)
  const size_t vl_off = ((size_t)ntiles * T * sizeof(df) + 15) & ~(size_t)15;
  GS_TRY(Q.alloc(vl_off + (size_t)T * sizeof(double2), stream));
  float* Bh = (float*)B.ptr;
  float* Bl = Bh + (size_t)N * T;
  double2* VL = (double2*)((char*)Q.ptr + vl_off);
  for (int64_t c0 = 0; c0 < a.ntl; c0 += T) {
    const int64_t tc = std::min<int64_t>(T, a.ntl - c0);
    KrigeArgs ca = a;
    ca.tx += c0;
    ca.ty += c0;
    if (ca.tz) ca.tz += c0;
    if (ca.tdrift) ca.tdrift += c0 * a.nv;
    ca.out_v += c0;
    ca.out_var += c0;
    if (ca.out_lag) ca.out_lag += c0;
    ca.out_st += c0;
    // Bh / Bl laid out with this chunk's count as the row stride
    float* bh = Bh;
    float* bl = Bh + (size_t)N * tc;
    const int rb = (int)std::min<int64_t>((tc + 31) / 32, (int64_t)sm_count() * 8);
    if (a.dim == 2)
      global_rhs_kernel<2><<<rb, 256, 0, stream>>>(ca, m, N, tc, lambda, arow, bh, bl, VL);
    else
      global_rhs_kernel<3><<<rb, 256, 0, stream>>>(ca, m, N, tc, lambda, arow, bh, bl, VL);
    dim3 grid((unsigned)((tc + kGT - 1) / kGT), (unsigned)ntiles);
    global_quad_kernel<<<grid, 256, 0, stream>>>(N, tc, Rh, Rl, bh, bl, (df*)Q.ptr);
    const int64_t fb = std::min<int64_t>((tc + 127) / 128, (int64_t)sm_count() * 16);
    global_finish_kernel<<<(int)fb, 128, 0, stream>>>(ca, m, tc, ntiles, VL, (const df*)Q.ptr);
    GS_CUDA(cudaGetLastError());
    count_launch(3);
  }
  return GS_OK;
}

int64_t fp64_scratch_doubles(int nmax, int64_t threads) {
  return ((int64_t)nmax * nmax + 2 * (int64_t)nmax) * threads;
}

int64_t fp64_threads_for(int nmax, int64_t budget_bytes) {
  const int64_t per = ((int64_t)nmax * nmax + 2 * (int64_t)nmax) * 8;
  int64_t t = budget_bytes / std::max<int64_t>(per, 1);
  t = std::min<int64_t>(t, (int64_t)sm_count() * 1024);
  t = (t / 128) * 128;
  return std::max<int64_t>(t, 128);
}

int krige_fp64_launch(const KrigeArgs& a, const DevModel& m, double* scratch, int64_t threads,
                      cudaStream_t stream) {
  if (a.ntl == 0) return GS_OK;
  const int tpb = 128;
  const int64_t T = ((std::min<int64_t>(threads, std::max<int64_t>(a.ntl, 1)) + tpb - 1) / tpb) * tpb;
  const int64_t Tl = std::min<int64_t>(T, threads);
  const int blocks = (int)((Tl + tpb - 1) / tpb);
  if (a.dim == 2) krige_fp64_kernel<2><<<blocks, tpb, 0, stream>>>(a, m, scratch, Tl);
  else krige_fp64_kernel<3><<<blocks, tpb, 0, stream>>>(a, m, scratch, Tl);
  GS_CUDA(cudaGetLastError());
  count_launch(1);
  return GS_OK;
}

template <int D>
__global__ void block_cbb_kernel(DevModel m, const double* off, int nu, double nugget, double* out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const double c0c = m.c0 - nugget;
  double s = 0.0;
  for (int u = 0; u < nu; ++u)
    for (int v = 0; v < nu; ++v) {
      if (u == v) {
        s += c0c;
      } else {
        double h[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int d = 0; d < D; ++d) h[d] = off[u * D + d] - off[v * D + d];
        s += cov_fp64<D>(m, h);
      }
    }
  const double fn = (double)nu;
  *out = s / (fn * fn);
}

int block_cbb_launch(int dim, const DevModel& m, const double* off, int noff, double nugget,
                     double* out, cudaStream_t stream) {
  if (dim == 2) block_cbb_kernel<2><<<1, 32, 0, stream>>>(m, off, noff, nugget, out);
  else block_cbb_kernel<3><<<1, 32, 0, stream>>>(m, off, noff, nugget, out);
  if (cudaGetLastError() != cudaSuccess) return fail(GS_ERR_CUDA, "block covariance launch failed");
  count_launch(1);
  return GS_OK;
}

int grid_centers_launch(int dim, const double* bmin, const double* step, const int64_t* ncell,
                        double* x, double* y, double* z, cudaStream_t stream) {
  int64_t total = ncell[0] * ncell[1] * (dim == 3 ? ncell[2] : 1);
  if (total == 0) return GS_OK;
  const int tpb = 256;
  const int blocks = (int)std::min<int64_t>((total + tpb - 1) / tpb, (int64_t)sm_count() * 64);
  if (dim == 2)
    grid_centers_kernel<2><<<blocks, tpb, 0, stream>>>(bmin[0], bmin[1], 0.0, step[0], step[1], 0.0,
                                                       ncell[0], ncell[1], total, x, y, z);
  else
    grid_centers_kernel<3><<<blocks, tpb, 0, stream>>>(bmin[0], bmin[1], bmin[2], step[0], step[1],
                                                       step[2], ncell[0], ncell[1], total, x, y, z);
  GS_CUDA(cudaGetLastError());
  return GS_OK;
}

}  // namespace gs
