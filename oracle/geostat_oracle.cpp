// geostat_oracle.cpp -- FP64 CPU restatement of geostat-rs's hot path.
//
// TEST INFRASTRUCTURE ONLY (the parity checker and the timed CPU baseline);
// the product never links or calls this file.
//
// Every function cites the reference file:line it restates (paths relative to
// the geostat-rs workspace).  Arithmetic follows the reference op-for-op:
// left-to-right sums starting from 0.0, no FMA contraction (build with
// -ffp-contract=off), glibc exp/log/sin/cos/sqrt/pow -- the same libm Rust
// calls on Linux.  Parity is pinned by the reference's own known-answer tests
// (gstat rotation golden values, Power-vs-gstat ordinary kriging, LU and
// Cholesky systems, exact-MVN Vecchia, brute-force searches); see tests/.
//
// One documented difference: the kd-tree here splits with std::nth_element
// instead of Rust's select_nth_unstable_by, so when the k-th and (k+1)-th
// candidates tie exactly on squared distance the surviving index may differ
// (the reference keeps whichever its traversal met first).  or_krige counts
// such boundary ties so callers can tell when that can matter.
#include "geostat_oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <queue>
#include <string>
#include <thread>
#include <unordered_map>
#include <utility>
#include <vector>

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

const double kInf = std::numeric_limits<double>::infinity();
const double kNaN = std::numeric_limits<double>::quiet_NaN();
const double kMinPositive = 2.2250738585072014e-308;  // f64::MIN_POSITIVE
const double kPi = 3.14159265358979323846;
const double kRadsPerDeg = kPi / 180.0;  // f64::to_radians constant

inline double to_radians(double deg) { return deg * kRadsPerDeg; }
// f64::max / f64::min: NaN-ignoring, like fmax/fmin.
inline double fmax_(double a, double b) { return std::fmax(a, b); }
inline double fmin_(double a, double b) { return std::fmin(a, b); }

inline uint64_t bits_of(double v) {
  uint64_t u;
  std::memcpy(&u, &v, 8);
  return u;
}
inline double from_bits(uint64_t u) {
  double v;
  std::memcpy(&v, &u, 8);
  return v;
}
// f64::total_cmp as a strict-weak "less".
inline int64_t total_key(double v) {
  int64_t b = (int64_t)bits_of(v);
  b ^= (int64_t)(((uint64_t)(b >> 63)) >> 1);
  return b;
}
inline bool total_lt(double a, double b) { return total_key(a) < total_key(b); }

// ---------------------------------------------------------------------------
// rng.rs:7-79
uint64_t splitmix64(uint64_t& state) {
  state += 0x9E3779B97F4A7C15ull;
  uint64_t z = state;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

struct Rng {
  uint64_t s[4];
  bool has_spare = false;
  double spare = 0.0;
  explicit Rng(uint64_t seed) {
    uint64_t sm = seed;
    for (int i = 0; i < 4; ++i) s[i] = splitmix64(sm);
  }
  uint64_t next_u64() {
    uint64_t result = rotl(s[0] + s[3], 23) + s[0];
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return result;
  }
  double uniform() { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }
  double normal() {
    if (has_spare) {
      has_spare = false;
      return spare;
    }
    for (;;) {
      double u1 = uniform();
      if (u1 > 0.0) {
        double u2 = uniform();
        double r = std::sqrt(-2.0 * std::log(u1));
        double a = 2.0 * kPi * u2;
        double sn = std::sin(a), cs = std::cos(a);
        spare = r * sn;
        has_spare = true;
        return r * cs;
      }
    }
  }
};

// ---------------------------------------------------------------------------
// variogram/model.rs
struct Anis {
  double azimuth_deg, ratio, ratio_z, dip_deg, rake_deg;
};

// model.rs:407-433 rotation_matrix_3d (GSLIB setrot).
void rotation_matrix_3d(const Anis& a, double rot[3][3]) {
  double alpha = (a.azimuth_deg >= 0.0 && a.azimuth_deg < 270.0) ? to_radians(90.0 - a.azimuth_deg)
                                                                 : to_radians(450.0 - a.azimuth_deg);
  double beta = to_radians(-a.dip_deg);
  double theta = to_radians(a.rake_deg);
  double sina = std::sin(alpha), cosa = std::cos(alpha);
  double sinb = std::sin(beta), cosb = std::cos(beta);
  double sint = std::sin(theta), cost = std::cos(theta);
  double afac1 = 1.0 / a.ratio;
  double afac2 = 1.0 / a.ratio_z;
  rot[0][0] = cosb * cosa;
  rot[0][1] = cosb * sina;
  rot[0][2] = -sinb;
  rot[1][0] = afac1 * (-cost * sina + sint * sinb * cosa);
  rot[1][1] = afac1 * (cost * cosa + sint * sinb * sina);
  rot[1][2] = afac1 * (sint * cosb);
  rot[2][0] = afac2 * (sint * sina + cost * sinb * cosa);
  rot[2][1] = afac2 * (-sint * cosa + cost * sinb * sina);
  rot[2][2] = afac2 * (cost * cosb);
}

// model.rs:353-367 transform_vector.
void transform_vector(const Anis& a, int dim, const double* dh, double* out) {
  if (dim == 3) {
    double rot[3][3];
    rotation_matrix_3d(a, rot);
    double h0 = dh[0], h1 = dh[1], h2 = dh[2];
    out[0] = rot[0][0] * h0 + rot[0][1] * h1 + rot[0][2] * h2;
    out[1] = rot[1][0] * h0 + rot[1][1] * h1 + rot[1][2] * h2;
    out[2] = rot[2][0] * h0 + rot[2][1] * h1 + rot[2][2] * h2;
  } else {
    double r = to_radians(a.azimuth_deg);
    double s = std::sin(r), c = std::cos(r);
    out[0] = dh[0] * s + dh[1] * c;
    out[1] = (dh[0] * c - dh[1] * s) / a.ratio;
  }
}

// model.rs:378-405 Anisotropy::validate.
int validate_anis(const Anis& a) {
  if (!(a.ratio_z > 0.0) || !std::isfinite(a.ratio_z))
    return fail(OR_INVALID_PARAMETER, "anisotropy ratio_z must be finite and > 0");
  if (!(a.ratio > 0.0) || !std::isfinite(a.ratio))
    return fail(OR_INVALID_PARAMETER, "anisotropy ratio must be finite and > 0");
  if (!std::isfinite(a.azimuth_deg))
    return fail(OR_INVALID_PARAMETER, "anisotropy azimuth must be finite");
  if (!std::isfinite(a.dip_deg) || !std::isfinite(a.rake_deg))
    return fail(OR_INVALID_PARAMETER, "anisotropy dip/rake must be finite");
  return OR_OK;
}

Anis anis_of(const or_structure& s) {
  return Anis{s.azimuth_deg, s.ratio, s.ratio_z, s.dip_deg, s.rake_deg};
}

// model.rs:122-181 ModelKind::g (unit-sill shapes).  The general Matern
// (Bessel quadrature) is not part of this path.
double kind_g(int kind, double param, double h, double a) {
  double d = h / a;
  switch (kind) {
    case OR_SPHERICAL:
      if (d >= 1.0) return 1.0;
      return 1.5 * d - 0.5 * d * d * d;
    case OR_EXPONENTIAL:
      return 1.0 - std::exp(-d);
    case OR_GAUSSIAN:
      return 1.0 - std::exp(-(d * d));
    case OR_MATERN15: {
      double s = std::sqrt(3.0) * d;
      return 1.0 - (1.0 + s) * std::exp(-s);
    }
    case OR_MATERN25: {
      double s = std::sqrt(5.0) * d;
      return 1.0 - (1.0 + s + s * s / 3.0) * std::exp(-s);
    }
    case OR_CIRCULAR: {
      double dd = fmin_(d, 1.0);
      return 1.0 - (2.0 / kPi) * (std::acos(dd) - dd * std::sqrt(1.0 - dd * dd));
    }
    case OR_STABLE:
      return 1.0 - std::exp(-std::pow(d, param));
    case OR_HOLE:
      if (d <= 0.0) return 0.0;
      return 1.0 - std::sin(d) / d;
    case OR_POWER:
      return std::pow(std::fabs(h), param);
    case OR_WAVE: {
      if (d <= 0.0) return 0.0;
      double pd = kPi * d;
      return 1.0 - std::sin(pd) / pd;
    }
  }
  return kNaN;
}

// model.rs:521-539 Structure::effective_h.
double effective_h(const or_structure& s, int dim, const double* dh) {
  double acc = 0.0;
  if (!s.has_anis) {
    for (int d = 0; d < dim; ++d) acc += dh[d] * dh[d];
    return std::sqrt(acc);
  }
  double e[3];
  transform_vector(anis_of(s), dim, dh, e);
  for (int d = 0; d < dim; ++d) acc += e[d] * e[d];
  return std::sqrt(acc);
}

// model.rs:636-646 gamma_dh.
double gamma_dh(const or_model& m, int dim, const double* dh) {
  bool all_zero = true;
  for (int d = 0; d < dim; ++d)
    if (dh[d] != 0.0) all_zero = false;
  if (all_zero) return 0.0;
  double sum = 0.0;
  for (int k = 0; k < m.n_structures; ++k) {
    const or_structure& s = m.s[k];
    sum += s.sill * kind_g(s.kind, s.param, effective_h(s, dim, dh), s.range);
  }
  return m.nugget + sum;
}

// model.rs:658-660.
double total_sill(const or_model& m) {
  double sum = 0.0;
  for (int k = 0; k < m.n_structures; ++k) sum += m.s[k].sill;
  return m.nugget + sum;
}

bool has_power(const or_model& m) {
  for (int k = 0; k < m.n_structures; ++k)
    if (m.s[k].kind == OR_POWER) return true;
  return false;
}

// model.rs:554-630 VariogramModel::new.
int validate_model(const or_model& m) {
  if (m.n_structures < 0 || m.n_structures > 4)
    return fail(OR_INVALID_PARAMETER, "at most 4 structures are supported");
  if (!(m.nugget >= 0.0) || !std::isfinite(m.nugget))
    return fail(OR_INVALID_PARAMETER, "nugget must be finite and >= 0");
  for (int k = 0; k < m.n_structures; ++k) {
    const or_structure& s = m.s[k];
    if (s.kind < 0 || s.kind > OR_POWER) return fail(OR_INVALID_PARAMETER, "unknown model kind");
    if (!(s.sill >= 0.0) || !std::isfinite(s.sill))
      return fail(OR_INVALID_PARAMETER, "partial sill must be finite and >= 0");
    if (!(s.range > 0.0) || !std::isfinite(s.range))
      return fail(OR_INVALID_PARAMETER, "range must be finite and > 0");
    if (s.kind == OR_STABLE && (!(s.param > 0.0) || s.param > 2.0))
      return fail(OR_INVALID_PARAMETER, "Stable alpha must be in (0, 2]");
    if (s.kind == OR_POWER && (!(s.param > 0.0) || s.param >= 2.0))
      return fail(OR_INVALID_PARAMETER, "Power theta must be in (0, 2)");
    if (s.has_anis) {
      int rc = validate_anis(anis_of(s));
      if (rc) return rc;
    }
  }
  if (!(total_sill(m) > 0.0)) return fail(OR_INVALID_PARAMETER, "total sill must be positive");
  return OR_OK;
}

bool valid_in_dim(const or_model& m, int dim) {
  for (int k = 0; k < m.n_structures; ++k)
    if (m.s[k].kind == OR_CIRCULAR && dim > 2) return false;
  return true;
}

// ---------------------------------------------------------------------------
// linalg.rs
struct Lu {
  std::vector<double> a;  // n x n row-major combined factors
  std::vector<size_t> piv;
  size_t n = 0;
};

// linalg.rs:27-76 lu_factor.
int lu_factor(std::vector<double> a, size_t n, Lu& out) {
  double scale = 0.0;
  for (double v : a) scale = fmax_(scale, std::fabs(v));
  scale = fmax_(scale, kMinPositive);
  std::vector<size_t> piv(n, 0);
  for (size_t k = 0; k < n; ++k) {
    size_t p = k;
    double mx = std::fabs(a[k * n + k]);
    for (size_t i = k + 1; i < n; ++i) {
      double v = std::fabs(a[i * n + k]);
      if (v > mx) {
        mx = v;
        p = i;
      }
    }
    if (mx < 1e-12 * scale) return fail(OR_SINGULAR_SYSTEM, "singular pivot");
    piv[k] = p;
    if (p != k)
      for (size_t j = 0; j < n; ++j) std::swap(a[k * n + j], a[p * n + j]);
    double pivot = a[k * n + k];
    for (size_t i = k + 1; i < n; ++i) {
      double f = a[i * n + k] / pivot;
      a[i * n + k] = f;
      if (f != 0.0)
        for (size_t j = k + 1; j < n; ++j) a[i * n + j] -= f * a[k * n + j];
    }
  }
  out.a = std::move(a);
  out.piv = std::move(piv);
  out.n = n;
  return OR_OK;
}

// linalg.rs:87-111 Lu::solve.
std::vector<double> lu_solve(const Lu& lu, std::vector<double> b) {
  size_t n = lu.n;
  for (size_t k = 0; k < n; ++k) std::swap(b[k], b[lu.piv[k]]);
  for (size_t i = 0; i < n; ++i) {
    double s = b[i];
    for (size_t j = 0; j < i; ++j) s -= lu.a[i * n + j] * b[j];
    b[i] = s;
  }
  for (size_t ii = n; ii-- > 0;) {
    double s = b[ii];
    for (size_t j = ii + 1; j < n; ++j) s -= lu.a[ii * n + j] * b[j];
    b[ii] = s / lu.a[ii * n + ii];
  }
  return b;
}

// linalg.rs:81-83.
double lu_ln_det_abs(const Lu& lu) {
  double s = 0.0;
  for (size_t i = 0; i < lu.n; ++i) s += std::log(std::fabs(lu.a[i * lu.n + i]));
  return s;
}

// linalg.rs:123-156 cholesky_factor_in_place.
int cholesky_factor(double* a, size_t n) {
  double scale = 0.0;
  for (size_t i = 0; i < n; ++i) scale = fmax_(scale, a[i * n + i]);
  scale = fmax_(scale, kMinPositive);
  for (size_t k = 0; k < n; ++k) {
    double d = a[k * n + k];
    for (size_t j = 0; j < k; ++j) d -= a[k * n + j] * a[k * n + j];
    if (!(d > 1e-12 * scale)) return fail(OR_SINGULAR_SYSTEM, "non-positive Cholesky pivot");
    d = std::sqrt(d);
    a[k * n + k] = d;
    for (size_t i = k + 1; i < n; ++i) {
      double s = a[i * n + k];
      for (size_t j = 0; j < k; ++j) s -= a[i * n + j] * a[k * n + j];
      a[i * n + k] = s / d;
    }
  }
  return OR_OK;
}

// linalg.rs:160-180.
void cholesky_forward(const double* a, size_t n, double* b) {
  for (size_t i = 0; i < n; ++i) {
    double s = b[i];
    for (size_t j = 0; j < i; ++j) s -= a[i * n + j] * b[j];
    b[i] = s / a[i * n + i];
  }
}
void cholesky_back(const double* a, size_t n, double* b) {
  for (size_t ii = n; ii-- > 0;) {
    double s = b[ii];
    for (size_t j = ii + 1; j < n; ++j) s -= a[j * n + ii] * b[j];
    b[ii] = s / a[ii * n + ii];
  }
}
// linalg.rs:192-203.
int cholesky_solve(double* a, size_t n, double* b) {
  int rc = cholesky_factor(a, n);
  if (rc) return rc;
  cholesky_forward(a, n, b);
  cholesky_back(a, n, b);
  return OR_OK;
}

// ---------------------------------------------------------------------------
// search.rs:15-36 heap helpers.  Max-heap on (d2 bits, idx).
typedef std::pair<uint64_t, uint32_t> Entry;
typedef std::priority_queue<Entry> Heap;

inline void push_candidate(Heap& heap, size_t k, double d2, uint32_t idx) {
  if (heap.size() < k) {
    heap.push(Entry(bits_of(d2), idx));
  } else if (bits_of(d2) < heap.top().first) {
    heap.push(Entry(bits_of(d2), idx));
    heap.pop();
  }
}
inline double heap_worst(const Heap& heap, size_t k) {
  return heap.size() == k ? from_bits(heap.top().first) : kInf;
}
std::vector<size_t> into_sorted(Heap heap, std::vector<Entry>* entries = nullptr) {
  std::vector<Entry> v;
  v.reserve(heap.size());
  while (!heap.empty()) {
    v.push_back(heap.top());
    heap.pop();
  }
  std::sort(v.begin(), v.end());
  std::vector<size_t> out(v.size());
  for (size_t i = 0; i < v.size(); ++i) out[i] = v[i].second;
  if (entries) *entries = std::move(v);
  return out;
}

inline double dist2(const double* p, const double* t, int dim) {
  double d2 = 0.0;
  for (int d = 0; d < dim; ++d) {
    double dd = p[d] - t[d];
    d2 += dd * dd;
  }
  return d2;
}

// search.rs:38-113 KdTree.
struct KdTree {
  int dim = 2;
  std::vector<uint32_t> idx;
  std::vector<double> coords;  // n x dim

  void build(const double* c, size_t n, int dim_) {
    dim = dim_;
    coords.assign(c, c + n * dim);
    idx.resize(n);
    for (size_t i = 0; i < n; ++i) idx[i] = (uint32_t)i;
    build_rec(idx.data(), n, 0);
  }
  void build_rec(uint32_t* node, size_t len, int axis) {
    if (len <= 1) return;
    size_t mid = len / 2;
    const double* cs = coords.data();
    int D = dim;
    std::nth_element(node, node + mid, node + len, [cs, D, axis](uint32_t a, uint32_t b) {
      return total_lt(cs[(size_t)a * D + axis], cs[(size_t)b * D + axis]);
    });
    build_rec(node, mid, (axis + 1) % dim);
    build_rec(node + mid + 1, len - mid - 1, (axis + 1) % dim);
  }
  void search(const uint32_t* node, size_t len, int axis, const double* target, size_t k,
              double r2, Heap& heap) const {
    if (len == 0) return;
    size_t mid = len / 2;
    const double* p = &coords[(size_t)node[mid] * dim];
    double d2 = dist2(p, target, dim);
    if (d2 <= r2) push_candidate(heap, k, d2, node[mid]);
    double diff = target[axis] - p[axis];
    const uint32_t *near_, *far_;
    size_t nlen, flen;
    if (diff <= 0.0) {
      near_ = node;
      nlen = mid;
      far_ = node + mid + 1;
      flen = len - mid - 1;
    } else {
      near_ = node + mid + 1;
      nlen = len - mid - 1;
      far_ = node;
      flen = mid;
    }
    search(near_, nlen, (axis + 1) % dim, target, k, r2, heap);
    if (diff * diff <= fmin_(heap_worst(heap, k), r2))
      search(far_, flen, (axis + 1) % dim, target, k, r2, heap);
  }
  std::vector<size_t> k_nearest(const double* target, size_t k, bool has_r, double radius,
                                std::vector<Entry>* entries = nullptr) const {
    if (k == 0 || idx.empty()) return {};
    double r2 = has_r ? radius * radius : kInf;
    Heap heap;
    search(idx.data(), idx.size(), 0, target, k, r2, heap);
    return into_sorted(std::move(heap), entries);
  }
};

// search.rs:318-349 k_nearest_brute (stable sort on d2 after a select).
std::vector<size_t> knn_brute(const double* coords, size_t n, int dim, const double* target,
                              size_t k, bool has_r, double radius) {
  if (k == 0) return {};
  double r2 = radius * radius;
  std::vector<std::pair<double, size_t>> cand;
  for (size_t i = 0; i < n; ++i) {
    double d2 = dist2(&coords[i * dim], target, dim);
    if (has_r && d2 > r2) continue;
    cand.push_back({d2, i});
  }
  // The reference selects by d2 then sorts by d2 only; with tie-free inputs
  // this equals a (d2, idx) sort, which is what is used here.
  std::stable_sort(cand.begin(), cand.end(),
                   [](const std::pair<double, size_t>& a, const std::pair<double, size_t>& b) {
                     return total_lt(a.first, b.first);
                   });
  if (cand.size() > k) cand.resize(k);
  std::vector<size_t> out;
  for (auto& c : cand) out.push_back(c.second);
  return out;
}

// search.rs:115-313 BucketGrid.
struct BucketGrid {
  int dim = 2;
  double origin[3] = {0, 0, 0};
  double cell = 1.0;
  size_t n[3] = {1, 1, 1};
  size_t strides[3] = {1, 1, 1};
  std::vector<std::vector<uint32_t>> buckets;
  std::vector<double> pts;

  BucketGrid(const double* mn, const double* mx, size_t expected, int dim_) {
    dim = dim_;
    double extents[3];
    double max_extent = 0.0;
    for (int d = 0; d < dim; ++d) {
      extents[d] = mx[d] - mn[d];
      max_extent = fmax_(max_extent, extents[d]);
    }
    double tol = max_extent * 1e-9;
    bool active[3];
    size_t n_active = 0;
    for (int d = 0; d < dim; ++d) {
      active[d] = extents[d] > tol;
      if (active[d]) ++n_active;
    }
    if (n_active == 0) n_active = 1;
    double volume = 1.0;
    for (int d = 0; d < dim; ++d)
      if (active[d]) volume *= extents[d];
    size_t e1 = expected > 0 ? expected : 1;
    cell = fmax_(std::pow(volume, 1.0 / (double)n_active), 1e-12) *
           (1.0 / std::pow((double)e1, 1.0 / (double)n_active));
    size_t cap = std::max<size_t>(e1 > SIZE_MAX / 4 ? SIZE_MAX : e1 * 4, 64);
    for (;;) {
      size_t total = 1;
      bool overflowed = false;
      for (int d = 0; d < dim; ++d) {
        if (active[d]) {
          double c = std::ceil(extents[d] / cell);
          // Rust `as usize` saturates; values here are finite and >= 0.
          size_t v = c >= 1.8446744073709552e19 ? SIZE_MAX : (size_t)c;
          n[d] = std::max<size_t>(v, 1);
        } else {
          n[d] = 1;
        }
        if (n[d] != 0 && total > SIZE_MAX / n[d]) {
          overflowed = true;
          break;
        }
        total *= n[d];
      }
      if (!overflowed && total <= cap) break;
      cell *= 2.0;
    }
    size_t total = 1;
    for (int d = 0; d < dim; ++d) {
      strides[d] = total;
      total *= n[d];
    }
    for (int d = 0; d < dim; ++d) origin[d] = mn[d];
    buckets.assign(total, {});
    pts.reserve(expected * dim);
  }
  void cell_of(const double* p, long long* c) const {
    for (int d = 0; d < dim; ++d) {
      double q = (p[d] - origin[d]) / cell;
      long long v;
      if (!(q == q)) v = 0;  // NaN -> 0 (Rust `as` cast)
      else if (q >= 9.2e18) v = INT64_MAX;
      else if (q <= -9.2e18) v = INT64_MIN;
      else v = (long long)q;  // truncation toward zero
      long long hi = (long long)n[d] - 1;
      c[d] = v < 0 ? 0 : (v > hi ? hi : v);
    }
  }
  size_t bucket_index(const long long* c) const {
    size_t s = 0;
    for (int d = 0; d < dim; ++d) s += (size_t)c[d] * strides[d];
    return s;
  }
  size_t size() const { return pts.size() / dim; }
  void insert(const double* p) {
    long long c[3];
    cell_of(p, c);
    buckets[bucket_index(c)].push_back((uint32_t)size());
    for (int d = 0; d < dim; ++d) pts.push_back(p[d]);
  }
  template <class F>
  void for_shell_cells(const long long* tc, size_t ring, F&& f) const {
    long long r = (long long)ring;
    long long t[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) t[d] = tc[d];
    auto visit = [&](const long long* cur) {
      for (int d = 0; d < dim; ++d)
        if (cur[d] < 0 || cur[d] >= (long long)n[d]) return;
      f(buckets[bucket_index(cur)]);
    };
    if (ring == 0) {
      visit(t);
      return;
    }
    for (int fd = 0; fd < dim; ++fd) {
      for (int si = 0; si < 2; ++si) {
        long long side = si == 0 ? -r : r;
        long long lo[3], hi[3];
        bool empty = false;
        for (int d = 0; d < dim; ++d) {
          if (d < fd) {
            lo[d] = t[d] - r + 1;
            hi[d] = t[d] + r - 1;
          } else if (d == fd) {
            lo[d] = t[d] + side;
            hi[d] = t[d] + side;
          } else {
            lo[d] = t[d] - r;
            hi[d] = t[d] + r;
          }
          if (lo[d] > hi[d]) empty = true;
        }
        if (empty) continue;
        long long cur[3];
        for (int d = 0; d < dim; ++d) cur[d] = lo[d];
        for (;;) {
          visit(cur);
          int d = 0;
          for (; d < dim; ++d) {
            cur[d] += 1;
            if (cur[d] <= hi[d]) break;
            cur[d] = lo[d];
          }
          if (d == dim) break;
        }
      }
    }
  }
  std::vector<size_t> k_nearest(const double* target, size_t k, bool has_r, double radius) const {
    if (k == 0 || pts.empty()) return {};
    double r2 = has_r ? radius * radius : kInf;
    long long tc[3];
    cell_of(target, tc);
    size_t max_ring = 1;
    for (int d = 0; d < dim; ++d) max_ring = d == 0 ? n[0] : std::max(max_ring, n[d]);
    Heap heap;
    for (size_t ring = 0; ring <= max_ring; ++ring) {
      double ring_min = fmax_((double)ring - 1.0, 0.0) * cell;
      if (ring_min * ring_min > fmin_(heap_worst(heap, k), r2)) break;
      for_shell_cells(tc, ring, [&](const std::vector<uint32_t>& bucket) {
        for (uint32_t i : bucket) {
          double d2 = dist2(&pts[(size_t)i * dim], target, dim);
          if (d2 <= r2) push_candidate(heap, k, d2, i);
        }
      });
    }
    return into_sorted(std::move(heap));
  }
};

// data.rs:384-397 duplicate_coord_pair.
struct KeyHash {
  size_t operator()(const std::array<uint64_t, 3>& k) const {
    uint64_t h = 1469598103934665603ull;
    for (uint64_t v : k) h = (h ^ v) * 1099511628211ull;
    return (size_t)h;
  }
};
bool duplicate_pair(const double* coords, size_t n, int dim, size_t* oi, size_t* oj) {
  std::unordered_map<std::array<uint64_t, 3>, size_t, KeyHash> seen;
  seen.reserve(n);
  for (size_t i = 0; i < n; ++i) {
    std::array<uint64_t, 3> key = {0, 0, 0};
    for (int d = 0; d < dim; ++d) key[d] = bits_of(coords[i * dim + d] + 0.0);
    auto it = seen.find(key);
    if (it != seen.end()) {
      *oi = it->second;
      *oj = i;
      return true;
    }
    seen.emplace(key, i);
  }
  return false;
}

// data.rs:244-283 PointSet::new validation.
int validate_pointset(const double* coords, const double* values, size_t n, int dim) {
  if (n == 0) return fail(OR_INSUFFICIENT_DATA, "no points provided");
  for (size_t i = 0; i < n * dim; ++i)
    if (!std::isfinite(coords[i])) return fail(OR_INVALID_PARAMETER, "non-finite coordinate");
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(values[i])) return fail(OR_INVALID_PARAMETER, "non-finite value");
  return OR_OK;
}

// data.rs:344-346.
double mean_of(const double* v, size_t n) {
  double s = 0.0;
  for (size_t i = 0; i < n; ++i) s += v[i];
  return s / (double)n;
}

// ---------------------------------------------------------------------------
// kriging.rs
struct Predictor {
  int dim = 2;
  size_t n = 0;
  const double* coords = nullptr;
  const double* values = nullptr;
  or_model model{};
  or_kcfg cfg{};
  bool use_tree = false;
  KdTree tree;
  double center[3] = {0, 0, 0};
  double scale = 1.0;
  size_t n_vars = 0;
  std::vector<double> drift;  // n x n_vars
  std::vector<double> drift_mean, drift_scale;
  std::vector<double> meas_err;
  bool has_global_lu = false;
  Lu global_lu;
  bool power = false;
  double c0 = 0.0;
  Anis search_anis{};
  bool aniso_search = false;

  // kriging.rs:46-60 n_drift.
  size_t n_drift() const {
    switch (cfg.method) {
      case 0:
        return 0;
      case 1:
        return 1;
      case 2:
        if (cfg.uk_degree == 1) return 1 + dim;
        if (cfg.uk_degree == 2) return 1 + dim + dim * (dim + 1) / 2;
        return 0;
      case 3:
        return 1 + (size_t)cfg.ked_nvars;
    }
    return 0;
  }
  void search_point(const double* p, double* out) const {
    if (aniso_search) transform_vector(search_anis, dim, p, out);
    else
      for (int d = 0; d < dim; ++d) out[d] = p[d];
  }
  // kriging.rs:410-439 fill_basis.
  void fill_basis(const double* p, const double* dr, double* out) const {
    switch (cfg.method) {
      case 0:
        break;
      case 1:
        out[0] = 1.0;
        break;
      case 2: {
        double xn[3];
        for (int d = 0; d < dim; ++d) xn[d] = (p[d] - center[d]) / scale;
        out[0] = 1.0;
        for (int d = 0; d < dim; ++d) out[1 + d] = xn[d];
        if (cfg.uk_degree == 2) {
          size_t idx = 1 + dim;
          for (int a = 0; a < dim; ++a)
            for (int b = a; b < dim; ++b) out[idx++] = xn[a] * xn[b];
        }
        break;
      }
      case 3:
        out[0] = 1.0;
        for (size_t k = 0; k < n_vars; ++k) out[1 + k] = (dr[k] - drift_mean[k]) / drift_scale[k];
        break;
    }
  }
  double entry(const double* h) const {
    return power ? gamma_dh(model, dim, h) : c0 - gamma_dh(model, dim, h);
  }
  // kriging.rs:527-567 build_lhs.
  std::vector<double> build_lhs(const std::vector<size_t>& nb) const {
    size_t m = n_drift();
    size_t nn = nb.size();
    size_t dimm = nn + m;
    std::vector<double> a(dimm * dimm, 0.0);
    std::vector<double> f(m, 0.0);
    double zero[3] = {0, 0, 0};
    for (size_t ii = 0; ii < nn; ++ii) {
      size_t i = nb[ii];
      const double* pi = &coords[i * dim];
      a[ii * dimm + ii] = entry(zero) + (meas_err.empty() ? 0.0 : meas_err[i]);
      for (size_t jj = ii + 1; jj < nn; ++jj) {
        const double* pj = &coords[nb[jj] * dim];
        double h[3];
        for (int d = 0; d < dim; ++d) h[d] = pi[d] - pj[d];
        double c = entry(h);
        a[ii * dimm + jj] = c;
        a[jj * dimm + ii] = c;
      }
      fill_basis(pi, n_vars ? &drift[i * n_vars] : nullptr, f.data());
      for (size_t k = 0; k < m; ++k) {
        a[ii * dimm + nn + k] = f[k];
        a[(nn + k) * dimm + ii] = f[k];
      }
    }
    return a;
  }
  // kriging.rs:441-490 neighbors.
  std::vector<size_t> neighbors(const double* target, bool* tie) const {
    *tie = false;
    if (!use_tree) {
      std::vector<size_t> all(n);
      for (size_t i = 0; i < n; ++i) all[i] = i;
      return all;
    }
    double st[3];
    search_point(target, st);
    bool has_r = cfg.has_search_radius != 0;
    if (cfg.max_per_octant < 0) {
      size_t k = cfg.max_neighbors >= 0 ? (size_t)cfg.max_neighbors : n;
      if (k < n) {
        // Detect a boundary tie with one extra candidate.
        std::vector<Entry> ent;
        tree.k_nearest(st, k + 1, has_r, cfg.search_radius, &ent);
        if (ent.size() == k + 1 && ent[k - 1].first == ent[k].first) *tie = true;
      }
      return tree.k_nearest(st, k, has_r, cfg.search_radius);
    }
    std::vector<size_t> cand = tree.k_nearest(st, n, has_r, cfg.search_radius);
    std::vector<double> sc(cand.size() * dim);
    for (size_t q = 0; q < cand.size(); ++q) search_point(&coords[cand[q] * dim], &sc[q * dim]);
    std::vector<std::pair<double, size_t>> keyed(cand.size());
    for (size_t q = 0; q < cand.size(); ++q) {
      double s = 0.0;
      for (int d = 0; d < dim; ++d) {
        double dd = sc[q * dim + d] - st[d];
        s += dd * dd;
      }
      keyed[q] = {s, q};
    }
    std::stable_sort(keyed.begin(), keyed.end(),
                     [](const std::pair<double, size_t>& a, const std::pair<double, size_t>& b) {
                       return total_lt(a.first, b.first);
                     });
    std::vector<size_t> counts((size_t)1 << dim, 0);
    std::vector<size_t> selected;
    for (auto& kq : keyed) {
      size_t q = kq.second;
      int oct = 0;
      for (int d = 0; d < dim; ++d)
        if (sc[q * dim + d] >= st[d]) oct |= 1 << d;
      if (counts[oct] < (size_t)cfg.max_per_octant) {
        counts[oct] += 1;
        selected.push_back(cand[q]);
      }
    }
    if (cfg.max_neighbors >= 0 && selected.size() > (size_t)cfg.max_neighbors)
      selected.resize((size_t)cfg.max_neighbors);
    return selected;
  }
  // kriging.rs:569-644 predict_inner.
  int predict_inner(const double* target, const double* tdrift, double* value, double* variance,
                    double* lagrange, std::vector<size_t>* nb_out, bool* tie) const {
    std::vector<size_t> nb = neighbors(target, tie);
    if (nb_out) *nb_out = nb;
    size_t min_nb = cfg.min_neighbors >= 0 ? (size_t)cfg.min_neighbors : 1;
    if (nb.size() < min_nb) return OR_NO_NEIGHBORS;
    size_t m = n_drift();
    size_t nn = nb.size();
    if (nn < m) return OR_INSUFFICIENT_DATA;
    size_t dimm = nn + m;
    std::vector<double> b(dimm, 0.0);
    for (size_t ii = 0; ii < nn; ++ii) {
      const double* p = &coords[nb[ii] * dim];
      double h[3];
      for (int d = 0; d < dim; ++d) h[d] = p[d] - target[d];
      b[ii] = power ? gamma_dh(model, dim, h) : c0 - gamma_dh(model, dim, h);
    }
    std::vector<double> f(m, 0.0);
    fill_basis(target, tdrift, f.data());
    for (size_t k = 0; k < m; ++k) b[nn + k] = f[k];
    std::vector<double> b0 = b;
    std::vector<double> w;
    if (has_global_lu) {
      w = lu_solve(global_lu, b);
    } else {
      Lu lu;
      int rc = lu_factor(build_lhs(nb), dimm, lu);
      if (rc) return rc;
      w = lu_solve(lu, b);
    }
    double v, var;
    if (cfg.method == 0) {
      double mean = cfg.sk_mean;
      v = mean;
      double reduction = 0.0;
      for (size_t ii = 0; ii < nn; ++ii) {
        v += w[ii] * (values[nb[ii]] - mean);
        reduction += w[ii] * b0[ii];
      }
      var = c0 - reduction;
      *lagrange = kNaN;
    } else {
      v = 0.0;
      for (size_t ii = 0; ii < nn; ++ii) v += w[ii] * values[nb[ii]];
      double reduction = 0.0;
      for (size_t i = 0; i < dimm; ++i) reduction += w[i] * b0[i];
      var = power ? reduction : c0 - reduction;
      *lagrange = w[nn];
    }
    *value = v;
    *variance = fmax_(var, 0.0);
    return OR_OK;
  }
  // kriging.rs:674-779 predict_block: the point-to-block covariances are
  // means over the discretisation points centre + offset; C(B,B) (coincident
  // points without the nugget) replaces c0 in the variance.
  int predict_block(const double* ctr, const double* offsets, size_t noff, double* value,
                    double* variance, double* lagrange) const {
    bool tie = false;
    std::vector<size_t> nb = neighbors(ctr, &tie);
    size_t min_nb = cfg.min_neighbors >= 0 ? (size_t)cfg.min_neighbors : 1;
    if (nb.size() < min_nb) return OR_NO_NEIGHBORS;
    const size_t m = n_drift();
    const size_t nn = nb.size();
    const size_t dimm = nn + m;
    const double nu = (double)noff;
    std::vector<double> a(dimm * dimm, 0.0), b(dimm, 0.0);
    for (size_t ii = 0; ii < nn; ++ii) {
      const double* pi = &coords[nb[ii] * dim];
      a[ii * dimm + ii] = c0 + (meas_err.empty() ? 0.0 : meas_err[nb[ii]]);
      for (size_t jj = ii + 1; jj < nn; ++jj) {
        const double* pj = &coords[nb[jj] * dim];
        double h[3];
        for (int d = 0; d < dim; ++d) h[d] = pi[d] - pj[d];
        const double c = c0 - gamma_dh(model, dim, h);
        a[ii * dimm + jj] = c;
        a[jj * dimm + ii] = c;
      }
      if (m == 1) {
        a[ii * dimm + nn] = 1.0;
        a[nn * dimm + ii] = 1.0;
      }
      double s = 0.0;
      for (size_t u = 0; u < noff; ++u) {
        double h[3];
        for (int d = 0; d < dim; ++d) h[d] = pi[d] - (ctr[d] + offsets[u * dim + d]);
        s += c0 - gamma_dh(model, dim, h);
      }
      b[ii] = s / nu;
    }
    if (m == 1) b[nn] = 1.0;
    const double c0c = c0 - model.nugget;
    double cbb = 0.0;
    for (size_t u = 0; u < noff; ++u)
      for (size_t v = 0; v < noff; ++v) {
        if (u == v) {
          cbb += c0c;
        } else {
          double h[3];
          for (int d = 0; d < dim; ++d) h[d] = offsets[u * dim + d] - offsets[v * dim + d];
          cbb += c0 - gamma_dh(model, dim, h);
        }
      }
    cbb /= nu * nu;
    std::vector<double> b0 = b;
    Lu lu;
    int rc = lu_factor(a, dimm, lu);
    if (rc) return rc;
    std::vector<double> w = lu_solve(lu, b);
    double v = 0.0, red = 0.0;
    if (cfg.method == 0) {
      v = cfg.sk_mean;
      for (size_t ii = 0; ii < nn; ++ii) {
        v += w[ii] * (values[nb[ii]] - cfg.sk_mean);
        red += w[ii] * b0[ii];
      }
      *lagrange = kNaN;
    } else {
      for (size_t ii = 0; ii < nn; ++ii) v += w[ii] * values[nb[ii]];
      for (size_t q = 0; q < dimm; ++q) red += w[q] * b0[q];
      *lagrange = w[nn];
    }
    *value = v;
    *variance = fmax_(cbb - red, 0.0);
    return OR_OK;
  }
};

// kriging.rs:262-408 Kriging::build (plus the three constructors).
int build_predictor(Predictor& P, int dim, size_t n, const double* coords, const double* values,
                    const double* drift, const double* meas_err, int ctor, const or_model& model,
                    const or_kcfg& cfg) {
  int rc = validate_pointset(coords, values, n, dim);
  if (rc) return rc;
  rc = validate_model(model);
  if (rc) return rc;
  P.dim = dim;
  P.n = n;
  P.coords = coords;
  P.values = values;
  P.model = model;
  P.cfg = cfg;
  if (ctor == 0) {
    if (cfg.method == 3)
      return fail(OR_INVALID_PARAMETER,
                  "external drift kriging requires Kriging::with_external_drift");
  } else if (ctor == 2) {
    if (cfg.method == 3)
      return fail(OR_INVALID_PARAMETER, "measurement error with external drift is not supported yet");
    if (has_power(model))
      return fail(OR_INVALID_PARAMETER,
                  "measurement error with Power (IRF-0) models is not supported yet");
    for (size_t i = 0; i < n; ++i)
      if (!(std::isfinite(meas_err[i]) && meas_err[i] >= 0.0))
        return fail(OR_INVALID_PARAMETER,
                    "measurement-error variances must be finite and non-negative");
    P.meas_err.assign(meas_err, meas_err + n);
  } else if (ctor == 1) {
    if (cfg.method != 3)
      return fail(OR_INVALID_PARAMETER, "with_external_drift requires KrigingMethod::ExternalDrift");
    if (cfg.ked_nvars == 0)
      return fail(OR_INVALID_PARAMETER, "external drift requires at least one covariate");
    size_t nv = (size_t)cfg.ked_nvars;
    for (size_t i = 0; i < n * nv; ++i)
      if (!std::isfinite(drift[i])) return fail(OR_INVALID_PARAMETER, "non-finite drift value");
    P.n_vars = nv;
    P.drift.assign(drift, drift + n * nv);
  }
  if (cfg.method == 2 && !(cfg.uk_degree >= 1 && cfg.uk_degree <= 2))
    return fail(OR_INVALID_PARAMETER, "universal kriging drift degree must be 1 or 2");
  if (has_power(model) && cfg.method == 0)
    return fail(OR_INVALID_PARAMETER, "Power (unbounded) models have no covariance function");
  if (!valid_in_dim(model, dim))
    return fail(OR_INVALID_PARAMETER, "this model is not a valid covariance in this dimension");
  if (cfg.has_search_radius && !(cfg.search_radius > 0.0))
    return fail(OR_INVALID_PARAMETER, "search radius must be positive");
  if (cfg.has_anisotropic_search) {
    Anis a{cfg.search_azimuth_deg, cfg.search_ratio, cfg.search_ratio_z, cfg.search_dip_deg,
           cfg.search_rake_deg};
    rc = validate_anis(a);
    if (rc) return rc;
    P.aniso_search = true;
    P.search_anis = a;
  }
  if (cfg.max_neighbors == 0) return fail(OR_INVALID_PARAMETER, "max_neighbors must be at least 1");
  size_t di, dj;
  if (duplicate_pair(coords, n, dim, &di, &dj))
    return fail(OR_DUPLICATE_POINTS, "duplicate data points: indices " + std::to_string(di) +
                                         " and " + std::to_string(dj));
  if (cfg.max_per_octant == 0) return fail(OR_INVALID_PARAMETER, "max_per_octant must be at least 1");
  if (cfg.min_neighbors >= 0) {
    if (cfg.min_neighbors == 0) return fail(OR_INVALID_PARAMETER, "min_neighbors must be at least 1");
    if ((size_t)cfg.min_neighbors > n)
      return fail(OR_INSUFFICIENT_DATA, "min_neighbors exceeds the number of data points");
    if (cfg.max_neighbors >= 0 && cfg.min_neighbors > cfg.max_neighbors)
      return fail(OR_INVALID_PARAMETER, "min_neighbors exceeds max_neighbors");
  }
  double mn[3] = {kInf, kInf, kInf}, mx[3] = {-kInf, -kInf, -kInf};
  for (size_t i = 0; i < n; ++i)
    for (int d = 0; d < dim; ++d) {
      mn[d] = fmin_(mn[d], coords[i * dim + d]);
      mx[d] = fmax_(mx[d], coords[i * dim + d]);
    }
  double spread = 0.0;
  for (int d = 0; d < dim; ++d) {
    P.center[d] = 0.5 * (mn[d] + mx[d]);
    spread = fmax_(spread, mx[d] - mn[d]);
  }
  P.scale = fmax_(0.5 * spread, kMinPositive);
  if (P.n_vars > 0) {
    P.drift_mean.assign(P.n_vars, 0.0);
    P.drift_scale.assign(P.n_vars, 1.0);
    double nd = (double)n;
    for (size_t k = 0; k < P.n_vars; ++k) {
      double s = 0.0;
      for (size_t i = 0; i < n; ++i) s += P.drift[i * P.n_vars + k];
      double mean = s / nd;
      double v = 0.0;
      for (size_t i = 0; i < n; ++i) {
        double t = P.drift[i * P.n_vars + k] - mean;
        v += t * t;
      }
      v = v / nd;
      P.drift_mean[k] = mean;
      P.drift_scale[k] = fmax_(std::sqrt(v), kMinPositive);
    }
  }
  P.power = has_power(model);
  double zero[3] = {0, 0, 0};
  P.c0 = total_sill(model) - gamma_dh(model, dim, zero);
  P.use_tree = cfg.max_neighbors >= 0 || cfg.has_search_radius || cfg.max_per_octant >= 0;
  if (P.use_tree) {
    std::vector<double> tr(n * dim);
    for (size_t i = 0; i < n; ++i) P.search_point(&coords[i * dim], &tr[i * dim]);
    P.tree.build(tr.data(), n, dim);
  } else {
    std::vector<size_t> nb(n);
    for (size_t i = 0; i < n; ++i) nb[i] = i;
    size_t m = P.n_drift();
    if (n >= m) {
      Lu lu;
      if (lu_factor(P.build_lhs(nb), n + m, lu) == OR_OK) {
        P.global_lu = std::move(lu);
        P.has_global_lu = true;
      }
    }
  }
  return OR_OK;
}

// ---------------------------------------------------------------------------
// vecchia.rs
struct MaxminKey {
  double d2;
  size_t idx;
  bool operator<(const MaxminKey& o) const {
    int64_t a = total_key(d2), b = total_key(o.d2);
    if (a != b) return a < b;
    return idx < o.idx;
  }
  bool operator>=(const MaxminKey& o) const { return !(*this < o); }
};

void bbox_from_first(const double* coords, size_t n, int dim, double* mn, double* mx) {
  for (int d = 0; d < dim; ++d) mn[d] = mx[d] = coords[d];
  for (size_t i = 0; i < n; ++i)
    for (int d = 0; d < dim; ++d) {
      mn[d] = fmin_(mn[d], coords[i * dim + d]);
      mx[d] = fmax_(mx[d], coords[i * dim + d]);
    }
}

size_t centroid_first(const double* coords, size_t n, int dim) {
  double c[3] = {0, 0, 0};
  for (size_t i = 0; i < n; ++i)
    for (int d = 0; d < dim; ++d) c[d] += coords[i * dim + d] / (double)n;
  size_t first = 0;
  double best = dist2(&coords[0], c, dim);
  for (size_t i = 1; i < n; ++i) {
    double v = dist2(&coords[i * dim], c, dim);
    if (total_lt(v, best)) {
      best = v;
      first = i;
    }
  }
  return first;
}

// vecchia.rs:144-215 maxmin_order.
std::vector<size_t> maxmin_order(const double* coords, size_t n, int dim) {
  if (n == 0) return {};
  size_t first = centroid_first(coords, n, dim);
  double mn[3], mx[3];
  bbox_from_first(coords, n, dim, mn, mx);
  BucketGrid grid(mn, mx, n, dim);
  std::vector<double> sel;
  sel.reserve(n * dim);
  std::vector<size_t> order;
  order.reserve(n);
  order.push_back(first);
  grid.insert(&coords[first * dim]);
  for (int d = 0; d < dim; ++d) sel.push_back(coords[first * dim + d]);
  std::vector<MaxminKey> init;
  init.reserve(n);
  for (size_t i = 0; i < n; ++i)
    if (i != first) init.push_back({dist2(&coords[i * dim], &coords[first * dim], dim), i});
  std::priority_queue<MaxminKey> heap(std::less<MaxminKey>(), std::move(init));
  const size_t kBrute = 48;
  while (!heap.empty()) {
    MaxminKey top = heap.top();
    heap.pop();
    size_t i = top.idx;
    size_t nsel = sel.size() / dim;
    double current;
    if (nsel <= kBrute) {
      current = kInf;
      for (size_t s = 0; s < nsel; ++s) current = fmin_(current, dist2(&coords[i * dim], &sel[s * dim], dim));
    } else {
      std::vector<size_t> nb = grid.k_nearest(&coords[i * dim], 1, false, 0.0);
      current = dist2(&coords[i * dim], &sel[nb[0] * dim], dim);
    }
    MaxminKey refreshed{current, i};
    if (heap.empty() || refreshed >= heap.top()) {
      order.push_back(i);
      grid.insert(&coords[i * dim]);
      for (int d = 0; d < dim; ++d) sel.push_back(coords[i * dim + d]);
    } else {
      heap.push(refreshed);
    }
  }
  return order;
}

// vecchia.rs:2244-2275 (test helper) O(n^2) farthest-point traversal.
std::vector<size_t> maxmin_brute(const double* coords, size_t n, int dim) {
  size_t first = centroid_first(coords, n, dim);
  std::vector<size_t> order{first};
  std::vector<char> chosen(n, 0);
  chosen[first] = 1;
  std::vector<double> md(n);
  for (size_t i = 0; i < n; ++i) md[i] = dist2(&coords[i * dim], &coords[first * dim], dim);
  for (size_t it = 1; it < n; ++it) {
    size_t next = SIZE_MAX;
    for (size_t i = 0; i < n; ++i) {
      if (chosen[i]) continue;
      // Iterator::max_by returns the last maximal element.
      if (next == SIZE_MAX || !total_lt(md[i], md[next])) next = i;
    }
    order.push_back(next);
    chosen[next] = 1;
    for (size_t i = 0; i < n; ++i)
      if (!chosen[i]) md[i] = fmin_(md[i], dist2(&coords[i * dim], &coords[next * dim], dim));
  }
  return order;
}

struct Plan {
  std::vector<size_t> order;
  std::vector<std::vector<size_t>> nb;
};

// vecchia.rs:232-282 vecchia_plan.
int vecchia_plan(const double* coords, size_t n, int dim, size_t m, const int64_t* order_in,
                 Plan& plan) {
  if (n < 2) return fail(OR_INSUFFICIENT_DATA, "Vecchia requires at least 2 points");
  if (m == 0) return fail(OR_INVALID_PARAMETER, "conditioning size m must be at least 1");
  size_t di, dj;
  if (duplicate_pair(coords, n, dim, &di, &dj))
    return fail(OR_DUPLICATE_POINTS, "duplicate data points");
  if (order_in) {
    plan.order.resize(n);
    for (size_t i = 0; i < n; ++i) plan.order[i] = (size_t)order_in[i];
  } else {
    plan.order = maxmin_order(coords, n, dim);
  }
  double mn[3], mx[3];
  bbox_from_first(coords, n, dim, mn, mx);
  BucketGrid grid(mn, mx, n, dim);
  plan.nb.assign(n, {});
  for (size_t k = 0; k < n; ++k) {
    size_t i = plan.order[k];
    std::vector<size_t> pos = grid.k_nearest(&coords[i * dim], m, false, 0.0);
    for (size_t& p : pos) p = plan.order[p];
    plan.nb[k] = std::move(pos);
    grid.insert(&coords[i * dim]);
  }
  return OR_OK;
}

// vecchia.rs:285-336 loglik_with_plan.
int loglik_with_plan(const double* coords, const double* values, size_t n, int dim,
                     const or_model& model, const Plan& plan, double* out, double* terms) {
  double mean = mean_of(values, n);
  std::vector<double> z(n);
  for (size_t i = 0; i < n; ++i) z[i] = values[i] - mean;
  double sill = total_sill(model);
  std::vector<double> kss, ki, w;
  double loglik = 0.0;
  const double ln2pi = std::log(2.0 * kPi);
  for (size_t k = 0; k < plan.order.size(); ++k) {
    size_t i = plan.order[k];
    const std::vector<size_t>& nb = plan.nb[k];
    double mu, var;
    if (nb.empty()) {
      mu = 0.0;
      var = sill;
    } else {
      size_t s = nb.size();
      kss.assign(s * s, 0.0);
      ki.assign(s, 0.0);
      for (size_t a = 0; a < s; ++a) {
        double h[3];
        for (int d = 0; d < dim; ++d) h[d] = coords[i * dim + d] - coords[nb[a] * dim + d];
        ki[a] = sill - gamma_dh(model, dim, h);
        for (size_t b = a; b < s; ++b) {
          for (int d = 0; d < dim; ++d) h[d] = coords[nb[a] * dim + d] - coords[nb[b] * dim + d];
          double c = sill - gamma_dh(model, dim, h);
          kss[a * s + b] = c;
          kss[b * s + a] = c;
        }
      }
      w = ki;
      int rc = cholesky_solve(kss.data(), s, w.data());
      if (rc) return rc;
      mu = 0.0;
      for (size_t a = 0; a < s; ++a) mu += w[a] * z[nb[a]];
      double red = 0.0;
      for (size_t a = 0; a < s; ++a) red += w[a] * ki[a];
      var = fmax_(sill - red, 1e-12);
    }
    double r = z[i] - mu;
    double term = -0.5 * (ln2pi + std::log(var) + r * r / var);
    if (terms) terms[k] = term;
    loglik += term;
  }
  *out = loglik;
  return OR_OK;
}

// vecchia.rs:570-602 guinness_blocks: consecutive ordered points join a
// block while at most 34 % of a new member's predecessors are new to it.
std::vector<std::pair<size_t, size_t>> guinness_blocks(const Plan& plan, size_t group_size) {
  const size_t n = plan.order.size();
  std::vector<std::pair<size_t, size_t>> blocks;
  std::vector<size_t> v_ids;
  auto contains = [](const std::vector<size_t>& v, size_t x) {
    return std::find(v.begin(), v.end(), x) != v.end();
  };
  size_t k0 = 0;
  while (k0 < n) {
    v_ids.assign(plan.nb[k0].begin(), plan.nb[k0].end());
    size_t k1 = k0 + 1;
    while (k1 < n && (k1 - k0) < group_size) {
      const std::vector<size_t>& nb = plan.nb[k1];
      const size_t m = std::max<size_t>(nb.size(), 1);
      auto in_block = [&](size_t j) {
        for (size_t q = k0; q < k1; ++q)
          if (plan.order[q] == j) return true;
        return false;
      };
      size_t new_count = 0;
      for (size_t j : nb)
        if (!contains(v_ids, j) && !in_block(j)) ++new_count;
      if ((double)new_count > 0.34 * (double)m) break;
      for (size_t j : nb)
        if (!contains(v_ids, j) && !in_block(j)) v_ids.push_back(j);
      ++k1;
    }
    blocks.emplace_back(k0, k1);
    k0 = k1;
  }
  return blocks;
}

// vecchia.rs:613-668 loglik_with_blocks: per block, the union S of the
// members' predecessors (members excluded) followed by the members; one
// Cholesky of the joint covariance; each member's term from its pivot and
// its forward-solved value.
int loglik_with_blocks(const double* coords, const double* values, size_t n, int dim,
                       const or_model& model, const Plan& plan,
                       const std::vector<std::pair<size_t, size_t>>& blocks, double* out) {
  const double mean = mean_of(values, n);
  std::vector<double> z(n);
  for (size_t i = 0; i < n; ++i) z[i] = values[i] - mean;
  const double sill = total_sill(model);
  const double ln2pi = std::log(2.0 * kPi);
  std::vector<size_t> v_ids;
  std::vector<double> kvv, w;
  double loglik = 0.0;
  for (const auto& blk : blocks) {
    const size_t k0 = blk.first, k1 = blk.second;
    auto in_block = [&](size_t j) {
      for (size_t q = k0; q < k1; ++q)
        if (plan.order[q] == j) return true;
      return false;
    };
    v_ids.clear();
    for (size_t k = k0; k < k1; ++k)
      for (size_t j : plan.nb[k])
        if (!in_block(j) && std::find(v_ids.begin(), v_ids.end(), j) == v_ids.end())
          v_ids.push_back(j);
    const size_t s_len = v_ids.size();
    for (size_t k = k0; k < k1; ++k) v_ids.push_back(plan.order[k]);
    const size_t vn = v_ids.size();
    kvv.assign(vn * vn, 0.0);
    for (size_t a = 0; a < vn; ++a) {
      kvv[a * vn + a] = sill;
      for (size_t b = a + 1; b < vn; ++b) {
        double h[3];
        for (int d = 0; d < dim; ++d) h[d] = coords[v_ids[a] * dim + d] - coords[v_ids[b] * dim + d];
        const double c = sill - gamma_dh(model, dim, h);
        kvv[a * vn + b] = c;
        kvv[b * vn + a] = c;
      }
    }
    int rc = cholesky_factor(kvv.data(), vn);
    if (rc) return rc;
    w.resize(vn);
    for (size_t a = 0; a < vn; ++a) w[a] = z[v_ids[a]];
    cholesky_forward(kvv.data(), vn, w.data());
    for (size_t t = s_len; t < vn; ++t) {
      const double l_tt = kvv[t * vn + t];
      const double var = l_tt * l_tt;
      loglik += -0.5 * (ln2pi + std::log(var) + w[t] * w[t]);
    }
  }
  *out = loglik;
  return OR_OK;
}

// vecchia.rs:1181-1196 monomials: exponent tuples of total degree <= degree,
// the first dimension's exponent varying slowest.
void monomials(int d, int dim, int rem, int* cur, std::vector<std::array<int, 3>>& out) {
  if (d == dim) {
    out.push_back({cur[0], cur[1], cur[2]});
    return;
  }
  for (int e = 0; e <= rem; ++e) {
    cur[d] = e;
    monomials(d + 1, dim, rem - e, cur, out);
  }
  cur[d] = 0;
}

// vecchia.rs:1199-1233 poly_basis: monomials of the centred, scaled
// coordinates (row-major n x p).
std::vector<double> poly_basis(const double* coords, size_t n, int dim, int degree, size_t* p_out) {
  double mean[3] = {0, 0, 0}, scale[3] = {1, 1, 1};
  for (size_t i = 0; i < n; ++i)
    for (int d = 0; d < dim; ++d) mean[d] += coords[i * dim + d] / (double)n;
  for (int d = 0; d < dim; ++d) {
    double var = 0.0;
    for (size_t i = 0; i < n; ++i) {
      double t = coords[i * dim + d] - mean[d];
      var += t * t;
    }
    var /= (double)n;
    scale[d] = fmax_(std::sqrt(var), 1e-12);
  }
  std::vector<std::array<int, 3>> exps;
  int cur[3] = {0, 0, 0};
  monomials(0, dim, degree, cur, exps);
  const size_t p = exps.size();
  std::vector<double> f(n * p);
  for (size_t i = 0; i < n; ++i) {
    double cs[3];
    for (int d = 0; d < dim; ++d) cs[d] = (coords[i * dim + d] - mean[d]) / scale[d];
    for (size_t c = 0; c < p; ++c) {
      double v = 1.0;
      for (int d = 0; d < dim; ++d)
        for (int e = 0; e < exps[c][d]; ++e) v *= cs[d];
      f[i * p + c] = v;
    }
  }
  *p_out = p;
  return f;
}

// vecchia.rs:1246-1272 standardized_drift_basis: intercept, then each
// covariate centred and divided by its standard deviation (floored at 1e-12).
std::vector<double> drift_basis(const double* drift, size_t n, size_t ncov) {
  std::vector<double> mean(ncov, 0.0), scale(ncov, 1.0);
  for (size_t i = 0; i < n; ++i)
    for (size_t k = 0; k < ncov; ++k) mean[k] += drift[i * ncov + k] / (double)n;
  for (size_t k = 0; k < ncov; ++k) {
    double var = 0.0;
    for (size_t i = 0; i < n; ++i) {
      double t = drift[i * ncov + k] - mean[k];
      var += t * t;
    }
    scale[k] = fmax_(std::sqrt(var / (double)n), 1e-12);
  }
  const size_t p = ncov + 1;
  std::vector<double> f(n * p);
  for (size_t i = 0; i < n; ++i) {
    f[i * p] = 1.0;
    for (size_t k = 0; k < ncov; ++k) f[i * p + 1 + k] = (drift[i * ncov + k] - mean[k]) / scale[k];
  }
  return f;
}

// vecchia.rs:1347-1356 (and 1447-1456): the GLS step on the accumulated
// whitened sums and the restricted log-likelihood.
int reml_finish(size_t n, size_t p, double logdet, double uz_uz, const std::vector<double>& a,
                const std::vector<double>& c, double* out) {
  Lu lu;
  int rc = lu_factor(a, p, lu);
  if (rc) return rc;
  std::vector<double> beta = lu_solve(lu, c);
  const double ln_det_a = lu_ln_det_abs(lu);
  double cb = 0.0;
  for (size_t i = 0; i < p; ++i) cb += c[i] * beta[i];
  const double resid = uz_uz - cb;
  const double nm = (double)(n - p);
  *out = -0.5 * (nm * std::log(2.0 * kPi) + logdet + ln_det_a + resid);
  return OR_OK;
}

// vecchia.rs:1278-1357 reml_loglik_with_plan: per ordered point the
// whitened value and trend row from w = K_SS^-1 k_i (Cholesky), accumulated
// into log det, z'z, F'z and F'F.
int reml_loglik_with_plan(const double* coords, const double* values, size_t n, int dim,
                          const or_model& model, const Plan& plan, const double* basis, size_t p,
                          double* out) {
  const double sill = total_sill(model);
  double logdet = 0.0, uz_uz = 0.0;
  std::vector<double> a(p * p, 0.0), c(p, 0.0), uf(p);
  std::vector<double> kss, ki, w;
  for (size_t k = 0; k < plan.order.size(); ++k) {
    const size_t i = plan.order[k];
    const std::vector<size_t>& nb = plan.nb[k];
    double uz, d;
    if (nb.empty()) {
      const double sd = std::sqrt(sill);
      for (size_t col = 0; col < p; ++col) uf[col] = basis[i * p + col] / sd;
      uz = values[i] / sd;
      d = sill;
    } else {
      const size_t s = nb.size();
      kss.assign(s * s, 0.0);
      ki.assign(s, 0.0);
      for (size_t aa = 0; aa < s; ++aa) {
        double h[3];
        for (int dd = 0; dd < dim; ++dd) h[dd] = coords[i * dim + dd] - coords[nb[aa] * dim + dd];
        ki[aa] = sill - gamma_dh(model, dim, h);
        for (size_t bb = aa; bb < s; ++bb) {
          for (int dd = 0; dd < dim; ++dd)
            h[dd] = coords[nb[aa] * dim + dd] - coords[nb[bb] * dim + dd];
          const double cv = sill - gamma_dh(model, dim, h);
          kss[aa * s + bb] = cv;
          kss[bb * s + aa] = cv;
        }
      }
      w = ki;
      int rc = cholesky_solve(kss.data(), s, w.data());
      if (rc) return rc;
      double red = 0.0;
      for (size_t aa = 0; aa < s; ++aa) red += w[aa] * ki[aa];
      d = fmax_(sill - red, 1e-12);
      const double sd = std::sqrt(d);
      double wz = 0.0;
      for (size_t aa = 0; aa < s; ++aa) wz += w[aa] * values[nb[aa]];
      uz = (values[i] - wz) / sd;
      for (size_t col = 0; col < p; ++col) {
        double wf = 0.0;
        for (size_t aa = 0; aa < s; ++aa) wf += w[aa] * basis[nb[aa] * p + col];
        uf[col] = (basis[i * p + col] - wf) / sd;
      }
    }
    logdet += std::log(d);
    uz_uz += uz * uz;
    for (size_t aa = 0; aa < p; ++aa) {
      c[aa] += uf[aa] * uz;
      for (size_t bb = 0; bb < p; ++bb) a[aa * p + bb] += uf[aa] * uf[bb];
    }
  }
  return reml_finish(n, p, logdet, uz_uz, a, c, out);
}

// vecchia.rs:1366-1457 reml_loglik_with_blocks: each block's joint
// Cholesky factor whitens z and every basis column by forward solves.
int reml_loglik_with_blocks(const double* coords, const double* values, size_t n, int dim,
                            const or_model& model, const Plan& plan, const double* basis, size_t p,
                            const std::vector<std::pair<size_t, size_t>>& blocks, double* out) {
  const double sill = total_sill(model);
  double logdet = 0.0, uz_uz = 0.0;
  std::vector<double> a(p * p, 0.0), c(p, 0.0);
  std::vector<size_t> v_ids;
  std::vector<double> kvv, wz;
  std::vector<std::vector<double>> wf(p);
  for (const auto& blk : blocks) {
    const size_t k0 = blk.first, k1 = blk.second;
    auto in_block = [&](size_t j) {
      for (size_t q = k0; q < k1; ++q)
        if (plan.order[q] == j) return true;
      return false;
    };
    v_ids.clear();
    for (size_t k = k0; k < k1; ++k)
      for (size_t j : plan.nb[k])
        if (!in_block(j) && std::find(v_ids.begin(), v_ids.end(), j) == v_ids.end())
          v_ids.push_back(j);
    const size_t s_len = v_ids.size();
    for (size_t k = k0; k < k1; ++k) v_ids.push_back(plan.order[k]);
    const size_t vn = v_ids.size();
    kvv.assign(vn * vn, 0.0);
    for (size_t aa = 0; aa < vn; ++aa) {
      kvv[aa * vn + aa] = sill;
      for (size_t bb = aa + 1; bb < vn; ++bb) {
        double h[3];
        for (int d = 0; d < dim; ++d)
          h[d] = coords[v_ids[aa] * dim + d] - coords[v_ids[bb] * dim + d];
        const double cv = sill - gamma_dh(model, dim, h);
        kvv[aa * vn + bb] = cv;
        kvv[bb * vn + aa] = cv;
      }
    }
    int rc = cholesky_factor(kvv.data(), vn);
    if (rc) return rc;
    wz.resize(vn);
    for (size_t q = 0; q < vn; ++q) wz[q] = values[v_ids[q]];
    cholesky_forward(kvv.data(), vn, wz.data());
    for (size_t col = 0; col < p; ++col) {
      wf[col].resize(vn);
      for (size_t q = 0; q < vn; ++q) wf[col][q] = basis[v_ids[q] * p + col];
      cholesky_forward(kvv.data(), vn, wf[col].data());
    }
    for (size_t t = s_len; t < vn; ++t) {
      const double l_tt = kvv[t * vn + t];
      const double uz = wz[t];
      logdet += std::log(l_tt * l_tt);
      uz_uz += uz * uz;
      for (size_t aa = 0; aa < p; ++aa) {
        c[aa] += wf[aa][t] * uz;
        for (size_t bb = 0; bb < p; ++bb) a[aa * p + bb] += wf[aa][t] * wf[bb][t];
      }
    }
  }
  return reml_finish(n, p, logdet, uz_uz, a, c, out);
}

int reject_vecchia_model(const or_model& model, int dim) {
  int rc = validate_model(model);
  if (rc) return rc;
  if (has_power(model))
    return fail(OR_INVALID_PARAMETER, "Vecchia cannot use the unbounded Power model");
  if (!valid_in_dim(model, dim))
    return fail(OR_INVALID_PARAMETER, "model is not a valid covariance in this dimension");
  return OR_OK;
}

// vecchia.rs:748-866 vecchia_predict.
int vecchia_predict(const double* coords, const double* values, size_t n, int dim,
                    const or_model& model, const double* targets, size_t nt, size_t m,
                    double* out_v, double* out_var) {
  int rc = reject_vecchia_model(model, dim);
  if (rc) return rc;
  if (m == 0) return fail(OR_INVALID_PARAMETER, "conditioning size m must be at least 1");
  if (nt == 0) return OR_OK;
  size_t di, dj;
  if (duplicate_pair(coords, n, dim, &di, &dj))
    return fail(OR_DUPLICATE_POINTS, "duplicate data points");
  double mean = mean_of(values, n);
  std::vector<double> z(n);
  for (size_t i = 0; i < n; ++i) z[i] = values[i] - mean;
  double zero[3] = {0, 0, 0};
  double c0 = total_sill(model) - gamma_dh(model, dim, zero);
  double mn[3], mx[3];
  for (int d = 0; d < dim; ++d) mn[d] = mx[d] = coords[d];
  for (size_t i = 0; i < n; ++i)
    for (int d = 0; d < dim; ++d) {
      mn[d] = fmin_(mn[d], coords[i * dim + d]);
      mx[d] = fmax_(mx[d], coords[i * dim + d]);
    }
  for (size_t i = 0; i < nt; ++i)
    for (int d = 0; d < dim; ++d) {
      mn[d] = fmin_(mn[d], targets[i * dim + d]);
      mx[d] = fmax_(mx[d], targets[i * dim + d]);
    }
  BucketGrid grid(mn, mx, n + nt, dim);
  std::vector<double> store(coords, coords + n * dim);
  std::vector<double> store_mean = z;
  for (size_t i = 0; i < n; ++i) grid.insert(&coords[i * dim]);
  std::vector<std::vector<std::pair<uint32_t, double>>> rows;
  rows.reserve(nt);
  std::vector<size_t> order = maxmin_order(targets, nt, dim);
  for (size_t i = 0; i < nt; ++i) out_v[i] = out_var[i] = kNaN;
  std::vector<double> kss, ki, w;
  std::map<uint32_t, double> acc;
  double coef_tol = 1e-8 * std::sqrt(c0);
  for (size_t t : order) {
    const double* target = &targets[t * dim];
    std::vector<size_t> nb = grid.k_nearest(target, m, false, 0.0);
    double mu, var;
    std::vector<std::pair<uint32_t, double>> row;
    if (nb.empty()) {
      mu = 0.0;
      var = c0;
      row.push_back({(uint32_t)rows.size(), std::sqrt(fmax_(c0, 0.0))});
    } else {
      size_t s = nb.size();
      kss.assign(s * s, 0.0);
      ki.assign(s, 0.0);
      for (size_t a = 0; a < s; ++a) {
        double h[3];
        for (int d = 0; d < dim; ++d) h[d] = target[d] - store[nb[a] * dim + d];
        ki[a] = c0 - gamma_dh(model, dim, h);
        for (size_t b = a; b < s; ++b) {
          for (int d = 0; d < dim; ++d) h[d] = store[nb[a] * dim + d] - store[nb[b] * dim + d];
          double c = c0 - gamma_dh(model, dim, h);
          kss[a * s + b] = c;
          kss[b * s + a] = c;
        }
      }
      w = ki;
      rc = cholesky_solve(kss.data(), s, w.data());
      if (rc) return rc;
      mu = 0.0;
      for (size_t a = 0; a < s; ++a) mu += w[a] * store_mean[nb[a]];
      double red = 0.0;
      for (size_t a = 0; a < s; ++a) red += w[a] * ki[a];
      double dd = fmax_(c0 - red, 0.0);
      acc.clear();
      for (size_t a = 0; a < s; ++a) {
        size_t j = nb[a];
        if (j >= n)
          for (auto& ic : rows[j - n]) acc[ic.first] += w[a] * ic.second;
      }
      for (auto& ic : acc)
        if (std::fabs(ic.second) > coef_tol) row.push_back(ic);
      row.push_back({(uint32_t)rows.size(), std::sqrt(dd)});
      var = 0.0;
      for (auto& ic : row) var += ic.second * ic.second;
    }
    out_v[t] = mean + mu;
    out_var[t] = var;
    grid.insert(target);
    for (int d = 0; d < dim; ++d) store.push_back(target[d]);
    store_mean.push_back(mu);
    rows.push_back(std::move(row));
  }
  return OR_OK;
}

// optim.rs:6-103 nelder_mead.
template <class F>
std::pair<std::vector<double>, double> nelder_mead(F&& f, const std::vector<double>& x0,
                                                   double step, size_t max_iter) {
  const double ALPHA = 1.0, GAMMA = 2.0, RHO = 0.5, SIGMA = 0.5;
  size_t n = x0.size();
  std::vector<std::vector<double>> simplex;
  simplex.push_back(x0);
  for (size_t i = 0; i < n; ++i) {
    std::vector<double> p = x0;
    p[i] += step;
    simplex.push_back(p);
  }
  std::vector<double> fv;
  for (auto& p : simplex) fv.push_back(f(p));
  for (size_t it = 0; it < max_iter; ++it) {
    std::vector<size_t> idx(n + 1);
    for (size_t i = 0; i <= n; ++i) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(),
                     [&](size_t a, size_t b) { return total_lt(fv[a], fv[b]); });
    std::vector<std::vector<double>> s2;
    std::vector<double> f2;
    for (size_t i : idx) {
      s2.push_back(simplex[i]);
      f2.push_back(fv[i]);
    }
    simplex = s2;
    fv = f2;
    if (std::fabs(fv[n] - fv[0]) <= 1e-12 * fmax_(std::fabs(fv[0]), 1e-12)) break;
    std::vector<double> centroid(n, 0.0);
    for (size_t i = 0; i < n; ++i)
      for (size_t j = 0; j < n; ++j) centroid[j] += simplex[i][j] / (double)n;
    std::vector<double> xr(n);
    for (size_t j = 0; j < n; ++j) xr[j] = centroid[j] + ALPHA * (centroid[j] - simplex[n][j]);
    double fr = f(xr);
    if (fr < fv[0]) {
      std::vector<double> xe(n);
      for (size_t j = 0; j < n; ++j) xe[j] = centroid[j] + GAMMA * (centroid[j] - simplex[n][j]);
      double fe = f(xe);
      if (fe < fr) {
        simplex[n] = xe;
        fv[n] = fe;
      } else {
        simplex[n] = xr;
        fv[n] = fr;
      }
    } else if (fr < fv[n - 1]) {
      simplex[n] = xr;
      fv[n] = fr;
    } else {
      std::vector<double> xc(n);
      double fc;
      if (fr < fv[n]) {
        for (size_t j = 0; j < n; ++j) xc[j] = centroid[j] + RHO * (xr[j] - centroid[j]);
      } else {
        for (size_t j = 0; j < n; ++j) xc[j] = centroid[j] - RHO * (centroid[j] - simplex[n][j]);
      }
      fc = f(xc);
      if (fc < fmin_(fr, fv[n])) {
        simplex[n] = xc;
        fv[n] = fc;
      } else {
        std::vector<double> best = simplex[0];
        for (size_t i = 1; i <= n; ++i) {
          for (size_t j = 0; j < n; ++j) simplex[i][j] = best[j] + SIGMA * (simplex[i][j] - best[j]);
          fv[i] = f(simplex[i]);
        }
      }
    }
  }
  size_t best = 0;
  for (size_t i = 1; i <= n; ++i)
    if (fv[i] < fv[best]) best = i;
  return {simplex[best], fv[best]};
}

// optim.rs:106-123 nelder_mead_multistart.
template <class F>
std::pair<std::vector<double>, double> nelder_mead_multistart(
    F&& f, const std::vector<std::vector<double>>& starts, double step, size_t max_iter) {
  bool have = false;
  std::pair<std::vector<double>, double> best;
  for (auto& x0 : starts) {
    auto r = nelder_mead(f, x0, step, max_iter);
    if (!have || r.second < best.second) {
      best = r;
      have = true;
    }
  }
  return best;
}

void plan_from_arrays(size_t n, size_t m, const int64_t* order, const int64_t* nb,
                      const int32_t* cnt, Plan& plan) {
  plan.order.resize(n);
  plan.nb.assign(n, {});
  for (size_t k = 0; k < n; ++k) {
    plan.order[k] = (size_t)order[k];
    for (int32_t a = 0; a < cnt[k]; ++a) plan.nb[k].push_back((size_t)nb[k * m + a]);
  }
}

// vecchia.rs:952-1016 (objective of mle_fit_with_plan).
double mle_objective(const double* coords, const double* values, size_t n, int dim, int kind,
                     double param, const Plan& plan, double range_max, const double* x) {
  double nugget = x[0] * x[0];
  double psill = std::exp(x[1]);
  double range = std::exp(x[2]);
  or_model m{};
  m.nugget = nugget;
  m.n_structures = 1;
  m.s[0].kind = kind;
  m.s[0].param = param;
  m.s[0].sill = psill;
  m.s[0].range = range;
  double reg = 0.0;
  if (range > range_max) {
    double t = (range - range_max) / range_max;
    reg = t * t;
  }
  double ll;
  int rc = loglik_with_plan(coords, values, n, dim, m, plan, &ll, nullptr);
  if (rc == OR_OK && std::isfinite(ll)) return -ll + 1e6 * reg;
  return 1e12;
}

void mle_setup(const double* coords, const double* values, size_t n, int dim, double* starts9,
               double* range_max) {
  double mean = mean_of(values, n);
  double s = 0.0;
  for (size_t i = 0; i < n; ++i) {
    double t = values[i] - mean;
    s += t * t;
  }
  double var0 = fmax_(s / (double)n, 1e-12);
  double lo[3] = {kInf, kInf, kInf}, hi[3] = {-kInf, -kInf, -kInf};
  for (size_t i = 0; i < n; ++i)
    for (int d = 0; d < dim; ++d) {
      lo[d] = fmin_(lo[d], coords[i * dim + d]);
      hi[d] = fmax_(hi[d], coords[i * dim + d]);
    }
  double e = 0.0;
  for (int d = 0; d < dim; ++d) {
    double t = hi[d] - lo[d];
    e += t * t;
  }
  double extent = std::sqrt(e);
  double range0 = fmax_(extent / 3.0, 1e-9);
  *range_max = 10.0 * extent;
  double lr0 = std::log(range0);
  const double fs[3] = {0.3, 1.0, 3.0};
  for (int i = 0; i < 3; ++i) {
    starts9[i * 3 + 0] = std::sqrt(0.1 * var0);
    starts9[i * 3 + 1] = std::log(0.9 * var0);
    starts9[i * 3 + 2] = lr0 + std::log(fs[i]);
  }
}

// Objective of mle_fit_with_plan with blocks (vecchia.rs:983, 1001-1016) and
// of reml_fit_with_basis (vecchia.rs:1609-1633): -loglik + 1e6 reg(range),
// 1e12 for a rejected candidate.
double fit_objective(const double* coords, const double* values, size_t n, int dim, int kind,
                     const Plan& plan, double range_max, const double* x, const double* basis,
                     size_t p, const std::vector<std::pair<size_t, size_t>>* blocks) {
  or_model m{};
  m.nugget = x[0] * x[0];
  m.n_structures = 1;
  m.s[0].kind = kind;
  m.s[0].sill = std::exp(x[1]);
  m.s[0].range = std::exp(x[2]);
  const double range = m.s[0].range;
  double reg = 0.0;
  if (range > range_max) {
    double t = (range - range_max) / range_max;
    reg = t * t;
  }
  double ll = 0.0;
  int rc;
  if (basis)
    rc = blocks ? reml_loglik_with_blocks(coords, values, n, dim, m, plan, basis, p, *blocks, &ll)
                : reml_loglik_with_plan(coords, values, n, dim, m, plan, basis, p, &ll);
  else
    rc = blocks ? loglik_with_blocks(coords, values, n, dim, m, plan, *blocks, &ll)
                : loglik_with_plan(coords, values, n, dim, m, plan, &ll, nullptr);
  if (rc == OR_OK && std::isfinite(ll)) return -ll + 1e6 * reg;
  return 1e12;
}

// vecchia.rs:353-389 g_and_dg: unit-sill variogram g(d) and dg/dd for the
// kinds with a closed-form range derivative.
bool g_and_dg(int kind, double d, double* g, double* dg) {
  switch (kind) {
    case OR_SPHERICAL:
      if (d >= 1.0) {
        *g = 1.0;
        *dg = 0.0;
      } else {
        *g = 1.5 * d - 0.5 * d * d * d;
        *dg = 1.5 - 1.5 * d * d;
      }
      return true;
    case OR_EXPONENTIAL: {
      double e = std::exp(-d);
      *g = 1.0 - e;
      *dg = e;
      return true;
    }
    case OR_GAUSSIAN: {
      double e = std::exp(-(d * d));
      *g = 1.0 - e;
      *dg = 2.0 * d * e;
      return true;
    }
    case OR_MATERN15: {
      double s = std::sqrt(3.0) * d;
      double e = std::exp(-s);
      *g = 1.0 - (1.0 + s) * e;
      *dg = 3.0 * d * e;
      return true;
    }
    case OR_MATERN25: {
      double s = std::sqrt(5.0) * d;
      double e = std::exp(-s);
      *g = 1.0 - (1.0 + s + s * s / 3.0) * e;
      *dg = 5.0 * d * (1.0 + s) / 3.0 * e;
      return true;
    }
    default:
      return false;
  }
}

// vecchia.rs:93-100 dist2.
double dist2_(const double* a, const double* b, int dim) {
  double s = 0.0;
  for (int d = 0; d < dim; ++d) {
    double v = a[d] - b[d];
    s += v * v;
  }
  return s;
}

// vecchia.rs:428-530 loglik_grad_inner: the log-likelihood and its gradient
// with respect to (nugget, psill, range) of a single isotropic structure.
int loglik_grad(const double* coords, const double* values, size_t n, int dim, int kind,
                double nugget, double psill, double range, const Plan& plan, double* ll_out,
                double* grad_out) {
  double gg, dgg;
  if (!g_and_dg(kind, 0.5, &gg, &dgg)) return fail(OR_INVALID_PARAMETER, "no closed-form gradient");
  double mean = mean_of(values, n);
  std::vector<double> z(n);
  for (size_t i = 0; i < n; ++i) z[i] = values[i] - mean;
  const double sill = nugget + psill;
  const double ln2pi = std::log(2.0 * kPi);
  std::vector<double> kss, ki, w, dk_psill, dk_range, dki_psill, dki_range, rhs, dw;
  double loglik = 0.0;
  double grad[3] = {0.0, 0.0, 0.0};
  for (size_t k = 0; k < plan.order.size(); ++k) {
    size_t i = plan.order[k];
    const std::vector<size_t>& nb = plan.nb[k];
    if (nb.empty()) {
      double var = sill;
      double r = z[i];
      loglik += -0.5 * (ln2pi + std::log(var) + r * r / var);
      double common = -0.5 / var + 0.5 * r * r / (var * var);
      grad[0] += common;
      grad[1] += common;
      continue;
    }
    size_t s = nb.size();
    kss.assign(s * s, 0.0);
    ki.assign(s, 0.0);
    dk_psill.assign(s * s, 0.0);
    dk_range.assign(s * s, 0.0);
    dki_psill.assign(s, 0.0);
    dki_range.assign(s, 0.0);
    for (size_t a = 0; a < s; ++a) {
      double h_ia = std::sqrt(dist2_(&coords[i * dim], &coords[nb[a] * dim], dim));
      double g_ia, dg_ia;
      g_and_dg(kind, h_ia / range, &g_ia, &dg_ia);
      ki[a] = sill - (nugget + psill * g_ia);
      dki_psill[a] = 1.0 - g_ia;
      dki_range[a] = psill * dg_ia * h_ia / (range * range);
      kss[a * s + a] = sill;
      dk_psill[a * s + a] = 1.0;
      for (size_t b = a + 1; b < s; ++b) {
        double h_ab = std::sqrt(dist2_(&coords[nb[a] * dim], &coords[nb[b] * dim], dim));
        double g_ab, dg_ab;
        g_and_dg(kind, h_ab / range, &g_ab, &dg_ab);
        double c = sill - (nugget + psill * g_ab);
        kss[a * s + b] = c;
        kss[b * s + a] = c;
        double dp = 1.0 - g_ab;
        dk_psill[a * s + b] = dp;
        dk_psill[b * s + a] = dp;
        double dr = psill * dg_ab * h_ab / (range * range);
        dk_range[a * s + b] = dr;
        dk_range[b * s + a] = dr;
      }
    }
    int rc = cholesky_factor(kss.data(), s);
    if (rc) return rc;
    w = ki;
    cholesky_forward(kss.data(), s, w.data());
    cholesky_back(kss.data(), s, w.data());
    double mu = 0.0;
    for (size_t a = 0; a < s; ++a) mu += w[a] * z[nb[a]];
    double reduction = 0.0;
    for (size_t a = 0; a < s; ++a) reduction += w[a] * ki[a];
    double raw_var = sill - reduction;
    double var = fmax_(raw_var, 1e-12);
    bool clamped = raw_var <= 1e-12;
    double r = z[i] - mu;
    loglik += -0.5 * (ln2pi + std::log(var) + r * r / var);
    auto solve_param = [&](double dsill_dp, const double* dk, const double* dki) {
      rhs.assign(s, 0.0);
      if (dk) {
        // vecchia.rs:391-398 matvec
        dw.assign(s, 0.0);
        for (size_t row = 0; row < s; ++row) {
          double acc = 0.0;
          for (size_t j = 0; j < s; ++j) acc += dk[row * s + j] * w[j];
          dw[row] = acc;
        }
        for (size_t a = 0; a < s; ++a) rhs[a] = dki[a] - dw[a];
      } else {
        for (size_t a = 0; a < s; ++a) rhs[a] = -w[a];
      }
      dw = rhs;
      cholesky_forward(kss.data(), s, dw.data());
      cholesky_back(kss.data(), s, dw.data());
      double dmu = 0.0;
      for (size_t a = 0; a < s; ++a) dmu += dw[a] * z[nb[a]];
      double d1 = 0.0, d2 = 0.0;
      for (size_t a = 0; a < s; ++a) d1 += dw[a] * ki[a];
      for (size_t a = 0; a < s; ++a) d2 += w[a] * dki[a];
      double dreduction = d1 + d2;
      double dvar = clamped ? 0.0 : dsill_dp - dreduction;
      return -0.5 * dvar / var + r * dmu / var + 0.5 * r * r / (var * var) * dvar;
    };
    std::vector<double> zeros(s, 0.0);
    grad[0] += solve_param(1.0, nullptr, zeros.data());
    grad[1] += solve_param(1.0, dk_psill.data(), dki_psill.data());
    grad[2] += solve_param(0.0, dk_range.data(), dki_range.data());
  }
  *ll_out = loglik;
  for (int q = 0; q < 3; ++q) grad_out[q] = grad[q];
  return OR_OK;
}

// optim.rs:125-182 helpers and the BFGS inverse-Hessian update.
double dot_(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}
std::vector<double> identity_flat(size_t n) {
  std::vector<double> m(n * n, 0.0);
  for (size_t i = 0; i < n * n; ++i) m[i] = (i % (n + 1) == 0) ? 1.0 : 0.0;
  return m;
}
std::vector<double> neg_mat_vec(const std::vector<double>& h, const std::vector<double>& v, size_t n) {
  std::vector<double> out(n);
  for (size_t i = 0; i < n; ++i) {
    double s = 0.0;
    for (size_t j = 0; j < n; ++j) s += h[i * n + j] * v[j];
    out[i] = -s;
  }
  return out;
}
std::vector<double> outer_(const std::vector<double>& u, const std::vector<double>& v, size_t n) {
  std::vector<double> m(n * n, 0.0);
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j < n; ++j) m[i * n + j] = u[i] * v[j];
  return m;
}
std::vector<double> mat_mat(const std::vector<double>& a, const std::vector<double>& b, size_t n) {
  std::vector<double> c(n * n, 0.0);
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j < n; ++j) {
      double s = 0.0;
      for (size_t k = 0; k < n; ++k) s += a[i * n + k] * b[k * n + j];
      c[i * n + j] = s;
    }
  return c;
}
std::vector<double> bfgs_update(const std::vector<double>& h, const std::vector<double>& s,
                                const std::vector<double>& y, double sy, size_t n) {
  double rho = 1.0 / sy;
  std::vector<double> left = identity_flat(n), right = identity_flat(n);
  std::vector<double> syt = outer_(s, y, n), yst = outer_(y, s, n), sst = outer_(s, s, n);
  for (size_t i = 0; i < n * n; ++i) left[i] -= rho * syt[i];
  for (size_t i = 0; i < n * n; ++i) right[i] -= rho * yst[i];
  std::vector<double> h_new = mat_mat(mat_mat(left, h, n), right, n);
  for (size_t i = 0; i < n * n; ++i) h_new[i] += rho * sst[i];
  return h_new;
}

// optim.rs:207-275 bfgs.
template <class F, class G>
std::pair<std::vector<double>, double> bfgs(F&& f, G&& grad, const std::vector<double>& x0,
                                            size_t max_iter) {
  size_t n = x0.size();
  std::vector<double> x = x0;
  std::vector<double> h = identity_flat(n);
  std::vector<double> g = grad(x);
  double fx = f(x);
  std::vector<double> best_x = x;
  double best_fx = fx;
  for (size_t it = 0; it < max_iter; ++it) {
    double gnorm = std::sqrt(dot_(g, g));
    if (gnorm < 1e-10) break;
    std::vector<double> p = neg_mat_vec(h, g, n);
    double slope = dot_(g, p);
    if (slope >= 0.0) {
      h = identity_flat(n);
      for (size_t i = 0; i < n; ++i) p[i] = -g[i];
      slope = dot_(g, p);
    }
    const double c1 = 1e-4;
    double alpha = 1.0;
    std::vector<double> x_new(n);
    double f_new;
    while (true) {
      for (size_t i = 0; i < n; ++i) x_new[i] = x[i] + alpha * p[i];
      double f_cand = f(x_new);
      if (f_cand <= fx + c1 * alpha * slope || alpha < 1e-12) {
        f_new = f_cand;
        break;
      }
      alpha *= 0.5;
    }
    std::vector<double> g_new = grad(x_new);
    std::vector<double> sv(n), yv(n);
    for (size_t i = 0; i < n; ++i) sv[i] = x_new[i] - x[i];
    for (size_t i = 0; i < n; ++i) yv[i] = g_new[i] - g[i];
    double sy = dot_(sv, yv);
    if (sy > 1e-10) h = bfgs_update(h, sv, yv, sy, n);
    bool stalled = std::fabs(fx - f_new) <= 1e-13 * (1.0 + std::fabs(fx)) &&
                   std::sqrt(dot_(sv, sv)) <= 1e-10 * (1.0 + std::sqrt(dot_(x, x)));
    x = x_new;
    g = g_new;
    fx = f_new;
    if (fx < best_fx) {
      best_fx = fx;
      best_x = x;
    }
    if (stalled) break;
  }
  return {best_x, best_fx};
}

// optim.rs:281-289 bfgs_multistart.
template <class F, class G>
std::pair<std::vector<double>, double> bfgs_multistart(F&& f, G&& grad,
                                                       const std::vector<std::vector<double>>& starts,
                                                       size_t max_iter) {
  bool have = false;
  std::pair<std::vector<double>, double> best;
  for (const auto& x0 : starts) {
    auto r = bfgs(f, grad, x0, max_iter);
    if (!have || r.second < best.second) {
      best = r;
      have = true;
    }
  }
  return best;
}

// vecchia.rs:1039-1061 objective_grad of mle_fit_with_plan.
std::vector<double> mle_objective_grad(const double* coords, const double* values, size_t n,
                                       int dim, int kind, const Plan& plan, double range_max,
                                       const std::vector<double>& x) {
  double nugget = x[0] * x[0];
  double psill = std::exp(x[1]);
  double range = std::exp(x[2]);
  double ll, g[3];
  if (loglik_grad(coords, values, n, dim, kind, nugget, psill, range, plan, &ll, g) != OR_OK)
    return {0.0, 0.0, 0.0};
  std::vector<double> gx = {-g[0] * 2.0 * x[0], -g[1] * psill, -g[2] * range};
  if (range > range_max) {
    double dreg_drange = 2.0 * (range - range_max) / (range_max * range_max);
    gx[2] += 1e6 * dreg_drange * range;
  }
  return gx;
}

void test_field_2d(size_t n, uint64_t seed, double* coords, double* values) {
  Rng rng(seed);
  for (size_t i = 0; i < n; ++i) {
    double x = rng.uniform() * 100.0;
    double y = rng.uniform() * 100.0;
    coords[2 * i] = x;
    coords[2 * i + 1] = y;
    values[i] = std::sin(x / 25.0) + std::cos(y / 30.0) + 0.1 * rng.normal();
  }
}
void test_field_3d(size_t n, uint64_t seed, double* coords, double* values) {
  Rng rng(seed);
  for (size_t i = 0; i < n; ++i) {
    double x = rng.uniform() * 100.0;
    double y = rng.uniform() * 100.0;
    double z = rng.uniform() * 40.0;
    coords[3 * i] = x;
    coords[3 * i + 1] = y;
    coords[3 * i + 2] = z;
    values[i] = std::sin(x / 15.0) + std::cos(y / 20.0) + std::sin(z / 8.0) + 0.05 * rng.normal();
  }
}

}  // namespace

// ===========================================================================
// C interface
extern "C" {

const char* or_last_error(void) { return g_err.c_str(); }

int or_model_validate(const or_model* m) { return validate_model(*m); }

double or_gamma_dh(const or_model* m, int dim, const double* dh) { return gamma_dh(*m, dim, dh); }

int or_lu_solve(int64_t n, const double* a, const double* b, double* x) {
  Lu lu;
  int rc = lu_factor(std::vector<double>(a, a + n * n), (size_t)n, lu);
  if (rc) return rc;
  std::vector<double> r = lu_solve(lu, std::vector<double>(b, b + n));
  std::copy(r.begin(), r.end(), x);
  return OR_OK;
}

int or_cholesky_solve(int64_t n, const double* a, const double* b, double* x) {
  std::vector<double> aw(a, a + n * n);
  std::copy(b, b + n, x);
  return cholesky_solve(aw.data(), (size_t)n, x);
}

int64_t or_kdtree_knn(int dim, int64_t n, const double* coords, const double* target, int64_t k,
                      int has_radius, double radius, int64_t* out) {
  KdTree t;
  t.build(coords, (size_t)n, dim);
  std::vector<size_t> r = t.k_nearest(target, (size_t)k, has_radius != 0, radius);
  for (size_t i = 0; i < r.size(); ++i) out[i] = (int64_t)r[i];
  return (int64_t)r.size();
}

int64_t or_knn_brute(int dim, int64_t n, const double* coords, const double* target, int64_t k,
                     int has_radius, double radius, int64_t* out) {
  std::vector<size_t> r = knn_brute(coords, (size_t)n, dim, target, (size_t)k, has_radius != 0, radius);
  for (size_t i = 0; i < r.size(); ++i) out[i] = (int64_t)r[i];
  return (int64_t)r.size();
}

int or_bucketgrid_queries(int dim, int64_t n, const double* coords, const double* bbox_min,
                          const double* bbox_max, int64_t expected, int64_t nq,
                          const int64_t* q_after, const double* q_target, int64_t k,
                          int has_radius, double radius, int64_t* out, int64_t* cnt,
                          int64_t* grid_dims) {
  BucketGrid g(bbox_min, bbox_max, (size_t)expected, dim);
  for (int d = 0; d < dim; ++d) grid_dims[d] = (int64_t)g.n[d];
  int64_t q = 0;
  for (int64_t i = 0; i < n && q < nq; ++i) {
    g.insert(&coords[i * dim]);
    while (q < nq && q_after[q] == i) {
      std::vector<size_t> r = g.k_nearest(&q_target[q * dim], (size_t)k, has_radius != 0, radius);
      cnt[q] = (int64_t)r.size();
      for (size_t a = 0; a < r.size(); ++a) out[q * k + a] = (int64_t)r[a];
      ++q;
    }
  }
  return OR_OK;
}

int or_duplicate_pair(int dim, int64_t n, const double* coords, int64_t* i, int64_t* j) {
  size_t a, b;
  if (duplicate_pair(coords, (size_t)n, dim, &a, &b)) {
    *i = (int64_t)a;
    *j = (int64_t)b;
    return 1;
  }
  return 0;
}

int or_grid_centers(int dim, const double* bmin, const double* bmax, const int64_t* ncell,
                    double* out) {
  for (int d = 0; d < dim; ++d) {
    if (ncell[d] == 0) return fail(OR_INVALID_PARAMETER, "grid must have at least one cell per axis");
    if (!(bmax[d] > bmin[d])) return fail(OR_INVALID_PARAMETER, "degenerate bbox");
  }
  double step[3];
  for (int d = 0; d < dim; ++d) step[d] = (bmax[d] - bmin[d]) / (double)ncell[d];
  size_t q = 0;
  if (dim == 2) {
    for (int64_t iy = 0; iy < ncell[1]; ++iy)
      for (int64_t ix = 0; ix < ncell[0]; ++ix) {
        out[q++] = bmin[0] + ((double)ix + 0.5) * step[0];
        out[q++] = bmin[1] + ((double)iy + 0.5) * step[1];
      }
  } else {
    for (int64_t iz = 0; iz < ncell[2]; ++iz)
      for (int64_t iy = 0; iy < ncell[1]; ++iy)
        for (int64_t ix = 0; ix < ncell[0]; ++ix) {
          out[q++] = bmin[0] + ((double)ix + 0.5) * step[0];
          out[q++] = bmin[1] + ((double)iy + 0.5) * step[1];
          out[q++] = bmin[2] + ((double)iz + 0.5) * step[2];
        }
  }
  return OR_OK;
}

int or_krige(int dim, int64_t n, const double* coords, const double* values, const double* drift,
             const double* meas_err, int ctor, const or_model* model, const or_kcfg* cfg,
             int64_t nt, const double* targets, const double* tdrift, double* value,
             double* variance, double* lagrange, int8_t* status, int32_t* nb_out, int64_t kcap,
             int32_t* nb_count, int64_t* boundary_ties, int nthreads) {
  if (dim != 2 && dim != 3) return fail(OR_DIMENSION_MISMATCH, "dim must be 2 or 3");
  Predictor P;
  int rc = build_predictor(P, dim, (size_t)n, coords, values, drift, meas_err, ctor, *model, *cfg);
  if (rc) return rc;
  if (nthreads < 1) nthreads = 1;
  std::vector<int64_t> ties(nthreads, 0);
  size_t nv = cfg->method == 3 ? (size_t)cfg->ked_nvars : 0;
  auto work = [&](int tid) {
    for (int64_t t = tid; t < nt; t += nthreads) {
      std::vector<size_t> nb;
      bool tie = false;
      double v = kNaN, var = kNaN, lag = kNaN;
      int st = P.predict_inner(&targets[t * dim], nv ? &tdrift[t * nv] : nullptr, &v, &var, &lag,
                               nb_out || nb_count ? &nb : nullptr, &tie);
      if (st != OR_OK) {
        v = kNaN;
        var = kNaN;
        lag = kNaN;
      }
      value[t] = v;
      variance[t] = var;
      if (lagrange) lagrange[t] = lag;
      if (status) status[t] = (int8_t)st;
      if (tie) ties[tid] += 1;
      if (nb_count) nb_count[t] = (int32_t)nb.size();
      if (nb_out)
        for (int64_t a = 0; a < kcap; ++a)
          nb_out[t * kcap + a] = a < (int64_t)nb.size() ? (int32_t)nb[a] : -1;
    }
  };
  if (nthreads == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (int i = 0; i < nthreads; ++i) th.emplace_back(work, i);
    for (auto& x : th) x.join();
  }
  if (boundary_ties) {
    int64_t s = 0;
    for (int64_t v : ties) s += v;
    *boundary_ties = s;
  }
  return OR_OK;
}

int or_maxmin_order(int dim, int64_t n, const double* coords, int64_t* order) {
  std::vector<size_t> o = maxmin_order(coords, (size_t)n, dim);
  for (size_t i = 0; i < o.size(); ++i) order[i] = (int64_t)o[i];
  return OR_OK;
}

int or_maxmin_order_brute(int dim, int64_t n, const double* coords, int64_t* order) {
  if (n == 0) return OR_OK;
  std::vector<size_t> o = maxmin_brute(coords, (size_t)n, dim);
  for (size_t i = 0; i < o.size(); ++i) order[i] = (int64_t)o[i];
  return OR_OK;
}

int or_vecchia_plan(int dim, int64_t n, const double* coords, int64_t m, const int64_t* order_in,
                    int64_t* order_out, int64_t* nb, int32_t* nb_count) {
  if (m < 0) return fail(OR_INVALID_PARAMETER, "conditioning size m must be at least 1");
  if (order_in == nullptr && false) return OR_OK;
  Plan plan;
  int rc = vecchia_plan(coords, (size_t)n, dim, (size_t)m, order_in, plan);
  if (rc) return rc;
  for (int64_t k = 0; k < n; ++k) {
    order_out[k] = (int64_t)plan.order[k];
    nb_count[k] = (int32_t)plan.nb[k].size();
    for (int64_t a = 0; a < m; ++a)
      nb[k * m + a] = a < (int64_t)plan.nb[k].size() ? (int64_t)plan.nb[k][a] : -1;
  }
  return OR_OK;
}

int or_vecchia_loglik_plan(int dim, int64_t n, const double* coords, const double* values,
                           const or_model* model, int64_t m, const int64_t* order,
                           const int64_t* nb, const int32_t* nb_count, double* ll,
                           double* terms) {
  int rc = reject_vecchia_model(*model, dim);
  if (rc) return rc;
  Plan plan;
  plan_from_arrays((size_t)n, (size_t)m, order, nb, nb_count, plan);
  return loglik_with_plan(coords, values, (size_t)n, dim, *model, plan, ll, terms);
}

// vecchia.rs:604-611 loglik_with_plan_grouped (group_size <= 1: ungrouped).
int or_vecchia_loglik_grouped(int dim, int64_t n, const double* coords, const double* values,
                              const or_model* model, int64_t m, const int64_t* order,
                              const int64_t* nb, const int32_t* nb_count, int64_t group_size,
                              double* ll) {
  int rc = reject_vecchia_model(*model, dim);
  if (rc) return rc;
  Plan plan;
  plan_from_arrays((size_t)n, (size_t)m, order, nb, nb_count, plan);
  if (group_size <= 1)
    return loglik_with_plan(coords, values, (size_t)n, dim, *model, plan, ll, nullptr);
  return loglik_with_blocks(coords, values, (size_t)n, dim, *model, plan,
                            guinness_blocks(plan, (size_t)group_size), ll);
}

int or_vecchia_loglik(int dim, int64_t n, const double* coords, const double* values,
                      const or_model* model, int64_t m, const int64_t* order, double* ll) {
  int rc = reject_vecchia_model(*model, dim);
  if (rc) return rc;
  if (m < 0) return fail(OR_INVALID_PARAMETER, "conditioning size m must be at least 1");
  Plan plan;
  rc = vecchia_plan(coords, (size_t)n, dim, (size_t)m, order, plan);
  if (rc) return rc;
  return loglik_with_plan(coords, values, (size_t)n, dim, *model, plan, ll, nullptr);
}

// vecchia.rs:1958-1974 exact_loglik (test oracle).
int or_exact_loglik(int dim, int64_t n, const double* coords, const double* values,
                    const or_model* model, double* ll) {
  size_t N = (size_t)n;
  double mean = mean_of(values, N);
  std::vector<double> z(N);
  for (size_t i = 0; i < N; ++i) z[i] = values[i] - mean;
  std::vector<double> cov(N * N);
  double sill = total_sill(*model);
  for (size_t a = 0; a < N; ++a)
    for (size_t b = 0; b < N; ++b) {
      double h[3];
      for (int d = 0; d < dim; ++d) h[d] = coords[a * dim + d] - coords[b * dim + d];
      cov[a * N + b] = sill - gamma_dh(*model, dim, h);
    }
  Lu lu;
  int rc = lu_factor(cov, N, lu);
  if (rc) return rc;
  std::vector<double> x = lu_solve(lu, z);
  double quad = 0.0;
  for (size_t i = 0; i < N; ++i) quad += z[i] * x[i];
  *ll = -0.5 * ((double)N * std::log(2.0 * kPi) + lu_ln_det_abs(lu) + quad);
  return OR_OK;
}

int or_vecchia_predict(int dim, int64_t n, const double* coords, const double* values,
                       const or_model* model, int64_t nt, const double* targets, int64_t m,
                       double* value, double* variance) {
  return vecchia_predict(coords, values, (size_t)n, dim, *model, targets, (size_t)nt, (size_t)m,
                         value, variance);
}

int or_vecchia_mle_objective(int dim, int64_t n, const double* coords, const double* values,
                             int32_t kind, double param, int64_t m, const int64_t* order,
                             const int64_t* nb, const int32_t* nb_count, double range_max,
                             int64_t nx, const double* x, double* fx) {
  Plan plan;
  plan_from_arrays((size_t)n, (size_t)m, order, nb, nb_count, plan);
  for (int64_t q = 0; q < nx; ++q)
    fx[q] = mle_objective(coords, values, (size_t)n, dim, kind, param, plan, range_max, &x[q * 3]);
  return OR_OK;
}

int or_vecchia_mle_setup(int dim, int64_t n, const double* coords, const double* values,
                         double* starts9, double* range_max) {
  mle_setup(coords, values, (size_t)n, dim, starts9, range_max);
  return OR_OK;
}

int or_vecchia_mle_nm(int dim, int64_t n, const double* coords, const double* values,
                      int32_t kind, double param, int64_t m, const int64_t* order_in,
                      int64_t nstarts, const double* starts, double step, int64_t max_iter,
                      double* x_out, double* f_out, int64_t* n_evals) {
  Plan plan;
  int rc = vecchia_plan(coords, (size_t)n, dim, (size_t)m, order_in, plan);
  if (rc) return rc;
  double s9[9], range_max;
  mle_setup(coords, values, (size_t)n, dim, s9, &range_max);
  int64_t evals = 0;
  auto f = [&](const std::vector<double>& x) {
    ++evals;
    return mle_objective(coords, values, (size_t)n, dim, kind, param, plan, range_max, x.data());
  };
  std::vector<std::vector<double>> st;
  for (int64_t i = 0; i < nstarts; ++i) st.push_back({starts[i * 3], starts[i * 3 + 1], starts[i * 3 + 2]});
  auto r = nelder_mead_multistart(f, st, step, (size_t)max_iter);
  for (int i = 0; i < 3; ++i) x_out[i] = r.first[i];
  *f_out = r.second;
  if (n_evals) *n_evals = evals;
  return OR_OK;
}

// Kriging::predict_block for nc blocks sharing one discretisation, with
// predict_block's own checks (kriging.rs:678-700) first.
int or_krige_block(int dim, int64_t n, const double* coords, const double* values,
                   const double* meas_err, int ctor, const or_model* model, const or_kcfg* cfg,
                   int64_t nc, const double* centers, const double* offsets, int64_t noff,
                   double* value, double* variance, double* lagrange, int8_t* status) {
  Predictor P;
  int rc = build_predictor(P, dim, (size_t)n, coords, values, nullptr, meas_err, ctor, *model, *cfg);
  if (rc) return rc;
  if (cfg->method != 0 && cfg->method != 1)
    return fail(OR_INVALID_PARAMETER, "block kriging supports simple and ordinary kriging only");
  if (has_power(*model)) return fail(OR_INVALID_PARAMETER, "block kriging with a Power model");
  if (noff <= 0) return fail(OR_INVALID_PARAMETER, "block discretization needs at least one point");
  for (int64_t t = 0; t < nc; ++t) {
    double v = kNaN, var = kNaN, lag = kNaN;
    int st = P.predict_block(&centers[t * dim], offsets, (size_t)noff, &v, &var, &lag);
    if (st != OR_OK) v = var = lag = kNaN;
    value[t] = v;
    variance[t] = var;
    lagrange[t] = lag;
    status[t] = (int8_t)st;
  }
  return OR_OK;
}

// validation.rs:298-328 spatial_block_assignment.
int or_spatial_block_assignment(int dim, int64_t n, const double* coords, const int64_t* bpd,
                                int64_t* fold_of) {
  double lo[3], hi[3];
  for (int d = 0; d < dim; ++d) lo[d] = hi[d] = coords[d];
  for (int64_t i = 0; i < n; ++i)
    for (int d = 0; d < dim; ++d) {
      lo[d] = fmin_(lo[d], coords[i * dim + d]);
      hi[d] = fmax_(hi[d], coords[i * dim + d]);
    }
  for (int64_t i = 0; i < n; ++i) {
    int64_t idx = 0, stride = 1;
    for (int d = 0; d < dim; ++d) {
      const double span = fmax_(hi[d] - lo[d], kMinPositive);
      double frac = (coords[i * dim + d] - lo[d]) / span;
      frac = frac < 0.0 ? 0.0 : (frac > 1.0 - 1e-12 ? 1.0 - 1e-12 : frac);
      int64_t bd = (int64_t)(frac * (double)bpd[d]);
      if (bd > bpd[d] - 1) bd = bpd[d] - 1;
      idx += bd * stride;
      stride *= bpd[d];
    }
    fold_of[i] = idx;
  }
  return OR_OK;
}

// vecchia.rs:577-602 guinness_blocks on a plan given as arrays: k1 of each
// block (block b covers [k1[b - 1], k1[b])), their number in *nblocks.
int or_guinness_blocks(int64_t n, int64_t m, const int64_t* order, const int64_t* nb,
                       const int32_t* nb_count, int64_t group_size, int64_t* k1,
                       int64_t* nblocks) {
  Plan plan;
  plan_from_arrays((size_t)n, (size_t)m, order, nb, nb_count, plan);
  auto blocks = guinness_blocks(plan, (size_t)group_size);
  for (size_t b = 0; b < blocks.size(); ++b) k1[b] = (int64_t)blocks[b].second;
  *nblocks = (int64_t)blocks.size();
  return OR_OK;
}

int64_t or_poly_basis_terms(int dim, int32_t degree) {
  std::vector<std::array<int, 3>> exps;
  int cur[3] = {0, 0, 0};
  monomials(0, dim, degree, cur, exps);
  return (int64_t)exps.size();
}

int or_poly_basis(int dim, int64_t n, const double* coords, int32_t degree, double* out) {
  size_t p = 0;
  std::vector<double> f = poly_basis(coords, (size_t)n, dim, degree, &p);
  std::copy(f.begin(), f.end(), out);
  return OR_OK;
}

int or_drift_basis(int64_t n, int64_t ncov, const double* drift, double* out) {
  std::vector<double> f = drift_basis(drift, (size_t)n, (size_t)ncov);
  std::copy(f.begin(), f.end(), out);
  return OR_OK;
}

// reml_loglik_with_plan / reml_loglik_with_blocks on a plan given as arrays
// (group_size <= 1: ungrouped).
int or_vecchia_reml_loglik(int dim, int64_t n, const double* coords, const double* values,
                           const or_model* model, int64_t m, const int64_t* order,
                           const int64_t* nb, const int32_t* nb_count, const double* basis,
                           int64_t p, int64_t group_size, double* ll) {
  int rc = reject_vecchia_model(*model, dim);
  if (rc) return rc;
  Plan plan;
  plan_from_arrays((size_t)n, (size_t)m, order, nb, nb_count, plan);
  if (group_size <= 1)
    return reml_loglik_with_plan(coords, values, (size_t)n, dim, *model, plan, basis, (size_t)p, ll);
  return reml_loglik_with_blocks(coords, values, (size_t)n, dim, *model, plan, basis, (size_t)p,
                                 guinness_blocks(plan, (size_t)group_size), ll);
}

// Nelder-Mead multistart fits: basis null = mle_fit_with_plan's grouped
// path (group_size > 1), else reml_fit_with_basis (vecchia.rs:1572-1644).
int or_vecchia_fit_nm(int dim, int64_t n, const double* coords, const double* values, int32_t kind,
                      int64_t m, const int64_t* order_in, const double* basis, int64_t p,
                      int64_t group_size, int64_t nstarts, const double* starts, double step,
                      int64_t max_iter, double* x_out, double* f_out, int64_t* n_evals) {
  Plan plan;
  int rc = vecchia_plan(coords, (size_t)n, dim, (size_t)m, order_in, plan);
  if (rc) return rc;
  if (basis && n <= p + 1)
    return fail(OR_INSUFFICIENT_DATA, "REML needs more points than trend terms plus one");
  double s9[9], range_max;
  mle_setup(coords, values, (size_t)n, dim, s9, &range_max);
  std::vector<std::pair<size_t, size_t>> blocks;
  if (group_size > 1) blocks = guinness_blocks(plan, (size_t)group_size);
  int64_t evals = 0;
  auto f = [&](const std::vector<double>& x) {
    ++evals;
    return fit_objective(coords, values, (size_t)n, dim, kind, plan, range_max, x.data(), basis,
                         (size_t)p, group_size > 1 ? &blocks : nullptr);
  };
  std::vector<std::vector<double>> st;
  for (int64_t i = 0; i < nstarts; ++i) st.push_back({starts[i * 3], starts[i * 3 + 1], starts[i * 3 + 2]});
  auto r = nelder_mead_multistart(f, st, step, (size_t)max_iter);
  for (int i = 0; i < 3; ++i) x_out[i] = r.first[i];
  *f_out = r.second;
  if (n_evals) *n_evals = evals;
  return OR_OK;
}

int or_g_and_dg(int32_t kind, double d, double* g, double* dg) {
  return g_and_dg(kind, d, g, dg) ? OR_OK : OR_INVALID_PARAMETER;
}

int or_vecchia_loglik_grad(int dim, int64_t n, const double* coords, const double* values,
                           int32_t kind, double nugget, double psill, double range, int64_t m,
                           const int64_t* order, const int64_t* nb, const int32_t* nb_count,
                           double* ll, double* grad3) {
  Plan plan;
  plan_from_arrays((size_t)n, (size_t)m, order, nb, nb_count, plan);
  return loglik_grad(coords, values, (size_t)n, dim, kind, nugget, psill, range, plan, ll, grad3);
}

int or_vecchia_mle_bfgs(int dim, int64_t n, const double* coords, const double* values,
                        int32_t kind, int64_t m, const int64_t* order_in, int64_t max_iter,
                        double* x_out, double* f_out, int64_t* n_evals) {
  Plan plan;
  int rc = vecchia_plan(coords, (size_t)n, dim, (size_t)m, order_in, plan);
  if (rc) return rc;
  double s9[9], range_max;
  mle_setup(coords, values, (size_t)n, dim, s9, &range_max);
  int64_t evals = 0;
  auto f = [&](const std::vector<double>& x) {
    ++evals;
    return mle_objective(coords, values, (size_t)n, dim, kind, 0.0, plan, range_max, x.data());
  };
  auto g = [&](const std::vector<double>& x) {
    ++evals;
    return mle_objective_grad(coords, values, (size_t)n, dim, kind, plan, range_max, x);
  };
  std::vector<std::vector<double>> st;
  for (int i = 0; i < 3; ++i) st.push_back({s9[i * 3], s9[i * 3 + 1], s9[i * 3 + 2]});
  auto r = bfgs_multistart(f, g, st, (size_t)max_iter);
  for (int i = 0; i < 3; ++i) x_out[i] = r.first[i];
  *f_out = r.second;
  if (n_evals) *n_evals = evals;
  if (r.second >= 1e12) return fail(OR_SINGULAR_SYSTEM, "Vecchia MLE did not converge");
  return OR_OK;
}

int or_bfgs_multistart(or_objective_fn f, or_gradient_fn g, void* ctx, int64_t n, int64_t nstarts,
                       const double* starts, int64_t max_iter, double* x_out, double* f_out) {
  std::vector<std::vector<double>> st;
  for (int64_t i = 0; i < nstarts; ++i) st.push_back(std::vector<double>(starts + i * n, starts + (i + 1) * n));
  auto obj = [&](const std::vector<double>& x) { return f(x.data(), n, ctx); };
  auto grad = [&](const std::vector<double>& x) {
    std::vector<double> out(n);
    g(x.data(), n, out.data(), ctx);
    return out;
  };
  auto r = bfgs_multistart(obj, grad, st, (size_t)max_iter);
  for (int64_t i = 0; i < n; ++i) x_out[i] = r.first[i];
  *f_out = r.second;
  return OR_OK;
}

int or_nelder_mead_multistart(or_objective_fn f, void* ctx, int64_t n, int64_t nstarts,
                              const double* starts, double step, int64_t max_iter, double* x_out,
                              double* f_out) {
  std::vector<std::vector<double>> st;
  for (int64_t i = 0; i < nstarts; ++i) st.push_back(std::vector<double>(starts + i * n, starts + (i + 1) * n));
  auto obj = [&](const std::vector<double>& x) { return f(x.data(), n, ctx); };
  auto r = nelder_mead_multistart(obj, st, step, (size_t)max_iter);
  for (int64_t i = 0; i < n; ++i) x_out[i] = r.first[i];
  *f_out = r.second;
  return OR_OK;
}

void or_rng_u64(uint64_t seed, int64_t count, uint64_t* out) {
  Rng r(seed);
  for (int64_t i = 0; i < count; ++i) out[i] = r.next_u64();
}
void or_rng_uniform(uint64_t seed, int64_t count, double* out) {
  Rng r(seed);
  for (int64_t i = 0; i < count; ++i) out[i] = r.uniform();
}
void or_rng_normal(uint64_t seed, int64_t count, double* out) {
  Rng r(seed);
  for (int64_t i = 0; i < count; ++i) out[i] = r.normal();
}
void or_rng_draw(uint64_t seed, int64_t n_uniform, int64_t n_normal, double* out) {
  Rng r(seed);
  for (int64_t i = 0; i < n_uniform; ++i) out[i] = r.uniform();
  for (int64_t i = 0; i < n_normal; ++i) out[n_uniform + i] = r.normal();
}
void or_test_field_2d(int64_t n, uint64_t seed, double* coords, double* values) {
  test_field_2d((size_t)n, seed, coords, values);
}
void or_test_field_3d(int64_t n, uint64_t seed, double* coords, double* values) {
  test_field_3d((size_t)n, seed, coords, values);
}

}  // extern "C"
