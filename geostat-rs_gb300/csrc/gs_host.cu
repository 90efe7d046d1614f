// gs_host.cu -- host-side runtime: error state, df constants, model
// conversion, xoshiro256++ RNG, max-min ordering and the Nelder-Mead state
// machine shared by the batched MLE driver.
//
// Compiled with -ffp-contract=off on the host side: max-min ordering and the
// Nelder-Mead simplex must take the same branch decisions as the reference's
// Rust code, which never contracts multiply-adds.
#include <math.h>

#include <algorithm>
#include <cstring>
#include <limits>
#include <queue>
#include <vector>

#include "gs_common.cuh"
#include "gs_host.h"
#include "gs_internal.h"

namespace gs {

static thread_local std::string g_error;

void set_error(const std::string& msg) { g_error = msg; }

int fail(int code, const std::string& msg) {
  g_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  g_error = std::string("CUDA error ") + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) +
            ") in " + what + " at " + file + ":" + std::to_string(line);
  return e == cudaErrorMemoryAllocation ? GS_ERR_OUT_OF_MEMORY : GS_ERR_CUDA;
}

const char* last_error() { return g_error.c_str(); }

// ---------------------------------------------------------- df constants --
static float round_to_bits(long double v, int bits) {
  int e;
  long double m = frexpl(v, &e);  // v = m * 2^e, 0.5 <= m < 1
  long double scaled = ldexpl(m, bits);
  scaled = roundl(scaled);
  return (float)ldexpl(scaled, e - bits);
}

void df_consts_host(ExpTable* tab, DfConsts* k) {
  const long double ln2 = 0.693147180559945309417232121458176568L;
  const long double L = ln2 / 256.0L;
  const float l1 = round_to_bits(L, 9);
  const long double rem = L - (long double)l1;
  const float l2 = (float)rem;
  const float l3 = (float)(rem - (long double)l2);
  k->l1 = l1;
  k->l2 = l2;
  k->l3 = l3;
  k->inv = (float)(256.0L / ln2);
  const long double s3 = sqrtl(3.0L), s5 = sqrtl(5.0L);
  k->s3h = (float)s3;
  k->s3l = (float)(s3 - (long double)k->s3h);
  k->s5h = (float)s5;
  k->s5l = (float)(s5 - (long double)k->s5h);
  for (int j = 0; j < 256; ++j) {
    const long double v = exp2l(-(long double)j / 256.0L);
    tab->v[j].hi = (float)v;
    tab->v[j].lo = (float)(v - (long double)tab->v[j].hi);
  }
}

void exp64_table_host(Exp64Table* t) {
  const long double ln2 = 0.693147180559945309417232121458176568L;
  const long double L = ln2 / 64.0L;
  int e;
  const long double mant = frexpl(L, &e);
  const double l1 = (double)ldexpl(roundl(ldexpl(mant, 36)), e - 36);  // 36 bits
  t->l1 = l1;
  t->l2 = (double)(L - (long double)l1);
  t->inv = (double)(64.0L / ln2);
  for (int j = 0; j < 64; ++j) {
    const long double v = exp2l(-(long double)j / 64.0L);
    t->hi[j] = (double)v;
    t->lo[j] = (double)(v - (long double)t->hi[j]);
  }
}

// ---------------------------------------------------------------- model --
static const double kRadsPerDeg = 3.14159265358979323846 / 180.0;

double total_sill(const gs_model& m) {
  double s = 0.0;
  for (int k = 0; k < m.n_structures; ++k) s += m.s[k].sill;
  return m.nugget + s;
}

bool has_power(const gs_model& m) {
  for (int k = 0; k < m.n_structures; ++k)
    if (m.s[k].kind == GS_KIND_POWER) return true;
  return false;
}

int validate_anisotropy(double az, double ratio, double ratio_z, double dip, double rake) {
  if (!(ratio_z > 0.0) || !std::isfinite(ratio_z))
    return fail(GS_ERR_INVALID_PARAMETER, "anisotropy ratio_z must be finite and > 0");
  if (!(ratio > 0.0) || !std::isfinite(ratio))
    return fail(GS_ERR_INVALID_PARAMETER, "anisotropy ratio must be finite and > 0");
  if (!std::isfinite(az)) return fail(GS_ERR_INVALID_PARAMETER, "anisotropy azimuth must be finite");
  if (!std::isfinite(dip) || !std::isfinite(rake))
    return fail(GS_ERR_INVALID_PARAMETER, "anisotropy dip/rake must be finite");
  return GS_OK;
}

// VariogramModel::new (model.rs:554-630).
int validate_model(const gs_model& m) {
  if (m.n_structures < 0 || m.n_structures > GS_MAX_STRUCTURES)
    return fail(GS_ERR_INVALID_PARAMETER, "at most 4 nested structures are supported");
  if (!(m.nugget >= 0.0) || !std::isfinite(m.nugget))
    return fail(GS_ERR_INVALID_PARAMETER, "nugget must be finite and >= 0");
  for (int k = 0; k < m.n_structures; ++k) {
    const gs_structure& s = m.s[k];
    if (s.kind < 0 || s.kind > GS_KIND_POWER)
      return fail(GS_ERR_INVALID_PARAMETER, "unknown model kind");
    if (!(s.sill >= 0.0) || !std::isfinite(s.sill))
      return fail(GS_ERR_INVALID_PARAMETER, "partial sill must be finite and >= 0");
    if (!(s.range > 0.0) || !std::isfinite(s.range))
      return fail(GS_ERR_INVALID_PARAMETER, "range must be finite and > 0");
    if (s.kind == GS_KIND_STABLE && (!(s.param > 0.0) || s.param > 2.0))
      return fail(GS_ERR_INVALID_PARAMETER, "Stable alpha must be in (0, 2]");
    if (s.kind == GS_KIND_POWER && (!(s.param > 0.0) || s.param >= 2.0))
      return fail(GS_ERR_INVALID_PARAMETER, "Power theta must be in (0, 2)");
    if (s.has_anis) GS_TRY(validate_anisotropy(s.azimuth_deg, s.ratio, s.ratio_z, s.dip_deg, s.rake_deg));
  }
  if (!(total_sill(m) > 0.0)) return fail(GS_ERR_INVALID_PARAMETER, "total sill must be positive");
  return GS_OK;
}

// Anisotropy::rotation_matrix_3d (model.rs:407-433), op for op.
void rotation_3d(double az, double ratio, double ratio_z, double dip, double rake, double r[9]) {
  double alpha = (az >= 0.0 && az < 270.0) ? (90.0 - az) * kRadsPerDeg : (450.0 - az) * kRadsPerDeg;
  double beta = (-dip) * kRadsPerDeg;
  double theta = rake * kRadsPerDeg;
  double sina = sin(alpha), cosa = cos(alpha);
  double sinb = sin(beta), cosb = cos(beta);
  double sint = sin(theta), cost = cos(theta);
  double afac1 = 1.0 / ratio, afac2 = 1.0 / ratio_z;
  r[0] = cosb * cosa;
  r[1] = cosb * sina;
  r[2] = -sinb;
  r[3] = afac1 * (-cost * sina + sint * sinb * cosa);
  r[4] = afac1 * (cost * cosa + sint * sinb * sina);
  r[5] = afac1 * (sint * cosb);
  r[6] = afac2 * (sint * sina + cost * sinb * cosa);
  r[7] = afac2 * (-sint * cosa + cost * sinb * sina);
  r[8] = afac2 * (cost * cosb);
}

void rotation_matrix(const gs_structure& s, int dim, double rot[9]) {
  for (int i = 0; i < 9; ++i) rot[i] = 0.0;
  if (dim == 3) {
    rotation_3d(s.azimuth_deg, s.ratio, s.ratio_z, s.dip_deg, s.rake_deg, rot);
  } else {
    // transform_vector 2-D (model.rs:362-365) written as a matrix.
    double a = s.azimuth_deg * kRadsPerDeg;
    double sn = sin(a), cs = cos(a);
    rot[0] = sn;
    rot[1] = cs;
    rot[3] = cs / s.ratio;
    rot[4] = -sn / s.ratio;
  }
}

int make_dev_model(const gs_model& m, int dim, DevModel* out, bool gpu_kinds_only) {
  GS_TRY(validate_model(m));
  std::memset(out, 0, sizeof(*out));
  out->ns = m.n_structures;
  out->dim = dim;
  out->nugget = m.nugget;
  out->c0 = total_sill(m);
  out->c0_df = df_from_double(out->c0);
  for (int k = 0; k < m.n_structures; ++k) {
    const gs_structure& s = m.s[k];
    if (gpu_kinds_only && s.kind > GS_KIND_MATERN25)
      return fail(GS_ERR_INVALID_PARAMETER,
                  "the CUDA path evaluates spherical, exponential, gaussian, matern15 and "
                  "matern25 structures only");
    DevStruct& d = out->s[k];
    d.kind = s.kind;
    d.aniso = s.has_anis ? 1 : 0;
    d.sill = s.sill;
    d.inv_range = 1.0 / s.range;
    d.sill_df = df_from_double(s.sill);
    d.inv_range_df = df_from_double(d.inv_range);
    if (s.has_anis) {
      rotation_matrix(s, dim, d.rot);
    } else {
      d.rot[0] = d.rot[4] = d.rot[8] = 1.0;
    }
    for (int i = 0; i < 9; ++i) d.rot_df[i] = df_from_double(d.rot[i]);
  }
  return GS_OK;
}

// ------------------------------------------------------------------ rng --
// xoshiro256++ seeded by splitmix64 (rng.rs:7-79).
Xoshiro::Xoshiro(uint64_t seed) {
  uint64_t sm = seed;
  for (int i = 0; i < 4; ++i) {
    sm += 0x9E3779B97F4A7C15ull;
    uint64_t z = sm;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    s[i] = z ^ (z >> 31);
  }
}
static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
uint64_t Xoshiro::next() {
  uint64_t result = rotl64(s[0] + s[3], 23) + s[0];
  uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl64(s[3], 45);
  return result;
}
double Xoshiro::uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
double Xoshiro::normal() {
  if (has_spare) {
    has_spare = false;
    return spare;
  }
  for (;;) {
    double u1 = uniform();
    if (u1 > 0.0) {
      double u2 = uniform();
      double r = sqrt(-2.0 * log(u1));
      double a = 2.0 * 3.14159265358979323846 * u2;
      spare = r * sin(a);
      has_spare = true;
      return r * cos(a);
    }
  }
}

// ------------------------------------------------------- max-min order --
// Farthest-point ordering with lazy key refresh (the algorithm of
// vecchia.rs:144-215).  Keys only decrease as points are selected, so a
// popped key that still dominates the heap after refreshing is exact.  The
// refresh needs the exact nearest selected point; it comes from a uniform
// grid over the selected points (any exact nearest-neighbour query yields
// the same squared distance, which is all the ordering consumes).
namespace {

struct Key {
  double d2;
  int64_t idx;
};
inline int64_t tkey(double v) {
  int64_t b;
  std::memcpy(&b, &v, 8);
  return b ^ (int64_t)(((uint64_t)(b >> 63)) >> 1);
}
struct KeyLess {
  bool operator()(const Key& a, const Key& b) const {
    int64_t x = tkey(a.d2), y = tkey(b.d2);
    if (x != y) return x < y;
    return a.idx < b.idx;
  }
};

// Multi-resolution grid over the selected points.  Level l has cells 2^l
// times wider than level 0 (about one point per cell when all n points are
// selected).  A query uses the finest level whose cells hold about one
// selected point each, so the exact nearest neighbour is found within a
// couple of rings whatever the current selected count.
class SelectedGrid {
 public:
  SelectedGrid(const std::vector<double>& pts, int dim, int64_t n) : dim_(dim) {
    for (int d = 0; d < dim; ++d) {
      lo_[d] = std::numeric_limits<double>::infinity();
      hi_[d] = -lo_[d];
    }
    for (int64_t i = 0; i < n; ++i)
      for (int d = 0; d < dim; ++d) {
        lo_[d] = std::min(lo_[d], pts[i * dim + d]);
        hi_[d] = std::max(hi_[d], pts[i * dim + d]);
      }
    double ext = 0.0;
    for (int d = 0; d < dim; ++d) ext = std::max(ext, hi_[d] - lo_[d]);
    if (!(ext > 0.0)) ext = 1.0;
    double vol = 1.0;
    int act = 0;
    for (int d = 0; d < dim; ++d)
      if (hi_[d] - lo_[d] > ext * 1e-9) {
        vol *= hi_[d] - lo_[d];
        ++act;
      }
    if (act == 0) act = 1;
    double cell = pow(vol / (double)std::max<int64_t>(n, 1), 1.0 / act);
    if (!(cell > 0.0)) cell = ext;
    for (int guard = 0; guard < 64; ++guard) {
      Level L;
      L.cell = cell;
      int64_t total = 1;
      for (int d = 0; d < dim; ++d) {
        double c = (hi_[d] - lo_[d] > ext * 1e-9) ? ceil((hi_[d] - lo_[d]) / cell) : 1.0;
        L.n[d] = std::max<int64_t>(1, (int64_t)std::min(c, 1e9));
        total *= L.n[d];
      }
      if (total <= 4 * std::max<int64_t>(n, 16) || levels_.size() > 0) {
        L.head.assign(total, -1);
        levels_.push_back(std::move(L));
      }
      if (total <= 4) break;
      cell *= 2.0;
    }
    pts_.reserve(n * dim);
  }
  void insert(const double* p) {
    const int64_t id = (int64_t)(pts_.size() / dim_);
    for (int d = 0; d < dim_; ++d) pts_.push_back(p[d]);
    for (auto& L : levels_) {
      int64_t c = cell_of(L, p);
      L.next.push_back(L.head[c]);
      L.head[c] = id;
    }
  }
  // Exact squared distance to the nearest inserted point.
  double nearest_d2(const double* p) const {
    const int64_t nsel = (int64_t)(pts_.size() / dim_);
    size_t lv = 0;
    while (lv + 1 < levels_.size() && (int64_t)levels_[lv].head.size() > 2 * nsel) ++lv;
    const Level& L = levels_[lv];
    int64_t tc[3] = {0, 0, 0};
    cell_coords(L, p, tc);
    double best = std::numeric_limits<double>::infinity();
    int64_t maxring = 0;
    for (int d = 0; d < dim_; ++d) maxring = std::max(maxring, L.n[d]);
    for (int64_t ring = 0; ring <= maxring; ++ring) {
      double rmin = std::max((double)ring - 1.0 - 1e-9, 0.0) * L.cell;
      if (rmin * rmin > best) break;
      visit_shell(L, tc, ring, [&](int64_t cell) {
        for (int64_t q = L.head[cell]; q >= 0; q = L.next[q]) {
          double s = 0.0;
          for (int d = 0; d < dim_; ++d) {
            double dd = pts_[q * dim_ + d] - p[d];
            s += dd * dd;
          }
          if (s < best) best = s;
        }
      });
    }
    return best;
  }

 private:
  struct Level {
    double cell = 1.0;
    int64_t n[3] = {1, 1, 1};
    std::vector<int64_t> head, next;
  };
  void cell_coords(const Level& L, const double* p, int64_t* c) const {
    for (int d = 0; d < dim_; ++d) {
      double q = floor((p[d] - lo_[d]) / L.cell);
      c[d] = q < 0 ? 0 : (q >= (double)L.n[d] ? L.n[d] - 1 : (int64_t)q);
    }
  }
  int64_t cell_of(const Level& L, const double* p) const {
    int64_t c[3] = {0, 0, 0};
    cell_coords(L, p, c);
    int64_t id = 0, stride = 1;
    for (int d = 0; d < dim_; ++d) {
      id += c[d] * stride;
      stride *= L.n[d];
    }
    return id;
  }
  template <class F>
  void visit_shell(const Level& L, const int64_t* tc, int64_t r, F&& f) const {
    int64_t lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int d = 0; d < dim_; ++d) {
      lo[d] = tc[d] - r;
      hi[d] = tc[d] + r;
    }
    const int64_t* n = L.n;
    int64_t zlo = dim_ == 3 ? std::max<int64_t>(lo[2], 0) : 0;
    int64_t zhi = dim_ == 3 ? std::min<int64_t>(hi[2], n[2] - 1) : 0;
    int64_t ylo = std::max<int64_t>(lo[1], 0), yhi = std::min<int64_t>(hi[1], n[1] - 1);
    int64_t xlo = std::max<int64_t>(lo[0], 0), xhi = std::min<int64_t>(hi[0], n[0] - 1);
    for (int64_t z = zlo; z <= zhi; ++z) {
      bool zface = dim_ == 3 && (z == lo[2] || z == hi[2]);
      for (int64_t y = ylo; y <= yhi; ++y) {
        bool yface = (y == lo[1] || y == hi[1]);
        if (zface || yface || r == 0) {
          for (int64_t x = xlo; x <= xhi; ++x) f(x + n[0] * (y + n[1] * z));
        } else {
          if (lo[0] >= 0) f(lo[0] + n[0] * (y + n[1] * z));
          if (hi[0] < n[0] && hi[0] != lo[0]) f(hi[0] + n[0] * (y + n[1] * z));
        }
      }
    }
  }
  int dim_;
  double lo_[3], hi_[3];
  std::vector<Level> levels_;
  std::vector<double> pts_;
};

inline double dist2(const double* a, const double* b, int dim) {
  double s = 0.0;
  for (int d = 0; d < dim; ++d) {
    double v = a[d] - b[d];
    s += v * v;
  }
  return s;
}

}  // namespace

void maxmin_order(const std::vector<double>& pts, int dim, int64_t n, int64_t* order) {
  NvtxRange nvtx_range("gs.maxmin_order");
  if (n == 0) return;
  double c[3] = {0, 0, 0};
  for (int64_t i = 0; i < n; ++i)
    for (int d = 0; d < dim; ++d) c[d] += pts[i * dim + d] / (double)n;
  int64_t first = 0;
  double best = dist2(&pts[0], c, dim);
  for (int64_t i = 1; i < n; ++i) {
    double v = dist2(&pts[i * dim], c, dim);
    if (tkey(v) < tkey(best)) {
      best = v;
      first = i;
    }
  }
  SelectedGrid grid(pts, dim, n);
  int64_t nsel = 0;
  order[nsel++] = first;
  grid.insert(&pts[first * dim]);
  std::vector<Key> init;
  init.reserve(n);
  for (int64_t i = 0; i < n; ++i)
    if (i != first) init.push_back({dist2(&pts[i * dim], &pts[first * dim], dim), i});
  std::priority_queue<Key, std::vector<Key>, KeyLess> heap(KeyLess(), std::move(init));
  KeyLess less;
  while (!heap.empty()) {
    Key top = heap.top();
    heap.pop();
    Key refreshed{grid.nearest_d2(&pts[top.idx * dim]), top.idx};
    if (heap.empty() || !less(refreshed, heap.top())) {
      order[nsel++] = top.idx;
      grid.insert(&pts[top.idx * dim]);
    } else {
      heap.push(refreshed);
    }
  }
}

// ---------------------------------------------------------- Nelder-Mead --
// optim.rs:6-103 recast as a resumable state machine: `pending()` lists the
// points whose objective values the simplex needs next; `supply()` feeds
// them back.  Branch decisions and arithmetic follow the reference exactly,
// so fed the same values it visits the same points.
NelderMead::NelderMead(const std::vector<double>& x0, double step, int64_t max_iter)
    : n_(x0.size()), max_iter_(max_iter) {
  simplex_.push_back(x0);
  for (size_t i = 0; i < n_; ++i) {
    std::vector<double> p = x0;
    p[i] += step;
    simplex_.push_back(p);
  }
  fv_.assign(n_ + 1, 0.0);
  pending_ = simplex_;
  stage_ = kInit;
}

static bool total_lt(double a, double b) { return tkey(a) < tkey(b); }

void NelderMead::begin_iteration() {
  if (it_ >= max_iter_) {
    stage_ = kDone;
    return;
  }
  std::vector<size_t> idx(n_ + 1);
  for (size_t i = 0; i <= n_; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return total_lt(fv_[a], fv_[b]); });
  std::vector<std::vector<double>> s2;
  std::vector<double> f2;
  for (size_t i : idx) {
    s2.push_back(simplex_[i]);
    f2.push_back(fv_[i]);
  }
  simplex_.swap(s2);
  fv_.swap(f2);
  if (fabs(fv_[n_] - fv_[0]) <= 1e-12 * std::max(fabs(fv_[0]), 1e-12)) {
    stage_ = kDone;
    return;
  }
  centroid_.assign(n_, 0.0);
  for (size_t i = 0; i < n_; ++i)
    for (size_t j = 0; j < n_; ++j) centroid_[j] += simplex_[i][j] / (double)n_;
  xr_.assign(n_, 0.0);
  for (size_t j = 0; j < n_; ++j) xr_[j] = centroid_[j] + 1.0 * (centroid_[j] - simplex_[n_][j]);
  pending_.assign(1, xr_);
  stage_ = kReflect;
}

void NelderMead::end_iteration() {
  ++it_;
  begin_iteration();
}

void NelderMead::supply(const std::vector<double>& f) {
  switch (stage_) {
    case kInit:
      fv_ = f;
      begin_iteration();
      return;
    case kReflect: {
      fr_ = f[0];
      if (fr_ < fv_[0]) {
        std::vector<double> xe(n_);
        for (size_t j = 0; j < n_; ++j) xe[j] = centroid_[j] + 2.0 * (centroid_[j] - simplex_[n_][j]);
        pending_.assign(1, xe);
        stage_ = kExpand;
      } else if (fr_ < fv_[n_ - 1]) {
        simplex_[n_] = xr_;
        fv_[n_] = fr_;
        end_iteration();
      } else {
        std::vector<double> xc(n_);
        if (fr_ < fv_[n_]) {
          for (size_t j = 0; j < n_; ++j) xc[j] = centroid_[j] + 0.5 * (xr_[j] - centroid_[j]);
        } else {
          for (size_t j = 0; j < n_; ++j) xc[j] = centroid_[j] - 0.5 * (centroid_[j] - simplex_[n_][j]);
        }
        pending_.assign(1, xc);
        stage_ = kContract;
      }
      return;
    }
    case kExpand: {
      double fe = f[0];
      if (fe < fr_) {
        simplex_[n_] = pending_[0];
        fv_[n_] = fe;
      } else {
        simplex_[n_] = xr_;
        fv_[n_] = fr_;
      }
      end_iteration();
      return;
    }
    case kContract: {
      double fc = f[0];
      if (fc < std::min(fr_, fv_[n_])) {
        simplex_[n_] = pending_[0];
        fv_[n_] = fc;
        end_iteration();
      } else {
        std::vector<double> best = simplex_[0];
        pending_.clear();
        for (size_t i = 1; i <= n_; ++i) {
          for (size_t j = 0; j < n_; ++j) simplex_[i][j] = best[j] + 0.5 * (simplex_[i][j] - best[j]);
          pending_.push_back(simplex_[i]);
        }
        stage_ = kShrink;
      }
      return;
    }
    case kShrink:
      for (size_t i = 1; i <= n_; ++i) fv_[i] = f[i - 1];
      end_iteration();
      return;
    case kDone:
      return;
  }
}

std::pair<std::vector<double>, double> NelderMead::best() const {
  size_t b = 0;
  for (size_t i = 1; i <= n_; ++i)
    if (fv_[i] < fv_[b]) b = i;
  return {simplex_[b], fv_[b]};
}

// optim.rs:106-123: the best of several independent runs (first wins ties).
std::pair<std::vector<double>, double> multistart_best(const std::vector<NelderMead>& runs) {
  bool have = false;
  std::pair<std::vector<double>, double> best;
  for (const auto& r : runs) {
    auto b = r.best();
    if (!have || b.second < best.second) {
      best = b;
      have = true;
    }
  }
  return best;
}


// ------------------------------------------------------------------ BFGS --
namespace {
double dotv(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}
std::vector<double> eye(size_t n) {
  std::vector<double> m(n * n, 0.0);
  for (size_t i = 0; i < n * n; ++i) m[i] = (i % (n + 1) == 0) ? 1.0 : 0.0;
  return m;
}
std::vector<double> matmul(const std::vector<double>& a, const std::vector<double>& b, size_t n) {
  std::vector<double> c(n * n, 0.0);
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j < n; ++j) {
      double s = 0.0;
      for (size_t k = 0; k < n; ++k) s += a[i * n + k] * b[k * n + j];
      c[i * n + j] = s;
    }
  return c;
}
// Nocedal & Wright eq. 6.17 in the operation order of optim.rs:166-182.
std::vector<double> inv_hessian_update(const std::vector<double>& h, const std::vector<double>& s,
                                       const std::vector<double>& y, double sy, size_t n) {
  const double rho = 1.0 / sy;
  std::vector<double> left = eye(n), right = eye(n);
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j < n; ++j) {
      left[i * n + j] -= rho * (s[i] * y[j]);
      right[i * n + j] -= rho * (y[i] * s[j]);
    }
  std::vector<double> out = matmul(matmul(left, h, n), right, n);
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j < n; ++j) out[i * n + j] += rho * (s[i] * s[j]);
  return out;
}
}  // namespace

Bfgs::Bfgs(const std::vector<double>& x0, int64_t max_iter)
    : n_(x0.size()), max_iter_(max_iter), x_(x0), h_(eye(x0.size())), req_(x0), best_x_(x0) {}

void Bfgs::begin_iteration() {
  if (it_ >= max_iter_ || std::sqrt(dotv(g_, g_)) < 1e-10) {
    stage_ = kDone;
    return;
  }
  p_.assign(n_, 0.0);
  for (size_t i = 0; i < n_; ++i) {
    double s = 0.0;
    for (size_t j = 0; j < n_; ++j) s += h_[i * n_ + j] * g_[j];
    p_[i] = -s;
  }
  slope_ = dotv(g_, p_);
  if (slope_ >= 0.0) {
    h_ = eye(n_);
    for (size_t i = 0; i < n_; ++i) p_[i] = -g_[i];
    slope_ = dotv(g_, p_);
  }
  alpha_ = 1.0;
  req_.assign(n_, 0.0);
  for (size_t i = 0; i < n_; ++i) req_[i] = x_[i] + alpha_ * p_[i];
  stage_ = kSearch;
}

void Bfgs::supply_g(const std::vector<double>& g) {
  if (stage_ == kInitG) {
    g_ = g;
    stage_ = kInitF;  // the objective at the same point comes next
    return;
  }
  if (stage_ != kGnew) return;
  std::vector<double> sv(n_), yv(n_);
  for (size_t i = 0; i < n_; ++i) sv[i] = xnew_[i] - x_[i];
  for (size_t i = 0; i < n_; ++i) yv[i] = g[i] - g_[i];
  const double sy = dotv(sv, yv);
  if (sy > 1e-10) h_ = inv_hessian_update(h_, sv, yv, sy, n_);
  const bool stalled = std::fabs(fx_ - fnew_) <= 1e-13 * (1.0 + std::fabs(fx_)) &&
                       std::sqrt(dotv(sv, sv)) <= 1e-10 * (1.0 + std::sqrt(dotv(x_, x_)));
  x_ = xnew_;
  g_ = g;
  fx_ = fnew_;
  if (fx_ < best_f_) {
    best_f_ = fx_;
    best_x_ = x_;
  }
  ++it_;
  if (stalled) {
    stage_ = kDone;
    return;
  }
  begin_iteration();
}

void Bfgs::supply_f(double f) {
  if (stage_ == kInitF) {
    fx_ = f;
    best_f_ = f;
    best_x_ = x_;
    begin_iteration();
    return;
  }
  if (stage_ != kSearch) return;
  const double c1 = 1e-4;
  if (f <= fx_ + c1 * alpha_ * slope_ || alpha_ < 1e-12) {
    xnew_ = req_;
    fnew_ = f;
    stage_ = kGnew;  // gradient at the accepted point
    return;
  }
  alpha_ *= 0.5;
  for (size_t i = 0; i < n_; ++i) req_[i] = x_[i] + alpha_ * p_[i];
}

std::pair<std::vector<double>, double> bfgs_multistart_best(const std::vector<Bfgs>& runs) {
  bool have = false;
  std::pair<std::vector<double>, double> best;
  for (const auto& r : runs) {
    auto b = r.best();
    if (!have || b.second < best.second) {
      best = b;
      have = true;
    }
  }
  return best;
}

}  // namespace gs
