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
// Farthest-point ordering (vecchia.rs:144-215): the first point is the one
// nearest the centroid; every later step takes the unselected point whose
// squared distance to its nearest selected point is largest, ties going to
// the larger index (the reference's heap order over (distance, index) under
// f64::total_cmp).  The reference finds that point with lazily refreshed
// heap keys; any exact search selects the same sequence.  Here every
// unselected point keeps its exact key, lowered as soon as a newly selected
// point lands closer, and a winner tree over the keys gives the maximum.  A
// selected point can only lower points within its own key distance (it was
// the maximum), so each step enumerates that ball.  The points are stored
// (as slots) in a spatial order that makes the ball cheap to enumerate: a
// uniform grid of about two points per cell when no cell is crowded, else a
// balanced k-d tree whose leaves are runs of 16-31 slots.
namespace {

inline int64_t tkey(double v) {
  int64_t b;
  std::memcpy(&b, &v, 8);
  return b ^ (int64_t)(((uint64_t)(b >> 63)) >> 1);
}

inline double dist2(const double* a, const double* b, int dim) {
  double s = 0.0;
  for (int d = 0; d < dim; ++d) {
    double v = a[d] - b[d];
    s += v * v;
  }
  return s;
}

class MaxminLayout {
 public:
  MaxminLayout(const std::vector<double>& pts, int dim, int64_t n) : dim_(dim), n_(n) {
    idx_.resize(n);
    for (int64_t i = 0; i < n; ++i) idx_[i] = i;
    if (!build_grid(pts)) build_tree(pts);
    xs_.resize(n * dim);
    for (int64_t j = 0; j < n; ++j)
      for (int d = 0; d < dim; ++d) xs_[j * dim + d] = pts[idx_[j] * dim + d];
    if (!grid_) tree_boxes();
  }
  int64_t point(int64_t j) const { return idx_[j]; }
  const double* at(int64_t j) const { return &xs_[j * dim_]; }

  // f(j) for every slot j whose point may lie closer than sqrt(R) to p:
  // a superset of them, never missing one (see the bounds below)
  template <class F>
  void visit_ball(const double* p, double R, F&& f) const {
    if (grid_) {
      // a point q with dist2(q, p) < R has |q_d - p_d| < sqrt(R) (1 + 3u)
      // per axis in exact terms (u = 2^-53); the slack (1e-9 relative, and
      // 1e-12 of |p_d| + r absolute) exceeds that and the rounding of
      // p_d -/+ r, and the cell index is monotone in its argument
      const double r = sqrt(R);
      int64_t clo[3] = {0, 0, 0}, chi[3] = {0, 0, 0};
      for (int d = 0; d < dim_; ++d) {
        const double rr = r + r * 1e-9 + 1e-12 * (fabs(p[d]) + r);
        clo[d] = cell_coord(p[d] - rr, d);
        chi[d] = cell_coord(p[d] + rr, d);
      }
      for (int64_t z = clo[2]; z <= chi[2]; ++z)
        for (int64_t y = clo[1]; y <= chi[1]; ++y) {
          const int64_t row = nc_[0] * (y + nc_[1] * z);
          for (int64_t j = cstart_[row + clo[0]], je = cstart_[row + chi[0] + 1]; j < je; ++j) f(j);
        }
      return;
    }
    // k-d tree: a node is skipped when the squared gap between p and its
    // box exceeds R; the gap per axis is computed from the box bound the
    // way dist2 computes it from a coordinate inside the box, and rounding
    // is monotone, so dist2 of every point inside is at least the gap
    int64_t stack[130];
    int sp = 0;
    stack[sp++] = 1;
    while (sp) {
      const int64_t v = stack[--sp];
      const double* lo = &blo_[v * 3];
      const double* hi = &bhi_[v * 3];
      double g2 = 0.0;
      for (int d = 0; d < dim_; ++d) {
        double g = 0.0;
        if (p[d] < lo[d]) g = lo[d] - p[d];
        else if (p[d] > hi[d]) g = p[d] - hi[d];
        g2 += g * g;
      }
      if (g2 > R) continue;
      if (v >= L_) {
        for (int64_t j = leaf_begin(v - L_), je = leaf_begin(v - L_ + 1); j < je; ++j) f(j);
      } else {
        stack[sp++] = 2 * v + 1;
        stack[sp++] = 2 * v;
      }
    }
  }

 private:
  static constexpr int64_t kCrowded = 32;  // most points a grid cell may hold

  // uniform grid of about two points per cell, slots sorted by cell; false
  // when a coordinate is not finite or a cell holds more than kCrowded
  bool build_grid(const std::vector<double>& pts) {
    double hi[3];
    for (int d = 0; d < dim_; ++d) {
      lo_[d] = std::numeric_limits<double>::infinity();
      hi[d] = -lo_[d];
    }
    for (int64_t i = 0; i < n_; ++i)
      for (int d = 0; d < dim_; ++d) {
        const double v = pts[i * dim_ + d];
        if (!std::isfinite(v)) return false;
        lo_[d] = std::min(lo_[d], v);
        hi[d] = std::max(hi[d], v);
      }
    double ext = 0.0;
    for (int d = 0; d < dim_; ++d) ext = std::max(ext, hi[d] - lo_[d]);
    if (!(ext > 0.0) || !std::isfinite(ext)) return false;
    double vol = 1.0;
    int act = 0;
    for (int d = 0; d < dim_; ++d)
      if (hi[d] - lo_[d] > ext * 1e-9) {
        vol *= hi[d] - lo_[d];
        ++act;
      }
    cell_ = pow(vol * 2.0 / (double)n_, 1.0 / act);
    if (!(cell_ > 0.0) || !std::isfinite(cell_)) return false;
    double total = 1.0;
    for (int d = 0; d < dim_; ++d) {
      nc_[d] = 1;
      if (hi[d] - lo_[d] > ext * 1e-9) {
        const double c = ceil((hi[d] - lo_[d]) / cell_);
        if (!(c < 1e12)) return false;
        nc_[d] = std::max<int64_t>(1, (int64_t)c);
      }
      total *= (double)nc_[d];
    }
    if (total > 4.0 * (double)n_ + 64.0) return false;
    const int64_t ncell = nc_[0] * nc_[1] * nc_[2];
    std::vector<int64_t> cell_of(n_);
    cstart_.assign(ncell + 1, 0);
    for (int64_t i = 0; i < n_; ++i) {
      int64_t id = 0, stride = 1;
      for (int d = 0; d < dim_; ++d) {
        id += cell_coord(pts[i * dim_ + d], d) * stride;
        stride *= nc_[d];
      }
      cell_of[i] = id;
      if (++cstart_[id + 1] > kCrowded) return false;
    }
    for (int64_t k = 0; k < ncell; ++k) cstart_[k + 1] += cstart_[k];
    std::vector<int64_t> fill(cstart_.begin(), cstart_.end() - 1);
    for (int64_t i = 0; i < n_; ++i) idx_[fill[cell_of[i]]++] = i;
    grid_ = true;
    return true;
  }
  int64_t cell_coord(double v, int d) const {
    const double q = floor((v - lo_[d]) / cell_);
    return q < 0.0 ? 0 : (q >= (double)nc_[d] ? nc_[d] - 1 : (int64_t)q);
  }

  // balanced k-d tree in heap layout: L_ leaves (a power of two), node v
  // (1 <= v < 2 L_) covering leaves [k0, k1) holds slots
  // [leaf_begin(k0), leaf_begin(k1)); each inner node splits its slots at
  // its middle leaf boundary along its widest axis (coordinates compared in
  // total order, so any input keeps the selection well defined)
  void build_tree(const std::vector<double>& pts) {
    L_ = 1;
    while (L_ * 32 <= n_) L_ <<= 1;
    for (int64_t v = 1; v < L_; ++v) {
      int depth = 0;
      while (((int64_t)2 << depth) <= v) ++depth;
      const int64_t span = L_ >> depth, k0 = (v - ((int64_t)1 << depth)) * span;
      const int64_t b = leaf_begin(k0), e = leaf_begin(k0 + span), mid = leaf_begin(k0 + span / 2);
      double lo[3], hi[3];
      for (int d = 0; d < dim_; ++d) {
        lo[d] = std::numeric_limits<double>::infinity();
        hi[d] = -lo[d];
      }
      for (int64_t k = b; k < e; ++k)
        for (int d = 0; d < dim_; ++d) {
          const double x = pts[idx_[k] * dim_ + d];
          lo[d] = std::min(lo[d], x);
          hi[d] = std::max(hi[d], x);
        }
      int ax = 0;
      double w = -1.0;
      for (int d = 0; d < dim_; ++d)
        if (hi[d] - lo[d] > w) {
          w = hi[d] - lo[d];
          ax = d;
        }
      if (mid > b && mid < e)
        std::nth_element(idx_.begin() + b, idx_.begin() + mid, idx_.begin() + e,
                         [&](int64_t a, int64_t c) {
                           return tkey(pts[a * dim_ + ax]) < tkey(pts[c * dim_ + ax]);
                         });
    }
  }
  // boxes of the leaves from their slots, of inner nodes from their children
  void tree_boxes() {
    blo_.assign(2 * L_ * 3, std::numeric_limits<double>::infinity());
    bhi_.assign(2 * L_ * 3, -std::numeric_limits<double>::infinity());
    for (int64_t k = 0; k < L_; ++k) {
      double* lo = &blo_[(L_ + k) * 3];
      double* hi = &bhi_[(L_ + k) * 3];
      for (int64_t j = leaf_begin(k), je = leaf_begin(k + 1); j < je; ++j)
        for (int d = 0; d < dim_; ++d) {
          lo[d] = std::min(lo[d], xs_[j * dim_ + d]);
          hi[d] = std::max(hi[d], xs_[j * dim_ + d]);
        }
    }
    for (int64_t v = L_ - 1; v >= 1; --v)
      for (int d = 0; d < 3; ++d) {
        blo_[v * 3 + d] = std::min(blo_[2 * v * 3 + d], blo_[(2 * v + 1) * 3 + d]);
        bhi_[v * 3 + d] = std::max(bhi_[2 * v * 3 + d], bhi_[(2 * v + 1) * 3 + d]);
      }
  }
  // first slot of leaf k: floor(n k / L) without overflow
  int64_t leaf_begin(int64_t k) const { return (n_ / L_) * k + (n_ % L_) * k / L_; }

  int dim_;
  int64_t n_;
  std::vector<int64_t> idx_;  // slot -> point
  std::vector<double> xs_;    // coordinates by slot
  bool grid_ = false;
  double lo_[3] = {0, 0, 0}, cell_ = 1.0;
  int64_t nc_[3] = {1, 1, 1};
  std::vector<int64_t> cstart_;  // grid: slots of cell c are [cstart_[c], cstart_[c + 1])
  int64_t L_ = 1;
  std::vector<double> blo_, bhi_;  // k-d tree: box of node v at [3 v, 3 v + 3)
};

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
  order[0] = first;
  if (n == 1) return;
  const MaxminLayout lay(pts, dim, n);
  // keys by slot in total order (INT64_MIN once selected); win[v] is the
  // slot of the largest (key, point index) below node v of a binary tree
  // over the slots (leaves at size + j; slot n stands for padding)
  std::vector<int64_t> key(n + 1), pid(n + 1);
  int64_t sfirst = 0;
  for (int64_t j = 0; j < n; ++j) {
    pid[j] = lay.point(j);
    key[j] = tkey(dist2(lay.at(j), &pts[first * dim], dim));
    if (pid[j] == first) sfirst = j;
  }
  key[n] = std::numeric_limits<int64_t>::min();
  pid[n] = -1;
  int64_t size = 1;
  while (size < n) size <<= 1;
  std::vector<int64_t> win(2 * size);
  auto better = [&](int64_t a, int64_t b) {
    return (key[a] != key[b] ? key[a] > key[b] : pid[a] > pid[b]) ? a : b;
  };
  for (int64_t j = 0; j < size; ++j) win[size + j] = j < n ? j : n;
  // slot j's key went down: a node changes only while j was its winner
  auto lowered = [&](int64_t j) {
    for (int64_t v = (size + j) >> 1; v >= 1; v >>= 1) {
      const int64_t old = win[v];
      win[v] = better(win[2 * v], win[2 * v + 1]);
      if (old != j && win[v] == old) break;
    }
  };
  key[sfirst] = std::numeric_limits<int64_t>::min();
  for (int64_t v = size - 1; v >= 1; --v) win[v] = better(win[2 * v], win[2 * v + 1]);
  for (int64_t nsel = 1; nsel < n; ++nsel) {
    const int64_t s = win[1];
    order[nsel] = pid[s];
    double R;
    std::memcpy(&R, &key[s], 8);
    key[s] = std::numeric_limits<int64_t>::min();
    lowered(s);
    const double* ps = lay.at(s);
    lay.visit_ball(ps, R, [&](int64_t j) {
      const int64_t e = tkey(dist2(lay.at(j), ps, dim));
      if (e < key[j]) {
        key[j] = e;
        lowered(j);
      }
    });
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
