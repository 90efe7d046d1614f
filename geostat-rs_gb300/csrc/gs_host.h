// gs_host.h -- host-side runtime declarations (see gs_host.cu).
#pragma once

#include <stdint.h>

#include <utility>
#include <vector>

namespace gs {

const char* last_error();
int validate_anisotropy(double az, double ratio, double ratio_z, double dip, double rake);
void rotation_3d(double az, double ratio, double ratio_z, double dip, double rake, double r[9]);

struct Xoshiro {
  uint64_t s[4];
  bool has_spare = false;
  double spare = 0.0;
  explicit Xoshiro(uint64_t seed);
  uint64_t next();
  double uniform();
  double normal();
};

// pts is n x dim row-major.
void maxmin_order(const std::vector<double>& pts, int dim, int64_t n, int64_t* order);

class NelderMead {
 public:
  NelderMead(const std::vector<double>& x0, double step, int64_t max_iter);
  bool done() const { return stage_ == kDone; }
  const std::vector<std::vector<double>>& pending() const { return pending_; }
  void supply(const std::vector<double>& f);
  std::pair<std::vector<double>, double> best() const;

 private:
  enum Stage { kInit, kReflect, kExpand, kContract, kShrink, kDone };
  void begin_iteration();
  void end_iteration();
  size_t n_;
  int64_t max_iter_;
  int64_t it_ = 0;
  Stage stage_ = kInit;
  std::vector<std::vector<double>> simplex_;
  std::vector<double> fv_;
  std::vector<double> centroid_, xr_;
  double fr_ = 0.0;
  std::vector<std::vector<double>> pending_;
};

std::pair<std::vector<double>, double> multistart_best(const std::vector<NelderMead>& runs);

}  // namespace gs
