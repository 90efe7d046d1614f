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

// optim.rs:207-275 bfgs as a state machine: each step asks for either the
// objective or the gradient at one point (pending_x / wants_gradient), and
// supply_f / supply_g feed the answer back, so several runs can be advanced
// in lock-step with their requests evaluated in one batched launch.  The
// iterates, line-search decisions and inverse-Hessian updates are those of the
// sequential algorithm.
class Bfgs {
 public:
  Bfgs(const std::vector<double>& x0, int64_t max_iter);
  bool done() const { return stage_ == kDone; }
  bool wants_gradient() const { return stage_ == kInitG || stage_ == kGnew; }
  const std::vector<double>& pending_x() const { return req_; }
  void supply_f(double f);
  void supply_g(const std::vector<double>& g);
  std::pair<std::vector<double>, double> best() const { return {best_x_, best_f_}; }

 private:
  enum Stage { kInitG, kInitF, kSearch, kGnew, kDone };
  void begin_iteration();
  size_t n_;
  int64_t max_iter_;
  int64_t it_ = 0;
  Stage stage_ = kInitG;
  std::vector<double> x_, g_, h_, p_, xnew_, req_, best_x_;
  double fx_ = 0.0, slope_ = 0.0, alpha_ = 1.0, fnew_ = 0.0, best_f_ = 0.0;
};

// optim.rs:281-289: the first run with the strictly smallest optimum.
std::pair<std::vector<double>, double> bfgs_multistart_best(const std::vector<Bfgs>& runs);

}  // namespace gs
