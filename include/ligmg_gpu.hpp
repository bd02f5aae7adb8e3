// ligmg_gpu.hpp — C++ facade over the C ABI (ligmg_gpu.h), shaped like the
// reference's ligmg::Solver (include/ligmg/ligmg.hpp:12-60):
//
//   ligmg::gpu::Solver s(n, rowptr, col, val);            // Solver(A)
//   ligmg::gpu::Solver s(n, rowptr, col, val, opts);      // Solver(A, Options)
//   ligmg::gpu::ConvergenceInfo r = s.solve(b);            // solve(b)
//   r = s.solve(b, from);                                  // solve(b, from)
//   s.print();                                             // print()
//   s.dump_csv(std::cout, r);                              // dump_csv(os, cvinfo)
//
// Errors become std::runtime_error, as PETSC_CHECK_ERROR does in the
// reference (util.hpp:653-660).  Header-only; link with -lligmg_gb300.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <ostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "ligmg_gpu.h"

namespace ligmg {
namespace gpu {

struct Options : ligmg_options {
  Options() { ligmg_default_options(this); }  // default_options(), options.hpp:136
};

inline void check(ligmg_status s, const char *what) {
  if (s != LIGMG_OK && s != LIGMG_NOT_CONVERGED)
    throw std::runtime_error(std::string(what) + ": " + ligmg_status_string(s));
}

// ConvergenceInfo (util.hpp:143-170), solution returned by value.
struct ConvergenceInfo {
  std::vector<double> residuals;
  int _iters = 0;
  double _time = 0, _work = 0;
  std::vector<double> solution;
  double true_rel_residual = 0;
  bool converged = false;

  int iters() const { return _iters; }
  double time() const { return _time; }
  double work() const { return _work; }
  double rel_residual() const {
    return residuals.empty() ? 0.0 : residuals.back() / residuals.front();
  }
  double cycle_complexity() const { return _iters ? _work / _iters : 0.0; }
  double cf() const { return std::pow(rel_residual(), 1.0 / _iters); }
  double ecf() const { return std::pow(rel_residual(), 1.0 / (_iters * cycle_complexity())); }
  double wda() const { return -1.0 / std::log10(ecf()); }
};

inline std::ostream &operator<<(std::ostream &os, const ConvergenceInfo &cv) {
  char buf[160];
  std::snprintf(buf, sizeof buf, "%5d %.2e %5.2f %.3f %.3f %5.2f %.2e", cv.iters(),
                cv.rel_residual(), cv.cycle_complexity(), cv.cf(), cv.ecf(), cv.wda(), cv.time());
  return os << "iters    error  comp  conv econv   wda     time\n" << buf;
}

class Solver {
 public:
  Options opts;
  double setup_time = 0;

  Solver(int64_t n, const int64_t *rowptr, const int32_t *col, const double *val,
         Options o = Options())
      : opts(o), n_(n) {
    check(ligmg_create(n, rowptr, col, val, &opts, &h_), "ligmg_create");
  }
  Solver(const Solver &) = delete;
  Solver &operator=(const Solver &) = delete;
  Solver(Solver &&o) noexcept : opts(o.opts), setup_time(o.setup_time), h_(o.h_), n_(o.n_) {
    o.h_ = nullptr;
  }
  ~Solver() {
    if (h_) ligmg_destroy(h_);
  }

  ConvergenceInfo solve(const std::vector<double> &b) const { return solve(b, 0); }

  ConvergenceInfo solve(const std::vector<double> &b, int from) const {
    ConvergenceInfo r;
    r.solution.resize(b.size());
    std::vector<double> hist(opts.iters + 1);
    ligmg_info info{};
    info.residual_history = hist.data();
    info.history_capacity = (int32_t)hist.size();
    ligmg_status s = from == 0 ? ligmg_solve(h_, b.data(), r.solution.data(), &info)
                               : ligmg_solve_from(h_, b.data(), r.solution.data(), from, &info);
    check(s, "ligmg_solve");
    hist.resize(info.history_len);
    r.residuals = hist;
    r._iters = info.iters;
    r._time = info.solve_seconds;
    r._work = info.work;
    r.true_rel_residual = info.true_rel_residual;
    r.converged = info.converged != 0;
    return r;
  }

  // print_hierarchy (multigrid.hpp:265-292)
  void print(std::FILE *f = stdout) const {
    int32_t L = 0;
    check(ligmg_hierarchy_levels(h_, &L), "ligmg_hierarchy_levels");
    std::fprintf(f, "%5s  %10s  %12s  %6s\n", "Level", "Size", "NNZ", "Type");
    for (int32_t l = 0; l < L; l++) {
      int32_t t;
      int64_t n, nnz, nc;
      check(ligmg_level_info(h_, l, &t, &n, &nnz, &nc), "ligmg_level_info");
      const char *name = t == LIGMG_LEVEL_ELIM ? "elim" : t == LIGMG_LEVEL_AGG ? "agg" : "coarse";
      std::fprintf(f, "%5d  %10lld  %12lld  %6s\n", l, (long long)n, (long long)nnz, name);
    }
  }

  // dump_csv (ligmg.hpp:42-45; columns of print_csv, util.hpp:187-205)
  void dump_csv(std::ostream &os, const ConvergenceInfo &cv) const {
    os << "graph,solver,iters,rel_error,cycle_complexity,wda,setup_time,solve_time,nnz,nodes\n"
       << "graph,ligmg," << cv.iters() << ',' << cv.rel_residual() << ','
       << cv.cycle_complexity() << ',' << cv.wda() << ',' << setup_time << ',' << cv.time()
       << ",," << 1 << '\n';
  }

  ligmg_handle handle() const { return h_; }
  int64_t size() const { return n_; }

 private:
  ligmg_handle h_ = nullptr;
  int64_t n_ = 0;
};

}  // namespace gpu
}  // namespace ligmg
