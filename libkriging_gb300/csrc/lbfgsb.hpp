// lbfgsb.hpp -- bound-constrained limited-memory BFGS (L-BFGS-B), written for this library from the published
// algorithm:
//   R. H. Byrd, P. Lu, J. Nocedal, C. Zhu, "A limited memory algorithm for bound constrained optimization",
//     SIAM J. Sci. Comput. 16(5), 1995  (generalized Cauchy point, compact L-BFGS matrices, subspace minimisation);
//   J. L. Morales, J. Nocedal, "Remark on Algorithm 778", ACM TOMS 38(1), 2011  (projected subspace step);
//   J. J. More, D. J. Thuente, "Line search algorithms with guaranteed sufficient decrease", ACM TOMS 20(3), 1994.
//
// Interface mirrors what libKriging's fit loop uses from its lbfgsb_cpp dependency (src/lib/Kriging.cpp:1950-1992):
// an Optimizer{n} with fields iprint, max_iter, pgtol, factr, and minimize(f, x, lb, ub, bounds_type) returning
// {f_opt, num_iters, task}; task strings follow the classic driver ("CONVERGENCE: ...", "ABNORMAL_TERMINATION_IN_LNSRCH",
// "STOP: TOTAL NO. of ITERATIONS REACHED LIMIT").
#pragma once
#include <functional>
#include <string>
#include <vector>

namespace lkg {

struct LbfgsbResult {
  double f_opt = 0.0;
  int num_iters = 0;
  int num_fg = 0;
  std::string task;
};

class Lbfgsb {
 public:
  explicit Lbfgsb(int n) : n_(n) {}
  int iprint = -1;
  int max_iter = 20;
  int m = 5;               // number of correction pairs
  int max_fun = 15000;     // function evaluations limit
  double pgtol = 1e-5;
  double factr = 1e7;
  // fg(x, g) returns f(x) and writes g.  x is updated in place to the best point found.
  // bounds_type per variable: 0 unbounded, 1 lower only, 2 both, 3 upper only.
  LbfgsbResult minimize(const std::function<double(const std::vector<double>&, std::vector<double>&)>& fg,
                        std::vector<double>& x, const double* lb, const double* ub, const int* bounds_type);

 private:
  int n_;
};

}  // namespace lkg
