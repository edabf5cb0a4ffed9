// lbfgsb.cpp -- L-BFGS-B written from Byrd-Lu-Nocedal-Zhu (1995), Morales-Nocedal (2011) and More-Thuente (1994).
// See lbfgsb.hpp for the references.  Dense linear algebra of the 2k x 2k middle matrices is done with a small
// partial-pivoting LU (k <= m corrections).
#include "lbfgsb.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <numeric>
#include <stdexcept>

namespace lkg {

namespace {

constexpr double EPSMCH = DBL_EPSILON;

// ---------------------------------------------------------------------------------------------------------------
// small dense LU solver
struct LU {
  int n = 0;
  std::vector<double> a;  // row-major n x n, factored in place
  std::vector<int> piv;
  bool factor(const std::vector<double>& A, int nn) {
    n = nn;
    a = A;
    piv.resize(n);
    for (int k = 0; k < n; ++k) {
      int p = k;
      for (int i = k + 1; i < n; ++i)
        if (std::fabs(a[i * n + k]) > std::fabs(a[p * n + k])) p = i;
      if (!(std::fabs(a[p * n + k]) > 0.0) || !std::isfinite(a[p * n + k])) return false;
      piv[k] = p;
      if (p != k)
        for (int j = 0; j < n; ++j) std::swap(a[k * n + j], a[p * n + j]);
      for (int i = k + 1; i < n; ++i) {
        a[i * n + k] /= a[k * n + k];
        for (int j = k + 1; j < n; ++j) a[i * n + j] -= a[i * n + k] * a[k * n + j];
      }
    }
    return true;
  }
  void solve(std::vector<double>& b) const {
    for (int k = 0; k < n; ++k)
      if (piv[k] != k) std::swap(b[k], b[piv[k]]);
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < i; ++k) b[i] -= a[i * n + k] * b[k];
    for (int i = n - 1; i >= 0; --i) {
      for (int k = i + 1; k < n; ++k) b[i] -= a[i * n + k] * b[k];
      b[i] /= a[i * n + i];
    }
  }
};

// ---------------------------------------------------------------------------------------------------------------
// limited-memory BFGS matrix B = theta I - W M W', W = [Y, theta S], M = K^-1, K = [[-D, L'], [L, theta S'S]]
struct Memory {
  int n, m;
  std::vector<std::vector<double>> S, Y;  // oldest first
  double theta = 1.0;
  LU Klu;
  std::vector<double> K;  // 2k x 2k row-major
  Memory(int n_, int m_) : n(n_), m(m_) {}
  int k() const { return (int)S.size(); }
  void reset() {
    S.clear();
    Y.clear();
    theta = 1.0;
  }
  void push(const std::vector<double>& s, const std::vector<double>& y) {
    if ((int)S.size() == m) {
      S.erase(S.begin());
      Y.erase(Y.begin());
    }
    S.push_back(s);
    Y.push_back(y);
  }
  static double dot(const std::vector<double>& a, const std::vector<double>& b) {
    double s = 0.0;
    for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
    return s;
  }
  bool form() {  // build and factor K
    const int kk = k(), k2 = 2 * kk;
    K.assign((size_t)k2 * k2, 0.0);
    for (int i = 0; i < kk; ++i) {
      K[i * k2 + i] = -dot(S[i], Y[i]);
      for (int j = 0; j < kk; ++j) {
        if (i > j) {  // L_ij = s_i' y_j
          const double l = dot(S[i], Y[j]);
          K[(kk + i) * k2 + j] = l;   // L block (lower-left)
          K[j * k2 + (kk + i)] = l;   // L' block (upper-right)
        }
        K[(kk + i) * k2 + (kk + j)] = theta * dot(S[i], S[j]);
      }
    }
    return kk == 0 || Klu.factor(K, k2);
  }
  // W row i (length 2k)
  void wrow(int i, std::vector<double>& w) const {
    const int kk = k();
    w.resize(2 * kk);
    for (int j = 0; j < kk; ++j) {
      w[j] = Y[j][i];
      w[kk + j] = theta * S[j][i];
    }
  }
  void Mv(const std::vector<double>& v, std::vector<double>& out) const {  // out = M v = K^-1 v
    out = v;
    if (k() > 0) Klu.solve(out);
  }
};

// ---------------------------------------------------------------------------------------------------------------
// More-Thuente line search (safeguarded step and search driver)
void dcstep(double& stx, double& fx, double& dx, double& sty, double& fy, double& dy, double& stp, double fp,
            double dp, bool& brackt, double stpmin, double stpmax) {
  const double p66 = 0.66;
  const double sgnd = dp * (dx / std::fabs(dx));
  double stpf;
  if (fp > fx) {
    const double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
    const double s = std::max({std::fabs(theta), std::fabs(dx), std::fabs(dp)});
    double gamma = s * std::sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
    if (stp < stx) gamma = -gamma;
    const double p = (gamma - dx) + theta;
    const double q = ((gamma - dx) + gamma) + dp;
    const double r = p / q;
    const double stpc = stx + r * (stp - stx);
    const double stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2.0) * (stp - stx);
    if (std::fabs(stpc - stx) < std::fabs(stpq - stx))
      stpf = stpc;
    else
      stpf = stpc + (stpq - stpc) / 2.0;
    brackt = true;
  } else if (sgnd < 0.0) {
    const double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
    const double s = std::max({std::fabs(theta), std::fabs(dx), std::fabs(dp)});
    double gamma = s * std::sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
    if (stp > stx) gamma = -gamma;
    const double p = (gamma - dp) + theta;
    const double q = ((gamma - dp) + gamma) + dx;
    const double r = p / q;
    const double stpc = stp + r * (stx - stp);
    const double stpq = stp + (dp / (dp - dx)) * (stx - stp);
    if (std::fabs(stpc - stp) > std::fabs(stpq - stp))
      stpf = stpc;
    else
      stpf = stpq;
    brackt = true;
  } else if (std::fabs(dp) < std::fabs(dx)) {
    const double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
    const double s = std::max({std::fabs(theta), std::fabs(dx), std::fabs(dp)});
    double gamma = s * std::sqrt(std::max(0.0, (theta / s) * (theta / s) - (dx / s) * (dp / s)));
    if (stp > stx) gamma = -gamma;
    const double p = (gamma - dp) + theta;
    const double q = (gamma + (dx - dp)) + gamma;
    const double r = p / q;
    double stpc;
    if (r < 0.0 && gamma != 0.0)
      stpc = stp + r * (stx - stp);
    else if (stp > stx)
      stpc = stpmax;
    else
      stpc = stpmin;
    const double stpq = stp + (dp / (dp - dx)) * (stx - stp);
    if (brackt) {
      stpf = (std::fabs(stpc - stp) < std::fabs(stpq - stp)) ? stpc : stpq;
      if (stp > stx)
        stpf = std::min(stp + p66 * (sty - stp), stpf);
      else
        stpf = std::max(stp + p66 * (sty - stp), stpf);
    } else {
      stpf = (std::fabs(stpc - stp) > std::fabs(stpq - stp)) ? stpc : stpq;
      stpf = std::min(stpmax, stpf);
      stpf = std::max(stpmin, stpf);
    }
  } else {
    if (brackt) {
      const double theta = 3.0 * (fp - fy) / (sty - stp) + dy + dp;
      const double s = std::max({std::fabs(theta), std::fabs(dy), std::fabs(dp)});
      double gamma = s * std::sqrt((theta / s) * (theta / s) - (dy / s) * (dp / s));
      if (stp > sty) gamma = -gamma;
      const double p = (gamma - dp) + theta;
      const double q = ((gamma - dp) + gamma) + dy;
      const double r = p / q;
      stpf = stp + r * (sty - stp);
    } else if (stp > stx) {
      stpf = stpmax;
    } else {
      stpf = stpmin;
    }
  }
  if (fp > fx) {
    sty = stp;
    fy = fp;
    dy = dp;
  } else {
    if (sgnd < 0.0) {
      sty = stx;
      fy = fx;
      dy = dx;
    }
    stx = stp;
    fx = fp;
    dx = dp;
  }
  stp = stpf;
}

struct LineSearch {
  double ftol = 1e-3, gtol = 0.9, xtol = 0.1, stpmin = 0.0, stpmax = 0.0;
  bool brackt = false;
  int stage = 1;
  double ginit = 0, gtest = 0, gx = 0, gy = 0, finit = 0, fx = 0, fy = 0, stx = 0, sty = 0, stmin = 0, stmax = 0,
         width = 0, width1 = 0;
  // returns "FG", "CONVERGENCE", "WARNING: ..." or "ERROR: ..."
  std::string start(double f, double g, double& stp) {
    if (stp < stpmin) return "ERROR: STP .LT. STPMIN";
    if (stp > stpmax) return "ERROR: STP .GT. STPMAX";
    if (g >= 0.0) return "ERROR: INITIAL G .GE. ZERO";
    brackt = false;
    stage = 1;
    finit = f;
    ginit = g;
    gtest = ftol * ginit;
    width = stpmax - stpmin;
    width1 = width / 0.5;
    stx = 0.0;
    fx = finit;
    gx = ginit;
    sty = 0.0;
    fy = finit;
    gy = ginit;
    stmin = 0.0;
    stmax = stp + 4.0 * stp;
    return "FG";
  }
  std::string step(double f, double g, double& stp) {
    const double xtrapl = 1.1, xtrapu = 4.0;
    const double ftest = finit + stp * gtest;
    if (stage == 1 && f <= ftest && g >= 0.0) stage = 2;
    std::string task;
    if (brackt && (stp <= stmin || stp >= stmax)) task = "WARNING: ROUNDING ERRORS PREVENT PROGRESS";
    if (brackt && stmax - stmin <= xtol * stmax) task = "WARNING: XTOL TEST SATISFIED";
    if (stp == stpmax && f <= ftest && g <= gtest) task = "WARNING: STP = STPMAX";
    if (stp == stpmin && (f > ftest || g >= gtest)) task = "WARNING: STP = STPMIN";
    if (f <= ftest && std::fabs(g) <= gtol * (-ginit)) task = "CONVERGENCE";
    if (!task.empty()) return task;
    if (stage == 1 && f <= fx && f > ftest) {
      const double fm = f - stp * gtest;
      double fxm = fx - stx * gtest, fym = fy - sty * gtest;
      const double gm = g - gtest;
      double gxm = gx - gtest, gym = gy - gtest;
      dcstep(stx, fxm, gxm, sty, fym, gym, stp, fm, gm, brackt, stmin, stmax);
      fx = fxm + stx * gtest;
      fy = fym + sty * gtest;
      gx = gxm + gtest;
      gy = gym + gtest;
    } else {
      dcstep(stx, fx, gx, sty, fy, gy, stp, f, g, brackt, stmin, stmax);
    }
    if (brackt) {
      if (std::fabs(sty - stx) >= 0.66 * width1) stp = stx + 0.5 * (sty - stx);
      width1 = width;
      width = std::fabs(sty - stx);
    }
    if (brackt) {
      stmin = std::min(stx, sty);
      stmax = std::max(stx, sty);
    } else {
      stmin = stp + xtrapl * (stp - stx);
      stmax = stp + xtrapu * (stp - stx);
    }
    stp = std::max(stp, stpmin);
    stp = std::min(stp, stpmax);
    if ((brackt && (stp <= stmin || stp >= stmax)) || (brackt && stmax - stmin <= xtol * stmax)) stp = stx;
    return "FG";
  }
};

double proj_grad_norm(const std::vector<double>& x, const std::vector<double>& g, const double* l, const double* u,
                      const int* nbd) {
  double s = 0.0;
  for (size_t i = 0; i < x.size(); ++i) {
    double gi = g[i];
    if (nbd[i] != 0) {
      if (gi < 0.0) {
        if (nbd[i] >= 2) gi = std::max(x[i] - u[i], gi);
      } else {
        if (nbd[i] <= 2) gi = std::min(x[i] - l[i], gi);
      }
    }
    s = std::max(s, std::fabs(gi));
  }
  return s;
}

// Generalized Cauchy point (BLNZ 1995, section 4).  iwhere: 0 free, 1 at lower, 2 at upper, -1 never bounded,
// -3 zero gradient.  c = W'(xcp - x).
void cauchy(const Memory& mem, const std::vector<double>& x, const std::vector<double>& g, const double* l,
            const double* u, const int* nbd, std::vector<double>& xcp, std::vector<double>& c,
            std::vector<int>& iwhere) {
  const int n = (int)x.size(), kk = mem.k(), k2 = 2 * kk;
  const double theta = mem.theta;
  std::vector<double> d(n, 0.0), p(k2, 0.0), wbp, v;
  std::vector<std::pair<double, int>> brk;
  double f1 = 0.0;
  bool bnded = true;
  int nfree_unbounded = 0;
  for (int i = 0; i < n; ++i) {
    const double neggi = -g[i];
    double tl = 0.0, tu = 0.0;
    if (nbd[i] == 0) {
      iwhere[i] = -1;
    } else {
      if (nbd[i] <= 2) tl = x[i] - l[i];
      if (nbd[i] >= 2) tu = u[i] - x[i];
      const bool xlower = nbd[i] <= 2 && tl <= 0.0;
      const bool xupper = nbd[i] >= 2 && tu <= 0.0;
      iwhere[i] = 0;
      if (xlower) {
        if (neggi <= 0.0) iwhere[i] = 1;
      } else if (xupper) {
        if (neggi >= 0.0) iwhere[i] = 2;
      } else if (std::fabs(neggi) <= 0.0) {
        iwhere[i] = -3;
      }
    }
    if (iwhere[i] != 0 && iwhere[i] != -1) {
      d[i] = 0.0;
    } else {
      d[i] = neggi;
      f1 -= neggi * neggi;
      for (int j = 0; j < kk; ++j) {
        p[j] += mem.Y[j][i] * neggi;
        p[kk + j] += mem.S[j][i] * neggi;
      }
      if (nbd[i] <= 2 && nbd[i] != 0 && neggi < 0.0) {
        brk.push_back({tl / (-neggi), i});
      } else if (nbd[i] >= 2 && neggi > 0.0) {
        brk.push_back({tu / neggi, i});
      } else {
        nfree_unbounded++;
        if (std::fabs(neggi) > 0.0) bnded = false;
      }
    }
  }
  for (int j = 0; j < kk; ++j) p[kk + j] *= theta;
  xcp = x;
  c.assign(k2, 0.0);
  if (brk.empty() && nfree_unbounded == 0) return;  // d is the zero vector
  double f2 = -theta * f1;
  const double f2_org = f2;
  if (kk > 0) {
    mem.Mv(p, v);
    double s = 0.0;
    for (int j = 0; j < k2; ++j) s += v[j] * p[j];
    f2 -= s;
  }
  double dtm = -f1 / f2;
  double tsum = 0.0;
  std::stable_sort(brk.begin(), brk.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  const int nbreak = (int)brk.size();
  double tj = 0.0;
  bool all_fixed = false;
  for (int it = 0; it < nbreak; ++it) {
    const double tj0 = tj;
    tj = brk[it].first;
    const int ibp = brk[it].second;
    const double dt = tj - tj0;
    if (dtm < dt) break;
    tsum += dt;
    const double dibp = d[ibp];
    d[ibp] = 0.0;
    double zibp;
    if (dibp > 0.0) {
      zibp = u[ibp] - x[ibp];
      xcp[ibp] = u[ibp];
      iwhere[ibp] = 2;
    } else {
      zibp = l[ibp] - x[ibp];
      xcp[ibp] = l[ibp];
      iwhere[ibp] = 1;
    }
    const int nleft = nbreak - it - 1;
    if (nleft == 0 && nbreak == n) {
      dtm = dt;
      all_fixed = true;
      break;
    }
    const double dibp2 = dibp * dibp;
    f1 = f1 + dt * f2 + dibp2 - theta * dibp * zibp;
    f2 = f2 - theta * dibp2;
    if (kk > 0) {
      for (int j = 0; j < k2; ++j) c[j] += dt * p[j];
      mem.wrow(ibp, wbp);
      mem.Mv(wbp, v);
      double wmc = 0.0, wmp = 0.0, wmw = 0.0;
      for (int j = 0; j < k2; ++j) {
        wmc += c[j] * v[j];
        wmp += p[j] * v[j];
        wmw += wbp[j] * v[j];
      }
      for (int j = 0; j < k2; ++j) p[j] -= dibp * wbp[j];
      f1 += dibp * wmc;
      f2 += 2.0 * dibp * wmp - dibp2 * wmw;
    }
    f2 = std::max(EPSMCH * f2_org, f2);
    if (nleft > 0) {
      dtm = -f1 / f2;
    } else if (bnded) {
      f1 = 0.0;
      f2 = 0.0;
      dtm = 0.0;
    } else {
      dtm = -f1 / f2;
    }
  }
  if (!all_fixed) {
    if (dtm <= 0.0) dtm = 0.0;
    tsum += dtm;
    for (int i = 0; i < n; ++i) xcp[i] += tsum * d[i];
  }
  if (kk > 0)
    for (int j = 0; j < k2; ++j) c[j] += dtm * p[j];
}

}  // namespace

LbfgsbResult Lbfgsb::minimize(const std::function<double(const std::vector<double>&, std::vector<double>&)>& fg,
                              std::vector<double>& x, const double* l, const double* u, const int* nbd) {
  const int n = n_;
  if ((int)x.size() != n) throw std::invalid_argument("Lbfgsb::minimize: x has wrong size");
  LbfgsbResult res;
  const double tol = factr * EPSMCH;
  bool boxed = true, cnstnd = false;
  for (int i = 0; i < n; ++i) {
    if (nbd[i] != 2) boxed = false;
    if (nbd[i] != 0) cnstnd = true;
    if (nbd[i] > 0) {  // project the starting point onto the box
      if (nbd[i] <= 2 && x[i] <= l[i]) x[i] = l[i];
      if (nbd[i] >= 2 && x[i] >= u[i]) x[i] = u[i];
    }
  }
  std::vector<double> g(n), xcp(n), c, d(n), t(n), r(n);
  std::vector<int> iwhere(n);
  double f = fg(x, g);
  res.num_fg = 1;
  double sbg = proj_grad_norm(x, g, l, u, nbd);
  if (sbg <= pgtol) {
    res.f_opt = f;
    res.task = "CONVERGENCE: NORM_OF_PROJECTED_GRADIENT_<=_PGTOL";
    return res;
  }
  Memory mem(n, m);
  int iter = 0;
  for (;;) {
    // ---- generalized Cauchy point and free variables ----
    std::vector<int> freev;
    if (!mem.form()) {
      mem.reset();
      continue;
    }
    if (!cnstnd && mem.k() > 0) {
      xcp = x;
      freev.resize(n);
      std::iota(freev.begin(), freev.end(), 0);
      c.assign(2 * mem.k(), 0.0);
    } else {
      cauchy(mem, x, g, l, u, nbd, xcp, c, iwhere);
      for (int i = 0; i < n; ++i)
        if (iwhere[i] <= 0) freev.push_back(i);
    }
    // ---- subspace minimisation over the free variables (projected Newton step, 2011 remark) ----
    if (!freev.empty() && mem.k() > 0) {
      const int kk = mem.k(), k2 = 2 * kk, ns = (int)freev.size();
      const double theta = mem.theta;
      // r = -Z'(B (xcp - x) + g) = -theta (xcp - x) - g + W M c
      std::vector<double> Mc;
      mem.Mv(c, Mc);
      std::vector<double> rr(ns);
      for (int a = 0; a < ns; ++a) {
        const int i = freev[a];
        double s = -theta * (xcp[i] - x[i]) - g[i];
        for (int j = 0; j < kk; ++j) s += mem.Y[j][i] * Mc[j] + theta * mem.S[j][i] * Mc[kk + j];
        rr[a] = s;
      }
      // Ktilde = K - (1/theta) W'Z Z'W ; v = W'Z r ; d = (1/theta) r + (1/theta^2) Z'W Ktilde^-1 v
      std::vector<double> Kt = mem.K, v(k2, 0.0);
      std::vector<double> wz((size_t)ns * k2);
      for (int a = 0; a < ns; ++a) {
        const int i = freev[a];
        for (int j = 0; j < kk; ++j) {
          wz[(size_t)a * k2 + j] = mem.Y[j][i];
          wz[(size_t)a * k2 + kk + j] = theta * mem.S[j][i];
        }
        for (int j = 0; j < k2; ++j) v[j] += wz[(size_t)a * k2 + j] * rr[a];
      }
      for (int p1 = 0; p1 < k2; ++p1)
        for (int p2 = 0; p2 < k2; ++p2) {
          double s = 0.0;
          for (int a = 0; a < ns; ++a) s += wz[(size_t)a * k2 + p1] * wz[(size_t)a * k2 + p2];
          Kt[p1 * k2 + p2] -= s / theta;
        }
      LU klu;
      if (!klu.factor(Kt, k2)) {
        mem.reset();
        continue;
      }
      klu.solve(v);
      std::vector<double> dsub(ns);
      for (int a = 0; a < ns; ++a) {
        double s = 0.0;
        for (int j = 0; j < k2; ++j) s += wz[(size_t)a * k2 + j] * v[j];
        dsub[a] = rr[a] / theta + s / (theta * theta);
      }
      // projection of the Newton point
      std::vector<double> xp = xcp;
      bool hit = false;
      for (int a = 0; a < ns; ++a) {
        const int i = freev[a];
        const double dk = dsub[a], xk = xcp[i];
        if (nbd[i] == 1) {
          xcp[i] = std::max(l[i], xk + dk);
          if (xcp[i] == l[i]) hit = true;
        } else if (nbd[i] == 2) {
          xcp[i] = std::min(u[i], std::max(l[i], xk + dk));
          if (xcp[i] == l[i] || xcp[i] == u[i]) hit = true;
        } else if (nbd[i] == 3) {
          xcp[i] = std::min(u[i], xk + dk);
          if (xcp[i] == u[i]) hit = true;
        } else {
          xcp[i] = xk + dk;
        }
      }
      if (hit) {
        double dd_p = 0.0;
        for (int i = 0; i < n; ++i) dd_p += (xcp[i] - x[i]) * g[i];
        if (dd_p > 0.0) {  // not a descent direction: truncated step from the Cauchy point
          xcp = xp;
          double alpha = 1.0, temp1 = alpha;
          int ibd = -1;
          for (int a = 0; a < ns; ++a) {
            const int i = freev[a];
            const double dk = dsub[a];
            if (nbd[i] != 0) {
              if (dk < 0.0 && nbd[i] <= 2) {
                const double temp2 = l[i] - xcp[i];
                if (temp2 >= 0.0) temp1 = 0.0;
                else if (dk * alpha < temp2) temp1 = temp2 / dk;
              } else if (dk > 0.0 && nbd[i] >= 2) {
                const double temp2 = u[i] - xcp[i];
                if (temp2 <= 0.0) temp1 = 0.0;
                else if (dk * alpha > temp2) temp1 = temp2 / dk;
              }
              if (temp1 < alpha) {
                alpha = temp1;
                ibd = a;
              }
            }
          }
          if (alpha < 1.0 && ibd >= 0) {
            const double dk = dsub[ibd];
            const int i = freev[ibd];
            if (dk > 0.0) {
              xcp[i] = u[i];
              dsub[ibd] = 0.0;
            } else if (dk < 0.0) {
              xcp[i] = l[i];
              dsub[ibd] = 0.0;
            }
          }
          for (int a = 0; a < ns; ++a) xcp[freev[a]] += alpha * dsub[a];
        }
      }
    }
    // ---- line search along d = xcp - x ----
    for (int i = 0; i < n; ++i) d[i] = xcp[i] - x[i];
    double dnorm = 0.0;
    for (int i = 0; i < n; ++i) dnorm += d[i] * d[i];
    dnorm = std::sqrt(dnorm);
    double stpmx = 1e10;
    if (cnstnd) {
      if (iter == 0) {
        stpmx = 1.0;
      } else {
        for (int i = 0; i < n; ++i) {
          const double a1 = d[i];
          if (nbd[i] != 0) {
            if (a1 < 0.0 && nbd[i] <= 2) {
              const double a2 = l[i] - x[i];
              if (a2 >= 0.0) stpmx = 0.0;
              else if (a1 * stpmx < a2) stpmx = a2 / a1;
            } else if (a1 > 0.0 && nbd[i] >= 2) {
              const double a2 = u[i] - x[i];
              if (a2 <= 0.0) stpmx = 0.0;
              else if (a1 * stpmx > a2) stpmx = a2 / a1;
            }
          }
        }
      }
    }
    double stp = (iter == 0 && !boxed) ? std::min(1.0 / dnorm, stpmx) : 1.0;
    t = x;
    r = g;
    const double fold = f;
    double gd = 0.0;
    for (int i = 0; i < n; ++i) gd += g[i] * d[i];
    const double gdold = gd;
    bool ls_ok = false;
    int ifun = 0;
    if (gd < 0.0 && dnorm > 0.0) {
      LineSearch ls;
      ls.stpmax = stpmx;
      if (stp > stpmx) stp = stpmx;
      std::string task = ls.start(f, gd, stp);
      while (task == "FG") {
        if (ifun >= 20 || res.num_fg >= max_fun) break;
        if (stp == 1.0)
          x = xcp;
        else
          for (int i = 0; i < n; ++i) x[i] = stp * d[i] + t[i];
        f = fg(x, g);
        res.num_fg++;
        ifun++;
        gd = 0.0;
        for (int i = 0; i < n; ++i) gd += g[i] * d[i];
        task = ls.step(f, gd, stp);
        if (task.rfind("CONV", 0) == 0 || task.rfind("WARN", 0) == 0) ls_ok = true;
      }
    }
    if (!ls_ok) {
      x = t;
      g = r;
      f = fold;
      if (mem.k() == 0) {
        res.f_opt = f;
        res.num_iters = iter + 1;
        res.task = "ABNORMAL_TERMINATION_IN_LNSRCH";
        return res;
      }
      mem.reset();  // refresh the memory and restart the iteration
      continue;
    }
    iter++;
    sbg = proj_grad_norm(x, g, l, u, nbd);
    if (iter >= max_iter) {
      res.f_opt = f;
      res.num_iters = iter;
      res.task = "STOP: TOTAL NO. of ITERATIONS REACHED LIMIT";
      return res;
    }
    if (res.num_fg >= max_fun) {
      res.f_opt = f;
      res.num_iters = iter;
      res.task = "STOP: TOTAL NO. of f AND g EVALUATIONS EXCEEDS LIMIT";
      return res;
    }
    if (sbg <= pgtol) {
      res.f_opt = f;
      res.num_iters = iter;
      res.task = "CONVERGENCE: NORM_OF_PROJECTED_GRADIENT_<=_PGTOL";
      return res;
    }
    const double ddum = std::max({std::fabs(fold), std::fabs(f), 1.0});
    if (fold - f <= tol * ddum) {
      res.f_opt = f;
      res.num_iters = iter;
      res.task = "CONVERGENCE: REL_REDUCTION_OF_F_<=_FACTR*EPSMCH";
      return res;
    }
    // ---- update the limited-memory matrix ----
    std::vector<double> s(n), y(n);
    for (int i = 0; i < n; ++i) y[i] = g[i] - r[i];
    double rr2 = 0.0;
    for (int i = 0; i < n; ++i) rr2 += y[i] * y[i];
    double dr, ddum2;
    if (stp == 1.0) {
      dr = gd - gdold;
      ddum2 = -gdold;
      s = d;
    } else {
      dr = (gd - gdold) * stp;
      for (int i = 0; i < n; ++i) s[i] = stp * d[i];
      ddum2 = -gdold * stp;
    }
    if (dr <= EPSMCH * ddum2) continue;  // skip the update
    mem.push(s, y);
    mem.theta = rr2 / dr;
  }
}

}  // namespace lkg
