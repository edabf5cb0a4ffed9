/*
 * lk_oracle.c -- CPU FP64 restatement of libKriging's likelihood hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  The GPU results are compared with it; the GPU product never links, loads or calls it.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 *
 * Each function restates one reference routine (paths relative to the libKriging source tree) in the same
 * operation order, so that results agree with the reference to the last few ulps:
 *   ora_cov / ora_dlncov        src/lib/Covariance.cpp:24-36, 38-50, 65-75, 77-88, 104-116, 118-130, 149-161, 163-179
 *   ora_build_R                 src/lib/LinearAlgebra.cpp:142-181  (cholCov: pair loop, *= factor, diag)
 *                               with dX from src/lib/LinearAlgebra.cpp:440-485 (compute_dX) recomputed per pair
 *   ora_grad_terms              src/lib/KrigingImpl.cpp:855-885    (compute_ll_grad_theta_vecs)
 *   ora_alpha_terms             src/lib/Kriging.cpp:307-326        (Nugget alpha-gradient dot products)
 *   ora_vecchia_sets            src/lib/Kriging.cpp:736-804        (maxmin ordering + m nearest earlier points)
 *   ora_vecchia_ll              src/lib/Kriging.cpp:806-924        (_logLikelihoodVecchia)
 *
 * Build:  gcc -O2 -ffp-contract=off -fPIC -shared -o oracle/_build/liblk_oracle.so oracle/lk_oracle.c -lm
 * (-ffp-contract=off keeps a*b+c as two roundings, as the reference's x86-64 build computes it).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { ORA_GAUSS = 0, ORA_EXP = 1, ORA_MATERN32 = 2, ORA_MATERN52 = 3 };

/* Covariance.cpp:24-36 (gauss), 65-75 (exp), 104-116 (matern3_2), 149-161 (matern5_2) */
double ora_cov(int kernel, const double* dx, const double* theta, int d) {
  const double SQRT_3 = sqrt(3.0), SQRT_5 = sqrt(5.0);
  double s = 0.0;
  switch (kernel) {
    case ORA_GAUSS:
      for (int i = 0; i < d; i++) {
        double v = dx[i] / theta[i];
        s += v * v;
      }
      return exp(-0.5 * s);
    case ORA_EXP:
      for (int i = 0; i < d; i++) s += fabs(dx[i] / theta[i]);
      return exp(-s);
    case ORA_MATERN32:
      for (int i = 0; i < d; i++) {
        double t = SQRT_3 * fabs(dx[i] / theta[i]);
        s += t - log1p(t);
      }
      return exp(-s);
    case ORA_MATERN52:
      for (int i = 0; i < d; i++) {
        double t = SQRT_5 * fabs(dx[i] / theta[i]);
        s += t - log1p(t + (t * t) / 3.0);
      }
      return exp(-s);
  }
  return NAN;
}

/* Covariance.cpp:38-50 (gauss), 77-88 (exp), 118-130 (matern3_2), 163-179 (matern5_2) */
void ora_dlncov(int kernel, const double* dx, const double* theta, int d, double* out) {
  const double SQRT_3 = sqrt(3.0), SQRT_5 = sqrt(5.0);
  for (int i = 0; i < d; i++) {
    double th = theta[i];
    switch (kernel) {
      case ORA_GAUSS:
        out[i] = (dx[i] * dx[i]) / (th * th * th);
        break;
      case ORA_EXP:
        out[i] = fabs(dx[i]) / (th * th);
        break;
      case ORA_MATERN32: {
        double t = SQRT_3 * fabs(dx[i] / th);
        out[i] = (t * t) / (1.0 + t) / th;
      } break;
      case ORA_MATERN52: {
        double t = SQRT_5 * fabs(dx[i] / th);
        double a = 1.0 + t;
        double b = (t * t) / 3.0;
        out[i] = (a * b) / (a + b) / th;
      } break;
      default:
        out[i] = NAN;
    }
  }
}

/* dX.col(i*n+j) for i>j holds X_j - X_i (LinearAlgebra.cpp:455-466: pair (a<b) stores X_a - X_b at a*n+b
 * and b*n+a).  X is n x d column-major. */
static void pair_dx(int n, int d, const double* X, int i, int j, double* dx) {
  for (int k = 0; k < d; k++) dx[k] = X[j + (size_t)k * n] - X[i + (size_t)k * n];
}

/* LinearAlgebra.cpp:142-181: R(i,j)=R(j,i)=Cov(dX_ij) for i>j, R *= factor, then diag = 1 or diag[]. */
void ora_build_R(int kernel, int n, int d, const double* X, const double* theta, double factor,
                 const double* diag, double* R) {
  double dx[64];
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < i; j++) {
      pair_dx(n, d, X, i, j, dx);
      double c = ora_cov(kernel, dx, theta, d);
      R[i + (size_t)j * n] = c;
      R[j + (size_t)i * n] = c;
    }
  }
  for (size_t q = 0; q < (size_t)n * n; q++) R[q] *= factor;
  for (int i = 0; i < n; i++) R[i + (size_t)i * n] = diag ? diag[i] : 1.0;
}

/* NestedKriging::corrMat (NestedKriging.cpp:101-115): R(i, j) = Cov(x1_i - x2_j; theta), no coincidence rule.
 * X1 n1 x d, X2 n2 x d, R n1 x n2, all column-major. */
void ora_cov_cross(int kernel, int n1, int n2, int d, const double* X1, const double* X2, const double* theta,
                   double* R) {
  double dx[64];
  for (int j = 0; j < n2; j++)
    for (int i = 0; i < n1; i++) {
      for (int k = 0; k < d; k++) dx[k] = X1[i + (size_t)k * n1] - X2[j + (size_t)k * n2];
      R[i + (size_t)j * n1] = ora_cov(kernel, dx, theta, d);
    }
}

/* Rows [i0, i1) of the cholCov pair loop (LinearAlgebra.cpp:150-155), serial like the reference: the timed sample of
 * the CPU baseline.  Writes both triangles of those rows. */
void ora_build_R_rows(int kernel, int n, int d, const double* X, const double* theta, int i0, int i1, double* R) {
  double dx[64];
  for (int i = i0; i < i1; i++) {
    for (int j = 0; j < i; j++) {
      pair_dx(n, d, X, i, j, dx);
      double c = ora_cov(kernel, dx, theta, d);
      R[i + (size_t)j * n] = c;
      R[j + (size_t)i * n] = c;
    }
  }
}

/* Full covariance build spread over OpenMP threads: set-up of the CPU baseline only (not a reference routine). */
void ora_build_R_parallel(int kernel, int n, int d, const double* X, const double* theta, double factor, double* R) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int i = 0; i < n; i++) {
    double dx[64];
    for (int j = 0; j < i; j++) {
      pair_dx(n, d, X, i, j, dx);
      double c = ora_cov(kernel, dx, theta, d) * factor;
      R[i + (size_t)j * n] = c;
      R[j + (size_t)i * n] = c;
    }
    R[i + (size_t)i * n] = 1.0;
  }
}

/* Rows [i0, i1) of the compute_ll_grad_theta_vecs loop (KrigingImpl.cpp:863-884), serial: timed sample. */
void ora_grad_terms_rows(int kernel, int n, int d, const double* X, const double* theta, const double* R,
                         const double* Rinv, const double* x, int i0, int i1, double* term1, double* term2) {
  double dx[64], dln[64];
  for (int i = i0; i < i1; i++) {
    for (int j = 0; j < i; j++) {
      pair_dx(n, d, X, i, j, dx);
      ora_dlncov(kernel, dx, theta, d, dln);
      double R_ij = R[i + (size_t)j * n];
      double x_i = x[i], x_j = x[j];
      double Rinv_ij = Rinv[i + (size_t)j * n];
      for (int k = 0; k < d; k++) {
        double g = R_ij * dln[k];
        term1[k] += 2.0 * x_i * g * x_j;
        term2[k] -= 2.0 * Rinv_ij * g;
      }
    }
  }
}

/* KrigingImpl.cpp:855-885: serial i>j loop; term1_k += 2 x_i gradR_k x_j, term2_k -= 2 Rinv_ij gradR_k,
 * gradR_k = R_ij * dlnCov_k.  term1/term2 are accumulated into (caller zeroes them). */
void ora_grad_terms(int kernel, int n, int d, const double* X, const double* theta, const double* R,
                    const double* Rinv, const double* x, double* term1, double* term2) {
  double dx[64], dln[64];
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < i; j++) {
      pair_dx(n, d, X, i, j, dx);
      ora_dlncov(kernel, dx, theta, d, dln);
      double R_ij = R[i + (size_t)j * n];
      double x_i = x[i], x_j = x[j];
      double Rinv_ij = Rinv[i + (size_t)j * n];
      for (int k = 0; k < d; k++) {
        double g = R_ij * dln[k];
        term1[k] += 2.0 * x_i * g * x_j;
        term2[k] -= 2.0 * Rinv_ij * g;
      }
    }
  }
}

/* The same pair loops spread over `threads` OpenMP threads, for the timed CPU baseline (the reference runs them in
 * one thread; every entry of R is computed with the identical per-pair arithmetic, so R is bit-identical to
 * ora_build_R's).  The gradient sums are per-thread partial sums over a static row schedule, added in thread order:
 * deterministic for a given thread count, equal to the serial loop's up to summation order. */
void ora_build_R_mt(int kernel, int n, int d, const double* X, const double* theta, double factor,
                    const double* diag, double* R, int threads) {
#pragma omp parallel for schedule(dynamic, 8) num_threads(threads)
  for (int i = 0; i < n; i++) {
    double dx[64];
    for (int j = 0; j < i; j++) {
      pair_dx(n, d, X, i, j, dx);
      double c = ora_cov(kernel, dx, theta, d) * factor;
      R[i + (size_t)j * n] = c;
      R[j + (size_t)i * n] = c;
    }
    R[i + (size_t)i * n] = diag ? diag[i] : 1.0;
  }
}

void ora_grad_terms_mt(int kernel, int n, int d, const double* X, const double* theta, const double* R,
                       const double* Rinv, const double* x, double* term1, double* term2, int threads) {
  double part[256][2][16];
  if (threads > 256) threads = 256;
  if (d > 16) return;
#pragma omp parallel num_threads(threads)
  {
    int tid = 0, nt = 1;
#ifdef _OPENMP
    tid = omp_get_thread_num();
    nt = omp_get_num_threads();
#endif
    double t1[16] = {0}, t2[16] = {0}, dx[64], dln[64];
    /* rows dealt round-robin in pairs (i, n-1-i) so that every thread gets the same number of pairs */
    for (int r = tid; r < (n + 1) / 2; r += nt) {
      for (int half = 0; half < 2; half++) {
        int i = half ? n - 1 - r : r;
        if (half && i == r) break;
        for (int j = 0; j < i; j++) {
          pair_dx(n, d, X, i, j, dx);
          ora_dlncov(kernel, dx, theta, d, dln);
          double R_ij = R[i + (size_t)j * n];
          double x_i = x[i], x_j = x[j];
          double Rinv_ij = Rinv[i + (size_t)j * n];
          for (int k = 0; k < d; k++) {
            double g = R_ij * dln[k];
            t1[k] += 2.0 * x_i * g * x_j;
            t2[k] -= 2.0 * Rinv_ij * g;
          }
        }
      }
    }
    for (int k = 0; k < d; k++) {
      part[tid][0][k] = t1[k];
      part[tid][1][k] = t2[k];
    }
#pragma omp barrier
#pragma omp single
    for (int q = 0; q < nt; q++)
      for (int k = 0; k < d; k++) {
        term1[k] += part[q][0][k];
        term2[k] += part[q][1][k];
      }
  }
}

/* ora_alpha_terms over `threads` threads: per-column partial sums, combined in column order. */
void ora_alpha_terms_mt(int n, const double* R, const double* Rinv, const double* x, double alpha,
                        double diag_value, double* out, int threads) {
  double* colv = (double*)malloc(sizeof(double) * 2 * (size_t)n);
#pragma omp parallel for schedule(static) num_threads(threads)
  for (int j = 0; j < n; j++) {
    double v = 0.0, dot = 0.0;
    for (int i = 0; i < n; i++) {
      double a = (i == j) ? diag_value : R[i + (size_t)j * n] / alpha;
      v += x[i] * a;
      dot += Rinv[i + (size_t)j * n] * a;
    }
    colv[j] = v * x[j];
    colv[n + j] = dot;
  }
  double xtAx = 0.0, dot = 0.0;
  for (int j = 0; j < n; j++) {
    xtAx += colv[j];
    dot += colv[n + j];
  }
  free(colv);
  out[0] = xtAx;
  out[1] = dot;
}

/* Kriging.cpp:307-326 building blocks: with dRdv = R/alpha (diagonal replaced by diag_value),
 *   out[0] = x' dRdv x,   out[1] = <Rinv, dRdv> (full-matrix dot).  Column-major order like arma. */
void ora_alpha_terms(int n, const double* R, const double* Rinv, const double* x, double alpha,
                     double diag_value, double* out) {
  double xtAx = 0.0, dot = 0.0;
  /* trans(x) * dRdv gives a row vector v_j = sum_i x_i dRdv_ij; then v * x. */
  for (int j = 0; j < n; j++) {
    double v = 0.0;
    for (int i = 0; i < n; i++) {
      double a = (i == j) ? diag_value : R[i + (size_t)j * n] / alpha;
      v += x[i] * a;
    }
    xtAx += v * x[j];
  }
  for (size_t q = 0; q < (size_t)n * n; q++) {
    size_t i = q % n, j = q / n;
    double a = (i == j) ? diag_value : R[q] / alpha;
    dot += Rinv[q] * a;
  }
  out[0] = xtAx;
  out[1] = dot;
}

/* ---- small dense helpers for the Vecchia conditionals (m <= 64) ---- */

/* In-place lower Cholesky of an m x m column-major matrix; returns 0 on success, -1 if not SPD. */
static int chol_lower(int m, double* A) {
  for (int j = 0; j < m; j++) {
    double s = A[j + j * m];
    for (int k = 0; k < j; k++) s -= A[j + k * m] * A[j + k * m];
    if (!(s > 0.0)) return -1;
    double ljj = sqrt(s);
    A[j + j * m] = ljj;
    for (int i = j + 1; i < m; i++) {
      double t = A[i + j * m];
      for (int k = 0; k < j; k++) t -= A[i + k * m] * A[j + k * m];
      A[i + j * m] = t / ljj;
    }
    for (int i = 0; i < j; i++) A[i + j * m] = 0.0;
  }
  return 0;
}

/* solve L L' a = r */
static void chol_solve(int m, const double* L, const double* r, double* a) {
  double t[128];
  for (int i = 0; i < m; i++) {
    double s = r[i];
    for (int k = 0; k < i; k++) s -= L[i + k * m] * t[k];
    t[i] = s / L[i + i * m];
  }
  for (int i = m - 1; i >= 0; i--) {
    double s = t[i];
    for (int k = i + 1; k < m; k++) s -= L[k + i * m] * a[k];
    a[i] = s / L[i + i * m];
  }
}

/* x <- L^-1 x (kind 1) or L^-T x (kind 2) for lower-triangular L (m x m column-major) */
static void tri_apply_inv(int m, const double* L, double* x, int kind) {
  if (kind == 1) {
    for (int i = 0; i < m; i++) {
      double s = x[i];
      for (int k = 0; k < i; k++) s -= L[i + k * m] * x[k];
      x[i] = s / L[i + i * m];
    }
  } else {
    for (int i = m - 1; i >= 0; i--) {
      double s = x[i];
      for (int k = i + 1; k < m; k++) s -= L[k + i * m] * x[k];
      x[i] = s / L[i + i * m];
    }
  }
}

/* rcond(L)^2 as LinearAlgebra::rcond_chol computes it (LinearAlgebra.cpp:106-115): LAPACK dtrcon('1', 'L', 'N'),
 * i.e. 1 / (|L|_1 * est(|L^-1|_1)) with the dlacn2 estimator (Hager / Higham). */
static double rcond2_small(int m, const double* L) {
  double anorm = 0.0;
  for (int j = 0; j < m; j++) {
    double s = 0.0;
    for (int i = j; i < m; i++) s += fabs(L[i + j * m]);
    if (s > anorm) anorm = s;
  }
  if (!(anorm > 0.0)) return 0.0;
  double x[128], xi[128], est;
  for (int i = 0; i < m; i++) x[i] = 1.0 / m;
  tri_apply_inv(m, L, x, 1);
  if (m == 1) {
    est = fabs(x[0]);
  } else {
    est = 0.0;
    for (int i = 0; i < m; i++) est += fabs(x[i]);
    for (int i = 0; i < m; i++) xi[i] = (x[i] >= 0.0) ? 1.0 : -1.0;
    for (int i = 0; i < m; i++) x[i] = xi[i];
    tri_apply_inv(m, L, x, 2);
    int j = 0;
    for (int i = 1; i < m; i++)
      if (fabs(x[i]) > fabs(x[j])) j = i;
    int iter = 2;
    for (;;) {
      for (int i = 0; i < m; i++) x[i] = (i == j) ? 1.0 : 0.0;
      tri_apply_inv(m, L, x, 1);
      double estold = est;
      est = 0.0;
      for (int i = 0; i < m; i++) est += fabs(x[i]);
      int same = 1;
      for (int i = 0; i < m; i++)
        if (((x[i] >= 0.0) ? 1.0 : -1.0) != xi[i]) same = 0;
      if (same || est <= estold) break;
      for (int i = 0; i < m; i++) xi[i] = (x[i] >= 0.0) ? 1.0 : -1.0;
      for (int i = 0; i < m; i++) x[i] = xi[i];
      tri_apply_inv(m, L, x, 2);
      int jlast = j;
      j = 0;
      for (int i = 1; i < m; i++)
        if (fabs(x[i]) > fabs(x[j])) j = i;
      if (x[jlast] != fabs(x[j]) && iter < 5) {
        iter++;
        continue;
      }
      break;
    }
    double altsgn = 1.0;
    for (int i = 0; i < m; i++) {
      x[i] = altsgn * (1.0 + (double)i / (double)(m - 1));
      altsgn = -altsgn;
    }
    tri_apply_inv(m, L, x, 1);
    double temp = 0.0;
    for (int i = 0; i < m; i++) temp += fabs(x[i]);
    temp = 2.0 * temp / (3.0 * m);
    if (temp > est) est = temp;
  }
  double rc = (1.0 / anorm) / est;
  return rc * rc;
}

static int g_rcond_check = 1;
static double g_min_rcond = 1e-18;
void ora_set_rcond_check(int check, double min_rcond) {
  g_rcond_check = check;
  g_min_rcond = min_rcond;
}

/* safe_chol_lower_retry (LinearAlgebra.cpp:68-98): on failure, or rcond(L)^2 < min_rcond when the check is on,
 * add num_nugget*10^k to the diagonal of a copy (cumulatively), k = 0..max_inc.  Returns increments or -1. */
static int safe_chol_small(int m, const double* A, double* L, double num_nugget, int max_inc) {
  double* W = L;
  memcpy(W, A, sizeof(double) * m * m);
  double* base = (double*)malloc(sizeof(double) * m * m);
  memcpy(base, A, sizeof(double) * m * m);
  for (int inc = 0;; inc++) {
    memcpy(W, base, sizeof(double) * m * m);
    if (chol_lower(m, W) == 0 && !(g_rcond_check && rcond2_small(m, W) < g_min_rcond)) {
      free(base);
      return inc;
    }
    if (inc > max_inc) {
      free(base);
      return -1;
    }
    for (int i = 0; i < m; i++) base[i + i * m] += num_nugget * pow(10.0, inc);
  }
}

/*
 * Kriging.cpp:736-804.  X is n x d column-major (normalised inputs).  order[n] receives the maxmin order;
 * nbr[n*m_max] (row t) the global row indices of the min(m,t) nearest earlier-ordered points, the
 * remaining slots set to -1.  Ties: index_min / index_max pick the lowest index (arma).  The neighbour
 * order inside a set is whatever selection gives (the likelihood does not depend on it).
 */
void ora_vecchia_sets(int n, int d, const double* X, int m_max, int32_t* order, int32_t* nbr) {
  int m = m_max < n - 1 ? m_max : n - 1;
  double* Xt = (double*)malloc(sizeof(double) * (size_t)n * d);
  for (int i = 0; i < n; i++)
    for (int k = 0; k < d; k++) Xt[(size_t)i * d + k] = X[i + (size_t)k * n];
  double* mind2 = (double*)malloc(sizeof(double) * n);
  double* centroid = (double*)calloc(d, sizeof(double));
  for (int k = 0; k < d; k++) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += Xt[(size_t)i * d + k];
    centroid[k] = s / n;
  }
  for (int i = 0; i < n; i++) {
    double s = 0.0;
    for (int k = 0; k < d; k++) {
      double dk = Xt[(size_t)i * d + k] - centroid[k];
      s += dk * dk;
    }
    mind2[i] = s;
  }
  int best = 0;
  for (int i = 1; i < n; i++)
    if (mind2[i] < mind2[best]) best = i;
  order[0] = best;
  for (int i = 0; i < n; i++) {
    double s = 0.0;
    for (int k = 0; k < d; k++) {
      double dk = Xt[(size_t)i * d + k] - Xt[(size_t)best * d + k];
      s += dk * dk;
    }
    mind2[i] = s;
  }
  mind2[best] = -INFINITY;
  for (int t = 1; t < n; t++) {
    int nx = 0;
    for (int i = 1; i < n; i++)
      if (mind2[i] > mind2[nx]) nx = i;
    order[t] = nx;
    for (int i = 0; i < n; i++) {
      if (mind2[i] == -INFINITY) continue;
      double s = 0.0;
      for (int k = 0; k < d; k++) {
        double dk = Xt[(size_t)i * d + k] - Xt[(size_t)nx * d + k];
        s += dk * dk;
      }
      if (s < mind2[i]) mind2[i] = s;
    }
    mind2[nx] = -INFINITY;
  }
  /* neighbours: the k smallest (dist2, index) pairs among the t earlier points (partial selection) */
  double* cd = (double*)malloc(sizeof(double) * n);
  int* ci = (int*)malloc(sizeof(int) * n);
  for (int t = 0; t < n; t++) {
    for (int q = 0; q < m_max; q++) nbr[(size_t)t * m_max + q] = -1;
    int k = m < t ? m : t;
    for (int j = 0; j < t; j++) {
      int oj = order[j], ot = order[t];
      double s = 0.0;
      for (int q = 0; q < d; q++) {
        double dk = Xt[(size_t)ot * d + q] - Xt[(size_t)oj * d + q];
        s += dk * dk;
      }
      cd[j] = s;
      ci[j] = oj;
    }
    /* selection of the k smallest by (distance, index) */
    for (int a = 0; a < k; a++) {
      int bi = a;
      for (int b = a + 1; b < t; b++)
        if (cd[b] < cd[bi] || (cd[b] == cd[bi] && ci[b] < ci[bi])) bi = b;
      double td = cd[a];
      cd[a] = cd[bi];
      cd[bi] = td;
      int ti = ci[a];
      ci[a] = ci[bi];
      ci[bi] = ti;
      nbr[(size_t)t * m_max + a] = ci[a];
    }
  }
  free(cd);
  free(ci);
  free(Xt);
  free(mind2);
  free(centroid);
}

/*
 * Timed sample of the per-point loop of _logLikelihoodVecchia (Kriging.cpp:829-889) with gradient: ordered points
 * [t0, t1) only, results discarded (the CPU baseline scales the time by n / (t1 - t0)).  Returns the number of
 * points whose conditional block needed numerical-nugget increments.
 */
int ora_vecchia_points_sample(int kernel, int n, int d, int p, const double* X, const double* y, const double* F,
                              const double* theta, const int32_t* order, const int32_t* nbr, int m_max,
                              double num_nugget, int t0, int t1) {
  int M = m_max, bumped = 0;
  double* RN = (double*)malloc(sizeof(double) * M * M);
  double* LN = (double*)malloc(sizeof(double) * M * M);
  double* dRN = (double*)malloc(sizeof(double) * (size_t)M * M * d);
  double* dr = (double*)malloc(sizeof(double) * M * d);
  double r[128], a_vec[128], rhs[128], da[128], dx[64], dln[64];
  volatile double sink = 0.0;
  for (int t = t0; t < t1; t++) {
    int oi = order[t];
    int mi = 0;
    while (mi < M && nbr[(size_t)t * M + mi] >= 0) mi++;
    const int32_t* Ni = nbr + (size_t)t * M;
    if (mi == 0) continue;
    for (int q = 0; q < mi * mi; q++) RN[q] = 1.0;
    memset(dRN, 0, sizeof(double) * mi * mi * d);
    for (int a = 0; a < mi; a++) {
      for (int b = a + 1; b < mi; b++) {
        for (int k = 0; k < d; k++) dx[k] = X[Ni[a] + (size_t)k * n] - X[Ni[b] + (size_t)k * n];
        double c = ora_cov(kernel, dx, theta, d);
        RN[a + b * mi] = RN[b + a * mi] = c;
        ora_dlncov(kernel, dx, theta, d, dln);
        for (int k = 0; k < d; k++) dRN[a + b * mi + k * mi * mi] = dRN[b + a * mi + k * mi * mi] = c * dln[k];
      }
      for (int k = 0; k < d; k++) dx[k] = X[Ni[a] + (size_t)k * n] - X[oi + (size_t)k * n];
      double c = ora_cov(kernel, dx, theta, d);
      r[a] = c;
      ora_dlncov(kernel, dx, theta, d, dln);
      for (int k = 0; k < d; k++) dr[a + k * mi] = c * dln[k];
    }
    for (int a = 0; a < mi; a++) RN[a + a * mi] += num_nugget;
    int inc = safe_chol_small(mi, RN, LN, num_nugget, 10);
    if (inc < 0) continue;
    bumped += inc > 0;
    chol_solve(mi, LN, r, a_vec);
    double ra = 0.0;
    for (int a = 0; a < mi; a++) ra += r[a] * a_vec[a];
    for (int k = 0; k < d; k++) {
      for (int a = 0; a < mi; a++) {
        double s = 0.0;
        for (int b = 0; b < mi; b++) s += dRN[a + b * mi + k * mi * mi] * a_vec[b];
        rhs[a] = dr[a + k * mi] - s;
      }
      chol_solve(mi, LN, rhs, da);
      double s2 = 0.0;
      for (int a = 0; a < mi; a++) s2 += r[a] * da[a] + da[a] * y[Ni[a]];
      sink += s2;
    }
    sink += ra;
    (void)F;
    (void)p;
  }
  free(RN);
  free(LN);
  free(dRN);
  free(dr);
  return bumped;
}

/*
 * Kriging.cpp:806-924 (_logLikelihoodVecchia) with p trend columns F (n x p, column-major) and
 * beta estimated by GLS (A += num_nugget I).  grad (length d) may be NULL.  Returns vll; beta_out (p) and
 * sigma2_out may be NULL.  Returns NAN if a conditional block stays non-SPD after the nugget retries.
 */
double ora_vecchia_ll(int kernel, int n, int d, int p, const double* X, const double* y, const double* F,
                      const double* theta, const int32_t* order, const int32_t* nbr, int m_max, double num_nugget,
                      double* grad, double* beta_out, double* sigma2_out) {
  const double v_floor = 1e-15;
  double* u = (double*)malloc(sizeof(double) * n);
  double* v = (double*)malloc(sizeof(double) * n);
  double* W = (double*)malloc(sizeof(double) * (size_t)p * n);
  double *du = NULL, *dv = NULL, *dW = NULL;
  if (grad) {
    du = (double*)calloc((size_t)n * d, sizeof(double));
    dv = (double*)calloc((size_t)n * d, sizeof(double));
    dW = (double*)calloc((size_t)p * n * d, sizeof(double));
  }
  int M = m_max;
  double* RN = (double*)malloc(sizeof(double) * M * M);
  double* LN = (double*)malloc(sizeof(double) * M * M);
  double* dRN = (double*)malloc(sizeof(double) * (size_t)M * M * d);
  double* dr = (double*)malloc(sizeof(double) * M * d);
  double r[128], a_vec[128], rhs[128], da[128], dx[64], dln[64];
  double result = NAN;
  for (int t = 0; t < n; t++) {
    int oi = order[t];
    int mi = 0;
    while (mi < M && nbr[(size_t)t * M + mi] >= 0) mi++;
    const int32_t* Ni = nbr + (size_t)t * M;
    if (mi == 0) {
      u[t] = y[oi];
      v[t] = 1.0;
      for (int q = 0; q < p; q++) W[q + (size_t)t * p] = F[oi + (size_t)q * n];
      continue;
    }
    for (int q = 0; q < mi * mi; q++) RN[q] = 1.0;
    if (grad) memset(dRN, 0, sizeof(double) * mi * mi * d);
    for (int a = 0; a < mi; a++) {
      for (int b = a + 1; b < mi; b++) {
        for (int k = 0; k < d; k++) dx[k] = X[Ni[a] + (size_t)k * n] - X[Ni[b] + (size_t)k * n];
        double c = ora_cov(kernel, dx, theta, d);
        RN[a + b * mi] = RN[b + a * mi] = c;
        if (grad) {
          ora_dlncov(kernel, dx, theta, d, dln);
          for (int k = 0; k < d; k++) dRN[a + b * mi + k * mi * mi] = dRN[b + a * mi + k * mi * mi] = c * dln[k];
        }
      }
      for (int k = 0; k < d; k++) dx[k] = X[Ni[a] + (size_t)k * n] - X[oi + (size_t)k * n];
      double c = ora_cov(kernel, dx, theta, d);
      r[a] = c;
      if (grad) {
        ora_dlncov(kernel, dx, theta, d, dln);
        for (int k = 0; k < d; k++) dr[a + k * mi] = c * dln[k];
      }
    }
    for (int a = 0; a < mi; a++) RN[a + a * mi] += num_nugget;
    if (safe_chol_small(mi, RN, LN, num_nugget, 10) < 0) goto done;
    chol_solve(mi, LN, r, a_vec);
    double ra = 0.0, ay = 0.0;
    for (int a = 0; a < mi; a++) ra += r[a] * a_vec[a];
    for (int a = 0; a < mi; a++) ay += a_vec[a] * y[Ni[a]];
    v[t] = fmax(1.0 - ra, v_floor);
    u[t] = y[oi] - ay;
    for (int q = 0; q < p; q++) {
      double s = 0.0;
      for (int a = 0; a < mi; a++) s += F[Ni[a] + (size_t)q * n] * a_vec[a];
      W[q + (size_t)t * p] = F[oi + (size_t)q * n] - s;
    }
    if (grad) {
      for (int k = 0; k < d; k++) {
        for (int a = 0; a < mi; a++) {
          double s = 0.0;
          for (int b = 0; b < mi; b++) s += dRN[a + b * mi + k * mi * mi] * a_vec[b];
          rhs[a] = dr[a + k * mi] - s;
        }
        chol_solve(mi, LN, rhs, da);
        double s1 = 0.0, s2 = 0.0, s3 = 0.0;
        for (int a = 0; a < mi; a++) s1 += dr[a + k * mi] * a_vec[a];
        for (int a = 0; a < mi; a++) s2 += r[a] * da[a];
        dv[t + (size_t)k * n] = -(s1 + s2);
        for (int a = 0; a < mi; a++) s3 += da[a] * y[Ni[a]];
        du[t + (size_t)k * n] = -s3;
        for (int q = 0; q < p; q++) {
          double s = 0.0;
          for (int a = 0; a < mi; a++) s += F[Ni[a] + (size_t)q * n] * da[a];
          dW[q + (size_t)t * p + (size_t)k * p * n] = -s;
        }
      }
    }
  }
  {
    /* GLS beta: A = sum W W'/v + num_nugget I, b = sum W u / v; A is p x p (p <= 64). */
    double A[64 * 64], bb[64], beta[64], LA[64 * 64];
    memset(A, 0, sizeof(A));
    memset(bb, 0, sizeof(bb));
    for (int t = 0; t < n; t++) {
      for (int q1 = 0; q1 < p; q1++) {
        for (int q2 = 0; q2 < p; q2++) A[q1 + q2 * p] += W[q1 + (size_t)t * p] * W[q2 + (size_t)t * p] / v[t];
        bb[q1] += W[q1 + (size_t)t * p] * u[t] / v[t];
      }
    }
    for (int q = 0; q < p; q++) A[q + q * p] += num_nugget;
    memcpy(LA, A, sizeof(double) * p * p);
    if (chol_lower(p, LA) != 0) goto done;
    chol_solve(p, LA, bb, beta);
    double Q = 0.0, slogv = 0.0;
    double* e = (double*)malloc(sizeof(double) * n);
    for (int t = 0; t < n; t++) {
      double s = 0.0;
      for (int q = 0; q < p; q++) s += W[q + (size_t)t * p] * beta[q];
      e[t] = u[t] - s;
    }
    for (int t = 0; t < n; t++) Q += e[t] * e[t] / v[t];
    for (int t = 0; t < n; t++) slogv += log(v[t]);
    double sigma2 = Q / n;
    if (beta_out)
      for (int q = 0; q < p; q++) beta_out[q] = beta[q];
    if (sigma2_out) *sigma2_out = sigma2;
    result = -0.5 * n * log(2 * M_PI * sigma2) - 0.5 * slogv - 0.5 * n;
    if (grad) {
      for (int k = 0; k < d; k++) {
        double dQ = 0.0, sdv = 0.0;
        for (int t = 0; t < n; t++) {
          double s = 0.0;
          for (int q = 0; q < p; q++) s += dW[q + (size_t)t * p + (size_t)k * p * n] * beta[q];
          double de = du[t + (size_t)k * n] - s;
          dQ += 2.0 * e[t] * de / v[t] - (e[t] * e[t] / (v[t] * v[t])) * dv[t + (size_t)k * n];
        }
        for (int t = 0; t < n; t++) sdv += dv[t + (size_t)k * n] / v[t];
        grad[k] = -0.5 * n * dQ / Q - 0.5 * sdv;
      }
    }
    free(e);
  }
done:
  free(u);
  free(v);
  free(W);
  free(du);
  free(dv);
  free(dW);
  free(RN);
  free(LN);
  free(dRN);
  free(dr);
  return result;
}
