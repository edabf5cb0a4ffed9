/*
 * libkriging_gb300.h -- C ABI of the GB300-native libKriging likelihood path.
 *
 * The entry points mirror libKriging's own C ABI (bindings/Julia/jlibkriging/csrc/libkriging_c.h, implementation
 * bindings/Julia/jlibkriging/csrc/libkriging_c.cpp) one for one, with the prefix lkg_ instead of lk_: same argument
 * order, sizes and meaning (column-major double arrays, int status 0 / -1, thread-local last error), so a binding
 * written against lk_* switches by renaming the symbols.  Entry points without a counterpart there say so.
 *
 * Everything computes on the GPU (sm_103a); there is no CPU fallback.  A call made without a usable CUDA device
 * returns -1 (or NULL / NaN) with the CUDA error in lkg_get_last_error().
 */
#ifndef LIBKRIGING_GB300_H
#define LIBKRIGING_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* libkriging_c.h:10 lk_get_last_error -- message of the last failed call on this thread. */
const char* lkg_get_last_error(void);

/* ---------------------------------------------------------------- Kriging ---------------------------------------- */
/* noise_model: "none" (or NULL) or "nugget".  "heterogeneous" is rejected (not part of this path). */

/* libkriging_c.h:17 lk_kriging_new */
void* lkg_kriging_new(const char* kernel, const char* noise_model);
/* libkriging_c.h:18-41 lk_kriging_new_fit (theta: one starting point of length theta_n, as there) */
void* lkg_kriging_new_fit(const double* y, int n, const double* noise, int noise_n, const double* X, int nX, int d,
                          const char* kernel, const char* noise_model, const char* regmodel, int normalize,
                          const char* optim, const char* objective, const double* sigma2, int is_sigma2_estim,
                          const double* theta, int theta_n, int is_theta_estim, const double* beta, int beta_n,
                          int is_beta_estim, const double* nugget, int is_nugget_estim);
/* libkriging_c.h:42 lk_kriging_delete */
void lkg_kriging_delete(void* ptr);
/* libkriging_c.h:45-56 lk_kriging_fit */
int lkg_kriging_fit(void* ptr, const double* y, int n, const double* noise, int noise_n, const double* X, int nX,
                    int d, const char* regmodel, int normalize, const char* optim, const char* objective);
/* No counterpart in the reference C ABI (its C++ Kriging::fit takes Kriging::Parameters, Kriging.hpp:113-119):
 * fit with parameters; theta is theta_rows x d column-major (one starting point per row). */
int lkg_kriging_fit_params(void* ptr, const double* y, int n, const double* X, int nX, int d, const char* regmodel,
                           int normalize, const char* optim, const char* objective, const double* sigma2,
                           int is_sigma2_estim, const double* theta, int theta_rows, int is_theta_estim,
                           const double* beta, int beta_n, int is_beta_estim, const double* nugget,
                           int is_nugget_estim);
/* libkriging_c.h:58-69 lk_kriging_predict: mean (m), stdev (m), cov (m x m), and with return_deriv the derivatives of
 * the mean and of the stdev with respect to the m points' coordinates (m x d each, column-major) */
int lkg_kriging_predict(void* ptr, const double* X_n, int m, int d, int return_stdev, int return_cov,
                        int return_deriv, double* mean_out, double* stdev_out, double* cov_out, double* mean_deriv_out,
                        double* stdev_deriv_out);
/* libkriging_c.h:43 lk_kriging_copy: a deep copy of the model (data, parameters and committed factor) */
void* lkg_kriging_copy(void* ptr);
/* libkriging_c.h:83-91 lk_kriging_update (Kriging.cpp:2433-2633): append n new points (X_u nX x d) in original units.
 * refit with optim != "none": NoiseModel nugget refits on the joined data, NoiseModel none runs one warm-started
 * L-BFGS-B from the current theta; otherwise theta is kept and the factor is extended by the incremental Cholesky on
 * the GPU.  noise_u must be NULL / 0 (per-observation noise is not part of this path). */
int lkg_kriging_update(void* ptr, const double* y_u, int n, const double* noise_u, int noise_n, const double* X_u,
                       int nX, int d, int refit);
/* libkriging_c.h:105 lk_kriging_save: libKriging's JSON model file, version 2 */
int lkg_kriging_save(void* ptr, const char* filename);
/* libkriging_c.h:106 lk_kriging_load: a model saved by lk_kriging_save or lkg_kriging_save (NULL on error) */
void* lkg_kriging_load(const char* filename);
/* libkriging_c.h:138 lk_kriging_cov_mat: cov_out (n1 x n2) = sigma2 C(X1, X2), X1 / X2 in original units */
int lkg_kriging_cov_mat(void* ptr, const double* X1, int n1, int d1, const double* X2, int n2, int d2,
                        double* cov_out);
/* libkriging_c.h:107 lk_kriging_summary */
const char* lkg_kriging_summary(void* ptr);
/* libkriging_c.h:109-116 lk_kriging_log_likelihood_fun (return_hess is rejected; hess_out untouched) */
int lkg_kriging_log_likelihood_fun(void* ptr, const double* theta, int theta_n, int return_grad, int return_hess,
                                   double* ll_out, double* grad_out, double* hess_out);
/* libkriging_c.h:132 lk_kriging_log_likelihood */
double lkg_kriging_log_likelihood(void* ptr);
/* libkriging_c.h:118-123 lk_kriging_leave_one_out_fun: LOO = |errorsLOO|^2 / n and dLOO/dtheta (theta_n = d) */
int lkg_kriging_leave_one_out_fun(void* ptr, const double* theta, int theta_n, int return_grad, double* loo_out,
                                  double* grad_out);
/* libkriging_c.h:133 lk_kriging_leave_one_out: leaveOneOutFun at the model's theta */
double lkg_kriging_leave_one_out(void* ptr);
/* libkriging_c.h:136 lk_kriging_leave_one_out_vec: yhat_out[n] = y - errorsLOO, stderr_out[n] = sqrt(sigma2LOO sigma2) */
int lkg_kriging_leave_one_out_vec(void* ptr, const double* theta, int theta_n, double* yhat_out, double* stderr_out);
/* libkriging_c.h:125-130 lk_kriging_log_marg_post_fun: log marginal posterior and its gradient (theta_n = d, or d + 1
 * with alpha for a NuggetKriging model; d alone takes the model's alpha) */
int lkg_kriging_log_marg_post_fun(void* ptr, const double* theta, int theta_n, int return_grad, double* lmp_out,
                                  double* grad_out);
/* libkriging_c.h:134 lk_kriging_log_marg_post */
double lkg_kriging_log_marg_post(void* ptr);
/* No counterpart in the reference: k candidates (k x theta_n column-major) evaluated in one batched GPU pass;
 * ll_out[k], grad_out k x theta_n column-major. */
int lkg_kriging_log_likelihood_fun_batch(void* ptr, const double* thetas, int k, int theta_n, int return_grad,
                                         double* ll_out, double* grad_out);
/* No counterpart in the reference: logLikelihoodFun(..., bench=true) writing the per-stage timings (ms, CUDA events)
 * as "key<TAB>value<LF>" lines; keys are the reference's Bench keys (src/lib/KrigingImpl.cpp:96-124). */
int lkg_kriging_log_likelihood_fun_bench(void* ptr, const double* theta, int theta_n, int return_grad, double* ll_out,
                                         double* grad_out, char* bench_out, int bench_cap);
/* No counterpart in the reference: lkg_kriging_log_likelihood_fun_batch writing the batched pass's per-stage
 * timings (ms, CUDA events on the model's stream, summed over the k candidates) like the entry point above. */
int lkg_kriging_log_likelihood_fun_batch_bench(void* ptr, const double* thetas, int k, int theta_n, int return_grad,
                                               double* ll_out, double* grad_out, char* bench_out, int bench_cap);

/* No counterpart in the reference (it has only the FP64 LAPACK path): precision of this model's objective
 * evaluations.  slices = 0 selects the FP64 path (default); 4..8 the mixed path, where the O(n^3) products of the
 * Cholesky, the triangular inverse and R^-1 run on the bf16 tensor cores by error-free splitting into `slices`
 * base-256 digits (7 ~ FP64-level products); a mixed factorisation that meets a non-positive pivot is redone on
 * the FP64 path.  lkg_kriging_last_slices reports what the last logLikelihoodFun used (0 after such a retreat). */
int lkg_kriging_set_precision(void* ptr, int slices);
int lkg_kriging_get_precision(void* ptr);
int lkg_kriging_last_slices(void* ptr);

/* No counterpart in the reference: objective evaluations this model has run since it was created, and the GPU
 * evaluation launches they took (a multistart fit runs every start's evaluation of one optimiser round as one
 * batched launch, so rounds < evaluations there).  Either pointer may be NULL. */
int lkg_kriging_eval_counts(void* ptr, long long* evaluations, long long* rounds);

/* No counterpart in the reference: the project's autotuner.  lkg_kriging_autotune_precision picks the fastest
 * precision of this model's objective -- 0 (FP64) or 5..7 slices of the mixed path -- whose LL and gradient at gamma
 * stay within tol_ll / tol_grad (relative, with a 10x margin) of the FP64 path's, by timing each candidate on the
 * GPU; it sets that precision and returns it (-1 on error).  Choices are tabled per problem shape and tolerance
 * (and persisted to $LKG_TUNE_FILE when set); LKG_AUTOTUNE=0 or lkg_autotune_enable(0) turns measuring off.
 * lkg_autotune_record tables a choice from given costs (lowest finite cost, ties to the earlier candidate) and
 * returns it; lkg_autotune_lookup returns a tabled choice or `fallback`; lkg_autotune_report writes
 * "key<TAB>choice<TAB>cost<LF>" lines and returns the size needed; save / load / clear manage the table. */
int lkg_kriging_autotune_precision(void* ptr, const double* gamma, int gamma_n, double tol_ll, double tol_grad);
/* No counterpart in the reference: times logLikelihoodFun(gamma, grad) of this (mixed-precision) model with 0, 12,
 * 16, 24 and 32 SMs kept for the Cholesky look-ahead's panel work and tables the fastest for the model's size; later
 * evaluations of that size use it unless lkg_set_lookahead fixed a value.  Returns the choice, -1 on error. */
int lkg_kriging_autotune_lookahead(void* ptr, const double* gamma, int gamma_n);
void lkg_autotune_enable(int on);
int lkg_autotune_record(const char* key, const int* candidates, const double* costs, int n);
int lkg_autotune_lookup(const char* key, int fallback);
int lkg_autotune_report(char* out, int cap);
int lkg_autotune_save(const char* path);
int lkg_autotune_load(const char* path);
void lkg_autotune_clear(void);

/* Vecchia approximation (objective "LLVecchia" / "LLVecchia(m)" of lkg_kriging_fit[_params]).  The reference
 * exposes these through its C++ Kriging class only (Kriging.hpp:145-173; no lk_* counterpart):
 *   logLikelihoodVecchiaFun(theta, return_grad) -> (vll, grad)  Kriging.hpp:145-150, Kriging.cpp:926-941
 *   set_vecchia_exact_commit, vecchia_neighbors, is_vecchia_light  Kriging.hpp:152-173
 * lkg_kriging_get_vecchia_sets returns the maxmin order (n) and the neighbour sets (n x m row-major, -1 padded) as
 * built by make_vecchia_sets (Kriging.cpp:736-804); lkg_vecchia_sets builds them on the GPU for a given X
 * (n x d column-major) without a model. */
int lkg_kriging_log_likelihood_vecchia_fun(void* ptr, const double* theta, int theta_n, int return_grad,
                                           double* vll_out, double* grad_out);
int lkg_kriging_set_vecchia_exact_commit(void* ptr, int b);
int lkg_kriging_vecchia_neighbors(void* ptr);
int lkg_kriging_is_vecchia_light(void* ptr);
int lkg_kriging_get_vecchia_sets(void* ptr, int* order_out, int* nbr_out, int* n, int* m);
int lkg_vecchia_sets(int n, int d, const double* X, int m, int* order_out, int* nbr_out);
/* Kriging::predictVecchia (Kriging.hpp:163-173, Kriging.cpp:950-1022; no lk_* counterpart): each of the q points
 * of X_n (q x d column-major) kriged on its m nearest observations (m = 0: the fit's Vecchia m, else 30); mean and,
 * when return_stdev, the simple-kriging stdev.  lkg_kriging_predict routes here after a light Vecchia fit. */
int lkg_kriging_predict_vecchia(void* ptr, const double* X_n, int q, int d, int return_stdev, int m,
                                double* mean_out, double* stdev_out);

/* lkg_vecchia_sets_noalloc: no counterpart in the reference (make_vecchia_sets is internal to Kriging.cpp there).
 * The same order and neighbour sets as lkg_vecchia_sets, bit for bit, for callers that may not allocate memory:
 * code that runs inside another allocator's budget (a caching allocator, a fixed memory pool), a serving loop that
 * cannot take the device-wide synchronisation a cudaFree implies, or code that queues work on a stream it does not
 * own.  X (n x d column-major), order (n) and nbr (n x m row-major, -1 padded) are caller-owned device (or managed)
 * buffers of the current device; stream is a cudaStream_t (NULL: the legacy default stream).  Every kernel is
 * queued on that stream and nothing is synchronised: the outputs are ready when the stream reaches that point.
 * The intermediates live in one fixed device array of this library, 2^20 doubles (8 MiB) per device, so calls are
 * limited to n * (2 d + 1) + 768 <= 1048576 (d = 3: n <= 149686; d = 8: n <= 61635), with 1 <= d <= 8 and
 * 0 <= m <= 32; larger or malformed calls fail with -1 and a message before any work is queued.  Nothing in that
 * array has to start at zero: every word is written before it is read within a call.  The first call on each device
 * (and the first after that device's context was reset) resolves the array's address with cudaGetSymbolAddress and
 * loads every kernel the entry point launches, whatever its m; loading a module can make the driver allocate, so
 * make that first call before any stream capture begins and outside any memory budget.  Later calls in the same
 * context load and resolve nothing.  Calls that overlap on one device -- from two threads, or on two streams that
 * are not ordered with each other -- share the array and race: order them.  The entry point calls no cudaMalloc,
 * cudaFree or allocating library routine and allocates no device memory; on failure the message is stored like
 * every other entry point's. */
int lkg_vecchia_sets_noalloc(int n, int d, const double* X, int m, int* order, int* nbr, void* stream);

/* Sharded Vecchia likelihood: no counterpart in the reference, whose _logLikelihoodVecchia (Kriging.cpp:806-924)
 * sums per-point terms over all ordered points in one loop.  Each rank owns the ordered positions [t0, t1) of the
 * same sets (X n x d, y n, F n x p column-major, normalised as the model holds them; order[n], nbr[n x m]):
 *   1. lkg_vecchia_shard_sums1: s1 = [A (p x p row-major), b (p), sum log v] over its positions, A = sum W W'/v,
 *      b = sum W u / v; failed_points counts conditionals that stayed non-SPD after the nugget increments;
 *   2. the ranks sum s1 (an all-reduce) and lkg_vecchia_gls_beta solves (A + num_nugget I) beta = b;
 *   3. lkg_vecchia_shard_sums2: s2 = [Q, dQ_k (d), sum dv_k / v (d)] at that beta;
 *   4. the ranks sum s2 and lkg_vecchia_finish gives sigma2 = Q / n, the VLL and its gradient (d).
 * The single-GPU evaluation runs the same four steps on one range. */
void* lkg_vecchia_shard_new(const char* kernel, int n, int d, int p, const double* X, const double* y,
                            const double* F, const int* order, const int* nbr, int m, int t0, int t1);
void lkg_vecchia_shard_delete(void* h);
int lkg_vecchia_shard_sums1(void* h, const double* theta, int with_grad, double* s1_out, long long* nugget_points,
                            int* failed_points);
int lkg_vecchia_shard_sums2(void* h, const double* beta, int with_grad, double* s2_out);
int lkg_vecchia_gls_beta(int p, const double* s1, double* beta_out);
int lkg_vecchia_finish(int n, int d, double slogv, const double* s2, int with_grad, double* vll_out,
                       double* sigma2_out, double* grad_out);

/* getters, libkriging_c.h:141-165 */
const char* lkg_kriging_kernel(void* ptr);
const char* lkg_kriging_optim(void* ptr);
const char* lkg_kriging_objective(void* ptr);
int lkg_kriging_is_normalize(void* ptr);
const char* lkg_kriging_regmodel(void* ptr);
int lkg_kriging_get_X(void* ptr, double* out, int* n, int* d);
int lkg_kriging_get_centerX(void* ptr, double* out, int* d);
int lkg_kriging_get_scaleX(void* ptr, double* out, int* d);
int lkg_kriging_get_y(void* ptr, double* out, int* n);
double lkg_kriging_get_centerY(void* ptr);
double lkg_kriging_get_scaleY(void* ptr);
int lkg_kriging_get_F(void* ptr, double* out, int* n, int* d);
int lkg_kriging_get_T(void* ptr, double* out, int* n, int* d);
int lkg_kriging_get_M(void* ptr, double* out, int* n, int* d);
int lkg_kriging_get_z(void* ptr, double* out, int* n);
int lkg_kriging_get_beta(void* ptr, double* out, int* n);
int lkg_kriging_is_beta_estim(void* ptr);
int lkg_kriging_get_theta(void* ptr, double* out, int* n);
int lkg_kriging_is_theta_estim(void* ptr);
double lkg_kriging_get_sigma2(void* ptr);
int lkg_kriging_is_sigma2_estim(void* ptr);
const char* lkg_kriging_noise_model(void* ptr);
double lkg_kriging_get_nugget(void* ptr);
int lkg_kriging_is_nugget_estim(void* ptr);

/* ------------------------------------------------------- numerical / optimiser settings --------------------------- */
/* LinearAlgebra::set_num_nugget / get_num_nugget (src/lib/LinearAlgebra.cpp:35-41) */
void lkg_set_num_nugget(double nugget);
double lkg_get_num_nugget(void);
/* LinearAlgebra::check_chol_rcond (src/lib/LinearAlgebra.cpp:53-55) */
void lkg_check_chol_rcond(int check);
/* LinearAlgebra::set_chol_warning (src/lib/LinearAlgebra.cpp:47-49) */
void lkg_set_chol_warning(int warn);
/* Optim setters (src/lib/Optim.cpp:44-139) */
void lkg_optim_use_reparametrize(int r);
void lkg_optim_set_theta_lower_factor(double f);
void lkg_optim_set_theta_upper_factor(double f);
void lkg_optim_use_variogram_bounds_heuristic(int v);
void lkg_optim_set_log_level(int l);
void lkg_optim_set_max_iteration(int m);
void lkg_optim_set_gradient_tolerance(double t);
void lkg_optim_set_objective_rel_tolerance(double t);
void lkg_optim_set_max_restart(int m);

/* ------------------------------------------------------------- diagnostics ---------------------------------------- */
/* No counterpart in the reference: name of CUDA device 0, or NULL without a device. */
const char* lkg_device_name(void);
/* No counterpart in the reference: measured FP64 FMA throughput (TFLOP/s) of this GPU, the roofline denominator of
 * the FP64 kernels (the DFMA pipe; FP64 mma.sync is slower on GB300). */
int lkg_probe_fp64_peak(double* tflops_out);
/* No counterpart in the reference: measured FP64 tensor-core (DMMA, mma.sync m8n8k4 f64) throughput in TFLOP/s --
 * the comparison that decides whether the FP64 tiles use DFMA or DMMA on this part. */
int lkg_probe_dmma_peak(double* tflops_out);
/* No counterpart in the reference (it times stages with Bench::tic/toc, src/lib/Bench.cpp): per-kernel launch
 * counts, and with timing enabled CUDA-event durations on each launch's own stream plus the launch's algorithmic
 * flops and bytes.  lkg_stats_report writes "name<TAB>launches<TAB>timed<TAB>ms<TAB>flops<TAB>bytes<LF>" lines and
 * returns the length needed (including the terminating NUL), or -1. */
void lkg_stats_enable(int on);
void lkg_stats_reset(void);
int lkg_stats_report(char* out, int cap);
/* No counterpart in the reference: C = A B^T (A M x K, B N x K, C M x N, column-major host buffers) through the
 * split-bf16 tensor-core GEMM -- the check hook of the mixed path's emulated products.  As in the engine, the
 * precision's `slices` become min(8, max(5, slices + 1)) 7-bit digits. */
int lkg_ozaki_gemm_check(int M, int N, int K, const double* A, const double* B, int slices, double* C);
/* No counterpart in the reference: the kernels of the mixed path's digit products.  One family remains: 3 =
 * tcgen05 on 7-bit digits with one exponent per 256-wide k block and two-level (256 / 64) blocked Cholesky and
 * triangular inverse.  lkg_set_tensor_path returns 3, or -1 for any other value. */
int lkg_set_tensor_path(int tc);
int lkg_get_tensor_path(void);
/* No counterpart in the reference: output tile width of the digit products, 32 (two TMEM accumulator sets, so the
 * fold of one tile overlaps the products of the next; the default) or 64 (one set; every A digit image serves
 * twice the columns).  Returns the width set, or -1 for another value. */
int lkg_set_digit_tile(int tn);
int lkg_get_digit_tile(void);
/* No counterpart in the reference: the mixed Cholesky's look-ahead (n >= 1024, single-matrix evaluations): the next
 * 256-wide panel is factored on a second stream on `ctas` SMs while the rest of the trailing update runs on the
 * others.  0 turns it off; -1 (the default, unless LKG_LOOKAHEAD_CTAS is set) uses the autotuned choice for the
 * matrix size (lkg_kriging_autotune_lookahead), else 16.  The factor is the same bit for bit either way.  Returns
 * the value set, or -2 on an argument outside -1 .. 64 (lkg_get_lookahead returns the setting). */
int lkg_set_lookahead(int ctas);
int lkg_get_lookahead(void);
/* No counterpart in the reference: CUDA graphs for the two launch sequences of an evaluation (covariance build +
 * factorisation; solves, GLS, R^-1 and adjoint sums), captured on the second run of a configuration and replayed
 * afterwards; on by default unless LKG_GRAPHS=0, and off while per-launch timing (lkg_stats_enable) is on.  Results
 * are the same bit for bit either way.  Returns the previous setting (1 on, 0 off). */
int lkg_set_graphs(int on);
/* No counterpart in the reference: one product of the 7-bit digit kernel on host data, S digits (5..8):
 * mode 0: C (M x N) = A B^T (A M x K, B N x K); mode 1: C = A A^T lower (M x M); mode 2: C = W^T W lower with
 * W = A (M x M, lower).  Returns 0, -1 (error text in lkg_get_last_error) or -2 when a wait of the kernel expired
 * (where_out, 8 ints, receives where). */
int lkg_oz7_mode_check(int mode, int M, int N, int K, const double* A, const double* B, int S, double* C,
                       int* where_out);

/* ------------------------------------------------------------- NestedKriging -------------------------------------- */
/* libkriging_c.h:394-455 lk_nested_kriging_* (NestedKriging.hpp:63-105): partition (kmeans | random), submodel
 * fits, common prior, aggregation PoE | gPoE | BCM | rBCM | NK.  warping must be empty (n_warping = 0): WarpKriging
 * submodels are not part of this library.  theta: one starting point of length theta_n, as there. */
void* lkg_nested_kriging_new_fit(const double* y, int n, const double* X, int nX, int d, const char* kernel,
                                 int nb_groups, const char* aggregation, const char* partition, int seed,
                                 const char** warping, int n_warping, const char* regmodel, const char* optim,
                                 const char* objective, const double* sigma2, int is_sigma2_estim, const double* theta,
                                 int theta_n, int is_theta_estim, const double* beta, int beta_n, int is_beta_estim);
void lkg_nested_kriging_delete(void* ptr);
int lkg_nested_kriging_fit(void* ptr, const double* y, int n, const double* X, int nX, int d, int nb_groups,
                           const char** warping, int n_warping, const char* regmodel, const char* optim,
                           const char* objective, const double* sigma2, int is_sigma2_estim, const double* theta,
                           int theta_n, int is_theta_estim, const double* beta, int beta_n, int is_beta_estim);
int lkg_nested_kriging_predict(void* ptr, const double* X_n, int m, int d, int return_stdev, double* mean_out,
                               double* stdev_out);
const char* lkg_nested_kriging_summary(void* ptr);
const char* lkg_nested_kriging_kernel(void* ptr);
const char* lkg_nested_kriging_aggregation(void* ptr);
int lkg_nested_kriging_nb_groups(void* ptr);
int lkg_nested_kriging_get_theta(void* ptr, double* out, int* n);
double lkg_nested_kriging_get_sigma2(void* ptr);
double lkg_nested_kriging_get_beta0(void* ptr);
/* No counterpart in the C ABI (NestedKriging(covType) + setters, NestedKriging.hpp:67, Python binding
 * NestedKriging(kernel)): an unfitted model with its aggregation, partition and seed. */
void* lkg_nested_kriging_new(const char* kernel, const char* aggregation, const char* partition, int seed);
/* No counterpart in the reference: fit on a given partition, labels[i] in [0, nb_groups) the group of row i. */
int lkg_nested_kriging_fit_groups(void* ptr, const double* y, int n, const double* X, int nX, int d,
                                  const int* labels, int nb_groups, const char* regmodel, const char* optim,
                                  const char* objective, const double* sigma2, int is_sigma2_estim,
                                  const double* theta, int theta_n, int is_theta_estim, const double* beta,
                                  int beta_n, int is_beta_estim);
/* NestedKriging::groups (NestedKriging.hpp:113) as labels: labels_out[i] = group of row i; *n = rows. */
int lkg_nested_kriging_get_groups(void* ptr, int* labels_out, int* n);
/* NestedKriging::submodel (NestedKriging.hpp:117): a Kriging handle owned by the nested model (valid until it is
 * refitted or deleted; never pass it to lkg_kriging_delete), usable with every lkg_kriging_* getter. */
void* lkg_nested_kriging_submodel(void* ptr, int i);
/* No counterpart in the reference: digit slices of the submodel objective evaluations (0 = FP64, 4..8 = mixed). */
int lkg_nested_kriging_set_precision(void* ptr, int slices);
/* NestedKriging::set_predict_chunk (NestedKriging.hpp:133). */
int lkg_nested_kriging_set_predict_chunk(void* ptr, int chunk);
/* No counterpart in the reference (each submodel's Kriging::logLikelihoodFun, Kriging.cpp:343-349, runs alone
 * there): the submodel fit objective of all p groups in one batched evaluation -- concentrated LL of group g at
 * theta row g of thetas (p x d row-major) into ll_out[g], theta-gradient into grad_out (p x d row-major) when
 * return_grad.  Needs a fit on the plain path (objective "LL"). */
int lkg_nested_kriging_log_likelihood_groups(void* ptr, const double* thetas, int p, int d, int return_grad,
                                             double* ll_out, double* grad_out);
/* No counterpart in the reference: the submodel estimates that entered unify_hyperparameters
 * (NestedKriging.cpp:283-310) -- theta_out p x d row-major, sigma2_out p, beta0_out p (0 without a constant trend);
 * *p = 0 after a fit that had no unify step (LLVecchia-unified path).  NULL outputs are skipped. */
int lkg_nested_kriging_get_group_estimates(void* ptr, double* theta_out, double* sigma2_out, double* beta0_out,
                                           int* p, int* d);

#ifdef __cplusplus
}
#endif

#endif /* LIBKRIGING_GB300_H */
