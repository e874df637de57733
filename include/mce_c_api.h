/*
 * C ABI of the GB300 MCE step path (libmce_gb300.so).
 *
 * Drop-in boundary for the reference's CauchyEstimator::step path
 * (natsnyder1/CauchyFriendly).  Plain pointers and sizes only; all device
 * state (terms, cell tables, arenas) stays inside the library.  Every entry
 * point returns a status instead of exiting the process.
 *
 * Arrays follow the reference's layouts: Phi is d x d row-major, Gamma is
 * d x pncc row-major, H is one measurement row (d), B is d x cmcc row-major,
 * complex outputs are interleaved (re, im) pairs.
 */
#ifndef MCE_C_API_H
#define MCE_C_API_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mce_handle mce_handle;

#ifdef __cplusplus
#define MCE_BOOL bool
#else
#define MCE_BOOL _Bool
#endif

/* status codes */
#define MCE_OK 0
#define MCE_ERR_ARG (-1)       /* invalid argument */
#define MCE_ERR_CUDA (-2)      /* CUDA runtime failure (message via mce_last_error) */
#define MCE_ERR_SHAPE (-3)     /* hyperplane count beyond what the build supports */
#define MCE_ERR_DEVICE (-4)    /* a kernel reported an error bit (see mce_device_errors) */
#define MCE_ERR_DONE (-5)      /* stepped past the last step; the reference calls exit(1) here */
#define MCE_ERR_NOMEM (-6)     /* device allocation failed */

/* Last error message of the calling thread (static storage). */
const char* mce_last_error(void);

/* Reproduces the reference constructor's libc rand() draws
 * (include/cauchy_estimator.hpp:127-128 root point, then num_cpus DCE helpers
 * drawing b_pert, include/cell_enumeration.hpp:467-470); helper 0's b_pert is
 * returned.  seed < 0 keeps the current rand() state (the reference never
 * seeds), otherwise srand(seed) is called first.  num_cpus 0 takes the
 * process-wide count below. */
int mce_draw_reference_constants(long long seed, int d, int max_shape, int num_cpus, double* root_point,
                                 double* b_pert);
/* How many DCE helpers an estimator made without explicit constants draws
 * b_pert for: the reference's compile-time NUM_CPUS
 * (include/cauchy_constants.hpp:69, 8 as shipped and the default here; 1 for
 * a serial build).  It only decides how far each estimator advances rand(),
 * so it matters when several estimators draw in turn.  Returns the previous
 * count (MCE_ERR_ARG below 1). */
int mce_set_reference_num_cpus(int num_cpus);

/* Batch of independent estimators stepped in lock-step.  Replaces
 * CauchyEstimator::CauchyEstimator (include/cauchy_estimator.hpp:87-185) for
 * n_est estimators at once.
 *   steps[n_est]            estimation steps per estimator
 *   A0 [n_est*d*d], p0 [n_est*d], b0 [n_est*d]
 *   root_point [n_est*d]    or NULL: drawn with rand() as the reference does
 *   b_pert [n_est*bpert_stride] or NULL: drawn with rand()
 * bpert_stride must be >= each estimator's max shape ((steps-1)*pncc + d). */
mce_handle* mce_batch_create(int n_est, int d, int cmcc, int pncc, int p, const int* steps, const double* A0,
                             const double* p0, const double* b0, const double* root_point, const double* b_pert,
                             int bpert_stride, int* status);

/* One measurement update for every estimator (CauchyEstimator::step,
 * include/cauchy_estimator.hpp:1211-1245).  shared_model != 0 means Phi,
 * Gamma, beta, H, gamma, B hold a single copy used by all estimators;
 * otherwise each is stacked per estimator.  msmt[n_est], u[n_est*cmcc].
 * err_out[n_est] receives each estimator's error bitmask (may be NULL). */
int mce_batch_step(mce_handle* h, const double* msmt, const double* Phi, const double* Gamma, const double* beta,
                   const double* H, const double* gamma, const double* B, const double* u, int shared_model,
                   int* err_out);

/* No counterpart in the reference.  mce_batch_step for callers that may not
 * allocate device memory while they estimate: a process whose device memory
 * is already handed out (a framework's caching allocator, a real-time loop
 * that sizes its memory at start-up), or one that cannot accept the
 * device-wide synchronisation of cudaMalloc/cudaFree.  Same arguments and
 * results as mce_batch_step; it calls no cudaMalloc, cudaFree or other
 * allocating routine:
 *  - the g-table kernel's scratch is a static 32 MiB device array of the
 *    library, and the kernel runs as many warps as it has slots for; a
 *    handle whose full-shape terms would need more than 4 warps' worth
 *    (above 524,288 half-cells per term) is refused with MCE_ERR_SHAPE
 *    before any work.  Under this build's limit of 24 hyperplanes per term
 *    the largest need is 390,656 half-cells (8 states), so every handle fits;
 *  - the handle's own device buffers must already be large enough (they grow
 *    only in the other calls: step the handle with mce_batch_step over a
 *    representative history, then mce_reset); a buffer that would have to
 *    grow stops the step with MCE_ERR_NOMEM, after which the handle must be
 *    reset.
 * The handle's device must be the current device (MCE_ERR_DEVICE otherwise:
 * the array's address is looked up on the current device).  The first call
 * on a device looks the array up (cudaGetSymbolAddress); make it before any
 * stream capture.  Every call on a device shares the array: calls that
 * overlap on the GPU race, so serialise them. */
int mce_batch_step_noalloc(mce_handle* h, const double* msmt, const double* Phi, const double* Gamma,
                           const double* beta, const double* H, const double* gamma, const double* B, const double* u,
                           int shared_model, int* err_out);

/* Runs every estimator through its whole measurement history
 * msmts[n_est * max_steps * p] (row e*max_steps*p + k*p + j), with a shared
 * model or per-estimator models as in mce_batch_step.  Per-update outputs are
 * optional (NULL): fz[n_est*max_updates*2], mean[...*2d], cov[...*2d*d],
 * err[n_est*max_updates], nt[n_est*max_updates]. */
int mce_batch_run(mce_handle* h, const double* msmts, int max_steps, const double* Phi, const double* Gamma,
                  const double* beta, const double* H, const double* gamma, const double* B, const double* u,
                  int shared_model, double* fz, double* mean, double* cov, int* err, long long* nt);

/* Single estimator, the CauchyEstimator constructor
 * (include/cauchy_estimator.hpp:87): a batch of one. */
mce_handle* mce_create(const double* A0, const double* p0, const double* b0, int steps, int d, int cmcc, int pncc,
                       int p, const double* root_point, const double* b_pert, int* status);

/* CauchyEstimator::step (include/cauchy_estimator.hpp:1211): returns the
 * error bitmask (>= 0) or a negative MCE_ERR_* status. */
int mce_step(mce_handle* h, double msmt, const double* Phi, const double* Gamma, const double* beta, const double* H,
             double gamma, const double* B, const double* u);

/* Reported moments after the numeric checks (the fields fz,
 * conditional_mean, conditional_variance the reference exposes,
 * include/cauchy_estimator.hpp:66-68): fz[2], mean[2d], cov[2d*d]. */
int mce_get_moments(mce_handle* h, int est, double* fz, double* mean, double* cov);
/* Raw moments of the last update before the checks, and G_SCALE_FACTOR. */
int mce_get_raw_moments(mce_handle* h, int est, double* fz, double* mean, double* cov, double* g_scale_factor);
/* numeric_moment_errors of one estimator. */
int mce_get_errors(mce_handle* h, int est);
/* Nt after the last update (post-reduction, or un-reduced after the final MU). */
long long mce_num_terms(mce_handle* h, int est);
/* terms_per_shape (n entries, shape index = hyperplane count). */
int mce_terms_per_shape(mce_handle* h, int est, int* out, int n);
/* Extended (nonlinear) mode helpers of CauchyEstimator
 * (include/cauchy_estimator.hpp:1312-1394), on one estimator's current terms:
 *  - mce_shift_cf_by_bias: every term's b += bias[d] (nothing after the
 *    final update, whose terms are not kept);
 *  - mce_deterministic_time_prop: every term's time_prop with Phi[d*d], and
 *    B[d*cmcc] u[cmcc] when both are given (A <- A Phi^T, b <- Phi b + B u);
 *  - mce_finalize_extended_moments: every term's b -= Re(mean) (not after
 *    the final update), then mean += x_bar and x_bar = Re(mean); x_bar[d] is
 *    read and written. */
int mce_shift_cf_by_bias(mce_handle* h, int est, const double* bias);
int mce_deterministic_time_prop(mce_handle* h, int est, const double* Phi, const double* B, const double* u);
int mce_finalize_extended_moments(mce_handle* h, int est, double* x_bar);

/* Marginal 1-D conditional pdf of estimator `est` on the grid
 * grid_low, grid_low + grid_res, ..., grid_high (the last point clamped), as
 * CauchyCPDFGridDispatcher1D (include/cpdf_ndim.hpp:2017-2139) evaluates
 * PointWiseNDimCauchyCPDF::evaluate_1D_marginal_cpdf (:1233-1352) and
 * pycauchy_get_marginal_1D_pointwise_cpdf returns it
 * (scripts/swig/cauchy/pycauchy.hpp:890-931).  bar_nu[d] is the pdf object's
 * random direction for rows orthogonal to the marginal axis
 * (mce_draw_bar_nu).  The first evaluation at a step and marginal index takes
 * the exact formula at the first grid point and caches per-term constants;
 * later evaluations at that step and index use the cache, as the reference
 * does.  x, y receive the points; with x or y NULL only the point count is
 * returned.  Returns the number of points or a negative status
 * (MCE_ERR_DONE after the last step, whose g-tables are skipped). */
int mce_cpdf_1d_grid(mce_handle* h, int est, int marg_idx, const double* bar_nu, double grid_low, double grid_high,
                     double grid_res, int max_points, double* x, double* y);

/* The conditional pdf of estimator `est` at npts points x[npts*d]:
 * PointWiseNDimCauchyCPDF::evaluate_cpdf (include/cpdf_ndim.hpp:677-904), the
 * characteristic function integrated one spectral dimension at a time.
 * out[2*npts] receives each value (re, im; the imaginary part is rounding).
 * Each (point, term) pair is lowered on its own (the reference merges terms
 * whose arrangements agree within 1e-8 between the lowerings): the same sum
 * up to rounding.  MCE_ERR_ARG before the first step or when the last step
 * reported moment errors (the reference asserts), MCE_ERR_DONE after the
 * last step, MCE_ERR_SHAPE when a current term has more than 16 hyperplanes
 * (the N-D pdf keeps its lowered terms' cell sets in shared memory; the
 * handle's capacity may be larger), MCE_ERR_DEVICE
 * where the reference exits (an anti-coaligned pair of rows that do not
 * enter the integration). */
int mce_cpdf_nd(mce_handle* h, int est, const double* x, int npts, double* out);

/* The marginal pdf of the states marg_idx[n_marg] (ascending, 0 < n_marg <
 * d) of estimator `est` at npts points x[npts*n_marg]:
 * PointWiseNDimCauchyCPDF::evaluate_marginal_cpdf (include/cpdf_ndim.hpp:
 * 918-1230).  Every term's columns are reordered so that the states
 * integrated out come first, the kept states are lowered out one at a time
 * as in mce_cpdf_nd, and the terms of the d - n_marg dimensions left are
 * looked up at the sign vector of A nu_bar; nu_bar[d - n_marg] stands for
 * the values the reference draws from rand() (any point off the
 * hyperplanes gives the same value up to rounding).  out[2*npts]; the same
 * errors as mce_cpdf_nd, MCE_ERR_ARG for indices that do not ascend within
 * [0, d). */
int mce_cpdf_marginal(mce_handle* h, int est, const int* marg_idx, int n_marg, const double* nu_bar, const double* x,
                      int npts, double* out);

/* Marginal 2-D conditional pdf of estimator `est` over states
 * marg_idx1 < marg_idx2 on the grid x = gridx_low ... gridx_high (step
 * gridx_res) by y = gridy_low ... gridy_high, x varying fastest, as
 * CauchyCPDFGridDispatcher2D (include/cpdf_ndim.hpp:1774-1919) evaluates
 * PointWiseNDimCauchyCPDF::evaluate_2D_marginal_cpdf (:1356-1455) and
 * pycauchy_get_marginal_2D_pointwise_cpdf returns it
 * (scripts/swig/cauchy/pycauchy.hpp:822-862).  The per-term cache (kept for
 * the same step and indices) is dropped after the grid when reset_cache != 0.
 * x, y, z receive the points; with any of them NULL only the point count is
 * returned.  Returns the number of points or a negative status (MCE_ERR_DONE
 * after the last step; MCE_ERR_DEVICE for a cell with gamma1 = gamma2 = 0,
 * where the reference exits). */
int mce_cpdf_2d_grid(mce_handle* h, int est, int marg_idx1, int marg_idx2, const double* bar_nu, double gridx_low,
                     double gridx_high, double gridx_res, double gridy_low, double gridy_high, double gridy_res,
                     int reset_cache, int max_points, double* x, double* y, double* z);

/* The draws of PointWiseNDimCauchyCPDF's constructor
 * (include/cpdf_ndim.hpp:385-388): bar_nu[i] = 2 (rand() + 1)/(RAND_MAX + 2)
 * for i < d.  seed >= 0 calls srand(seed) first. */
int mce_draw_bar_nu(long long seed, int d, double* bar_nu);

/* Relative-then-transformed 2-D system of two estimators, rel = secondary -
 * primary projected by the 2 x d matrix Trel (row-major): one cached 2-D term
 * per (primary term, secondary term) pair.  Replaces
 * get_marg2d_relative_and_transformed_cpdf
 * (include/cauchy_prediction.hpp:653-971, single-thread term order; the
 * container it returns is the mce_rel2d object) and, with the grid below,
 * pycauchy_single_step_eval_2d_rsys_cpdf (scripts/swig/cauchy/pycauchy.hpp:672-747).
 *   est_p / est_s      the estimators within their batches (may be one batch)
 *   bar_nu_full[d]     the point the reference draws as 2 u - 1,
 *                      u = (rand() + 1) / (RAND_MAX + 2), for rows that the
 *                      projection zeroes
 *   full_solve         FULL_SOLVE: all 2m cells of each term instead of m
 *   with_term_approx   drop terms whose bound on the pdf contribution is
 *                      below term_approx_eps (approx_out_rel_marg2d_term_for_cpdf)
 *   moments[14]        or NULL: the relative moments fz, mean[2], cov[2x2],
 *                      finalised, as (re, im) pairs
 *   counts[2]          or NULL: pairs, pairs approximated out
 * Returns NULL with *status < 0 on failure: MCE_ERR_ARG before the first
 * update or for differing dimensions, MCE_ERR_DONE after the last update (no
 * g-tables), MCE_ERR_SHAPE when the two estimators' hyperplanes exceed 31. */
typedef struct mce_rel2d mce_rel2d;
mce_rel2d* mce_rel2d_create(mce_handle* primary, int est_p, mce_handle* secondary, int est_s, const double* Trel,
                            const double* bar_nu_full, int full_solve, int with_term_approx, double term_approx_eps,
                            double* moments, long long* counts, int* status);

/* The relative pdf on the grid xlow..xhigh (step dx, last point xhigh) by
 * ylow..yhigh, x outermost: point (i, j) at i * ny + j, as
 * grid_eval_marg2d_relative_and_transformed_cpdf
 * (include/cauchy_prediction.hpp:1091-1186) lays it out; the value is the real
 * part of (2 - full) sum / (2 pi)^2 / (norm_factor_prim norm_factor_sec).
 * With x, y or z NULL only the point count is returned.  Returns the number
 * of points or a negative status (MCE_ERR_DEVICE for a cell with
 * gamma1 = gamma2 = 0, where the reference exits). */
int mce_rel2d_grid(mce_rel2d* r, double xlow, double xhigh, double dx, double ylow, double yhigh, double dy,
                   double norm_factor_prim, double norm_factor_sec, int max_points, double* x, double* y, double* z);
/* Pairs formed, and pairs kept after the term approximation. */
long long mce_rel2d_num_pairs(mce_rel2d* r);
long long mce_rel2d_num_terms(mce_rel2d* r);
/* Device time in ms (CUDA events on the object's stream) of the pair kernel
 * (which = 0), of the kept-pair compaction and moment sums (1) of
 * mce_rel2d_create, and of the last mce_rel2d_grid (2). */
double mce_rel2d_device_ms(mce_rel2d* r, int which);
/* Kernels launched by mce_rel2d_create and every mce_rel2d_grid so far. */
long long mce_rel2d_launch_count(mce_rel2d* r);
void mce_rel2d_destroy(mce_rel2d* r);

/* ---- window managers ---------------------------------------------------- */

/* Eigen-decomposition of the symmetric n x n matrix A (row-major): evals[n],
 * evecs[n*n] with eigenvector i in column i, by Householder tridiagonalisation
 * and implicit-shift QL as the reference's sym_eig (include/eig_solve.hpp:404)
 * computes it (same order and signs of the eigenvectors).  Host code. */
int mce_sym_eig(int n, const double* A, double* evals, double* evecs);

/* Speyer's restart statistics of a window about an estimate
 * (speyers_window_init, include/cauchy_util.hpp:23-113, as
 * pycauchy_speyers_window_init returns them, scripts/swig/cauchy/pycauchy.hpp:973):
 * A0[n*n] (rows = eigenvectors of P + P H^T H P / s, s = gamma^2 + (z - H x)^2),
 * p0[n], b0[n].  var_boost[n] (or NULL) is added to P's diagonal first; P is
 * not modified.  Returns 1 when P had an eigenvalue below -1e-5 and its
 * diagonal was raised (the reference prints a warning there), else MCE_OK.
 * Host code. */
int mce_speyers_window_init(int n, const double* xhat, const double* Phat, const double* H, double gamma, double z,
                            const double* var_boost, double* A0, double* p0, double* b0);

/* The reference's CauchyDynamicsUpdateContainer (include/dynamic_models.hpp:62-80),
 * the struct LTV dynamics callbacks receive (same field order and types). */
typedef struct mce_dynamics_container {
    double* x;
    double* u;
    double dt;
    int step;
    int n;
    int cmcc;
    int pncc;
    int p;
    double* Phi;
    double* Gamma;
    double* B;
    double* H;
    double* beta;
    double* gamma;
    MCE_BOOL is_xbar_set_for_ece;
    void* other_stuff;
} mce_dynamics_container;
typedef void (*mce_dynamics_callback)(mce_dynamics_container*);
/* The nonlinear measurement model of extended mode: zbar[p] = h(c->x). */
typedef void (*mce_msmt_model_callback)(mce_dynamics_container*, double* zbar);

/* Sliding-window manager of the C++ front end: SlidingWindowManager(num_windows,
 * num_sim_steps, A0, p0, b0, duc, ..., dyn_cb, ..., win_var_boost, ...)
 * (include/cauchy_windows.hpp:814-1022), .step(msmts, controls) (:1025-1165)
 * and .shutdown() (:1167), for n_mgr independent managers stepped together
 * (one batched GPU handle per window slot).  Per-manager arrays are stacked:
 * A0[n_mgr*d*d], p0, b0[n_mgr*d], Phi[n_mgr*d*d], Gamma[n_mgr*d*pncc],
 * B[n_mgr*d*cmcc], beta[n_mgr*pncc], H[n_mgr*p*d], gamma[n_mgr*p].  dyn_cb
 * (or NULL for LTI) is the LTV callback; each window and the manager call it
 * on their own copy of the container, as the reference's window processes do.
 * root_point[n_mgr*d] / b_pert[n_mgr*bpert_stride] (or both NULL: drawn with
 * rand()) are shared by a manager's windows, as the reference's forked windows
 * share the rand() state they inherit.  Logging options of the reference have
 * no counterpart. */
typedef struct mce_swm mce_swm;
mce_swm* mce_swm_create(int n_mgr, int num_windows, int num_sim_steps, int d, int cmcc, int pncc, int p,
                        const double* A0, const double* p0, const double* b0, const double* Phi,
                        const double* Gamma, const double* B, const double* beta, const double* H,
                        const double* gamma, double dt, int init_step, mce_dynamics_callback dyn_cb,
                        const double* win_var_boost, const double* root_point, const double* b_pert,
                        int bpert_stride, int* status);
/* The extended (nonlinear) manager: SlidingWindowManager with is_extended
 * (include/cauchy_windows.hpp:814-1022 with the three callbacks), as
 * pycauchy_initialize_nonlin_window_manager makes it
 * (scripts/swig/cauchy/pycauchy.hpp:152-184).  x0[n_mgr*d] is x_bar at the
 * first step; dyn_cb propagates c->x (x_hat -> x_bar) and sets Phi, Gamma,
 * beta and is_xbar_set_for_ece; msmt_cb gives z_bar = h(c->x); ext_cb sets H
 * and gamma at c->x.  The window estimators take no controls (controls reach
 * the callbacks through c->u).  Each window's update: z_bar and H at its
 * x_bar, the estimator steps on z - z_bar, finalize_extended_moments moves
 * x_bar to the estimate; restarts use Speyer's statistics of x_hat - x_bar
 * and z - h(x_bar) about the best window's reported x_bar. */
mce_swm* mce_swm_create_nonlin(int n_mgr, int num_windows, int num_sim_steps, int d, int cmcc, int pncc, int p,
                               const double* x0, const double* A0, const double* p0, const double* b0,
                               const double* beta, const double* gamma, double dt, int init_step,
                               mce_dynamics_callback dyn_cb, mce_msmt_model_callback msmt_cb,
                               mce_dynamics_callback ext_cb, const double* win_var_boost, const double* root_point,
                               const double* b_pert, int bpert_stride, int* status);
/* SlidingWindowManager::step + the read-out pycauchy_step returns
 * (scripts/swig/cauchy/pycauchy.hpp:187-221), per manager (each output may be
 * NULL): fz[n_mgr], xhat[n_mgr*d], Phat[n_mgr*d*d], cerr_fz, cerr_xhat,
 * cerr_Phat[n_mgr], win_idx[n_mgr], err_code[n_mgr].  msmts[n_mgr*p],
 * controls[n_mgr*cmcc] (or NULL).  MCE_ERR_DONE after num_sim_steps steps;
 * MCE_ERR_DEVICE when no window is usable (the reference exits). */
int mce_swm_step(mce_swm* s, const double* msmts, const double* controls, double* fz, double* xhat, double* Phat,
                 double* cerr_fz, double* cerr_xhat, double* cerr_Phat, int* win_idx, int* err_code);
/* Terms present after every MU of every window since creation. */
long long mce_swm_post_mu_terms(mce_swm* s);
/* The batched handle of window slot j (for read-outs), and the steps window j
 * has taken since its last restart. */
mce_handle* mce_swm_window(mce_swm* s, int j);
int mce_swm_window_count(mce_swm* s, int j);
void mce_swm_destroy(mce_swm* s);

/* ---- adjoint ------------------------------------------------------------ */

/* Gradient of sum_k w_k Re(fz_k) over one estimator's run -- and with
 * w_K = 1/Re(fz_K) on the last update alone, of the accumulated
 * log-likelihood sum_k log fz_k, fz_k = 1/(2 pi G_SCALE_FACTOR_k)
 * (include/cauchy_estimator.hpp:340-357) -- with respect to the model's
 * scales and matrices, holding the enumerated cell structure fixed.  No
 * counterpart in the reference (which has no derivatives); the forward run is
 * the GPU step path of CauchyEstimator::step.  LTI model, no controls.
 *   create: d states, pncc process-noise columns, p measurements per step,
 *           `steps` steps; A0[d*d], p0[d], b0[d]; root_point[d] and
 *           b_pert[(steps-1)*pncc+d] as for mce_create (required here).
 *   forward: runs every update (msmts[steps*p]; Phi[d*d], Gamma[d*pncc],
 *           beta[pncc], H[p*d], gamma[p]) and records it; fz_raw[steps*p]
 *           (or NULL) receives Re fz of every update.
 *   backward: w[steps*p] seeds; grad[mce_adjoint_num_params] receives the
 *           gradient in the order beta, gamma, p0, Phi (row-major), Gamma
 *           (row-major), H (row-major).
 *   check: the largest relative difference between the recorded tape and the
 *           GPU run (every kept g-table, every Re fz); both ~1e-15 when the
 *           tape describes the run. */
typedef struct mce_adjoint mce_adjoint;
mce_adjoint* mce_adjoint_create(int d, int pncc, int p, int steps, const double* A0, const double* p0,
                                const double* b0, const double* root_point, const double* b_pert, int* status);
int mce_adjoint_forward(mce_adjoint* a, const double* msmts, const double* Phi, const double* Gamma,
                        const double* beta, const double* H, const double* gamma, double* fz_raw);
/* mce_adjoint_forward for a time-varying model: Phis[steps*d*d], the Phi of
 * every step (step k's time propagation uses Phis[k]); the gradient's Phi
 * entries are then those of a perturbation common to every step's Phi. */
int mce_adjoint_forward_ltv(mce_adjoint* a, const double* msmts, const double* Phis, const double* Gamma,
                            const double* beta, const double* H, const double* gamma, double* fz_raw);
int mce_adjoint_num_params(mce_adjoint* a);
int mce_adjoint_backward(mce_adjoint* a, const double* w, double* grad);
int mce_adjoint_check(mce_adjoint* a, double* max_table_rel_err, double* max_fz_rel_err);
/* Wall ms spent since creation: [0] the forward step path, [1] the forward
 * tape (host records, GPU member values and checks), [2] the reverse over the
 * tables (GPU), [3] the record chain (GPU). */
int mce_adjoint_timing(mce_adjoint* a, double* ms4);
void mce_adjoint_destroy(mce_adjoint* a);

/* A batch of adjoint runs of one LTI model (the window lives of a sliding-
 * window log-likelihood, say), stepped together by one batched handle
 * (mce_batch_step per update) with their records and reverses spread over
 * the host's cores, each core's GPU work on its own stream.  Run r has
 * steps[r] steps from (A0[r], p0[r], b0[r]) with its own rand() constants
 * root_point[r*d...] and b_pert[r*bpert_stride...]; every run gives the same
 * gradient as an mce_adjoint of its own (the step path is the same doubles).
 *   forward: msmts[n_runs*max_steps*p] (run r's updates from
 *           r*max_steps*p); the model arrays as for mce_adjoint_forward;
 *           fz_raw[n_runs*max_steps*p] (or NULL), 0 past a run's last update.
 *   backward: w[n_runs*max_steps*p] seeds (a run whose seeds are all 0 is
 *           skipped and gets a zero gradient); grad[n_runs*num_params].
 *   timing: wall ms of the batched step path, of the forward records, of the
 *           reverse, and the runs' summed record-chain ms. */
typedef struct mce_adjoint_batch mce_adjoint_batch;
mce_adjoint_batch* mce_adjoint_batch_create(int n_runs, int d, int pncc, int p, const int* steps, const double* A0,
                                            const double* p0, const double* b0, const double* root_point,
                                            const double* b_pert, int bpert_stride, int* status);
int mce_adjoint_batch_forward(mce_adjoint_batch* b, const double* msmts, int max_steps, const double* Phi,
                              const double* Gamma, const double* beta, const double* H, const double* gamma,
                              double* fz_raw);
/* mce_adjoint_batch_forward for time-varying models, each run its own:
 * Phis[n_runs*max_steps*d*d] (run r's Phi of its step k at
 * (r*max_steps + k)*d*d), Gammas[n_runs*d*pncc], Hs[n_runs*p*d]; beta and
 * gamma are shared.  Each run's gradient is with respect to its own Phi
 * (a perturbation common to its steps), Gamma and H, and the shared scales. */
int mce_adjoint_batch_forward_ltv(mce_adjoint_batch* b, const double* msmts, int max_steps, const double* Phis,
                                  const double* Gammas, const double* beta, const double* Hs, const double* gamma,
                                  double* fz_raw);
int mce_adjoint_batch_backward(mce_adjoint_batch* b, const double* w, int max_steps, double* grad);
/* Every run of the batch starts with measurement first_sub of its first
 * step (0 by default): a sliding window restarted with the last measurement
 * of a step (first_sub = p - 1) runs that one update, then its master step
 * jumps to p (pycauchy_single_step_set_master_step), so its steps[r] steps
 * are steps[r] * p - first_sub updates; msmts, fz_raw and w hold them from
 * the run's offset on.  Clears the recorded runs. */
int mce_adjoint_batch_set_first_sub(mce_adjoint_batch* b, int first_sub);
int mce_adjoint_batch_num_params(mce_adjoint_batch* b);
int mce_adjoint_batch_check(mce_adjoint_batch* b, double* max_table_rel_err, double* max_fz_rel_err);
int mce_adjoint_batch_timing(mce_adjoint_batch* b, double* ms4);
void mce_adjoint_batch_destroy(mce_adjoint_batch* b);

/* Host wall time (ms) of the steps since the last mce_clear_profile: which = 0
 * whole steps, 1 input packing, 2 the moment checks after the device work. */
double mce_host_time_ms(mce_handle* h, int which);

/* Sum over all updates and estimators of the terms present after each MU. */
long long mce_post_mu_terms(mce_handle* h);
int mce_master_step(mce_handle* h);
/* Device error bits accumulated by the kernels (0 when healthy): 1 an
 * anti-coaligned orthogonal hyperplane (the reference exits,
 * cauchy_term.hpp:673-687), 2 a B table above its capacity, 4 more
 * hyperplanes than the handle's capacity, 8 the reduction's resolution
 * stalled, 16 a vertex enumeration above its capacity, 32 an MU record past
 * the step's record count, 64 a reduction root's cells above its table slot,
 * 128 a promoted member's cells above its table slot. */
int mce_device_errors(mce_handle* h);

/* Parity hooks: terms of one estimator in (shape, index) order.  Sizes:
 * shape[nt], A[nt*max_shape*d], p[nt*max_shape], b[nt*d], cells[nt],
 * keys[total_cells], g[2*total_cells]. */
long long mce_total_cells(mce_handle* h, int est);
int mce_dump_terms(mce_handle* h, int est, int max_shape, int* shape, double* A, double* p, double* b, int* cells,
                   int* keys, double* g);

/* CauchyEstimator::reset (include/cauchy_estimator.hpp:1247) for every estimator. */
int mce_reset(mce_handle* h);
/* Frees the device buffers that grow with the term count (term records,
 * g-tables, reduction and evaluation scratch) when together they hold at
 * least min_bytes (0: whatever they hold), returning the bytes released (0
 * below the threshold); the next step allocates what it needs again.  Only
 * between mce_reset (or creation) and the next step, else MCE_ERR_ARG.  The
 * window managers call it with 1 GiB on every window they reset, so that
 * only the windows that are large at the same time hold large buffers (the
 * reference's terms are reallocated each step, include/cauchy_estimator.hpp)
 * while small windows keep theirs. */
long long mce_trim_memory(mce_handle* h, long long min_bytes);
/* reinitialize_start_statistics (include/cauchy_estimator.hpp:1302). */
int mce_reinitialize_start_statistics(mce_handle* h, int est, const double* A0, const double* p0, const double* b0);
/* The constructor's print_basic_info (include/cauchy_estimator.hpp:87, 165)
 * for estimator est (est < 0: every estimator of the handle).  When set, the
 * moments reported after each update that rebuilds the tables (and after the
 * first update) are the post-reduction ones of compute_moments(false)
 * (include/cauchy_estimator.hpp:524-602, 1166-1177, 1197-1203), which also
 * replace G_SCALE_FACTOR; otherwise fz is reported as 1 there.  Nothing is
 * printed. */
int mce_set_print_basic_info(mce_handle* h, int est, int on);

/* master_step setter used by the window manager (pycauchy.hpp:776). */
int mce_set_master_step(mce_handle* h, int master_step);
int mce_set_window_number(mce_handle* h, int win_num);

/* Device time of the last step and since creation / mce_clear_profile
 * (CUDA events on the library's stream), ms. */
double mce_last_step_ms(mce_handle* h);
double mce_device_time_ms(mce_handle* h);
/* Kernels launched by this handle since creation / mce_clear_profile. */
long long mce_launch_count(mce_handle* h);
/* Profiling: 0 off, 1 time each kernel group with CUDA events, 2 also
 * accumulate each group's algorithmic bytes and FP64 flops (extra kernels and
 * synchronisation; for an untimed pass). */
int mce_set_profiling(mce_handle* h, int mode);
int mce_clear_profile(mce_handle* h);
int mce_num_kernel_groups(void);
const char* mce_kernel_group_name(int group);
int mce_kernel_group_stats(mce_handle* h, int group, double* ms, long long* launches, double* alg_bytes,
                           double* alg_flops);

/* Block-size autotuner of the thread-per-item kernels (kernel ids: 0 TP,
 * 1 vertex build of the new hyperplane arrangements, 2 MU rows, 3 g-table
 * evaluation, 4 g-table combination, 5 promoted-root g-table evaluation,
 * 6 compaction, 7 FTR resolution).  Process-wide: each (kernel, state
 * dimension, hyperplane capacity, log2 of the launch's item count) key tries
 * 64/128/256/512 threads on its first launches, timed with CUDA events on the
 * launching stream, and keeps the fastest.  Block size does not change any
 * result.  mce_autotune_configure drops every tuned key and turns the tuner
 * on (1, the default unless MCE_AUTOTUNE=0) or off (0, fixed block sizes).
 * mce_autotune_table writes up to max_rows settled keys as 5 ints each
 * (kernel, d, hyperplane capacity, log2 items, block) and the best sample's
 * ms, and returns how many keys are settled. */
int mce_autotune_configure(int enabled);
int mce_autotune_table(int* rows, float* best_ms, int max_rows);
const char* mce_autotune_kernel_name(int kernel);

void mce_destroy(mce_handle* h);

#ifdef __cplusplus
}
#endif

#endif /* MCE_C_API_H */
