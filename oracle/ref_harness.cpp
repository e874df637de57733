// Test infrastructure only: a C-ABI harness around the UNMODIFIED reference
// estimator (natsnyder1/CauchyFriendly, header-only C++), compiled from the
// reference headers where they lie.  Nothing in the product links this file.
//
// It is used (a) to generate the golden fixtures under tests/golden and
// (b) as the reference CPU baseline when the reference sources are present.
//
// Two build knobs are applied without touching the reference sources:
//   * HARNESS_NUM_CPUS replaces the compile-time thread count
//     (include/cauchy_constants.hpp:69-71).  The serial build (1) gives the
//     term order of step_tp_to_muc (include/cauchy_estimator.hpp:604-832);
//     the threaded build reproduces the stock threaded path.
//   * covariance_checker (include/cauchy_util.hpp:1882) is wrapped so the
//     harness can record the RAW moments (fz, mean, covariance) that
//     moments_numerical_check (include/cauchy_estimator.hpp:359) inspects
//     before it may revert them to the last good ones.  The wrapper calls the
//     original with with_warnings=false; the returned flags are identical.
#ifndef HARNESS_NUM_CPUS
#define HARNESS_NUM_CPUS 1
#endif

#define NUM_CPUS NUM_CPUS_REFERENCE_DEFAULT
#define NUM_CPUS_FTR NUM_CPUS_FTR_REFERENCE_DEFAULT
#include "cauchy_constants.hpp"
#undef NUM_CPUS
#undef NUM_CPUS_FTR
const int NUM_CPUS = HARNESS_NUM_CPUS;
const int NUM_CPUS_FTR = HARNESS_NUM_CPUS;

#include "cauchy_term.hpp"
#include "cauchy_types.hpp"
#include "cauchy_util.hpp"

#include <stdlib.h>
#include <string.h>
#include <time.h>

// ---- raw-moment capture -------------------------------------------------
static double g_raw_fz[2];
static double* g_raw_mean = nullptr;  // 2*d
static double* g_raw_cov = nullptr;   // 2*d*d
static const C_COMPLEX_TYPE* g_cur_mean = nullptr;
static const C_COMPLEX_TYPE* g_cur_fz = nullptr;
static int g_cur_d = 0;

static int harness_covariance_checker(C_COMPLEX_TYPE* cov, const int d, const int win_num,
                                      const int step, const int total_steps, bool with_warnings)
{
    (void)with_warnings;
    if (g_cur_fz && g_cur_mean && g_raw_mean && g_raw_cov && d == g_cur_d) {
        g_raw_fz[0] = creal(*g_cur_fz);
        g_raw_fz[1] = cimag(*g_cur_fz);
        for (int i = 0; i < d; i++) {
            g_raw_mean[2 * i] = creal(g_cur_mean[i]);
            g_raw_mean[2 * i + 1] = cimag(g_cur_mean[i]);
        }
        for (int i = 0; i < d * d; i++) {
            g_raw_cov[2 * i] = creal(cov[i]);
            g_raw_cov[2 * i + 1] = cimag(cov[i]);
        }
    }
    return covariance_checker(cov, d, win_num, step, total_steps, false);
}
#define covariance_checker harness_covariance_checker

#include "cauchy_estimator.hpp"
#include <vector>
#include "cpdf_ndim.hpp"
#include "cauchy_prediction.hpp"

struct RefHandle {
    CauchyEstimator* est;
    PointWiseNDimCauchyCPDF* cpdf;  // made on first use, as pycauchy does
    int d;
    double raw_fz[2];
    double* raw_mean;
    double* raw_cov;
    double last_step_seconds;
};

extern "C" {

int ref_num_cpus(void) { return NUM_CPUS; }

// Seeds libc rand() and constructs the estimator exactly as the reference
// does (root_point then NUM_CPUS DCE helpers draw from rand()).
void* ref_create(const double* A0, const double* p0, const double* b0, int steps, int d, int cmcc,
                 int pncc, int p, unsigned seed)
{
    srand(seed);
    RefHandle* h = new RefHandle();
    h->d = d;
    h->raw_mean = (double*)calloc(2 * d, sizeof(double));
    h->raw_cov = (double*)calloc(2 * d * d, sizeof(double));
    h->est = new CauchyEstimator((double*)A0, (double*)p0, (double*)b0, steps, d, cmcc, pncc, p, false);
    return h;
}

void ref_destroy(void* vh)
{
    // runs the reference's own destructor (its arenas are released), so a
    // process can step many estimators one after another
    RefHandle* h = (RefHandle*)vh;
    delete h->cpdf;
    delete h->est;
    free(h->raw_mean);
    free(h->raw_cov);
    delete h;
}

int ref_step(void* vh, double msmt, const double* Phi, const double* Gamma, const double* beta,
             const double* H, double gamma, const double* B, const double* u)
{
    RefHandle* h = (RefHandle*)vh;
    CauchyEstimator* e = h->est;
    g_cur_fz = &e->fz;
    g_cur_mean = e->conditional_mean;
    g_cur_d = h->d;
    g_raw_mean = h->raw_mean;
    g_raw_cov = h->raw_cov;
    g_raw_fz[0] = g_raw_fz[1] = 0;
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    int err = e->step(msmt, (double*)Phi, (double*)Gamma, (double*)beta, (double*)H, gamma, (double*)B,
                      (double*)u);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    h->last_step_seconds = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
    h->raw_fz[0] = g_raw_fz[0];
    h->raw_fz[1] = g_raw_fz[1];
    g_cur_fz = nullptr;
    g_cur_mean = nullptr;
    return err;
}

double ref_last_step_seconds(void* vh) { return ((RefHandle*)vh)->last_step_seconds; }

void ref_get_constants(void* vh, double* root_point, double* b_pert, int* max_shape)
{
    RefHandle* h = (RefHandle*)vh;
    CauchyEstimator* e = h->est;
    memcpy(root_point, e->root_point, h->d * sizeof(double));
    *max_shape = e->shape_range - 1;
    memcpy(b_pert, e->dce_helper[0].b_pert, (e->shape_range - 1) * sizeof(double));
}

// Reported moments (after the numeric checks) and the raw ones.
void ref_get_moments(void* vh, double* fz, double* mean, double* cov, double* raw_fz, double* raw_mean,
                     double* raw_cov, double* g_scale_factor)
{
    RefHandle* h = (RefHandle*)vh;
    CauchyEstimator* e = h->est;
    int d = h->d;
    fz[0] = creal(e->fz);
    fz[1] = cimag(e->fz);
    for (int i = 0; i < d; i++) {
        mean[2 * i] = creal(e->conditional_mean[i]);
        mean[2 * i + 1] = cimag(e->conditional_mean[i]);
    }
    for (int i = 0; i < d * d; i++) {
        cov[2 * i] = creal(e->conditional_variance[i]);
        cov[2 * i + 1] = cimag(e->conditional_variance[i]);
    }
    raw_fz[0] = h->raw_fz[0];
    raw_fz[1] = h->raw_fz[1];
    memcpy(raw_mean, h->raw_mean, 2 * d * sizeof(double));
    memcpy(raw_cov, h->raw_cov, 2 * d * d * sizeof(double));
    *g_scale_factor = e->G_SCALE_FACTOR;
}

int ref_num_terms(void* vh) { return ((RefHandle*)vh)->est->Nt; }
int ref_master_step(void* vh) { return ((RefHandle*)vh)->est->master_step; }
int ref_shape_range(void* vh) { return ((RefHandle*)vh)->est->shape_range; }
void ref_terms_per_shape(void* vh, int* out)
{
    CauchyEstimator* e = ((RefHandle*)vh)->est;
    memcpy(out, e->terms_per_shape, e->shape_range * sizeof(int));
}

// Total g-table cells over all (parent) terms; valid after a non-final step.
long long ref_total_cells(void* vh)
{
    CauchyEstimator* e = ((RefHandle*)vh)->est;
    long long tot = 0;
    for (int m = 1; m < e->shape_range; m++)
        for (int i = 0; i < e->terms_per_shape[m]; i++) tot += e->terms_dp[m][i].cells_gtable_p;
    return tot;
}

// Dumps every term in shape/index order: shape, A (padded to max_shape x d),
// p (padded), b, cells, sorted keys and complex g values of gtable_p.
void ref_dump_terms(void* vh, int* shape, double* A, double* p, double* b, int* cells, int* keys,
                    double* gvals)
{
    CauchyEstimator* e = ((RefHandle*)vh)->est;
    const int d = e->d;
    const int M = e->shape_range - 1;
    int t = 0;
    long long c = 0;
    for (int m = 1; m < e->shape_range; m++) {
        for (int i = 0; i < e->terms_per_shape[m]; i++) {
            CauchyTerm* term = e->terms_dp[m] + i;
            shape[t] = term->m;
            memset(A + (size_t)t * M * d, 0, M * d * sizeof(double));
            memset(p + (size_t)t * M, 0, M * sizeof(double));
            memcpy(A + (size_t)t * M * d, term->A, term->m * d * sizeof(double));
            memcpy(p + (size_t)t * M, term->p, term->m * sizeof(double));
            memcpy(b + (size_t)t * d, term->b, d * sizeof(double));
            cells[t] = term->cells_gtable_p;
            for (int k = 0; k < term->cells_gtable_p; k++) {
                keys[c] = (int)term->gtable_p[k].key;
                gvals[2 * c] = creal(term->gtable_p[k].value);
                gvals[2 * c + 1] = cimag(term->gtable_p[k].value);
                c++;
            }
            t++;
        }
    }
}

// Marginal 2-D pdf on a grid through the reference's CauchyCPDFGridDispatcher2D,
// as pycauchy_get_marginal_2D_pointwise_cpdf does (pycauchy.hpp:822-862),
// including its optional cache reset after the grid.
int ref_cpdf_2d_grid(void* vh, int i1, int i2, double lx, double hx, double rx, double ly, double hy, double ry,
                     int reset_cache, int max_points, double* xs, double* ys, double* zs, double* bar_nu)
{
    RefHandle* h = (RefHandle*)vh;
    if (!h->cpdf) h->cpdf = new PointWiseNDimCauchyCPDF(h->est);
    for (int i = 0; i < h->d; i++) bar_nu[i] = h->cpdf->bar_nu[i];
    CauchyCPDFGridDispatcher2D grid(h->cpdf, lx, hx, rx, ly, hy, ry);
    if (grid.num_grid_points > max_points) return -2;
    if (grid.evaluate_point_grid(i1, i2, 1)) return -5;
    if (reset_cache) h->cpdf->reset_2D_marginal_cpdf();
    for (int i = 0; i < grid.num_grid_points; i++) {
        xs[i] = grid.points[i].x;
        ys[i] = grid.points[i].y;
        zs[i] = grid.points[i].z;
    }
    return grid.num_grid_points;
}

// The constructor's print_basic_info (include/cauchy_estimator.hpp:87, 165),
// set after construction: the reference then reports the post-FTR moments of
// compute_moments(false) after every table build (and prints its progress).
void ref_set_print_basic_info(void* vh, int on) { ((RefHandle*)vh)->est->print_basic_info = on != 0; }

// The reference's extended-mode helpers (include/cauchy_estimator.hpp:1312-1394).
void ref_shift_cf_by_bias(void* vh, const double* bias) { ((RefHandle*)vh)->est->shift_cf_by_bias((double*)bias); }
void ref_deterministic_time_prop(void* vh, const double* Phi, const double* B, const double* u)
{
    ((RefHandle*)vh)->est->deterministic_time_prop((double*)Phi, (double*)B, (double*)u);
}
void ref_finalize_extended_moments(void* vh, double* x_bar) { ((RefHandle*)vh)->est->finalize_extended_moments(x_bar); }

// Marginal 1-D pdf on a grid through the reference's own
// PointWiseNDimCauchyCPDF and CauchyCPDFGridDispatcher1D
// (include/cpdf_ndim.hpp), as pycauchy_get_marginal_1D_pointwise_cpdf does
// (scripts/swig/cauchy/pycauchy.hpp:890-931): the pdf object is made on the
// first call (it draws bar_nu from rand()) and kept; a dispatcher per call.
// Returns the point count, -2 if it exceeds max_points, -5 if the reference
// refuses (the last step).  bar_nu[d] receives the pdf object's draws.
// PointWiseNDimCauchyCPDF::evaluate_cpdf (include/cpdf_ndim.hpp:677-904) at
// x[d] with the handle's pdf object; out[2] = (re, im).  -5 where the
// reference would assert (no step yet, or moment errors).
int ref_cpdf_nd(void* vh, const double* x, double* out)
{
    RefHandle* h = (RefHandle*)vh;
    if (h->est->master_step < 1 || h->est->numeric_moment_errors) return -5;
    if (!h->cpdf) h->cpdf = new PointWiseNDimCauchyCPDF(h->est);
    std::vector<double> xk(x, x + h->d);
    const C_COMPLEX_TYPE v = h->cpdf->evaluate_cpdf(xk.data());
    out[0] = __real__ v;
    out[1] = __imag__ v;
    return 0;
}

// PointWiseNDimCauchyCPDF::evaluate_marginal_cpdf (include/cpdf_ndim.hpp:918-1230)
// of the states idx[0..nm) at xm[nm] with the handle's pdf object, after
// srand(seed).  The function draws from rand() as it goes: each lowering's
// DiffCellEnumHelper::init draws one b_pert value per hyperplane of its
// largest shape (cell_enumeration.hpp:466-469; the shape range starts at the
// largest shape held + 1 and drops by one a lowering), then nu_bar[d - nm]
// = 2 U - 1 (cpdf_ndim.hpp:1187-1188).  nu_bar receives those values,
// reproduced from the same draws.  out[2] = (re, im); -5 where the reference
// would assert.
int ref_cpdf_marginal(void* vh, const double* xm, const int* idx, int nm, unsigned seed, double* nu_bar, double* out)
{
    RefHandle* h = (RefHandle*)vh;
    if (h->est->master_step < 1 || h->est->numeric_moment_errors || nm < 1 || nm >= h->d) return -5;
    if (!h->cpdf) h->cpdf = new PointWiseNDimCauchyCPDF(h->est);
    int top = 0;
    for (int i = 0; i < h->est->shape_range; i++)
        if (h->est->terms_per_shape[i] > 0) top = i;
    long long skip = 0;
    for (int l = 0; l < nm; l++) skip += (top + 1 - l) - 1;
    srand(seed);
    for (long long i = 0; i < skip; i++) rand();
    for (int i = 0; i < h->d - nm; i++) nu_bar[i] = 2 * random_uniform() - 1;
    srand(seed);
    std::vector<double> x(xm, xm + nm);
    std::vector<int> id(idx, idx + nm);
    const C_COMPLEX_TYPE v = h->cpdf->evaluate_marginal_cpdf(x.data(), id.data(), nm);
    out[0] = __real__ v;
    out[1] = __imag__ v;
    return 0;
}

int ref_cpdf_1d_grid(void* vh, int marg, double low, double high, double res, int max_points, double* xs,
                     double* ys, double* bar_nu)
{
    RefHandle* h = (RefHandle*)vh;
    if (!h->cpdf) h->cpdf = new PointWiseNDimCauchyCPDF(h->est);
    for (int i = 0; i < h->d; i++) bar_nu[i] = h->cpdf->bar_nu[i];
    CauchyCPDFGridDispatcher1D grid(h->cpdf, low, high, res);
    if (grid.num_grid_points > max_points) return -2;
    if (grid.evaluate_point_grid(marg, 1)) return -5;
    for (int i = 0; i < grid.num_grid_points; i++) {
        xs[i] = grid.points[i].x;
        ys[i] = grid.points[i].y;
    }
    return grid.num_grid_points;
}


// Relative-then-transformed system of two estimators through the reference's
// own get_marg2d_relative_and_transformed_cpdf and
// grid_eval_marg2d_relative_and_transformed_cpdf (include/cauchy_prediction.hpp),
// single-thread creation (its term order).  With center, the grid is offset by
// the relative mean as pycauchy_single_step_eval_2d_rsys_cpdf does
// (scripts/swig/cauchy/pycauchy.hpp:672-747).  rand() is seeded with bar_seed
// right before the call; bar_nu_full[d] receives the point it then draws.
// mom[14]: fz, mean[2], cov[4] as re/im pairs; counts[2]: pairs, pairs
// approximated out.  Returns the point count, -2 if it exceeds max_points,
// -5 if the reference refuses.
int ref_rel2d(void* vp, void* vs, const double* Trel, unsigned bar_seed, int full_solve, int with_term_approx,
              double term_approx_eps, double xlow, double xhigh, double dx, double ylow, double yhigh, double dy,
              int center, int max_points, double* bar_nu_full, double* mom, long long* counts, double* xs,
              double* ys, double* zs)
{
    RefHandle* p = (RefHandle*)vp;
    RefHandle* s = (RefHandle*)vs;
    const int d = p->d;
    srand(bar_seed);
    for (int i = 0; i < d; i++) bar_nu_full[i] = 2 * random_uniform_open() - 1;
    srand(bar_seed);
    C_COMPLEX_TYPE fz[1], mean[2], cov[4];
    Cached2DCPDFTermContainer* c = get_marg2d_relative_and_transformed_cpdf(
        p->est, s->est, (double*)Trel, full_solve != 0, false, true, fz, mean, cov, with_term_approx != 0,
        term_approx_eps, 1);
    if (!c) return -5;
    mom[0] = creal(fz[0]);
    mom[1] = cimag(fz[0]);
    for (int i = 0; i < 2; i++) {
        mom[2 + 2 * i] = creal(mean[i]);
        mom[3 + 2 * i] = cimag(mean[i]);
    }
    for (int i = 0; i < 4; i++) {
        mom[6 + 2 * i] = creal(cov[i]);
        mom[7 + 2 * i] = cimag(cov[i]);
    }
    const long long total = (long long)p->est->Nt * s->est->Nt;
    counts[0] = total;
    counts[1] = total - (long long)c->current_term_idx;
    const double ox = center ? mom[2] : 0.0, oy = center ? mom[4] : 0.0;
    const int nx = (int)ceil((xhigh - xlow) / dx + 1), ny = (int)ceil((yhigh - ylow) / dy + 1);
    if ((long long)nx * ny > max_points) {
        c->deinit();
        free(c);
        return -2;
    }
    int rx = 0, ry = 0;
    // two threads: the single-thread grid path prints every point
    CauchyPoint3D* pts = grid_eval_marg2d_relative_and_transformed_cpdf(
        c, xlow + ox, xhigh + ox, dx, ylow + oy, yhigh + oy, dy, creal(p->est->fz), creal(s->est->fz), &rx, &ry, 2,
        full_solve != 0, false);
    const int n = rx * ry;
    for (int i = 0; i < n; i++) {
        xs[i] = pts[i].x;
        ys[i] = pts[i].y;
        zs[i] = pts[i].z;
    }
    free(pts);
    c->deinit();
    free(c);
    return n;
}

}  // extern "C"
