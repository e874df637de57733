// Host-side pieces around the GPU step path, in C++:
//
//  * Speyer's restart statistics of a window (include/cauchy_util.hpp:23-113),
//    with the symmetric eigen-solver it needs: Householder reduction to
//    tridiagonal form followed by the QL iteration with implicit shifts, the
//    published pair of algorithms the reference also uses
//    (include/eig_solve.hpp:254-402; Numerical Recipes in C, 2nd ed.,
//    sections 11.2-11.3).  The restart's A0 rows are the eigenvectors, and
//    their order and signs fix the restarted window's term order and cell
//    keys, so the solver keeps the published arithmetic step for step.
//  * The C++ front end's sliding-window manager
//    (include/cauchy_windows.hpp:729-1165, SlidingWindowManager): W windows
//    per manager, one restarted each step about the fullest usable window.
//    The reference runs each window in a forked process fed through pipes;
//    here each window slot is one batched GPU handle over n_mgr managers that
//    advance in lock-step, so a step issues one launch sequence per slot and
//    measurement.
//
// Compiled as host code (no device code in this file), with
// -ffp-contract=off like the rest of the host side.
#include "../../include/mce_c_api.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

namespace mce {
void report_error(const std::string& s);
}

namespace {

// sqrt(a^2 + b^2) without destructive overflow or underflow.
double hypot_scaled(double a, double b)
{
    const double x = std::fabs(a), y = std::fabs(b);
    if (x > y) {
        const double r = y / x;
        return x * std::sqrt(1.0 + r * r);
    }
    if (y == 0.0) return 0.0;
    const double r = x / y;
    return y * std::sqrt(1.0 + r * r);
}

// Householder reduction of the symmetric n x n matrix z (row-major, in place)
// to tridiagonal form: diag[i] the diagonal, off[i] the sub-diagonal
// (off[0] = 0); z is replaced by the accumulated orthogonal transformation.
void householder_tridiagonal(double* z, int n, double* diag, double* off)
{
    auto Z = [z, n](int r, int c) -> double& { return z[(size_t)r * n + c]; };
    for (int i = n - 1; i > 0; i--) {
        const int l = i - 1;
        double h = 0.0, scale = 0.0;
        if (l > 0) {
            for (int k = 0; k <= l; k++) scale += std::fabs(Z(i, k));
            if (scale == 0.0) {
                off[i] = Z(i, l);
            } else {
                for (int k = 0; k <= l; k++) {
                    Z(i, k) /= scale;
                    h += Z(i, k) * Z(i, k);
                }
                double f = Z(i, l);
                double g = f >= 0.0 ? -std::sqrt(h) : std::sqrt(h);
                off[i] = scale * g;
                h -= f * g;
                Z(i, l) = f - g;
                f = 0.0;
                for (int j = 0; j <= l; j++) {
                    Z(j, i) = Z(i, j) / h;
                    g = 0.0;
                    for (int k = 0; k <= j; k++) g += Z(j, k) * Z(i, k);
                    for (int k = j + 1; k <= l; k++) g += Z(k, j) * Z(i, k);
                    off[j] = g / h;
                    f += off[j] * Z(i, j);
                }
                const double hh = f / (h + h);
                for (int j = 0; j <= l; j++) {
                    f = Z(i, j);
                    g = off[j] - hh * f;
                    off[j] = g;
                    for (int k = 0; k <= j; k++) Z(j, k) -= (f * off[k] + g * Z(i, k));
                }
            }
        } else {
            off[i] = Z(i, l);
        }
        diag[i] = h;
    }
    diag[0] = 0.0;
    off[0] = 0.0;
    // accumulate the transformations
    for (int i = 0; i < n; i++) {
        if (diag[i] != 0.0) {
            for (int j = 0; j < i; j++) {
                double g = 0.0;
                for (int k = 0; k < i; k++) g += Z(i, k) * Z(k, j);
                for (int k = 0; k < i; k++) Z(k, j) -= g * Z(k, i);
            }
        }
        diag[i] = Z(i, i);
        Z(i, i) = 1.0;
        for (int j = 0; j < i; j++) Z(j, i) = Z(i, j) = 0.0;
    }
}

// QL iteration with implicit shifts on the tridiagonal (diag, off) from
// householder_tridiagonal; eigenvalues end in diag, eigenvector i in column i
// of z.  Returns false if an eigenvalue needed more than 30 iterations.
bool ql_implicit(double* diag, double* off, int n, double* z)
{
    auto Z = [z, n](int r, int c) -> double& { return z[(size_t)r * n + c]; };
    bool ok = true;
    for (int i = 1; i < n; i++) off[i - 1] = off[i];
    off[n - 1] = 0.0;
    for (int l = 0; l < n; l++) {
        int iter = 0;
        int m;
        do {
            for (m = l; m < n - 1; m++) {
                const double dd = std::fabs(diag[m]) + std::fabs(diag[m + 1]);
                if (std::fabs(off[m]) + dd == dd) break;
            }
            if (m == l) break;
            if (iter++ == 30) {
                ok = false;
                break;
            }
            double g = (diag[l + 1] - diag[l]) / (2.0 * off[l]);
            double r = hypot_scaled(g, 1.0);
            g = diag[m] - diag[l] + off[l] / (g + (g >= 0.0 ? std::fabs(r) : -std::fabs(r)));
            double s = 1.0, c = 1.0, p = 0.0;
            bool underflow = false;
            for (int i = m - 1; i >= l; i--) {
                double f = s * off[i];
                const double b = c * off[i];
                r = hypot_scaled(f, g);
                off[i + 1] = r;
                if (r == 0.0) {
                    diag[i + 1] -= p;
                    off[m] = 0.0;
                    underflow = true;
                    break;
                }
                s = f / r;
                c = g / r;
                g = diag[i + 1] - p;
                r = (diag[i] - g) * s + 2.0 * c * b;
                p = s * r;
                diag[i + 1] = g + p;
                g = c * r - b;
                for (int k = 0; k < n; k++) {
                    f = Z(k, i + 1);
                    Z(k, i + 1) = s * Z(k, i) + c * f;
                    Z(k, i) = c * Z(k, i) - s * f;
                }
            }
            if (underflow) continue;
            diag[l] -= p;
            off[l] = g;
            off[m] = 0.0;
        } while (true);
    }
    return ok;
}

}  // namespace

extern "C" {

int mce_sym_eig(int n, const double* A, double* evals, double* evecs)
{
    if (n < 1 || !A || !evals || !evecs) return MCE_ERR_ARG;
    std::vector<double> off(n, 0.0);
    memcpy(evecs, A, sizeof(double) * n * n);
    householder_tridiagonal(evecs, n, evals, off.data());
    ql_implicit(evals, off.data(), n, evecs);
    return MCE_OK;
}

int mce_speyers_window_init(int n, const double* xhat, const double* Phat, const double* H, double gamma, double z,
                            const double* var_boost, double* A0, double* p0, double* b0)
{
    if (n < 1 || !xhat || !Phat || !H || !A0 || !p0 || !b0) return MCE_ERR_ARG;
    const size_t nn = (size_t)n * n;
    std::vector<double> V(Phat, Phat + nn), w1(nn), w2(nn), eig(n);
    if (var_boost)
        for (int i = 0; i < n; i++) V[(size_t)i * n + i] += var_boost[i];
    // make the covariance positive definite enough for the restart
    const double kCovEigTol = -1e-5;  // COV_EIGENVALUE_TOLERANCE (include/cauchy_constants.hpp:102)
    mce_sym_eig(n, V.data(), w2.data(), w1.data());
    double min_eig = w2[0];
    bool boost = false;
    for (int i = 0; i < n; i++) {
        if (w2[i] < kCovEigTol) boost = true;
        if (w2[i] < min_eig) min_eig = w2[i];
    }
    if (boost)
        for (int i = 0; i < n; i++) V[(size_t)i * n + i] += kCovEigTol - min_eig;
    // A = V + V H^T H V / s,  s = gamma^2 + (z - H x)^2
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) w1[(size_t)i * n + j] = 0.0 + H[i] * H[j];
    auto matmul = [n](const double* X, const double* Y, double* R) {
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                double s = 0.0;
                for (int k = 0; k < n; k++) s += X[(size_t)i * n + k] * Y[(size_t)k * n + j];
                R[(size_t)i * n + j] = s;
            }
    };
    matmul(V.data(), w1.data(), w2.data());
    matmul(w2.data(), V.data(), w1.data());
    double hx = 0.0;
    for (int i = 0; i < n; i++) hx += H[i] * xhat[i];
    const double innov = z - hx;
    const double scale = gamma * gamma + innov * innov;
    const double inv_scale = 1.0 / scale;
    for (size_t i = 0; i < nn; i++) w1[i] *= inv_scale;
    std::vector<double> A(nn);
    for (size_t i = 0; i < nn; i++) A[i] = V[i] + w1[i] * 1.0;
    // eigenvectors of A (columns of w2 after the solve)
    mce_sym_eig(n, A.data(), eig.data(), w2.data());
    // b0 = x - V H^T (z - H x) / s
    const double scale2 = innov / scale;
    std::vector<double> vh(n), hv(n);
    for (int i = 0; i < n; i++) {
        double s = 0.0;
        for (int j = 0; j < n; j++) s += V[(size_t)i * n + j] * H[j];
        vh[i] = s;
    }
    for (int i = 0; i < n; i++) b0[i] = xhat[i] - vh[i] * scale2;
    // p0_i = lambda_i / ((s + H V H^T) / gamma) * |v_i . H|
    for (int i = 0; i < n; i++) {
        double s = 0.0;
        for (int j = 0; j < n; j++) s += w2[i + (size_t)j * n] * H[j];
        hv[i] = s;
    }
    double hvh = 0.0;
    for (int i = 0; i < n; i++) hvh += H[i] * vh[i];
    const double scale3 = (scale + hvh) / gamma;
    for (int i = 0; i < n; i++) {
        double v = eig[i] / scale3;
        v *= hv[i];
        v /= (double)((hv[i] > 0.0) - (hv[i] < 0.0));
        p0[i] = v;
    }
    // rows of A0 are the eigenvectors
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) A0[(size_t)i * n + j] = w2[(size_t)j * n + i];
    return boost ? 1 : MCE_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Sliding-window manager of the C++ front end
// (include/cauchy_windows.hpp:729-1165 SlidingWindowManager, and the window
// processes' loop child_window_loop, :396-712).
//
// Schedule (the same for every manager of the object):
//  * step 0: window 0 takes the step's p measurements from the initial A0, p0, b0;
//  * step k >= 1: every started window except window k mod W (the
//    "initializee") takes the p measurements; the fullest of them whose error
//    bits show neither fz <= 0 nor a mean or covariance that does not exist
//    gives the step's estimate; the initializee is restarted about that
//    estimate with Speyer's statistics (the measurement model of the step's
//    last measurement) and takes the last measurement only;
//  * a window that has taken W steps reports, then is reset.
// LTV: a window calls the dynamics callback with its own conditional mean
// before each step but its first, the restarted window with the restart
// estimate, and the manager with the restart estimate before Speyer's
// statistics, each on its own copy of the dynamics container.
// Extended (nonlinear) mode: each window's container x holds its x_bar; the
// dynamics callback propagates it (and sets Phi, Gamma, beta) before each
// step but a window's first; every measurement update runs the measurement
// model (z_bar = h(x_bar)) and the extended update callback (H, gamma), steps
// the estimator (no controls) with z - z_bar and finalises the extended
// moments (x_bar <- the new estimate).  A restart is about the best window's
// x_bar: Speyer's statistics of dx = x_hat - x_bar and dz = z - h(x_bar),
// and the restarted window takes x_bar as its own
// (include/cauchy_windows.hpp:480-540, :600-660 and :1123-1139).
struct mce_swm {
    struct Duc {
        std::vector<double> x, Phi, Gamma, B, H, beta, gamma;
        mce_dynamics_container c;
    };
    int n_mgr = 0, W = 0, num_sim_steps = 0, d = 0, cmcc = 0, pncc = 0, p = 0, init_step = 0;
    double dt = 0;
    int est_cmcc = 0;  // controls of the window estimators (none in extended mode)
    mce_dynamics_callback cb = nullptr;
    bool ext = false;
    mce_msmt_model_callback msmt_cb = nullptr;
    mce_dynamics_callback ext_cb = nullptr;
    std::vector<double> xbar_win;    // W * n_mgr * d: the x_bar each window last reported
    std::vector<mce_handle*> slots;  // W batched handles over the managers
    std::vector<Duc> wduc;           // W * n_mgr window containers
    std::vector<Duc> mduc;           // n_mgr manager containers
    std::vector<double> u;           // n_mgr * cmcc controls of the current step
    std::vector<double> boost;       // window variance boost (empty: none)
    std::vector<int> win_count;      // steps each window has taken since its (re)start
    int msmt_count = 0;
    long long post_mu_done = 0;
    // latest moments per (window, manager): fz (re, im), mean, cov as (re, im)
    std::vector<double> fz, mean, cov;
    std::vector<int> err;

    ~mce_swm()
    {
        for (mce_handle* h : slots)
            if (h) mce_destroy(h);
    }

    void init_duc(Duc& q, int m, const double* Phi, const double* Gamma, const double* B, const double* beta,
                  const double* H, const double* gamma)
    {
        auto take = [](std::vector<double>& v, const double* src, size_t n, size_t off) {
            v.assign(std::max<size_t>(n, 1), 0.0);
            if (src && n) memcpy(v.data(), src + off * n, n * sizeof(double));
        };
        take(q.x, nullptr, d, 0);
        take(q.Phi, Phi, (size_t)d * d, m);
        take(q.Gamma, Gamma, (size_t)d * pncc, m);
        take(q.B, B, (size_t)d * cmcc, m);
        take(q.H, H, (size_t)p * d, m);
        take(q.beta, beta, pncc, m);
        take(q.gamma, gamma, p, m);
        memset(&q.c, 0, sizeof(q.c));
        q.c.x = q.x.data();
        q.c.u = u.data() + (size_t)m * std::max(cmcc, 1);
        q.c.dt = dt;
        q.c.step = init_step;
        q.c.n = d;
        q.c.cmcc = cmcc;
        q.c.pncc = pncc;
        q.c.p = p;
        q.c.Phi = q.Phi.data();
        q.c.Gamma = q.Gamma.data();
        q.c.B = q.B.data();
        q.c.H = q.H.data();
        q.c.beta = q.beta.data();
        q.c.gamma = q.gamma.data();
    }

    // One update of window slot j with measurement index i of every manager
    // (zs: the managers' measurements, else msmts[m * p + i]).
    int step_slot(int j, int i, const double* msmts, const double* zs = nullptr)
    {
        const size_t n = n_mgr;
        const int cm = est_cmcc;
        std::vector<double> z(n), Phi(n * d * d), Gam(n * d * std::max(pncc, 1)), beta(n * std::max(pncc, 1)),
            H(n * d), gam(n), B(n * d * std::max(cm, 1));
        for (int m = 0; m < n_mgr; m++) {
            const Duc& q = wduc[(size_t)j * n_mgr + m];
            z[m] = zs ? zs[m] : msmts[(size_t)m * p + i];
            memcpy(&Phi[(size_t)m * d * d], q.Phi.data(), sizeof(double) * d * d);
            if (pncc) memcpy(&Gam[(size_t)m * d * pncc], q.Gamma.data(), sizeof(double) * d * pncc);
            if (pncc) memcpy(&beta[(size_t)m * pncc], q.beta.data(), sizeof(double) * pncc);
            memcpy(&H[(size_t)m * d], q.H.data() + (size_t)i * d, sizeof(double) * d);
            gam[m] = q.gamma[i];
            if (cm) memcpy(&B[(size_t)m * d * cm], q.B.data(), sizeof(double) * d * cm);
        }
        std::vector<int> e(n);
        const int st = mce_batch_step(slots[j], z.data(), Phi.data(), Gam.data(), beta.data(), H.data(), gam.data(),
                                      cm ? B.data() : nullptr, cm ? u.data() : nullptr, 0, e.data());
        if (st < 0) return st;
        for (int m = 0; m < n_mgr; m++) err[(size_t)j * n_mgr + m] = e[m];
        return MCE_OK;
    }

    int read_moments(int j)
    {
        for (int m = 0; m < n_mgr; m++) {
            const size_t w = (size_t)j * n_mgr + m;
            const int st = mce_get_moments(slots[j], m, &fz[2 * w], &mean[2 * d * w], &cov[2 * (size_t)d * d * w]);
            if (st < 0) return st;
        }
        return MCE_OK;
    }

    void call_cb(Duc& q, const double* x, int step)
    {
        memcpy(q.x.data(), x, sizeof(double) * d);
        q.c.step = step;
        cb(&q.c);
    }

    // Extended-mode dynamics callback of a window: propagates its x_bar.
    int ext_propagate(Duc& q, int step)
    {
        q.c.is_xbar_set_for_ece = false;
        q.c.step = step;
        cb(&q.c);
        if (!q.c.is_xbar_set_for_ece) {
            mce::report_error("mce_swm_step: the dynamics callback did not set is_xbar_set_for_ece "
                              "(the reference asserts it, cauchy_windows.hpp:488)");
            return MCE_ERR_ARG;
        }
        return MCE_OK;
    }

    // Extended-mode update of window slot j with measurement index i of every
    // manager; save_xbar: the window reports the x_bar it starts this update
    // from (cauchy_windows.hpp:524 and :645).
    int ext_update(int j, int i, const double* msmts, bool save_xbar)
    {
        std::vector<double> z(n_mgr), zbar(p);
        for (int m = 0; m < n_mgr; m++) {
            Duc& q = wduc[(size_t)j * n_mgr + m];
            if (save_xbar) memcpy(&xbar_win[((size_t)j * n_mgr + m) * d], q.x.data(), sizeof(double) * d);
            msmt_cb(&q.c, zbar.data());
            z[m] = msmts[(size_t)m * p + i] - zbar[i];
            ext_cb(&q.c);
        }
        int st = step_slot(j, i, msmts, z.data());
        if (st < 0) return st;
        for (int m = 0; m < n_mgr; m++) {
            st = mce_finalize_extended_moments(slots[j], m, wduc[(size_t)j * n_mgr + m].x.data());
            if (st < 0) return st;
        }
        return MCE_OK;
    }
};

extern "C" {

static mce_swm* swm_make(int n_mgr, int num_windows, int num_sim_steps, int d, int cmcc, int pncc, int p,
                         const double* x0, const double* A0, const double* p0, const double* b0, const double* Phi,
                         const double* Gamma, const double* B, const double* beta, const double* H,
                         const double* gamma, double dt, int init_step, mce_dynamics_callback dyn_cb,
                         mce_msmt_model_callback msmt_cb, mce_dynamics_callback ext_cb,
                         const double* win_var_boost, const double* root_point, const double* b_pert,
                         int bpert_stride, int* status);

mce_swm* mce_swm_create(int n_mgr, int num_windows, int num_sim_steps, int d, int cmcc, int pncc, int p,
                        const double* A0, const double* p0, const double* b0, const double* Phi,
                        const double* Gamma, const double* B, const double* beta, const double* H,
                        const double* gamma, double dt, int init_step, mce_dynamics_callback dyn_cb,
                        const double* win_var_boost, const double* root_point, const double* b_pert,
                        int bpert_stride, int* status)
{
    if (!H || (!Phi && !dyn_cb)) {
        mce::report_error("mce_swm_create: invalid arguments");
        if (status) *status = MCE_ERR_ARG;
        return nullptr;
    }
    return swm_make(n_mgr, num_windows, num_sim_steps, d, cmcc, pncc, p, nullptr, A0, p0, b0, Phi, Gamma, B, beta, H,
                    gamma, dt, init_step, dyn_cb, nullptr, nullptr, win_var_boost, root_point, b_pert, bpert_stride,
                    status);
}

mce_swm* mce_swm_create_nonlin(int n_mgr, int num_windows, int num_sim_steps, int d, int cmcc, int pncc, int p,
                               const double* x0, const double* A0, const double* p0, const double* b0,
                               const double* beta, const double* gamma, double dt, int init_step,
                               mce_dynamics_callback dyn_cb, mce_msmt_model_callback msmt_cb,
                               mce_dynamics_callback ext_cb, const double* win_var_boost, const double* root_point,
                               const double* b_pert, int bpert_stride, int* status)
{
    if (!x0 || !dyn_cb || !msmt_cb || !ext_cb) {
        mce::report_error("mce_swm_create_nonlin: x0 and the three callbacks are required (cauchy_windows.hpp:866-884)");
        if (status) *status = MCE_ERR_ARG;
        return nullptr;
    }
    return swm_make(n_mgr, num_windows, num_sim_steps, d, cmcc, pncc, p, x0, A0, p0, b0, nullptr, nullptr, nullptr,
                    beta, nullptr, gamma, dt, init_step, dyn_cb, msmt_cb, ext_cb, win_var_boost, root_point, b_pert,
                    bpert_stride, status);
}

static mce_swm* swm_make(int n_mgr, int num_windows, int num_sim_steps, int d, int cmcc, int pncc, int p,
                         const double* x0, const double* A0, const double* p0, const double* b0, const double* Phi,
                         const double* Gamma, const double* B, const double* beta, const double* H,
                         const double* gamma, double dt, int init_step, mce_dynamics_callback dyn_cb,
                         mce_msmt_model_callback msmt_cb, mce_dynamics_callback ext_cb,
                         const double* win_var_boost, const double* root_point, const double* b_pert,
                         int bpert_stride, int* status)
{
    auto fail = [status](int st, const char* msg) -> mce_swm* {
        mce::report_error(msg);
        if (status) *status = st;
        return nullptr;
    };
    if (n_mgr < 1 || num_windows < 2 || num_sim_steps < 1 || d < 2 || p < 1 || pncc < 0 || cmcc < 0 || !A0 ||
        !p0 || !b0 || !gamma)
        return fail(MCE_ERR_ARG, "mce_swm_create: invalid arguments");
    if (init_step != 0 && init_step != 1)
        return fail(MCE_ERR_ARG, "mce_swm_create: the initial step must be 0 or 1 (cauchy_windows.hpp:871)");
    if ((root_point == nullptr) != (b_pert == nullptr))
        return fail(MCE_ERR_ARG, "mce_swm_create: give both root_point and b_pert or neither");
    std::unique_ptr<mce_swm> s(new mce_swm());
    s->n_mgr = n_mgr;
    s->W = num_windows;
    s->num_sim_steps = num_sim_steps;
    s->d = d;
    s->cmcc = cmcc;
    s->pncc = pncc;
    s->p = p;
    s->dt = dt;
    s->init_step = init_step;
    s->cb = dyn_cb;
    s->ext = msmt_cb != nullptr;
    s->msmt_cb = msmt_cb;
    s->ext_cb = ext_cb;
    s->est_cmcc = s->ext ? 0 : cmcc;
    if (win_var_boost) s->boost.assign(win_var_boost, win_var_boost + d);
    s->u.assign((size_t)n_mgr * std::max(cmcc, 1), 0.0);
    s->win_count.assign(num_windows, 0);
    s->fz.assign((size_t)num_windows * n_mgr * 2, 0.0);
    s->mean.assign((size_t)num_windows * n_mgr * 2 * d, 0.0);
    s->cov.assign((size_t)num_windows * n_mgr * 2 * d * d, 0.0);
    s->err.assign((size_t)num_windows * n_mgr, 0);
    s->mduc.resize(n_mgr);
    s->wduc.resize((size_t)num_windows * n_mgr);
    for (int m = 0; m < n_mgr; m++) {
        s->init_duc(s->mduc[m], m, Phi, Gamma, B, beta, H, gamma);
        for (int j = 0; j < num_windows; j++)
            s->init_duc(s->wduc[(size_t)j * n_mgr + m], m, Phi, Gamma, B, beta, H, gamma);
    }
    if (s->ext) {
        // every window process starts from a copy of the manager's container, x = x_bar_0
        s->xbar_win.assign((size_t)num_windows * n_mgr * d, 0.0);
        for (int m = 0; m < n_mgr; m++) {
            memcpy(s->mduc[m].x.data(), x0 + (size_t)m * d, sizeof(double) * d);
            for (int j = 0; j < num_windows; j++)
                memcpy(s->wduc[(size_t)j * n_mgr + m].x.data(), x0 + (size_t)m * d, sizeof(double) * d);
        }
    }
    // every window process of the reference constructs its estimator after the
    // fork, from the same rand() state: one set of constants per manager,
    // shared by its windows
    const int ms = (num_windows - 1) * pncc + d;
    std::vector<double> rp, bp;
    int stride = bpert_stride;
    if (!root_point) {
        rp.resize((size_t)n_mgr * d);
        bp.resize((size_t)n_mgr * ms);
        for (int m = 0; m < n_mgr; m++)
            mce_draw_reference_constants(-1, d, ms, 0, &rp[(size_t)m * d], &bp[(size_t)m * ms]);
        stride = ms;
    } else {
        if (bpert_stride < ms) return fail(MCE_ERR_ARG, "mce_swm_create: b_pert stride below the window's max shape");
        rp.assign(root_point, root_point + (size_t)n_mgr * d);
        bp.assign(b_pert, b_pert + (size_t)n_mgr * bpert_stride);
    }
    std::vector<int> steps(n_mgr, num_windows);
    s->slots.assign(num_windows, nullptr);
    for (int j = 0; j < num_windows; j++) {
        int st = MCE_OK;
        s->slots[j] = mce_batch_create(n_mgr, d, s->est_cmcc, pncc, p, steps.data(), A0, p0, b0, rp.data(), bp.data(),
                                       stride, &st);
        if (!s->slots[j]) {
            if (status) *status = st;
            return nullptr;
        }
        mce_set_window_number(s->slots[j], j);
    }
    if (status) *status = MCE_OK;
    return s.release();
}

int mce_swm_step(mce_swm* s, const double* msmts, const double* controls, double* fz, double* xhat, double* Phat,
                 double* cerr_fz, double* cerr_xhat, double* cerr_Phat, int* win_idx, int* err_code)
{
    if (!s || !msmts) return MCE_ERR_ARG;
    if (s->msmt_count >= s->num_sim_steps) {
        mce::report_error("mce_swm_step: the manager has taken all its simulation steps");
        return MCE_ERR_DONE;
    }
    const int W = s->W, d = s->d, p = s->p, nm = s->n_mgr;
    const int mc = s->msmt_count;
    const int step_k = s->init_step + mc;
    const int initializee = mc == 0 ? -1 : mc % W;
    if (s->cmcc && controls) memcpy(s->u.data(), controls, sizeof(double) * nm * s->cmcc);
    for (auto& q : s->wduc) q.c.step = step_k;
    for (auto& q : s->mduc) q.c.step = step_k;
    // windows that keep going take the step's p measurements
    std::vector<char> active(W, 0);
    std::vector<double> xr(d);
    const bool first_loop = mc < W;
    for (int j = 0; j < W; j++) {
        if (j == initializee || (mc < W && j > mc)) continue;
        active[j] = 1;
        s->win_count[j] += 1;
        if (s->cb && s->win_count[j] != 1) {
            for (int m = 0; m < nm; m++) {
                if (s->ext) {
                    // x_bar already equals Re(mean): finalising the last update set it
                    const int st = s->ext_propagate(s->wduc[(size_t)j * nm + m], step_k);
                    if (st < 0) return st;
                    continue;
                }
                const double* mu = &s->mean[2 * d * ((size_t)j * nm + m)];
                for (int i = 0; i < d; i++) xr[i] = mu[2 * i];
                s->call_cb(s->wduc[(size_t)j * nm + m], xr.data(), step_k);
            }
        }
        for (int i = 0; i < p; i++) {
            const int st = s->ext ? s->ext_update(j, i, msmts, i == p - 1 && (first_loop || s->win_count[j] == W))
                                  : s->step_slot(j, i, msmts);
            if (st < 0) return st;
        }
        const int st = s->read_moments(j);
        if (st < 0) return st;
    }
    // the fullest usable window of each manager (stratgey_choose_fullest_window_first)
    const int kBad = (1 << 9) | (1 << 3) | (1 << 7);  // fz <= 0, covariance DNE, mean DNE
    std::vector<int> order;
    for (int j = 0; j < W; j++)
        if (active[j]) order.push_back(j);
    std::stable_sort(order.begin(), order.end(), [s](int a, int b) { return s->win_count[a] > s->win_count[b]; });
    std::vector<int> best(nm, -1);
    for (int m = 0; m < nm; m++) {
        for (int j : order)
            if (!(s->err[(size_t)j * nm + m] & kBad)) {
                best[m] = j;
                break;
            }
        if (best[m] < 0) {
            mce::report_error("mce_swm_step: no window is usable (the reference exits here, cauchy_windows.hpp:1560)");
            return MCE_ERR_DEVICE;
        }
    }
    // outputs: the best window's latest moments
    for (int m = 0; m < nm; m++) {
        const size_t w = (size_t)best[m] * nm + m;
        const double* f = &s->fz[2 * w];
        const double* mu = &s->mean[2 * d * w];
        const double* cv = &s->cov[2 * (size_t)d * d * w];
        if (fz) fz[m] = f[0];
        if (cerr_fz) cerr_fz[m] = f[1];
        double ex = 0, ep = 0;
        for (int i = 0; i < d; i++) {
            if (xhat) xhat[(size_t)m * d + i] = mu[2 * i];
            ex = std::max(ex, std::fabs(mu[2 * i + 1]));
        }
        for (int i = 0; i < d * d; i++) {
            if (Phat) Phat[(size_t)m * d * d + i] = cv[2 * i];
            ep = std::max(ep, std::fabs(cv[2 * i + 1]));
        }
        if (cerr_xhat) cerr_xhat[m] = ex;
        if (cerr_Phat) cerr_Phat[m] = ep;
        if (win_idx) win_idx[m] = best[m];
        if (err_code) err_code[m] = s->err[w];
    }
    // restart the initializee about each manager's best estimate
    if (initializee >= 0 && s->ext) {
        const int j = initializee;
        std::vector<double> Pr((size_t)d * d), A0((size_t)d * d), p0(d), b0(d), xb(d), zbar(p);
        for (int m = 0; m < nm; m++) {
            const size_t w = (size_t)best[m] * nm + m;
            memcpy(xb.data(), &s->xbar_win[w * d], sizeof(double) * d);
            for (int i = 0; i < d; i++) xr[i] = s->mean[2 * d * w + 2 * i] - xb[i];  // dx
            for (int i = 0; i < d * d; i++) Pr[i] = s->cov[2 * (size_t)d * d * w + 2 * i];
            mce_swm::Duc& q = s->mduc[m];
            memcpy(q.x.data(), xb.data(), sizeof(double) * d);
            q.c.step = step_k;
            s->ext_cb(&q.c);
            s->msmt_cb(&q.c, zbar.data());
            const double dz = msmts[(size_t)m * p + p - 1] - zbar[p - 1];
            mce_speyers_window_init(d, xr.data(), Pr.data(), q.H.data() + (size_t)(p - 1) * d, q.gamma[p - 1], dz,
                                    s->boost.empty() ? nullptr : s->boost.data(), A0.data(), p0.data(), b0.data());
            int st = mce_reinitialize_start_statistics(s->slots[j], m, A0.data(), p0.data(), b0.data());
            if (st < 0) return st;
            mce_swm::Duc& wq = s->wduc[(size_t)j * nm + m];
            memcpy(wq.x.data(), xb.data(), sizeof(double) * d);
            wq.c.step = step_k;
        }
        s->win_count[j] = 1;
        int st = s->ext_update(j, p - 1, msmts, first_loop);
        if (st < 0) return st;
        st = mce_set_master_step(s->slots[j], p);
        if (st < 0) return st;
        st = s->read_moments(j);
        if (st < 0) return st;
    } else if (initializee >= 0) {
        const int j = initializee;
        std::vector<double> Pr((size_t)d * d), A0((size_t)d * d), p0(d), b0(d);
        for (int m = 0; m < nm; m++) {
            const size_t w = (size_t)best[m] * nm + m;
            for (int i = 0; i < d; i++) xr[i] = s->mean[2 * d * w + 2 * i];
            for (int i = 0; i < d * d; i++) Pr[i] = s->cov[2 * (size_t)d * d * w + 2 * i];
            mce_swm::Duc& q = s->mduc[m];
            if (s->cb) s->call_cb(q, xr.data(), step_k);
            mce_speyers_window_init(d, xr.data(), Pr.data(), q.H.data() + (size_t)(p - 1) * d, q.gamma[p - 1],
                                    msmts[(size_t)m * p + p - 1], s->boost.empty() ? nullptr : s->boost.data(),
                                    A0.data(), p0.data(), b0.data());
            int st = mce_reinitialize_start_statistics(s->slots[j], m, A0.data(), p0.data(), b0.data());
            if (st < 0) return st;
            if (s->cb) s->call_cb(s->wduc[(size_t)j * nm + m], xr.data(), step_k);
        }
        s->win_count[j] = 1;
        int st = s->step_slot(j, p - 1, msmts);
        if (st < 0) return st;
        st = mce_set_master_step(s->slots[j], p);
        if (st < 0) return st;
        st = s->read_moments(j);
        if (st < 0) return st;
    }
    // full windows are reset after they report
    for (int j = 0; j < W; j++)
        if (s->win_count[j] == W) {
            s->post_mu_done += mce_post_mu_terms(s->slots[j]);
            const int st = mce_reset(s->slots[j]);
            if (st < 0) return st;
            // the window restarts from one term: buffers of a gigabyte or more go back to the device
            const long long tr = mce_trim_memory(s->slots[j], 1LL << 30);
            if (tr < 0) return (int)tr;
            s->win_count[j] = 0;
        }
    s->msmt_count += 1;
    return MCE_OK;
}

long long mce_swm_post_mu_terms(mce_swm* s)
{
    if (!s) return MCE_ERR_ARG;
    long long t = s->post_mu_done;
    for (mce_handle* h : s->slots) t += mce_post_mu_terms(h);
    return t;
}

mce_handle* mce_swm_window(mce_swm* s, int j) { return (s && j >= 0 && j < s->W) ? s->slots[j] : nullptr; }

int mce_swm_window_count(mce_swm* s, int j) { return (s && j >= 0 && j < s->W) ? s->win_count[j] : MCE_ERR_ARG; }

void mce_swm_destroy(mce_swm* s) { delete s; }

}  // extern "C"
