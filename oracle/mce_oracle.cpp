// ORACLE — test infrastructure only.
//
// A plain, serial CPU restatement of the reference's per-step term
// propagation (natsnyder1/CauchyFriendly, CauchyEstimator::step,
// include/cauchy_estimator.hpp:1211-1245), written from the reference's
// algorithm, used only by tests/, __graft_entry__.smoke() and bench.py's
// cpu_baseline / reference arm as the CHECKER.  The shipped product never
// links or calls this file.
//
// Pinned against the compiled reference (oracle/ref_harness.cpp) through the
// golden fixtures in tests/golden (tests/test_oracle_golden.py).
//
// Storage mode mirrored: binary-search g-tables with half storage (the
// reference defaults, include/cauchy_types.hpp:22-35).  Term order mirrors the
// serial path (NUM_CPUS == 1): parents in shape/index order, then children in
// (parent, hyperplane) order (include/cauchy_estimator.hpp:741-780).
//
// Floating point: every sum is evaluated sequentially in the reference's
// index order and complex numbers use the C99 complex type, so with
// -ffp-contract=off the results are bit-identical to the reference build.
#include <algorithm>
#include <cmath>
#include <complex.h>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>
#include <chrono>

typedef double __complex__ cplx;

static inline cplx mkc(double re, double im)
{
    cplx z;
    __real__ z = re;
    __imag__ z = im;
    return z;
}
static inline cplx cconj(cplx z)
{
    __imag__ z = -__imag__ z;
    return z;
}
// Complex division by Smith's method (CACM 5(8), 1962), evaluated here
// unfused.  On x86-64 this is bit-identical to the compiler runtime's
// division the reference uses; spelling it out keeps the oracle identical on
// hosts whose runtime division is built with fused multiply-adds (aarch64).
static inline cplx cdiv(cplx x, cplx y)
{
    const double a = __real__ x, b = __imag__ x, c = __real__ y, d = __imag__ y;
    if (fabs(c) < fabs(d)) {
        const double r = c / d;
        const double den = c * r + d;
        return mkc((a * r + b) / den, (b * r - a) / den);
    }
    const double r = d / c;
    const double den = d * r + c;
    return mkc((b * r + a) / den, (b - a * r) / den);
}

// Constants: include/cauchy_constants.hpp:27-81
static const double kTwoPiInv = 1.0 / (2.0 * M_PI);
static const double kCoalignEps = 1e-8;   // COALIGN_TP_EPS / COALIGN_MU_EPS
static const double kMuEps = 1e-10;       // MU_EPS
static const double kTermApproxEps = 1e-15;
static const double kPluEps = 1e-15;
static const double kCondEps = 1e12;
static const double kReductionEps = 1e-8;

enum {
    ERR_FZ_NEGATIVE = 9,
    ERR_FZ_UNSTABLE = 8,
    ERR_MEAN_DNE = 7,
    ERR_MEAN_UNSTABLE_NOT_FINAL = 6,
    ERR_MEAN_UNSTABLE_FINAL = 5,
    ERR_MEAN_UNSTABLE_ANY = 4,
    ERR_COV_DNE = 3,
    ERR_COV_UNSTABLE_NOT_FINAL = 2,
    ERR_COV_UNSTABLE_FINAL = 1,
    ERR_COV_UNSTABLE_ANY = 0,
};

enum { ORC_OK = 0, ORC_ERR_BOTH_HORTHOG_NEG = 1, ORC_ERR_SHAPE = 2, ORC_ERR_DONE = 3 };

// ----------------------------------------------------------------------------
// Combinatorics: include/cell_enumeration.hpp:11-56, 71-119
static long long binom(int n, int k)
{
    if (k < 0 || k > n) return 0;
    long long r = 1;
    if (k > n - k) k = n - k;
    for (int i = 0; i < k; i++) {
        r *= (n - i);
        r /= (i + 1);
    }
    return r;
}
static int cells_central(int m, int d)
{
    if (m < d) return 1 << m;
    long long s = 0;
    for (int i = 0; i < d; i++) s += binom(m - 1, i);
    return (int)(2 * s);
}
static int cells_general(int m, int d)
{
    if (m < d) return 1 << m;
    long long s = 0;
    for (int i = 0; i <= d; i++) s += binom(m, i);
    return (int)s;
}
// d-subsets of {0..m-1} in lexicographic order (the order std::prev_permutation
// on a leading-ones mask produces, cell_enumeration.hpp:71-92).
static void lex_combos(int m, int d, std::vector<int>& out)
{
    out.clear();
    if (d > m || d <= 0) return;
    std::vector<int> c(d);
    for (int i = 0; i < d; i++) c[i] = i;
    while (true) {
        out.insert(out.end(), c.begin(), c.end());
        int i = d - 1;
        while (i >= 0 && c[i] == m - d + i) i--;
        if (i < 0) break;
        c[i]++;
        for (int j = i + 1; j < d; j++) c[j] = c[j - 1] + 1;
    }
}

// ----------------------------------------------------------------------------
// Small dense linear algebra with the reference's exact operation order.
// PLU with partial pivoting: cauchy_linalg.hpp:1180-1231
static int plu(double* A, int* P, int n, double tol)
{
    double tmp[32];
    for (int j = 0; j < n; j++) {
        double piv = tol;
        int pi = -1;
        for (int i = j; i < n; i++)
            if (fabs(A[i * n + j]) > fabs(piv)) {
                piv = A[i * n + j];
                pi = i;
            }
        if (pi == -1) return 1;
        if (pi != j) {
            memcpy(tmp, A + j * n, n * sizeof(double));
            memcpy(A + j * n, A + pi * n, n * sizeof(double));
            memcpy(A + pi * n, tmp, n * sizeof(double));
        }
        P[j] = pi;
        for (int k = j + 1; k < n; k++) {
            A[k * n + j] /= A[j * n + j];
            double t = A[k * n + j];
            for (int q = j + 1; q < n; q++) A[k * n + q] -= t * A[j * n + q];
        }
    }
    return 0;
}
// forward/back solves on a packed LU: cauchy_linalg.hpp:1234-1256
static void lu_forward(const double* LU, double* b, int n)
{
    for (int i = 0; i < n; i++) {
        double s = b[i];
        for (int j = 0; j < i; j++) s -= LU[i * n + j] * b[j];
        b[i] = s;
    }
}
static void lu_back(const double* LU, double* b, int n)
{
    for (int i = n - 1; i >= 0; i--) {
        double s = b[i];
        for (int j = n - 1; j > i; j--) s -= LU[i * n + j] * b[j];
        b[i] = s / LU[i * n + i];
    }
}
// Inverse row permutation of the pivot list: cauchy_linalg.hpp:1258-1277
static void pivots_to_inverse_perm(const int* P, int* PT, int n)
{
    int Preg[32];
    for (int i = 0; i < n; i++) Preg[i] = i;
    for (int i = 0; i < n; i++) {
        int t = Preg[i];
        Preg[i] = Preg[P[i]];
        Preg[P[i]] = t;
    }
    for (int i = 0; i < n; i++) PT[Preg[i]] = i;
}
// 1-norm condition number through an explicit inverse: cauchy_linalg.hpp:1337-1390
static double cond1(double* A, int* P, int n)
{
    double nrm = -1;
    for (int c = 0; c < n; c++) {
        double s = 0;
        for (int r = 0; r < n; r++) s += fabs(A[r * n + c]);
        if (s > nrm) nrm = s;
    }
    if (plu(A, P, n, kPluEps)) return 1.79769313486231570815e+308;
    int PT[32];
    pivots_to_inverse_perm(P, PT, n);
    double W[32 * 32];
    memset(W, 0, sizeof(double) * n * n);
    for (int i = 0; i < n; i++) {
        W[i * n + PT[i]] = 1;
        lu_forward(A, W + i * n, n);
        lu_back(A, W + i * n, n);
    }
    // The reference transposes W and takes column sums; that equals row sums of W.
    double inrm = -1;
    for (int i = 0; i < n; i++) {
        double s = 0;
        for (int j = 0; j < n; j++) s += fabs(W[i * n + j]);
        if (s > inrm) inrm = s;
    }
    return nrm * inrm;
}
// solve_trf: cauchy_linalg.hpp:1280-1299
static void solve_lu(const double* LU, const int* P, const double* b, double* x, int n)
{
    int PT[32];
    pivots_to_inverse_perm(P, PT, n);
    for (int i = 0; i < n; i++) x[PT[i]] = b[i];
    lu_forward(LU, x, n);
    lu_back(LU, x, n);
}

// Symmetric eigenvalues (Jacobi rotations) for the covariance check.  The
// reference uses tred2/tqli (eig_solve.hpp:404); only the sign test against
// -1e-5 consumes the result.
static void sym_eigvals(const double* S, double* ev, int n)
{
    double a[64];
    memcpy(a, S, sizeof(double) * n * n);
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0;
        for (int i = 0; i < n; i++)
            for (int j = i + 1; j < n; j++) off += a[i * n + j] * a[i * n + j];
        if (off < 1e-300) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                double apq = a[p * n + q];
                if (apq == 0) continue;
                double th = (a[q * n + q] - a[p * n + p]) / (2 * apq);
                double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1));
                double c = 1 / sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; k++) {
                    double akp = a[k * n + p], akq = a[k * n + q];
                    a[k * n + p] = c * akp - s * akq;
                    a[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    double apk = a[p * n + k], aqk = a[q * n + k];
                    a[p * n + k] = c * apk - s * aqk;
                    a[q * n + k] = s * apk + c * aqk;
                }
            }
    }
    for (int i = 0; i < n; i++) ev[i] = a[i * n + i];
}

// covariance_checker: cauchy_util.hpp:1882-2004
static int covariance_flags(const cplx* cov, int d)
{
    int flags = 0;
    double re[64], im[64], ev[8];
    for (int i = 0; i < d * d; i++) {
        re[i] = __real__ cov[i];
        im[i] = __imag__ cov[i];
    }
    sym_eigvals(re, ev, d);
    for (int i = 0; i < d; i++)
        if (ev[i] < -1e-5) flags |= 1;
    for (int i = 0; i < d - 1; i++) {
        double sii = sqrt(re[i * d + i]);
        for (int j = i + 1; j < d; j++) {
            double sjj = sqrt(re[j * d + j]);
            double c = re[i * d + j] / (sii * sjj);
            if (fabs(c) > 1) flags |= 2;
        }
    }
    for (int i = 0; i < d; i++)
        for (int j = i; j < d; j++) {
            double r = fabs(im[i * d + j]) / (fabs(re[i * d + j]) + 1e-15);
            if (r > 10) flags |= 4;
        }
    for (int i = 0; i < d * d; i++)
        if (fabs(im[i]) > 2000) flags |= 8;
    return flags;
}

// ----------------------------------------------------------------------------
// g-table: sorted keys with complex values (half storage).
struct GTable {
    std::vector<int> keys;
    std::vector<cplx> vals;
    int find(int key) const
    {
        // binsearch: gtable.hpp:283-301
        int lo = 0, hi = (int)keys.size() - 1;
        while (lo <= hi) {
            int mid = (lo + hi) / 2;
            int mk = keys[mid];
            if (mk == key) return mid;
            if ((unsigned)mk > (unsigned)key) hi = mid - 1;
            else lo = mid + 1;
        }
        return -1;
    }
};

// g numerator lookup in the parent table with half storage: eval_gs.hpp:94-153
static inline cplx lookup_num(const GTable* gp, int enc, int phc)
{
    const int top = 1 << (phc - 1);
    const int rev = (1 << phc) - 1;
    if (enc & top) {
        int idx = gp->find(rev ^ enc);
        if (idx < 0) return mkc(0, 0);
        return cconj(gp->vals[idx]);
    }
    int idx = gp->find(enc);
    if (idx < 0) return mkc(0, 0);
    return gp->vals[idx];
}

struct Term {
    int m = 0;
    std::vector<double> A, p, q, b;
    double c_val = 0, d_val = 0;
    unsigned horthog = 0;
    int phc = 0, pbc = 0, z = 0, enc_lhp = 0;
    bool is_new_child = false;
    bool has_cmap = false;
    std::vector<int> cmap, csmap;
    std::shared_ptr<GTable> gp;             // parent table (keys in phc-bit space)
    std::shared_ptr<std::vector<int>> encB;  // own B (parents) or shared B_mu (new children)
    std::vector<int> own_B;                  // B built for this term in make_gtables
    GTable g;                                // table built at this step
};

// Per-term constants of the 1-D marginal pdf (Cached1DCPDFTerm, cpdf_ndim.hpp:216-222).
struct Cpdf1DTerm {
    double a, b, w, s;
};

// Per-term cache of the 2-D marginal pdf (Cached2DCPDFTerm, cpdf_ndim.hpp:205-214).
struct Cpdf2DTerm {
    std::vector<double> sin_t, cos_t, g1r, g2r;
    std::vector<cplx> g;
    double b[2];
    int m;
};

struct Estimator {
    int d, cmcc, pncc, p, num_steps, shape_range;
    int master_step = 0;
    std::vector<double> A0, p0, b0, root, bpert;
    std::vector<Term> terms;  // ordered by shape then index
    int Nt = 1;
    std::vector<int> terms_per_shape;
    cplx fz, last_fz;
    std::vector<cplx> mean, cov, last_mean, last_cov;
    cplx raw_fz;
    std::vector<cplx> raw_mean, raw_cov;
    double gscale = 0;
    int errors = 0;
    bool skip_post_mu = false;
    bool print_basic_info = false;  // compute_moments(false) after each table build
    std::vector<std::vector<int>> combos;  // per shape
    long long post_mu_terms = 0;           // sum over steps of terms after MU
    // 1-D marginal pdf cache, keyed like the reference's by (master step, index)
    std::vector<Cpdf1DTerm> cpdf1d_cache;
    int cpdf1d_step = -1, cpdf1d_marg = -1;
    std::vector<Cpdf2DTerm> cpdf2d_cache;
    int cpdf2d_step = -1, cpdf2d_m1 = -1, cpdf2d_m2 = -1;
};

// ----------------------------------------------------------------------------
// Term operations (include/cauchy_term.hpp)

// time_prop: cauchy_term.hpp:435-456
static void time_prop(Term& t, int d, const double* Phi, const double* B, const double* u, int cmcc)
{
    std::vector<double> w(t.A.begin(), t.A.begin() + t.m * d);
    for (int i = 0; i < t.m; i++)
        for (int j = 0; j < d; j++) {
            double s = 0.0;
            for (int k = 0; k < d; k++) s += w[i * d + k] * Phi[k + j * d];
            t.A[i * d + j] = s;
        }
    double wb[16];
    memcpy(wb, t.b.data(), d * sizeof(double));
    for (int i = 0; i < d; i++) {
        double s = 0.0;
        for (int j = 0; j < d; j++) s += Phi[i * d + j] * wb[j];
        t.b[i] = s;
    }
    if (cmcc > 0) {
        for (int i = 0; i < d; i++) {
            double s = 0.0;
            for (int j = 0; j < cmcc; j++) s += B[i * cmcc + j] * u[j];
            wb[i] = s;
        }
        for (int i = 0; i < d; i++) t.b[i] += 1.0 * wb[i];
    }
}

// normalize_hps: cauchy_term.hpp:458-472
static void normalize_rows(Term& t, int d, bool set_q)
{
    if (set_q) t.q.assign(t.p.begin(), t.p.begin() + t.m);
    for (int i = 0; i < t.m; i++) {
        double n1 = 0;
        for (int j = 0; j < d; j++) n1 += fabs(t.A[i * d + j]);
        t.p[i] *= n1;
        for (int j = 0; j < d; j++) t.A[i * d + j] /= n1;
    }
}

// row-vs-row coalignment gate used by TP and MU coalignment
// (cauchy_term.hpp:494-504, 565-576): returns +1 (same), -1 (opposite), 0.
static inline int coalign_gate(const double* r, const double* c, int d)
{
    bool pos = true, neg = true;
    for (int l = 0; l < d; l++) {
        if (pos) pos &= fabs(r[l] - c[l]) < kCoalignEps;
        if (neg) neg &= fabs(r[l] + c[l]) < kCoalignEps;
        if (!(pos || neg)) break;
    }
    if (pos) return 1;
    if (neg) return -1;
    return 0;
}

// tp_coalign: cauchy_term.hpp:475-531
static void tp_coalign(Term& t, int d, const double* Gt, const double* bt, int cnt)
{
    normalize_rows(t, d, false);
    bool F[32];
    for (int j = 0; j < cnt; j++) F[j] = true;
    for (int j = 0; j < cnt; j++)
        for (int k = 0; k < t.m; k++)
            if (F[j] && coalign_gate(Gt + j * d, t.A.data() + k * d, d) != 0) {
                F[j] = false;
                t.p[k] += bt[j];
            }
    for (int j = 0; j < cnt; j++)
        if (F[j]) {
            t.A.resize((t.m + 1) * d);
            t.p.resize(t.m + 1);
            memcpy(t.A.data() + t.m * d, Gt + j * d, d * sizeof(double));
            t.p[t.m] = bt[j];
            t.m++;
        }
}

// precoalign_Gamma_beta: cauchy_util.hpp:128-210
static int precoalign_gamma(const double* Gamma, const double* beta, int pncc, int d, double* Gt, double* bt)
{
    for (int i = 0; i < pncc; i++) {
        for (int j = 0; j < d; j++) Gt[i * d + j] = Gamma[j * pncc + i];
        bt[i] = beta[i];
    }
    for (int i = 0; i < pncc; i++) {
        double nf = 0;
        for (int j = 0; j < d; j++) nf += fabs(Gt[i * d + j]);
        for (int j = 0; j < d; j++) Gt[i * d + j] /= nf;
        bt[i] *= nf;
    }
    bool F[32];
    for (int i = 0; i < pncc; i++) F[i] = true;
    for (int i = 0; i < pncc - 1; i++)
        if (F[i])
            for (int j = i + 1; j < pncc; j++)
                if (F[j] && coalign_gate(Gt + i * d, Gt + j * d, d) != 0) {
                    F[j] = false;
                    bt[i] += bt[j];
                }
    int cnt = 0;
    for (int i = 0; i < pncc; i++) cnt += F[i];
    if (cnt != pncc) {
        int u = 1;
        for (int j = 1; j < pncc; j++)
            if (F[j]) {
                if (u < j) {
                    memcpy(Gt + u * d, Gt + j * d, d * sizeof(double));
                    bt[u] = bt[j];
                }
                u++;
            }
    }
    return cnt;
}

// make_time_prop_btable: cell_enumeration.hpp:676-855 (the FAST_TP_DCE=false path)
static void tp_enumerate(Estimator& E, Term& t)
{
    const int m = t.m, d = E.d;
    std::vector<int> out;
    if (m < d) {
        for (int i = 0; i < (1 << (m - 1)); i++) out.push_back(i);
        t.encB = std::make_shared<std::vector<int>>(out);
        return;
    }
    const int phc = t.phc;
    const int gmask = (1 << phc) - 1, ptop = 1 << (phc - 1);
    const int mtop = 1 << (m - 1), mrev = (1 << m) - 1;
    const int cells_gen = cells_general(m, d);
    std::vector<char> seen((size_t)1 << m, 0);
    std::vector<int> found;
    std::vector<char> in_set((size_t)1 << m, 0);
    const std::vector<int>& cmb = E.combos[m];
    const int ncomb = m > d ? (int)(cmb.size() / d) : 0;  // the reference has no combos for m == d
    double Ac[64], bc[8], v[8];
    int P[8];
    for (int i = 0; i < ncomb; i++) {
        const int* c = &cmb[i * d];
        for (int j = 0; j < d; j++) {
            memcpy(Ac + j * d, t.A.data() + c[j] * d, d * sizeof(double));
            bc[j] = E.bpert[c[j]];
        }
        if (cond1(Ac, P, d) > kCondEps) continue;
        solve_lu(Ac, P, bc, v, d);
        int niv = 0;
        for (int a = 0; a < m; a++) {
            bool inc = false;
            for (int j = 0; j < d; j++)
                if (c[j] == a) inc = true;
            if (inc) continue;
            double s = 0.0;
            for (int j = 0; j < d; j++) s += t.A[a * d + j] * v[j];
            if (s - E.bpert[a] < 0) niv |= 1 << a;
        }
        for (int j = 0; j < (1 << d); j++) {
            int sv = niv;
            for (int k = 0; k < d; k++)
                if ((j >> k) & 1) sv |= 1 << c[k];
            if (seen[sv]) continue;
            seen[sv] = 1;
            int psv = sv & gmask;
            if (psv & ptop) psv ^= gmask;
            if (t.gp->find(psv) >= 0) {
                found.push_back(sv);
                in_set[sv] = 1;
            }
        }
        if ((int)found.size() == cells_gen) break;
    }
    std::vector<char> used(found.size(), 0);
    for (size_t i = 0; i < found.size(); i++) {
        if (used[i]) continue;
        int b = found[i], br = b ^ mrev;
        if (in_set[br]) {
            used[i] = 1;
            // mark the partner as consumed
            for (size_t k = i + 1; k < found.size(); k++)
                if (found[k] == br) {
                    used[k] = 1;
                    break;
                }
            out.push_back((b & mtop) ? br : b);
        }
    }
    t.encB = std::make_shared<std::vector<int>>(out);
}

// msmt_update: cauchy_term.hpp:84-310.  `t` is the parent; integrable children
// are appended to `kids`.  Returns the number of children.
static int msmt_update(Term& t, int d, std::vector<Term>& kids, double msmt, const double* H, double gamma,
                       bool first, bool last)
{
    const int m = t.m;
    std::vector<double> mu((m + 1) * d), rho(m + 1);
    std::vector<int> sgn(m);
    std::vector<char> Fi(m + 1);
    memcpy(mu.data(), t.A.data(), m * d * sizeof(double));
    memcpy(rho.data(), t.p.data(), m * sizeof(double));
    rho[m] = gamma;
    for (int j = 0; j < d; j++) mu[m * d + j] = 0;
    Fi[m] = 1;
    for (int l = 0; l < m; l++) {
        double h = 0.0;
        for (int j = 0; j < d; j++) h += H[j] * mu[l * d + j];
        double ah = fabs(h);
        if (ah < kMuEps) {
            rho[l] = t.p[l];
            sgn[l] = 1;
            Fi[l] = 0;
        } else {
            double r = 1.0 / h;
            for (int j = 0; j < d; j++) mu[l * d + j] *= r;
            rho[l] = t.p[l] * ah;
            sgn[l] = h > 0 ? 1 : -1;
            Fi[l] = 1;
        }
    }
    double hb = 0.0;
    for (int j = 0; j < d; j++) hb += H[j] * t.b[j];
    const double zeta = msmt - hb;
    const size_t kid0 = kids.size();
    std::vector<double> b_old(t.b);
    for (int tt = 0; tt <= m; tt++) {
        if (!Fi[tt]) continue;
        Term* c;
        Term tmp;
        if (tt == m) c = &t;
        else c = &tmp;
        if (!first) {
            c->gp = t.gp;
            c->phc = t.phc;
            c->pbc = m;
            c->z = tt;
        }
        c->c_val = zeta;
        c->d_val = rho[tt];
        c->m = m;
        std::vector<double> nb(d), nA(m * d), np(m);
        for (int j = 0; j < d; j++) nb[j] = b_old[j] + zeta * mu[tt * d + j];
        int l = 0;
        unsigned hof = 0;
        for (int ll = 0; ll <= m; ll++) {
            if (ll == tt) continue;
            np[l] = rho[ll];
            if (Fi[ll])
                for (int j = 0; j < d; j++) nA[l * d + j] = mu[ll * d + j] - mu[tt * d + j];
            else {
                for (int j = 0; j < d; j++) nA[l * d + j] = mu[ll * d + j];
                hof |= 1u << l;
            }
            l++;
        }
        c->A = nA;
        c->p = np;
        c->b = nb;
        c->horthog = hof;
        if (tt != m) kids.push_back(std::move(tmp));
    }
    t.is_new_child = false;
    if (!first) {
        int esg = 0;
        for (int l = 0; l < m; l++)
            if (sgn[l] == -1) esg |= 1 << l;
        int lhp = esg;
        if (t.phc < m) lhp &= (1 << t.phc) - 1;
        t.enc_lhp = lhp;
        if (esg & (1 << (m - 1))) esg ^= (1 << m) - 1;
        for (size_t i = kid0; i < kids.size(); i++) {
            kids[i].enc_lhp = lhp;
            kids[i].is_new_child = true;
            kids[i].encB = t.encB;  // shared: sees the parent's XOR below (B_mu)
        }
        if (!last)
            for (auto& k : *t.encB) k ^= esg;
    }
    return (int)(kids.size() - kid0);
}

// eval_g_yei: cauchy_term.hpp:312-401
static cplx eval_g_yei(const Term& t, int d, const double* root, cplx* yei, bool first)
{
    const int m = t.m;
    double sA[32], ty[16];
    for (int j = 0; j < d; j++) ty[j] = 0;
    double ygi = 0;
    for (int l = 0; l < m; l++) {
        double s = 0.0;
        for (int j = 0; j < d; j++) s += t.A[l * d + j] * root[j];
        sA[l] = s > 0 ? 1 : -1;
        double sc = t.p[l] * sA[l];
        for (int j = 0; j < d; j++) ty[j] += sc * t.A[l * d + j];
    }
    if (t.horthog) {
        for (int l = 0; l < m; l++)
            if (!(t.horthog & (1u << l))) ygi += t.p[l] * sA[l];
    } else {
        double z = 0.0;
        for (int l = 0; l < m; l++) z += t.p[l] * sA[l];
        ygi = z;
    }
    cplx gp, gm;
    if (first) {
        gp = mkc(1, 0);
        gm = mkc(1, 0);
    } else {
        int lp = 0, lm = 0, k = 0;
        for (int l = 0; l < m; l++) {
            if (k < t.phc) {
                if (k == t.z) {
                    lm |= 1 << k;
                    k++;
                    if (k == t.phc) continue;
                }
                if (sA[l] < 0) {
                    lp |= 1 << k;
                    lm |= 1 << k;
                }
                k++;
            }
        }
        gp = lookup_num(t.gp.get(), lp ^ t.enc_lhp, t.phc);
        gm = lookup_num(t.gp.get(), lm ^ t.enc_lhp, t.phc);
    }
    cplx g = cdiv(gp, mkc(ygi + t.d_val, t.c_val)) - cdiv(gm, mkc(ygi - t.d_val, t.c_val));
    g *= kTwoPiInv;
    for (int j = 0; j < d; j++) yei[j] = mkc(-ty[j], t.b[j]);
    return g;
}

// mu_coalign: cauchy_term.hpp:533-745.  Returns the new shape or -1 on the
// reference's fatal condition (two H-orthogonal rows anti-coaligned).
static int mu_coalign(Term& t, int d)
{
    normalize_rows(t, d, true);
    const int m = t.m;
    std::vector<char> F(m, 1);
    std::vector<char> hflag(m, 0);
    t.cmap.assign(m, 255);
    t.csmap.assign(m, 1);
    if (t.horthog)
        for (int j = 0; j < m; j++) hflag[j] = (t.horthog >> j) & 1;
    int uc = 0;
    for (int j = 0; j < m - 1; j++) {
        if (!F[j]) continue;
        t.cmap[j] = uc;
        for (int k = j + 1; k < m; k++) {
            if (!F[k]) continue;
            int g = coalign_gate(t.A.data() + j * d, t.A.data() + k * d, d);
            if (g == 1) {
                if (t.horthog) {
                    bool hj = hflag[j], hk = hflag[k];
                    if (!hj && !hk) t.q[j] += t.q[k];
                    else if (hj && !hk) {
                        t.q[j] = t.q[k];
                        hflag[j] = 0;
                    } else if (!hj && hk) hflag[k] = 0;
                    else {
                        hflag[k] = 0;
                        t.q[j] += t.q[k];
                    }
                } else
                    t.q[j] += t.q[k];
                F[k] = 0;
                t.p[j] += t.p[k];
                t.cmap[k] = uc;
                t.csmap[k] = 1;
            } else if (g == -1) {
                if (t.horthog) {
                    bool hj = hflag[j], hk = hflag[k];
                    if (!hj && !hk) t.q[j] -= t.q[k];
                    else if (hj && !hk) {
                        t.q[j] = -t.q[k];
                        hflag[j] = 0;
                    } else if (!hj && hk) hflag[k] = 0;
                    else return -1;
                } else
                    t.q[j] -= t.q[k];
                F[k] = 0;
                t.p[j] += t.p[k];
                t.cmap[k] = uc;
                t.csmap[k] = -1;
            }
        }
        uc++;
    }
    if (F[m - 1]) t.cmap[m - 1] = uc;
    int ns = 0;
    for (int i = 0; i < m; i++) ns += F[i];
    if (ns != m) {
        int u = 1;
        for (int j = 1; j < m; j++)
            if (F[j]) {
                if (u < j) {
                    memcpy(t.A.data() + u * d, t.A.data() + j * d, d * sizeof(double));
                    t.p[u] = t.p[j];
                    t.q[u] = t.q[j];
                }
                u++;
            }
        if (t.horthog) {
            unsigned nh = 0;
            int c = 0;
            for (int j = 0; j < m; j++)
                if (F[j]) nh |= (unsigned)hflag[j] << c++;
            t.horthog = nh;
        }
        t.m = ns;
        t.A.resize(ns * d);
        t.p.resize(ns);
        t.q.resize(ns);
    }
    return t.m;
}

// make_new_child_btable: cell_enumeration.hpp:206-371 (the MU-side DCE)
static void new_child_btable(Term& t, int d)
{
    const int m = t.m;
    std::vector<int> out;
    if (m <= d) {
        for (int i = 0; i < (1 << (m - 1)); i++) out.push_back(i);
        t.own_B = out;
        return;
    }
    const std::vector<int>& Bmu = *t.encB;
    const int pbc = t.pbc, z = t.z;
    const int mz = 1 << z, hb = 1 << (pbc - 1), rev = (1 << pbc) - 1, low = mz - 1;
    std::vector<int> pos((size_t)1 << pbc, -1);
    for (size_t j = 0; j < Bmu.size(); j++) pos[Bmu[j]] = (int)j;
    std::vector<char> F(Bmu.size(), 1);
    std::vector<int> buc;
    for (size_t j = 0; j < Bmu.size(); j++) {
        if (!F[j]) continue;
        int b = Bmu[j];
        int bq = b ^ mz;
        if (bq & hb) bq ^= rev;
        int k = pos[bq];
        if (k < 0) continue;
        F[j] = 0;
        F[k] = 0;
        int zb = (b & mz) >> z;
        int c1 = ((b >> (z + 1)) << z) | (b & low) | (zb << (pbc - 1));
        int c2 = c1 ^ hb;
        buc.push_back((c1 & hb) ? (c1 ^ rev) : c1);
        buc.push_back((c2 & hb) ? (c2 ^ rev) : c2);
    }
    if (m < pbc) {
        // projection through the coalignment map, first occurrence kept
        std::vector<int> bitmask;
        std::vector<char> Fc(pbc, 1);
        for (int j = 0; j < pbc; j++) {
            int ci = t.cmap[j];
            if (Fc[ci]) {
                Fc[ci] = 0;
                bitmask.push_back(1 << j);
            }
        }
        std::vector<char> seen((size_t)1 << bitmask.size(), 0);
        for (int b : buc) {
            int bc = 0;
            for (size_t l = 0; l < bitmask.size(); l++)
                if (b & bitmask[l]) bc |= 1 << l;
            if (!seen[bc]) {
                seen[bc] = 1;
                out.push_back(bc);
            }
        }
    } else
        out = buc;
    t.own_B = out;
}

// make_lowered_child_btable: cell_enumeration.hpp:1121-1279 (the N-D pdf's
// lowering).  The child keeps the parent cells b (in the frame of enc_lhp)
// whose neighbour across hyperplane z is a parent cell too, with bit z
// removed; the last child keeps the smaller of the two opposite keys.
static void lowered_child_btable(Term& t, int d)
{
    const int m = t.m;
    std::vector<int> out;
    if (m == d) {
        for (int i = 0; i < (1 << d) / 2; i++) out.push_back(i);
        t.own_B = out;
        return;
    }
    const std::vector<int>& Bmu = *t.encB;
    const int phc = t.phc, z = t.z;
    const int top = 1 << (phc - 1), rev = (1 << phc) - 1, mz = 1 << z;
    int lhp = t.enc_lhp;
    if (lhp & top) lhp ^= rev;
    std::vector<int> pos((size_t)1 << phc, -1);
    for (size_t j = 0; j < Bmu.size(); j++)
        if (pos[Bmu[j] ^ lhp] < 0) pos[Bmu[j] ^ lhp] = (int)j;
    std::vector<char> F(Bmu.size(), 1);
    const bool last = z == phc - 1;
    auto remove_bit = [](int b, int bit) { return ((b >> (bit + 1)) << bit) | (b & ((1 << bit) - 1)); };
    std::vector<int> buc;
    for (size_t j = 0; j < Bmu.size(); j++) {
        if (!F[j]) continue;
        const int b = Bmu[j] ^ lhp;
        int bq = b ^ mz;
        if (last) bq ^= rev;
        const int k = pos[bq];
        if (k < 0) continue;
        F[j] = 0;
        F[k] = 0;
        const int c1 = remove_bit(b, z);
        if (last) {
            const int c2 = remove_bit(bq, z);
            buc.push_back(c1 < c2 ? c1 : c2);
        } else
            buc.push_back(c1);
    }
    if (t.has_cmap) {
        // projection through the coalignment map, first occurrence kept.  The
        // reference runs j up to phc, one past the child's phc - 1 mapped rows;
        // that extra entry can only add a mask bit no key has, so the rows stop
        // at phc - 1 here
        std::vector<int> bitmask;
        std::vector<char> Fc(phc, 1);
        for (int j = 0; j < (int)t.cmap.size(); j++) {
            const int ci = t.cmap[j];
            if (Fc[ci]) {
                Fc[ci] = 0;
                bitmask.push_back(1 << j);
            }
        }
        std::vector<char> seen((size_t)1 << bitmask.size(), 0);
        for (int bb : buc) {
            int bc = 0;
            for (size_t l = 0; l < bitmask.size(); l++)
                if (bb & bitmask[l]) bc |= 1 << l;
            if (!seen[bc]) {
                seen[bc] = 1;
                out.push_back(bc);
            }
        }
    } else
        out = buc;
    t.own_B = out;
}

// Orientation mask between two equal arrangements (first component that is
// significant in both rows decides): cell_enumeration.hpp:630-640 and
// flattening.hpp:279-288.
static int orientation_mask(const double* Ai, const double* Aj, int m, int d)
{
    int s = 0;
    for (int k = 0; k < m; k++) {
        int l = 0;
        while (l < d - 1 && ((fabs(Ai[k * d + l]) < kReductionEps) || (fabs(Aj[k * d + l]) < kReductionEps))) l++;
        if (Ai[k * d + l] * Aj[k * d + l] < 0) s |= 1 << k;
    }
    return s;
}
// update_btable: cell_enumeration.hpp:584-625
static std::vector<int> reorient(const double* Ai, const std::vector<int>& Bi, const double* Aj, int n, int m, int d)
{
    int s = orientation_mask(Ai, Aj, m, d);
    if (s & (1 << (m - 1))) s ^= (1 << m) - 1;
    std::vector<int> out(Bi.begin(), Bi.begin() + n);
    if (s)
        for (auto& k : out) k ^= s;
    return out;
}

// make_gtable: flattening.hpp:77-255.  Returns true when the term is negligible.
static bool make_gtable(Term& t, const std::vector<int>& B, double gscale)
{
    const int m = t.m, phc = t.phc;
    double ps = 0;
    for (int i = 0; i < m; i++) ps += t.p[i];
    ps *= ps;
    bool negl = true;
    std::vector<std::pair<int, cplx>> kv;
    kv.reserve(B.size());
    int sb[32];
    for (int be : B) {
        double ygi = 0;
        if (t.horthog) {
            for (int k = 0; k < m; k++) {
                sb[k] = ((be >> k) & 1) ? -1 : 1;
                if (!(t.horthog & (1u << k))) ygi += t.q[k] * sb[k];
            }
        } else
            for (int k = 0; k < m; k++) {
                sb[k] = ((be >> k) & 1) ? -1 : 1;
                ygi += t.q[k] * sb[k];
            }
        int lp = 0, lm = 0;
        if (!t.is_new_child) {
            lp = be & ((1 << phc) - 1);
            lm = lp;
        } else {
            int k = 0, l = 0;
            while (k < phc) {
                if (k == t.z) {
                    lm |= 1 << k;
                    k++;
                    if (k == phc) break;
                }
                int bv = t.has_cmap ? sb[t.cmap[l]] * t.csmap[l] : sb[l];
                if (bv < 0) {
                    lp |= 1 << k;
                    lm |= 1 << k;
                }
                k++;
                l++;
            }
        }
        cplx gp = lookup_num(t.gp.get(), lp ^ t.enc_lhp, phc);
        cplx gm = lookup_num(t.gp.get(), lm ^ t.enc_lhp, phc);
        cplx v = cdiv(gp, mkc(ygi + t.d_val, t.c_val)) - cdiv(gm, mkc(ygi - t.d_val, t.c_val));
        v *= gscale;
        kv.push_back({be, v});
        if (negl && ps * hypot(__real__ v, __imag__ v) > kTermApproxEps) negl = false;  // cabs == hypot
    }
    std::stable_sort(kv.begin(), kv.end(), [](const std::pair<int, cplx>& a, const std::pair<int, cplx>& b) {
        return a.first < b.first;
    });
    t.g.keys.resize(kv.size());
    t.g.vals.resize(kv.size());
    for (size_t i = 0; i < kv.size(); i++) {
        t.g.keys[i] = kv[i].first;
        t.g.vals[i] = kv[i].second;
    }
    return negl;
}

// add_gtables: flattening.hpp:259-315
static void add_gtables(Term& ti, const std::vector<int>& Bi, const Term& tj, int d)
{
    const int m = ti.m;
    int s = orientation_mask(ti.A.data(), tj.A.data(), m, d);
    const int top = 1 << (m - 1), rev = (1 << m) - 1;
    for (int bi : Bi) {
        int bj = bi ^ s;
        bool cj = false;
        if (bj & top) {
            cj = true;
            bj ^= rev;
        }
        int ii = ti.g.find(bi), jj = tj.g.find(bj);
        if (ii >= 0 && jj >= 0) ti.g.vals[ii] += cj ? cconj(tj.g.vals[jj]) : tj.g.vals[jj];
    }
}

static void become_parent(Term& t)
{
    t.phc = t.m;
    t.gp = std::make_shared<GTable>(std::move(t.g));
    t.g = GTable();
    t.is_new_child = false;
    t.has_cmap = false;
    t.encB.reset();
    t.own_B.clear();
}

// ----------------------------------------------------------------------------
// Fast term reduction: term_reduction.hpp:159-276 (serial path).  The window
// test on every axis is the value test qp-eps < v <= qp+eps that the
// reference's sorted-axis binary searches implement.  The hyperplane check
// compares the first m entries of the row-major A arrays, as the reference
// does (it indexes Ai[k] / Aj[k] inside the per-component loop).
static void ftr(const std::vector<Term*>& T, int d, std::vector<int>& F)
{
    const int n = (int)T.size();
    F.resize(n);
    for (int i = 0; i < n; i++) F[i] = i;
    if (n == 0) return;
    const int m = T[0]->m;
    const double ep = kReductionEps;
    // index sorted along axis 0 for the candidate window
    std::vector<int> ord(n);
    for (int i = 0; i < n; i++) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return T[a]->b[0] < T[b]->b[0]; });
    std::vector<double> v0(n);
    for (int i = 0; i < n; i++) v0[i] = T[ord[i]]->b[0];
    for (int i = 0; i < n; i++) {
        if (F[i] != i) continue;
        const double* bi = T[i]->b.data();
        double lo = bi[0] - ep, hi = bi[0] + ep;
        int s = (int)(std::upper_bound(v0.begin(), v0.end(), lo) - v0.begin());
        int e = (int)(std::upper_bound(v0.begin(), v0.end(), hi) - v0.begin());
        for (int w = s; w < e; w++) {
            int j = ord[w];
            if (j <= i || F[j] != j) continue;
            const double* bj = T[j]->b.data();
            bool ok = true;
            for (int a = 1; a < d && ok; a++) {
                double l2 = bi[a] - ep, h2 = bi[a] + ep;
                if (!(bj[a] > l2 && bj[a] <= h2)) ok = false;
            }
            if (!ok) continue;
            for (int k = 0; k < m && ok; k++)
                if (fabs(T[j]->p[k] - T[i]->p[k]) > ep) ok = false;
            if (!ok) continue;
            for (int k = 0; k < m && ok; k++) {
                double r = T[i]->A[k], c = T[j]->A[k];
                if (!(fabs(r - c) < ep || fabs(r + c) < ep)) ok = false;
            }
            if (ok) F[j] = i;
        }
    }
}

// make_gtables for one shape: flattening.hpp:318-568.
static void make_gtables_shape(std::vector<Term*>& T, const std::vector<int>& F, int d, double gscale,
                               std::vector<Term*>& out, bool lowered = false)
{
    const int n = (int)T.size();
    std::vector<std::vector<int>> members(n);
    for (int j = 0; j < n; j++)
        if (F[j] != j) members[F[j]].push_back(j);
    for (int j = 0; j < n; j++) {
        if (F[j] != j) continue;
        Term* root = T[j];
        bool have_root = true;
        std::vector<int> rootB;
        if (root->is_new_child) {
            if (lowered) lowered_child_btable(*root, d);
            else new_child_btable(*root, d);
            rootB = root->own_B;
        } else
            rootB = *root->encB;
        if (make_gtable(*root, rootB, gscale)) have_root = false;
        size_t k = 0;
        const std::vector<int>& mem = members[j];
        if (!have_root) {
            // the root approximated out: the next member that survives becomes root
            std::vector<int> grpB = rootB;
            const double* Alfr = root->A.data();
            while (k < mem.size()) {
                Term* c = T[mem[k++]];
                std::vector<int> cB;
                if (c->is_new_child) {
                    grpB = reorient(Alfr, grpB, c->A.data(), (int)grpB.size(), c->m, d);
                    cB = grpB;
                } else {
                    // a parent keeps its own B; the group's cell list becomes its list
                    grpB = *c->encB;
                    cB = grpB;
                }
                if (!make_gtable(*c, cB, gscale)) {
                    root = c;
                    rootB = cB;
                    have_root = true;
                    break;
                } else
                    Alfr = c->A.data();
            }
        }
        while (k < mem.size()) {
            Term* c = T[mem[k++]];
            std::vector<int> cB;
            if (c->is_new_child)
                cB = reorient(root->A.data(), rootB, c->A.data(), (int)rootB.size(), c->m, d);
            else {
                if (c->encB->size() != rootB.size())
                    cB = reorient(root->A.data(), rootB, c->A.data(), (int)rootB.size(), c->m, d);
                else
                    cB = *c->encB;
            }
            if (!make_gtable(*c, cB, gscale)) add_gtables(*root, rootB, *c, d);
        }
        if (have_root) {
            become_parent(*root);
            out.push_back(root);
        }
    }
}

// ----------------------------------------------------------------------------
// Estimator (include/cauchy_estimator.hpp)

static void numeric_check(Estimator& E)
{
    // moments_numerical_check: cauchy_estimator.hpp:359-461
    const int d = E.d;
    const int ph = E.master_step % E.p;
    const bool first = ph == 0, not_last = ph != E.p - 1, last = ph == E.p - 1;
    if (first) {
        E.errors |= (1 << ERR_MEAN_DNE) | (1 << ERR_COV_DNE);
        E.errors &= ~((1 << ERR_MEAN_UNSTABLE_FINAL) | (1 << ERR_MEAN_UNSTABLE_NOT_FINAL) |
                      (1 << ERR_COV_UNSTABLE_NOT_FINAL) | (1 << ERR_COV_UNSTABLE_FINAL));
    }
    int ne = 0;
    if (__real__ E.fz <= 0) ne |= 1 << ERR_FZ_NEGATIVE;
    if (fabs(__imag__ E.fz / (1e-15 + __real__ E.fz)) > 1e-3) ne |= 1 << ERR_FZ_UNSTABLE;
    bool mean_ok = true;
    for (int i = 0; i < d; i++) {
        double re = fabs(__real__ E.mean[i]), im = fabs(__imag__ E.mean[i]);
        double r = im / (1e-15 + re);
        if (r > 1e-1 || im > 0.001) {
            ne |= 1 << ERR_MEAN_UNSTABLE_ANY;
            if (not_last) ne |= 1 << ERR_MEAN_UNSTABLE_NOT_FINAL;
            if (last) ne |= 1 << ERR_MEAN_UNSTABLE_FINAL;
            mean_ok = false;
        }
    }
    bool cov_ok = true;
    if (covariance_flags(E.cov.data(), d)) {
        ne |= 1 << ERR_COV_UNSTABLE_ANY;
        if (not_last) ne |= 1 << ERR_COV_UNSTABLE_NOT_FINAL;
        if (last) ne |= 1 << ERR_COV_UNSTABLE_FINAL;
        cov_ok = false;
    }
    E.errors |= ne;
    if (mean_ok) E.errors &= ~(1 << ERR_MEAN_DNE);
    if (cov_ok) E.errors &= ~(1 << ERR_COV_DNE);
    if (mean_ok) E.last_mean = E.mean;
    else E.mean = E.last_mean;
    if (cov_ok) E.last_cov = E.cov;
    else E.cov = E.last_cov;
    if (!mean_ok && !cov_ok) E.fz = E.last_fz;
    else E.last_fz = E.fz;
}

static void accumulate(Estimator& E, cplx g, const cplx* y)
{
    // cache_moments: cauchy_estimator.hpp:307-338
    const int d = E.d;
    E.fz += g;
    for (int j = 0; j < d; j++) {
        cplx yy = y[j];
        E.mean[j] += g * yy;
        for (int k = 0; k < d; k++) E.cov[j * d + k] -= g * yy * y[k];
    }
}

static void finalize_moments(Estimator& E)
{
    // finalize_cached_moments: cauchy_estimator.hpp:340-357
    const int d = E.d;
    E.gscale = kTwoPiInv / __real__ E.fz;
    cplx ifz = mkc(0, __real__ E.fz);
    for (int i = 0; i < d; i++) E.mean[i] = cdiv(E.mean[i], ifz);
    for (int i = 0; i < d; i++)
        for (int j = 0; j < d; j++) E.cov[i * d + j] = cdiv(E.cov[i * d + j], E.fz) - E.mean[i] * E.mean[j];
    E.raw_fz = E.fz;
    E.raw_mean = E.mean;
    E.raw_cov = E.cov;
    numeric_check(E);
}

// compute_moments(false) (cauchy_estimator.hpp:524-602), run after the
// tables are built when print_basic_info is set: every current term in shape
// and index order through eval_g_yei_after_ftr (cauchy_term.hpp:403-433) --
// the sign vector of the rows at the root point (0 counts as negative), the
// parent-table value there, yei = -sum p_l s_l A_l + i b -- summed as in
// cache_moments, then fz, G_SCALE_FACTOR, mean and covariance replaced.
static void post_ftr_moments(Estimator& E)
{
    const int d = E.d;
    E.fz = mkc(0, 0);
    E.mean.assign(d, mkc(0, 0));
    E.cov.assign(d * d, mkc(0, 0));
    for (const Term& t : E.terms) {
        int enc = 0;
        double ty[16] = {0};
        for (int l = 0; l < t.m; l++) {
            double s = 0.0;
            for (int j = 0; j < d; j++) s += t.A[l * d + j] * E.root[j];
            const double sg = s > 0 ? 1 : -1;
            const double sc = t.p[l] * sg;
            for (int j = 0; j < d; j++) ty[j] += sc * t.A[l * d + j];
            if (sg < 0) enc |= 1 << l;
        }
        const cplx g = lookup_num(t.gp.get(), enc, t.m);
        cplx y[16];
        for (int j = 0; j < d; j++) y[j] = mkc(-ty[j], t.b[j]);
        accumulate(E, g, y);
    }
    E.gscale = kTwoPiInv / __real__ E.fz;
    cplx ifz = mkc(0, __real__ E.fz);
    for (int i = 0; i < d; i++) E.mean[i] = cdiv(E.mean[i], ifz);
    for (int i = 0; i < d; i++)
        for (int j = 0; j < d; j++) E.cov[i * d + j] = cdiv(E.cov[i * d + j], E.fz) - E.mean[i] * E.mean[j];
}

static void reset_terms(Estimator& E)
{
    E.terms.clear();
    Term t;
    t.m = E.d;
    t.A = E.A0;
    t.p = E.p0;
    t.b = E.b0;
    E.terms.push_back(t);
    E.Nt = 1;
    E.terms_per_shape.assign(E.shape_range, 0);
    E.terms_per_shape[E.d] = 1;
    E.master_step = 0;
    E.errors = 0;
    E.post_mu_terms = 0;  // counts since the last reset, as mce_post_mu_terms does
}

// step_first: cauchy_estimator.hpp:1179-1208 with make_gtable_first flattening.hpp:14-67
static void step_first(Estimator& E, double msmt, const double* H, double gamma)
{
    const int d = E.d;
    std::vector<Term> kids;
    Term parent = E.terms[0];
    msmt_update(parent, d, kids, msmt, H, gamma, true, false);
    std::vector<Term> all;
    all.push_back(parent);
    for (auto& k : kids) all.push_back(std::move(k));
    E.fz = mkc(0, 0);
    E.mean.assign(d, mkc(0, 0));
    E.cov.assign(d * d, mkc(0, 0));
    cplx y[16];
    for (auto& t : all) {
        cplx g = eval_g_yei(t, d, E.root.data(), y, true);
        accumulate(E, g, y);
    }
    E.gscale = kTwoPiInv / __real__ E.fz;
    cplx ifz = mkc(0, __real__ E.fz);
    for (int i = 0; i < d; i++) E.mean[i] = cdiv(E.mean[i], ifz);
    for (int i = 0; i < d; i++)
        for (int j = 0; j < d; j++) E.cov[i * d + j] = cdiv(E.cov[i * d + j], E.fz) - E.mean[i] * E.mean[j];
    E.raw_fz = E.fz;
    E.raw_mean = E.mean;
    E.raw_cov = E.cov;
    const int cells = cells_central(d, d) / 2;
    for (auto& t : all) {
        t.g = GTable();
        for (int j = 0; j < cells; j++) {
            double ygi = 0;
            for (int k = 0; k < d; k++)
                if (!(t.horthog & (1u << k))) ygi += t.p[k] * (((j >> k) & 1) == 0 ? 1.0 : -1.0);
            cplx v = cdiv(mkc(1, 0), mkc(ygi + t.d_val, t.c_val)) - cdiv(mkc(1, 0), mkc(ygi - t.d_val, t.c_val));
            v *= E.gscale;
            t.g.keys.push_back(j);
            t.g.vals.push_back(v);
        }
        become_parent(t);
    }
    E.terms = std::move(all);
    E.Nt = (int)E.terms.size();
    E.terms_per_shape.assign(E.shape_range, 0);
    E.terms_per_shape[d] = E.Nt;
    E.post_mu_terms += E.Nt;
    if (E.print_basic_info) post_ftr_moments(E);
    else E.fz = mkc(1, 0);
    E.last_mean = E.mean;
    E.last_cov = E.cov;
    E.last_fz = E.fz;
}

// step_tp_to_muc (serial): cauchy_estimator.hpp:604-832, then
// fast_term_reduction_and_create_gtables: cauchy_estimator.hpp:981-1177.
static void step_rest(Estimator& E, double msmt, const double* Phi, const double* Gamma, const double* beta,
                      const double* H, double gamma, const double* B, const double* u)
{
    const int d = E.d;
    const bool with_tp = (E.master_step % E.p) == 0;
    const bool skip = E.skip_post_mu;
    double Gt[8 * 32], bt[32];
    int gcnt = 0;
    if (with_tp) gcnt = precoalign_gamma(Gamma, beta, E.pncc, d, Gt, bt);
    E.fz = mkc(0, 0);
    E.mean.assign(d, mkc(0, 0));
    E.cov.assign(d * d, mkc(0, 0));
    std::vector<Term> kids;
    std::vector<Term>& P = E.terms;
    cplx y[16];
    long long skip_children = 0;
    std::vector<int> skip_tps(E.shape_range, 0);
    for (auto& t : P) {
        if (with_tp) {
            time_prop(t, d, Phi, B, u, E.cmcc);
            tp_coalign(t, d, Gt, bt, gcnt);
            if (!skip) {
                if (t.m == t.phc) t.encB = std::make_shared<std::vector<int>>(t.gp->keys);
                else tp_enumerate(E, t);
            }
        } else if (!skip) {
            t.encB = std::make_shared<std::vector<int>>(t.gp->keys);
        }
        size_t k0 = kids.size();
        msmt_update(t, d, kids, msmt, H, gamma, false, skip);
        cplx g = eval_g_yei(t, d, E.root.data(), y, false);
        accumulate(E, g, y);
        for (size_t k = k0; k < kids.size(); k++) {
            g = eval_g_yei(kids[k], d, E.root.data(), y, false);
            accumulate(E, g, y);
        }
        if (!skip) {
            normalize_rows(t, d, true);
            t.has_cmap = false;
            for (size_t k = k0; k < kids.size(); k++) {
                int pre = kids[k].m;
                int ns = mu_coalign(kids[k], d);
                if (ns < 0) {
                    fprintf(stderr, "oracle: anti-coaligned H-orthogonal hyperplanes\n");
                    ns = kids[k].m;
                }
                kids[k].has_cmap = ns < pre;
            }
        } else {
            // the final MU keeps only the counts (cauchy_estimator.hpp:749-751, 806-812)
            const long long nk = (long long)(kids.size() - k0);
            skip_children += nk;
            skip_tps[t.m] += (int)nk + 1;
            kids.resize(k0);
        }
    }
    const long long n_after = (long long)P.size() + (long long)kids.size() + skip_children;
    finalize_moments(E);
    E.post_mu_terms += n_after;
    if (skip) {
        E.Nt = (int)n_after;
        E.terms_per_shape = skip_tps;
        return;
    }
    // regroup by shape: parents then children (cauchy_estimator.hpp:741-780)
    std::vector<std::vector<Term*>> byshape(E.shape_range);
    for (auto& t : P) byshape[t.m].push_back(&t);
    for (auto& t : kids) byshape[t.m].push_back(&t);
    std::vector<Term> next;
    std::vector<Term*> survivors;
    std::vector<int> tps(E.shape_range, 0);
    for (int m = 0; m < E.shape_range; m++) {
        if (byshape[m].empty()) continue;
        std::vector<int> F;
        ftr(byshape[m], d, F);
        std::vector<Term*> outm;
        make_gtables_shape(byshape[m], F, d, E.gscale, outm);
        tps[m] = (int)outm.size();
        for (auto* t : outm) survivors.push_back(t);
    }
    next.reserve(survivors.size());
    for (auto* t : survivors) next.push_back(std::move(*t));
    E.terms = std::move(next);
    E.Nt = (int)E.terms.size();
    E.terms_per_shape = tps;
    if (E.print_basic_info) post_ftr_moments(E);
    else E.fz = mkc(1, 0);
}

// ----------------------------------------------------------------------------
// C ABI
// ----------------------------------------------------------------------------
// Marginal 1-D conditional pdf: PointWiseNDimCauchyCPDF::evaluate_1D_marginal_cpdf
// (cpdf_ndim.hpp:1233-1352) over the current terms in shape/index order, and
// the grid of CauchyCPDFGridDispatcher1D (cpdf_ndim.hpp:2055-2139), which
// evaluates every point with caching on: the first evaluation at a master step
// and marginal index takes the exact complex formula and fills the per-term
// cache (a, b, w, s); every later one at that step and index sums
// (a x + b) / (w^2 + (x - s)^2).

// number of grid points: reset_grid (cpdf_ndim.hpp:2055-2072)
// ----------------------------------------------------------------------------
// Point-wise N-D conditional pdf: PointWiseNDimCauchyCPDF::evaluate_cpdf
// (cpdf_ndim.hpp:677-904).  The terms are lowered one spectral dimension at
// a time (construct_lowered_parent_elements :392-443, construct_lowered_children
// :520-641), each lowered child coaligned as after an MU, the children of each
// shape reduced (FTR) and given g-tables (make_gtables with
// make_lowered_child_btable, G_SCALE_FACTOR 1), and the 1-D terms left are
// integrated in closed form (evaluate_1d_cf :643-666).

// The lowered children of parent P (dimension ld) into out; xk (the point)
// on the first lowering only.
static void lower_children(const Term& P, int ld, const double* xk, std::vector<Term>& out)
{
    const int m = P.m, l1 = ld - 1;
    std::vector<double> Alp((size_t)m * l1), Ald(m), plp(m), blp(l1);
    std::vector<char> nz(m);
    int lam = 0;
    for (int i = 0; i < m; i++) {
        Ald[i] = -P.A[i * ld + ld - 1];
        nz[i] = fabs(Ald[i]) > kMuEps;
    }
    for (int i = 0; i < m; i++) {
        if (nz[i]) {
            for (int j = 0; j < l1; j++) Alp[i * l1 + j] = P.A[i * ld + j] / Ald[i];
            if (Ald[i] < 0) lam |= 1 << i;
            plp[i] = P.p[i] * fabs(Ald[i]);
        } else {
            for (int j = 0; j < l1; j++) Alp[i * l1 + j] = P.A[i * ld + j];
            plp[i] = P.p[i];
        }
    }
    double tb;
    if (xk) {
        for (int i = 0; i < l1; i++) blp[i] = P.b[i] - xk[i];
        tb = P.b[l1] - xk[l1];
    } else {
        for (int i = 0; i < l1; i++) blp[i] = P.b[i];
        tb = P.b[l1];
    }
    auto keys = std::make_shared<std::vector<int>>(P.gp->keys);
    for (int t = 0; t < m; t++) {
        if (!nz[t]) continue;
        Term c;
        c.m = m - 1;
        c.A.assign((size_t)(m - 1) * l1, 0.0);
        c.p.assign(m - 1, 0.0);
        c.b.assign(l1, 0.0);
        const double* mu_t = Alp.data() + t * l1;
        int l_ = 0;
        unsigned unint = 0;
        for (int l = 0; l < m; l++) {
            if (l == t) continue;
            const double* mu_l = Alp.data() + l * l1;
            double* row = c.A.data() + l_ * l1;
            if (nz[l]) {
                for (int j = 0; j < l1; j++) row[j] = mu_l[j] - mu_t[j];
            } else {
                for (int j = 0; j < l1; j++) row[j] = mu_l[j];
                unint |= 1u << l_;
            }
            c.p[l_] = plp[l];
            l_++;
        }
        for (int j = 0; j < l1; j++) c.b[j] = blp[j] + tb * mu_t[j];
        c.c_val = tb;
        c.d_val = plp[t];
        c.z = t;
        c.horthog = unint;
        c.is_new_child = true;
        c.enc_lhp = lam;
        c.gp = P.gp;
        c.encB = keys;
        c.phc = m;
        c.pbc = m;
        out.push_back(std::move(c));
    }
}

// Returns 0 and the complex value, or -1 before the first step / with
// moment errors (the reference asserts), -3 when a lowered child
// anti-coaligns two unintegrable rows (the reference exits).
static int cpdf_nd_eval(Estimator& E, const double* xk, cplx* out, bool reduce = true)
{
    if (E.master_step < 1 || E.errors) return -1;
    const int dim = E.d;
    int top = 0;
    for (int i = 0; i < E.shape_range; i++)
        if (E.terms_per_shape[i] > 0) top = i;
    int shape_range = top + 1;
    // parents by shape, in term order
    std::vector<std::vector<Term>> par(shape_range);
    for (const Term& t : E.terms)
        if (t.m < shape_range) par[t.m].push_back(t);
    for (int d = dim; d > 1; d--) {
        const int dl = d - 1;
        std::vector<Term> kids;
        for (int m = d; m < shape_range; m++)
            for (const Term& P : par[m]) {
                const size_t k0 = kids.size();
                lower_children(P, d, d == dim ? xk : nullptr, kids);
                for (size_t k = k0; k < kids.size(); k++) {
                    const int pre = kids[k].m;
                    const int ns = mu_coalign(kids[k], dl);
                    if (ns < 0) return -3;
                    kids[k].has_cmap = ns < pre;
                }
            }
        std::vector<std::vector<Term*>> byshape(shape_range);
        for (Term& c : kids) byshape[c.m].push_back(&c);
        std::vector<std::vector<Term>> next(shape_range);
        for (int m = 0; m < shape_range; m++) {
            if (byshape[m].empty() || m < dl) continue;
            std::vector<int> F;
            if (reduce) ftr(byshape[m], dl, F);
            else
                for (size_t i = 0; i < byshape[m].size(); i++) F.push_back((int)i);
            std::vector<Term*> roots;
            make_gtables_shape(byshape[m], F, dl, 1.0, roots, true);
            for (Term* r : roots) next[m].push_back(std::move(*r));
        }
        par.swap(next);
        shape_range -= 1;
    }
    cplx f = mkc(0, 0);
    if (shape_range > 1)
        for (const Term& t : par[1]) {
            const int lp = t.A[0] > 0 ? 1 : 0, lm = t.A[0] > 0 ? 0 : 1;
            const cplx gp = lookup_num(t.gp.get(), lp, 1);
            const cplx gm = lookup_num(t.gp.get(), lm, 1);
            f += cdiv(gp, mkc(t.p[0], t.b[0])) - cdiv(gm, mkc(-t.p[0], t.b[0]));
        }
    // unnormalized_f_x / norm_factor * pow(RECIPRICAL_TWO_PI, dim)
    const double nf = __real__ E.fz;
    f = mkc(__real__ f / nf, __imag__ f / nf);
    const double s = pow(kTwoPiInv, dim);
    *out = mkc(__real__ f * s, __imag__ f * s);
    return 0;
}

// PointWiseNDimCauchyCPDF::evaluate_marginal_cpdf (cpdf_ndim.hpp:918-1230):
// the marginal pdf of the states idx[0..nm) (ascending, 0 < nm < d) at
// xm[nm].  Every term's A columns and b are reordered so that the states
// integrated out come first and the kept states last, b less the point at
// the kept states (construct_lowered_marginal_parent_elements :445-517); nm
// lowerings as in evaluate_cpdf; then every term of the d - nm dimensions
// left is looked up at the sign vector of A nu_bar (:1180-1212); the sum
// / Re fz * (2 pi)^-nm.  Returns as cpdf_nd_eval.
static int cpdf_marginal_eval(Estimator& E, const double* xm, const int* idx, int nm, const double* nu_bar,
                              cplx* out, bool reduce = true)
{
    if (E.master_step < 1 || E.errors) return -1;
    const int dim = E.d, nz = dim - nm;
    if (nm < 1 || nm >= dim) return -2;
    std::vector<int> reo(dim);
    std::vector<char> F(dim, 1);
    for (int i = 0; i < nm; i++) {
        reo[nz + i] = idx[i];
        F[idx[i]] = 0;
    }
    for (int i = 0, c = 0; i < dim; i++)
        if (F[i]) reo[c++] = i;
    int top = 0;
    for (int i = 0; i < E.shape_range; i++)
        if (E.terms_per_shape[i] > 0) top = i;
    int shape_range = top + 1;
    std::vector<std::vector<Term>> par(shape_range);
    for (const Term& t : E.terms) {
        if (t.m >= shape_range) continue;
        Term r = t;
        std::vector<double> tb(t.b);
        for (int i = 0; i < nm; i++) tb[reo[nz + i]] -= xm[i];
        for (int i = 0; i < t.m; i++)
            for (int j = 0; j < dim; j++) r.A[i * dim + j] = t.A[i * dim + reo[j]];
        for (int j = 0; j < dim; j++) r.b[j] = tb[reo[j]];
        par[t.m].push_back(std::move(r));
    }
    for (int d = dim; d > nz; d--) {
        const int dl = d - 1;
        std::vector<Term> kids;
        for (int m = d; m < shape_range; m++)
            for (const Term& P : par[m]) {
                const size_t k0 = kids.size();
                lower_children(P, d, nullptr, kids);
                for (size_t k = k0; k < kids.size(); k++) {
                    const int pre = kids[k].m;
                    const int ns = mu_coalign(kids[k], dl);
                    if (ns < 0) return -3;
                    kids[k].has_cmap = ns < pre;
                }
            }
        std::vector<std::vector<Term*>> byshape(shape_range);
        for (Term& c : kids) byshape[c.m].push_back(&c);
        std::vector<std::vector<Term>> next(shape_range);
        for (int m = 0; m < shape_range; m++) {
            if (byshape[m].empty() || m < dl) continue;
            std::vector<int> Fr;
            if (reduce) ftr(byshape[m], dl, Fr);
            else
                for (size_t i = 0; i < byshape[m].size(); i++) Fr.push_back((int)i);
            std::vector<Term*> roots;
            make_gtables_shape(byshape[m], Fr, dl, 1.0, roots, true);
            for (Term* r : roots) next[m].push_back(std::move(*r));
        }
        par.swap(next);
        shape_range -= 1;
    }
    cplx f = mkc(0, 0);
    for (int m = nz; m < shape_range; m++)
        for (const Term& t : par[m]) {
            int enc = 0;
            for (int k = 0; k < m; k++) {
                double w = 0;
                for (int j = 0; j < nz; j++) w += t.A[k * nz + j] * nu_bar[j];
                if (w < 0) enc |= 1 << k;
            }
            f += lookup_num(t.gp.get(), enc, m);
        }
    const double nf = __real__ E.fz;
    f = mkc(__real__ f / nf, __imag__ f / nf);
    const double s = pow(kTwoPiInv, nm);
    *out = mkc(__real__ f * s, __imag__ f * s);
    return 0;
}

static int cpdf_grid_points(double low, double high, double res)
{
    return (int)((high - low + res - 1e-15) / res) + 1;
}

static double cpdf1d_eval(Estimator& E, int marg, double x, const double* bar_nu)
{
    const int d = E.d;
    const bool use_cache = E.cpdf1d_step == E.master_step && E.cpdf1d_marg == marg;
    double fx = 0;
    if (use_cache) {
        for (const Cpdf1DTerm& c : E.cpdf1d_cache) {
            const double w2 = c.w * c.w;
            double xms = x - c.s;
            xms *= xms;
            fx += (c.a * x + c.b) / (w2 + xms);
        }
        return fx / __real__ E.fz;
    }
    E.cpdf1d_step = E.master_step;
    E.cpdf1d_marg = marg;
    E.cpdf1d_cache.clear();
    for (const Term& T : E.terms) {
        const int m = T.m;
        const double b_c = T.b[marg] - x;
        double p_cc = 0;
        int lhs = 0, rhs = 0;
        for (int j = 0; j < m; j++) {
            const double a_cj = T.A[j * d + marg];
            const double fa = fabs(a_cj);
            p_cc += T.p[j] * fa;
            bool left;
            if (fa > 1e-15) {
                left = a_cj > 0;
            } else {
                double ip = 0.0;  // dot_prod, cauchy_linalg.hpp:559-565
                for (int l = 0; l < d; l++) ip += T.A[j * d + l] * bar_nu[l];
                left = ip > 0;
            }
            if (left) lhs |= 1 << j;
            else rhs |= 1 << j;
        }
        const cplx gl = lookup_num(T.gp.get(), lhs, m);
        const cplx gr = lookup_num(T.gp.get(), rhs, m);
        const cplx g = cdiv(gl, mkc(p_cc, b_c)) - cdiv(gr, mkc(-p_cc, b_c));
        fx += __real__ g;
        Cpdf1DTerm c;
        c.s = T.b[marg];
        c.w = p_cc;
        c.a = __imag__ gr / M_PI;
        c.b = (__real__ gr * c.w - __imag__ gr * c.s) / M_PI;
        E.cpdf1d_cache.push_back(c);
    }
    return fx * kTwoPiInv / __real__ E.fz;
}

// ----------------------------------------------------------------------------
// Marginal 2-D conditional pdf: PointWiseNDimCauchyCPDF::evaluate_2D_marginal_cpdf
// (cpdf_ndim.hpp:1356-1455) with marg2d_eval_term_for_cpdf (:1474-1658), the
// cached evaluation (:1660-1748) and the helpers marg2d_extract_2D_HPA,
// marg2d_remove_zeros_and_coalign, marg2d_get_cell_wall_angles and
// marg2d_get_SVs (:31-203); the grid of CauchyCPDFGridDispatcher2D
// (:1816-1919).  Per term: the two marginal columns of A, normalised and
// coaligned; the 2m cell-wall angles; each of the m half-plane cells'
// sign vector (at its mid angle), g value and closed-form integral.

static const double kIntegralGammaEps = 1e-8;  // INTEGRAL_GAMMA_EPS
static const int kZeroHpMarker = 32;           // ZERO_HP_MARKER_VALUE

// the integral of one cell; returns false on the reference's singularity exit
static bool marg2d_cell(double sin_t1, double cos_t1, double sin_t2, double cos_t2, double g1r, double g1i,
                        double g2r, double g2i, bool check_gamma1, cplx g, double* out)
{
    cplx gamma1 = mkc(g1r, g1i), gamma2 = mkc(g2r, g2i);
    bool fast = true;
    if (check_gamma1 && fabs(g1r) < kIntegralGammaEps) {
        fast = false;
        if (fabs(g2r) < kIntegralGammaEps && fabs(g2i) < kIntegralGammaEps) return false;
    }
    cplx lo, hi, cell;
    if (fast) {
        gamma2 *= gamma1;
        gamma1 *= gamma1;
        lo = cdiv(mkc(sin_t1, 0), gamma1 * cos_t1 + gamma2 * sin_t1);
        hi = cdiv(mkc(sin_t2, 0), gamma1 * cos_t2 + gamma2 * sin_t2);
        cell = hi - lo;
        cell *= g;
    } else {
        lo = cdiv(gamma1 * sin_t1 - gamma2 * cos_t1, gamma1 * cos_t1 + gamma2 * sin_t1);
        hi = cdiv(gamma1 * sin_t2 - gamma2 * cos_t2, gamma1 * cos_t2 + gamma2 * sin_t2);
        cell = hi - lo;
        gamma1 *= gamma1;
        gamma2 *= gamma2;
        cell *= cdiv(g, gamma1 + gamma2);
    }
    *out = __real__ cell;
    return true;
}

static double cpdf2d_eval(Estimator& E, int i1, int i2, double x1, double x2, const double* bar_nu, int* err)
{
    const int d = E.d;
    const bool use_cache = E.cpdf2d_step == E.master_step && E.cpdf2d_m1 == i1 && E.cpdf2d_m2 == i2;
    double fx = 0;
    if (use_cache) {
        for (const Cpdf2DTerm& c : E.cpdf2d_cache) {
            const double g1i = c.b[0] - x1, g2i = c.b[1] - x2;
            const bool check = fabs(g1i) < kIntegralGammaEps;
            double t = 0;
            for (int i = 0; i < c.m; i++) {
                double v;
                if (!marg2d_cell(c.sin_t[i], c.cos_t[i], c.sin_t[i + 1], c.cos_t[i + 1], c.g1r[i], g1i, c.g2r[i], g2i,
                                 check, c.g[i], &v)) {
                    *err = 1;
                    v = 0;
                }
                t += v;
            }
            fx += t;
        }
        return 2 * fx * kTwoPiInv * kTwoPiInv / __real__ E.fz;
    }
    E.cpdf2d_step = E.master_step;
    E.cpdf2d_m1 = i1;
    E.cpdf2d_m2 = i2;
    E.cpdf2d_cache.clear();
    for (const Term& T : E.terms) {
        const int m = T.m;
        // marg2d_extract_2D_HPA
        double A[2 * 32], p[32], A2[2 * 32], p2[32], b[2];
        int cmap[32], csmap[32], fidx[32];
        bool F[32];
        for (int i = 0; i < m; i++) {
            A[2 * i] = T.A[i * d + i1];
            A[2 * i + 1] = T.A[i * d + i2];
            p[i] = T.p[i];
            F[i] = true;
        }
        b[0] = T.b[i1];
        b[1] = T.b[i2];
        // marg2d_remove_zeros_and_coalign
        for (int i = 0; i < m; i++) {
            const double f0 = fabs(A[2 * i]), f1 = fabs(A[2 * i + 1]);
            if (f0 < kMuEps && f1 < kMuEps) {
                cmap[i] = csmap[i] = fidx[i] = kZeroHpMarker;
                F[i] = false;
                continue;
            }
            const double s = f0 + f1;
            A[2 * i] /= s;
            A[2 * i + 1] /= s;
            p[i] *= s;
        }
        int mu = 0;
        for (int i = 0; i < m; i++) {
            if (!F[i]) continue;
            cmap[i] = mu;
            csmap[i] = 1;
            fidx[i] = i;
            p2[mu] = p[i];
            for (int j = i + 1; j < m; j++) {
                if (!F[j]) continue;
                if (fabs(A[2 * i] - A[2 * j]) < kCoalignEps && fabs(A[2 * i + 1] - A[2 * j + 1]) < kCoalignEps) {
                    cmap[j] = mu;
                    csmap[j] = 1;
                    F[j] = false;
                    fidx[j] = i;
                    p2[mu] += p[j];
                    continue;
                }
                if (fabs(A[2 * i] + A[2 * j]) < kCoalignEps && fabs(A[2 * i + 1] + A[2 * j + 1]) < kCoalignEps) {
                    cmap[j] = mu;
                    csmap[j] = -1;
                    F[j] = false;
                    fidx[j] = i;
                    p2[mu] += p[j];
                }
            }
            mu++;
        }
        const int mn = mu;
        if (mn < m) {
            int u = 0;
            for (int i = 0; i < m; i++)
                if (fidx[i] == i) {
                    A2[2 * u] = A[2 * i];
                    A2[2 * u + 1] = A[2 * i + 1];
                    u++;
                }
        } else {
            memcpy(A2, A, sizeof(double) * 2 * m);
        }
        // marg2d_get_cell_wall_angles
        double th[64];
        for (int i = 0; i < mn; i++) {
            const double* a = A2 + 2 * i;
            double pt0, pt1;
            if (fabs(a[0]) < fabs(a[1])) {
                pt0 = 1;
                pt1 = -a[0] / a[1];
            } else {
                pt0 = -a[1] / a[0];
                pt1 = 1;
            }
            double t1 = atan2(pt1, pt0);
            if (t1 < 0) t1 += M_PI;
            th[2 * i] = t1;
            th[2 * i + 1] = t1 + M_PI;
        }
        std::sort(th, th + 2 * mn);
        // cells
        Cpdf2DTerm c;
        c.m = mn;
        c.b[0] = b[0];
        c.b[1] = b[1];
        const double g1i = b[0] - x1, g2i = b[1] - x2;
        const bool check = fabs(g1i) < kIntegralGammaEps;
        double t = 0, s2 = 0, c2 = 0;
        for (int i = 0; i < mn; i++) {
            // marg2d_get_SVs: the signs at the cell's mid angle
            const double tm = (th[i + 1] + th[i]) / 2.0;
            const double ct = cos(tm), st = sin(tm);
            double sv[32];
            for (int j = 0; j < mn; j++) sv[j] = (A2[2 * j] * ct + A2[2 * j + 1] * st > 0) ? 1 : -1;
            int enc = 0;
            if (mn == m) {
                for (int j = 0; j < m; j++)
                    if (sv[j] < 0) enc |= 1 << j;
            } else {
                for (int j = 0; j < m; j++) {
                    if (cmap[j] == kZeroHpMarker) {
                        double ip = 0.0;
                        for (int l = 0; l < d; l++) ip += T.A[j * d + l] * bar_nu[l];
                        if (ip < 0) enc |= 1 << j;
                    } else {
                        const int s = (int)(sv[cmap[j]] * csmap[j]);
                        if (s < 0) enc |= 1 << j;
                    }
                }
            }
            const cplx g = lookup_num(T.gp.get(), enc, m);
            double g1r = 0, g2r = 0;
            for (int j = 0; j < mn; j++) {
                g1r -= (A2[2 * j] * p2[j]) * sv[j];
                g2r -= (A2[2 * j + 1] * p2[j]) * sv[j];
            }
            const double t1 = th[i], t2 = th[i + 1];
            const double s1 = sin(t1), c1 = cos(t1);
            s2 = sin(t2);
            c2 = cos(t2);
            c.sin_t.push_back(s1);
            c.cos_t.push_back(c1);
            c.g1r.push_back(g1r);
            c.g2r.push_back(g2r);
            c.g.push_back(g);
            double v;
            if (!marg2d_cell(s1, c1, s2, c2, g1r, g1i, g2r, g2i, check, g, &v)) {
                *err = 1;
                v = 0;
            }
            t += v;
        }
        c.sin_t.push_back(s2);
        c.cos_t.push_back(c2);
        E.cpdf2d_cache.push_back(std::move(c));
        fx += t;
    }
    return 2 * fx * kTwoPiInv * kTwoPiInv / __real__ E.fz;
}

// ----------------------------------------------------------------------------
// Relative-then-transformed system of two estimators
// (include/cauchy_prediction.hpp).  rel = secondary - primary, projected by
// the 2 x d matrix Trel.  Every (primary term, secondary term) pair becomes
// one 2-D term: A_rel = [-A_prim; A_sec], p_rel = [p_prim; p_sec],
// b_rel = b_sec - b_prim (:573-584), A_2d = A_rel Trel^T, b_2d = Trel b_rel
// (:587-588), then marg2d_remove_zeros_and_coalign (cpdf_ndim.hpp:42-138).
// Pairs run over primary shapes, secondary shapes, primary terms, secondary
// terms (:789-800, the single-thread order).

struct RelSys {
    int full = 0;
    std::vector<Cpdf2DTerm> terms;
    long long total = 0, approxed_out = 0;
};

static double rel_sgn(double x) { return (double)((x > 0) - (x < 0)); }

// one pair; returns false on the reference's singular-cell exit (never here:
// caching evaluates no integral) -- the moments go into acc[7] when given
static void rel2d_pair(const Term& P, const Term& S, int d, const double* Trel, const double* bar_nu_full,
                       const double* bar_nu, int full, cplx* acc, Cpdf2DTerm& c)
{
    const int mp = P.m, ms = S.m, mps = mp + ms;
    double Arel[32 * 8], prel[32], brel[8], A2[2 * 32], b2[2], Ac[2 * 32], pc[32];
    int cmap[32], csmap[32], fidx[32];
    bool F[32];
    for (int i = 0; i < d; i++) brel[i] = S.b[i] - P.b[i];
    for (int i = 0; i < mp * d; i++) Arel[i] = P.A[i] * -1;
    for (int i = 0; i < ms * d; i++) Arel[mp * d + i] = S.A[i];
    for (int i = 0; i < mp; i++) prel[i] = P.p[i];
    for (int i = 0; i < ms; i++) prel[mp + i] = S.p[i];
    // matmatmul(A_rel, Trel, A_2d, mps, d, 2, d, false, true) (cauchy_linalg.hpp:352-367)
    for (int i = 0; i < mps; i++)
        for (int j = 0; j < 2; j++) {
            double s = 0.0;
            for (int k = 0; k < d; k++) s += Arel[i * d + k] * Trel[j * d + k];
            A2[i * 2 + j] = s;
        }
    for (int i = 0; i < 2; i++) {
        double s = 0.0;
        for (int j = 0; j < d; j++) s += Trel[i * d + j] * brel[j];
        b2[i] = s;
    }
    // marg2d_remove_zeros_and_coalign: A2 and prel are normalised in place
    for (int i = 0; i < mps; i++) {
        F[i] = true;
        const double f0 = fabs(A2[2 * i]), f1 = fabs(A2[2 * i + 1]);
        if (f0 < kMuEps && f1 < kMuEps) {
            cmap[i] = csmap[i] = fidx[i] = kZeroHpMarker;
            F[i] = false;
            continue;
        }
        const double s = f0 + f1;
        A2[2 * i] /= s;
        A2[2 * i + 1] /= s;
        prel[i] *= s;
    }
    int mn = 0;
    for (int i = 0; i < mps; i++) {
        if (!F[i]) continue;
        cmap[i] = mn;
        csmap[i] = 1;
        fidx[i] = i;
        pc[mn] = prel[i];
        for (int j = i + 1; j < mps; j++) {
            if (!F[j]) continue;
            if (fabs(A2[2 * i] - A2[2 * j]) < kCoalignEps && fabs(A2[2 * i + 1] - A2[2 * j + 1]) < kCoalignEps) {
                cmap[j] = mn;
                csmap[j] = 1;
                F[j] = false;
                fidx[j] = i;
                pc[mn] += prel[j];
                continue;
            }
            if (fabs(A2[2 * i] + A2[2 * j]) < kCoalignEps && fabs(A2[2 * i + 1] + A2[2 * j + 1]) < kCoalignEps) {
                cmap[j] = mn;
                csmap[j] = -1;
                F[j] = false;
                fidx[j] = i;
                pc[mn] += prel[j];
            }
        }
        mn++;
    }
    {
        int u = 0;
        for (int i = 0; i < mps; i++)
            if (mn == mps || fidx[i] == i) {
                Ac[2 * u] = A2[2 * i];
                Ac[2 * u + 1] = A2[2 * i + 1];
                u++;
            }
    }
    // eval_rel_sys_moments_for_term (cauchy_prediction.hpp:207-285), on the
    // normalised, un-coalesced rows; zero rows take the sign of the full row
    if (acc) {
        double ty[2] = {0, 0};
        int encp = 0, encs = 0;
        for (int i = 0; i < mps; i++) {
            double v;
            if (cmap[i] != kZeroHpMarker) v = A2[2 * i] * bar_nu[0] + A2[2 * i + 1] * bar_nu[1];
            else {
                v = 0.0;
                for (int l = 0; l < d; l++) v += Arel[i * d + l] * bar_nu_full[l];
            }
            const double s = rel_sgn(v);
            const double sc = prel[i] * s;
            ty[0] += sc * A2[2 * i];
            ty[1] += sc * A2[2 * i + 1];
            if (s < 0) {
                if (i < mp) encp |= 1 << i;
                else encs |= 1 << (i - mp);
            }
        }
        const cplx g = lookup_num(P.gp.get(), encp, mp) * lookup_num(S.gp.get(), encs, ms);
        const cplx y[2] = {mkc(-ty[0], b2[0]), mkc(-ty[1], b2[1])};
        acc[0] += g;
        for (int j = 0; j < 2; j++) {
            acc[1 + j] += g * y[j];
            for (int k = 0; k < 2; k++) acc[3 + j * 2 + k] -= g * y[j] * y[k];
        }
    }
    // cache_rel_marg2d_term_for_cpdf (cauchy_prediction.hpp:306-443)
    double th[2 * 32 + 1];
    for (int i = 0; i < mn; i++) {
        const double* a = Ac + 2 * i;
        double pt0, pt1;
        if (fabs(a[0]) < fabs(a[1])) {
            pt0 = 1;
            pt1 = -a[0] / a[1];
        } else {
            pt0 = -a[1] / a[0];
            pt1 = 1;
        }
        double t1 = atan2(pt1, pt0);
        if (t1 < 0) t1 += M_PI;
        th[2 * i] = t1;
        th[2 * i + 1] = t1 + M_PI;
    }
    std::sort(th, th + 2 * mn);
    if (full && mn > 0) th[2 * mn] = th[0] + 2 * M_PI;
    const int cells = mn * (1 + full);
    c.m = mn;
    c.b[0] = b2[0];
    c.b[1] = b2[1];
    c.sin_t.clear();
    c.cos_t.clear();
    c.g1r.clear();
    c.g2r.clear();
    c.g.clear();
    const int maskp = (1 << mp) - 1;
    for (int i = 0; i < cells; i++) {
        // marg2d_get_SVs: the half at the mid angles, the other half flipped
        const int h = i < mn ? i : i - mn;
        const double tm = (th[h + 1] + th[h]) / 2.0;
        const double ct = cos(tm), st = sin(tm);
        double sv[32];
        for (int j = 0; j < mn; j++) {
            sv[j] = (Ac[2 * j] * ct + Ac[2 * j + 1] * st > 0) ? 1 : -1;
            if (i >= mn) sv[j] = -1 * sv[j];
        }
        int enc = 0;
        for (int j = 0; j < mps; j++) {
            if (cmap[j] == kZeroHpMarker) {
                double ip = 0.0;
                for (int l = 0; l < d; l++) ip += Arel[j * d + l] * bar_nu_full[l];
                if (ip < 0) enc |= 1 << j;
            } else {
                const int s = (int)(sv[cmap[j]] * csmap[j]);
                if (s < 0) enc |= 1 << j;
            }
        }
        const cplx g = lookup_num(P.gp.get(), enc & maskp, mp) * lookup_num(S.gp.get(), enc >> mp, ms);
        double g1r = 0, g2r = 0;
        for (int j = 0; j < mn; j++) {
            g1r -= (Ac[2 * j] * pc[j]) * sv[j];
            g2r -= (Ac[2 * j + 1] * pc[j]) * sv[j];
        }
        c.sin_t.push_back(sin(th[i]));
        c.cos_t.push_back(cos(th[i]));
        c.g1r.push_back(g1r);
        c.g2r.push_back(g2r);
        c.g.push_back(g);
    }
    c.sin_t.push_back(cells > 0 ? sin(th[cells]) : 0.0);
    c.cos_t.push_back(cells > 0 ? cos(th[cells]) : 0.0);
}

// approx_out_rel_marg2d_term_for_cpdf (cauchy_prediction.hpp:445-470)
static bool rel2d_negligible(const Cpdf2DTerm& c, double norm_fact, double eps)
{
    double total = 0;
    for (int i = 0; i < c.m; i++) {
        const double a1 = c.g1r[i], a2 = c.g2r[i];
        const double c1 = c.cos_t[i], s1 = c.sin_t[i], c2 = c.cos_t[i + 1], s2 = c.sin_t[i + 1];
        const double den1 = a1 * (a1 * c1 + a2 * s1);
        const double den2 = a1 * (a1 * c2 + a2 * s2);
        if (fabs(den1) < 1e-14) return false;
        if (fabs(den2) < 1e-14) return false;
        const double gr = hypot(__real__ c.g[i], __imag__ c.g[i]);
        total += fabs((gr * s2) / den2) + fabs((gr * s1) / den1);
    }
    total *= (2 * norm_fact);
    return fabs(total) < eps;
}

extern "C" {

void* orc_create(const double* A0, const double* p0, const double* b0, int steps, int d, int cmcc, int pncc,
                 int p, const double* root_point, const double* b_pert)
{
    Estimator* E = new Estimator();
    E->d = d;
    E->cmcc = cmcc;
    E->pncc = pncc;
    E->p = p;
    E->num_steps = p * steps;
    int max_shape = d > 1 ? (steps - 1) * pncc + d : d + pncc;
    E->shape_range = max_shape + 1;
    E->A0.assign(A0, A0 + d * d);
    E->p0.assign(p0, p0 + d);
    E->b0.assign(b0, b0 + d);
    E->root.assign(root_point, root_point + d);
    E->bpert.assign(b_pert, b_pert + max_shape);
    E->combos.resize(E->shape_range);
    for (int m = d + 1; m < E->shape_range; m++) lex_combos(m, d, E->combos[m]);
    E->mean.assign(d, mkc(0, 0));
    E->cov.assign(d * d, mkc(0, 0));
    E->last_mean = E->mean;
    E->last_cov = E->cov;
    E->fz = E->last_fz = mkc(0, 0);
    reset_terms(*E);
    return E;
}

void orc_destroy(void* h) { delete (Estimator*)h; }

int orc_step(void* h, double msmt, const double* Phi, const double* Gamma, const double* beta, const double* H,
             double gamma, const double* B, const double* u)
{
    Estimator& E = *(Estimator*)h;
    if (E.errors & (1 << ERR_FZ_NEGATIVE)) return E.errors;
    if (E.master_step == E.num_steps) return -1;
    E.skip_post_mu = E.master_step == E.num_steps - 1;
    if (E.master_step == 0) step_first(E, msmt, H, gamma);
    else step_rest(E, msmt, Phi, Gamma, beta, H, gamma, B, u);
    E.master_step++;
    return E.errors;
}

// reset (cauchy_estimator.hpp:1247), reinitialize_start_statistics (:1302),
// and the master_step setter the window manager uses (pycauchy.hpp:767).
void orc_reset(void* h) { reset_terms(*(Estimator*)h); }
void orc_reinit(void* h, const double* A0, const double* p0, const double* b0)
{
    Estimator& E = *(Estimator*)h;
    E.A0.assign(A0, A0 + E.d * E.d);
    E.p0.assign(p0, p0 + E.d);
    E.b0.assign(b0, b0 + E.d);
}
void orc_set_master_step(void* h, int ms) { ((Estimator*)h)->master_step = ms; }
// print_basic_info of the constructor (cauchy_estimator.hpp:87, 165): the
// moments reported after each table build come from compute_moments(false)
void orc_set_print_basic_info(void* h, int on) { ((Estimator*)h)->print_basic_info = on != 0; }
int orc_errors(void* h) { return ((Estimator*)h)->errors; }

int orc_num_terms(void* h) { return ((Estimator*)h)->Nt; }
long long orc_post_mu_terms(void* h) { return ((Estimator*)h)->post_mu_terms; }
int orc_shape_range(void* h) { return ((Estimator*)h)->shape_range; }
void orc_terms_per_shape(void* h, int* out)
{
    Estimator& E = *(Estimator*)h;
    for (int i = 0; i < E.shape_range; i++) out[i] = E.terms_per_shape[i];
}

void orc_get_moments(void* h, double* fz, double* mean, double* cov, double* raw_fz, double* raw_mean,
                     double* raw_cov, double* gscale)
{
    Estimator& E = *(Estimator*)h;
    const int d = E.d;
    fz[0] = __real__ E.fz;
    fz[1] = __imag__ E.fz;
    raw_fz[0] = __real__ E.raw_fz;
    raw_fz[1] = __imag__ E.raw_fz;
    for (int i = 0; i < d; i++) {
        mean[2 * i] = __real__ E.mean[i];
        mean[2 * i + 1] = __imag__ E.mean[i];
        raw_mean[2 * i] = __real__ E.raw_mean[i];
        raw_mean[2 * i + 1] = __imag__ E.raw_mean[i];
    }
    for (int i = 0; i < d * d; i++) {
        cov[2 * i] = __real__ E.cov[i];
        cov[2 * i + 1] = __imag__ E.cov[i];
        raw_cov[2 * i] = __real__ E.raw_cov[i];
        raw_cov[2 * i + 1] = __imag__ E.raw_cov[i];
    }
    *gscale = E.gscale;
}

long long orc_total_cells(void* h)
{
    Estimator& E = *(Estimator*)h;
    long long s = 0;
    for (auto& t : E.terms) s += t.gp ? (long long)t.gp->keys.size() : 0;
    return s;
}

void orc_dump_terms(void* h, int* shape, double* A, double* p, double* b, int* cells, int* keys, double* gvals)
{
    Estimator& E = *(Estimator*)h;
    const int d = E.d, M = E.shape_range - 1;
    long long c = 0;
    for (size_t t = 0; t < E.terms.size(); t++) {
        const Term& T = E.terms[t];
        shape[t] = T.m;
        memset(A + t * M * d, 0, sizeof(double) * M * d);
        memset(p + t * M, 0, sizeof(double) * M);
        memcpy(A + t * M * d, T.A.data(), sizeof(double) * T.m * d);
        memcpy(p + t * M, T.p.data(), sizeof(double) * T.m);
        memcpy(b + t * d, T.b.data(), sizeof(double) * d);
        int nc = T.gp ? (int)T.gp->keys.size() : 0;
        cells[t] = nc;
        for (int k = 0; k < nc; k++) {
            keys[c] = T.gp->keys[k];
            gvals[2 * c] = __real__ T.gp->vals[k];
            gvals[2 * c + 1] = __imag__ T.gp->vals[k];
            c++;
        }
    }
}

// Extended (nonlinear) mode helpers, cauchy_estimator.hpp:1312-1394.
// shift_cf_by_bias: every term's b += bias, unless the last update was the
// final MU (whose terms are not kept).
void orc_shift_cf_by_bias(void* h, const double* bias)
{
    Estimator& E = *(Estimator*)h;
    if (E.skip_post_mu) return;
    for (Term& T : E.terms)
        for (int j = 0; j < E.d; j++) T.b[j] += bias[j];
}

// deterministic_time_prop: time_prop of every term with (Phi) or (Phi, B, u).
void orc_deterministic_time_prop(void* h, const double* Phi, const double* B, const double* u)
{
    Estimator& E = *(Estimator*)h;
    const int cm = (B && u) ? E.cmcc : 0;
    for (Term& T : E.terms) time_prop(T, E.d, Phi, B, u, cm);
}

// finalize_extended_moments: every term's b -= Re(mean) (not after the final
// MU), then mean += x_bar and x_bar = Re(mean).
void orc_finalize_extended_moments(void* h, double* x_bar)
{
    Estimator& E = *(Estimator*)h;
    const int d = E.d;
    if (!E.skip_post_mu) {
        std::vector<double> dx(d);
        for (int i = 0; i < d; i++) dx[i] = __real__ E.mean[i];
        for (Term& T : E.terms)
            for (int j = 0; j < d; j++) T.b[j] -= dx[j];
    }
    for (int i = 0; i < d; i++) __real__ E.mean[i] += x_bar[i];
    for (int i = 0; i < d; i++) x_bar[i] = __real__ E.mean[i];
}

// Marginal 1-D pdf grid: CauchyCPDFGridDispatcher1D::reset_grid and
// evaluate_point_grid (cpdf_ndim.hpp:2055-2139).  Returns the point count, -2
// if it exceeds max_points, -1 before the first step, -5 at the last step
// (its g-tables are skipped).
// the N-D conditional pdf at x[d]; out[2] = (re, im).  reduce 0 skips the
// term reduction between the lowerings (every lowered child kept apart: the
// same sum up to rounding), for comparisons with the GPU's formulation.
int orc_cpdf_nd(void* h, const double* x, double* out, int reduce)
{
    cplx v;
    const int st = cpdf_nd_eval(*(Estimator*)h, x, &v, reduce != 0);
    if (st == 0) {
        out[0] = __real__ v;
        out[1] = __imag__ v;
    }
    return st;
}

int orc_cpdf_marginal(void* h, const double* xm, const int* idx, int nm, const double* nu_bar, double* out, int reduce)
{
    cplx v;
    const int st = cpdf_marginal_eval(*(Estimator*)h, xm, idx, nm, nu_bar, &v, reduce != 0);
    if (st) return st;
    out[0] = __real__ v;
    out[1] = __imag__ v;
    return 0;
}

int orc_cpdf_1d_grid(void* h, int marg, const double* bar_nu, double low, double high, double res, int max_points,
                     double* xs, double* ys)
{
    Estimator& E = *(Estimator*)h;
    const int n = cpdf_grid_points(low, high, res);
    if (n > max_points) return -2;
    if (E.master_step < 1) return -1;
    if (E.master_step >= E.num_steps) return -5;  // num_steps counts updates (p * steps)
    for (int i = 0; i < n; i++) {
        double x = low + i * res;
        if (x > high) x = high;
        xs[i] = x;
        ys[i] = cpdf1d_eval(E, marg, x, bar_nu);
    }
    return n;
}

// Marginal 2-D pdf grid: CauchyCPDFGridDispatcher2D::reset_grid and
// evaluate_point_grid (cpdf_ndim.hpp:1816-1919), x varying fastest; with
// reset_cache the cache is dropped afterwards (pycauchy.hpp:856-859).
// Returns the point count, -2 if it exceeds max_points, -1 before the first
// step, -5 at the last step, -6 on the reference's singular-cell exit.
int orc_cpdf_2d_grid(void* h, int i1, int i2, const double* bar_nu, double lx, double hx, double rx, double ly,
                     double hy, double ry, int reset_cache, int max_points, double* xs, double* ys, double* zs)
{
    Estimator& E = *(Estimator*)h;
    const int nx = cpdf_grid_points(lx, hx, rx), ny = cpdf_grid_points(ly, hy, ry);
    if ((long long)nx * ny > max_points) return -2;
    if (E.master_step < 1) return -1;
    if (E.master_step >= E.num_steps) return -5;
    int err = 0;
    for (int i = 0; i < ny; i++) {
        double y = ly + i * ry;
        if (y > hy) y = hy;
        for (int j = 0; j < nx; j++) {
            double x = lx + j * rx;
            if (x > hx) x = hx;
            const int q = i * nx + j;
            xs[q] = x;
            ys[q] = y;
            zs[q] = cpdf2d_eval(E, i1, i2, x, y, bar_nu, &err);
        }
    }
    if (reset_cache) E.cpdf2d_step = E.cpdf2d_m1 = E.cpdf2d_m2 = -1;
    return err ? -6 : nx * ny;
}


// get_marg2d_relative_and_transformed_cpdf (cauchy_prediction.hpp:653-971),
// single-thread order.  bar_nu_full[d] is the point the reference draws
// (2 u - 1, u = random_uniform_open()).  mom[14] receives the relative
// moments finalised (fz re/im, mean 2 x re/im, covariance 4 x re/im) when
// get_moments; counts[2] the pairs and the pairs approximated out.  *status:
// 0, -1 before the first step, -5 at the last step of either estimator,
// -3 dimension mismatch or too many rows.  pair_stride > 1 takes only the
// pairs whose index is pair_offset modulo pair_stride (a bounded sample for
// timing, which several processes can share).
void* orc_rel2d_create(void* hp, void* hs, const double* Trel, const double* bar_nu_full, int full_solve,
                       int get_moments, int with_term_approx, double term_approx_eps, double* mom, long long* counts,
                       int* status, long long pair_stride, long long pair_offset)
{
    Estimator& P = *(Estimator*)hp;
    Estimator& S = *(Estimator*)hs;
    *status = 0;
    if (P.d != S.d) {
        *status = -3;
        return nullptr;
    }
    if (P.master_step < 1 || S.master_step < 1) {
        *status = -1;
        return nullptr;
    }
    if (P.master_step >= P.num_steps || S.master_step >= S.num_steps) {
        *status = -5;
        return nullptr;
    }
    const int d = P.d;
    if ((P.shape_range - 1) + (S.shape_range - 1) >= 32) {
        *status = -3;
        return nullptr;
    }
    const double nf = kTwoPiInv * kTwoPiInv / __real__ P.fz / __real__ S.fz;
    double bar_nu[2];
    for (int i = 0; i < 2; i++) {
        double s = 0.0;
        for (int j = 0; j < d; j++) s += Trel[i * d + j] * bar_nu_full[j];
        bar_nu[i] = s;
    }
    // terms by shape, in order
    std::vector<std::vector<const Term*>> bp(P.shape_range), bs(S.shape_range);
    for (const Term& t : P.terms) bp[t.m].push_back(&t);
    for (const Term& t : S.terms) bs[t.m].push_back(&t);
    RelSys* R = new RelSys();
    R->full = full_solve ? 1 : 0;
    cplx acc[7];
    for (int i = 0; i < 7; i++) acc[i] = mkc(0, 0);
    long long pair_index = 0;
    for (int mp = 1; mp < P.shape_range; mp++)
        for (int ms = 1; ms < S.shape_range; ms++)
            for (const Term* tp : bp[mp])
                for (const Term* ts : bs[ms]) {
                    if (pair_stride > 1 && (pair_index++ % pair_stride) != pair_offset) continue;
                    Cpdf2DTerm c;
                    rel2d_pair(*tp, *ts, d, Trel, bar_nu_full, bar_nu, R->full, get_moments ? acc : nullptr, c);
                    R->total++;
                    if (with_term_approx && rel2d_negligible(c, nf, term_approx_eps)) {
                        R->approxed_out++;
                        continue;
                    }
                    R->terms.push_back(std::move(c));
                }
    if (get_moments) {
        // finalize_rel_sys_moments (cauchy_prediction.hpp:288-303)
        const cplx fz = acc[0];
        const cplx ifz = mkc(0, __real__ fz);
        cplx mean[2], cov[4];
        for (int i = 0; i < 2; i++) mean[i] = cdiv(acc[1 + i], ifz);
        for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++) cov[i * 2 + j] = cdiv(acc[3 + i * 2 + j], fz) - mean[i] * mean[j];
        mom[0] = __real__ fz;
        mom[1] = __imag__ fz;
        for (int i = 0; i < 2; i++) {
            mom[2 + 2 * i] = __real__ mean[i];
            mom[3 + 2 * i] = __imag__ mean[i];
        }
        for (int i = 0; i < 4; i++) {
            mom[6 + 2 * i] = __real__ cov[i];
            mom[7 + 2 * i] = __imag__ cov[i];
        }
    }
    counts[0] = R->total;
    counts[1] = R->approxed_out;
    return R;
}

void orc_rel2d_destroy(void* r) { delete (RelSys*)r; }

// grid_eval_marg2d_relative_and_transformed_cpdf (cauchy_prediction.hpp:1091-1186)
// with eval_marg2d_relative_and_transformed_cpdf (:1062-1073): x outermost,
// point (i, j) at i * ny + j.  Returns the point count, -2 if it exceeds
// max_points, -3 for a grid of fewer than two points per axis, -6 on the
// reference's singular-cell exit.
int orc_rel2d_grid(void* r, double xlow, double xhigh, double dx, double ylow, double yhigh, double dy,
                   double nf_prim, double nf_sec, int max_points, double* xs, double* ys, double* zs)
{
    RelSys& R = *(RelSys*)r;
    if (!(xhigh > xlow) || !(yhigh > ylow)) return -3;
    const int nx = (int)ceil((xhigh - xlow) / dx + 1), ny = (int)ceil((yhigh - ylow) / dy + 1);
    if (nx <= 1 || ny <= 1) return -3;
    if ((long long)nx * ny > max_points) return -2;
    int err = 0;
    for (int i = 0; i < nx; i++) {
        const double x = i == nx - 1 ? xhigh : xlow + dx * i;
        for (int j = 0; j < ny; j++) {
            const double y = j == ny - 1 ? yhigh : ylow + dy * j;
            double fx = 0;
            for (const Cpdf2DTerm& c : R.terms) {
                const double g1i = c.b[0] - x, g2i = c.b[1] - y;
                const bool check = fabs(g1i) < kIntegralGammaEps;
                double t = 0;
                const int cells = c.m * (1 + R.full);
                for (int k = 0; k < cells; k++) {
                    double v;
                    if (!marg2d_cell(c.sin_t[k], c.cos_t[k], c.sin_t[k + 1], c.cos_t[k + 1], c.g1r[k], g1i, c.g2r[k],
                                     g2i, check, c.g[k], &v)) {
                        err = 1;
                        v = 0;
                    }
                    t += v;
                }
                fx += t;
            }
            const int q = i * ny + j;
            xs[q] = x;
            ys[q] = y;
            zs[q] = ((double)(2 - R.full)) * fx * kTwoPiInv * kTwoPiInv / (nf_prim * nf_sec);
        }
    }
    return err ? -6 : nx * ny;
}

}  // extern "C"
