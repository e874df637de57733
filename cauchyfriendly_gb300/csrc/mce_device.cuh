// Device-side building blocks of the MCE step path (sm_103a, FP64).
//
// Every arithmetic helper here evaluates in the same operation order as the
// reference's C++ (natsnyder1/CauchyFriendly include/*.hpp) and the kernels are
// compiled with --fmad=false, so the floating-point decisions that fix the
// integer structure (coalignment, MU orthogonality, cond() vertex skipping,
// term reduction, term approximation) take the same branches as the reference.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mce {

constexpr int kMaxRows = 31;    // keys are 32-bit sign masks (cauchy_estimator.hpp:231-235)
constexpr int kMaxDim = 8;
constexpr int kMaxGamma = 8;   // process-noise columns per step
constexpr double kPi = 3.14159265358979323846;                      // PI (M_PI)
constexpr double kTwoPiInv = 1.0 / (2.0 * 3.14159265358979323846);  // RECIPRICAL_TWO_PI
constexpr double kCoalignEps = 1e-8;   // COALIGN_TP_EPS == COALIGN_MU_EPS
constexpr double kMuEps = 1e-10;       // MU_EPS
constexpr double kTermApproxEps = 1e-15;
constexpr double kPluEps = 1e-15;
constexpr double kCondEps = 1e12;
constexpr double kReductionEps = 1e-8;

// term flags
constexpr int kFlagNewChild = 1;
constexpr int kFlagHasCmap = 2;

// device error bits (reported through the engine's status word)
constexpr int kErrAntiCoalignedHorthog = 1;  // cauchy_term.hpp:673-687 exits the process
constexpr int kErrTableOverflow = 2;  // a parent's B table above its capacity
constexpr int kErrShapeTooLarge = 4;
constexpr int kErrResolveStalled = 8;
constexpr int kErrDceOverflow = 16;
constexpr int kErrRecordOverflow = 32;       // an MU record past the step's record count
constexpr int kErrRootCellsOverflow = 64;    // a reduction root's cells above its table slot
constexpr int kErrMemberCellsOverflow = 128;  // a promoted member's cells above its table slot

struct cd {
    double re, im;
};
__host__ __device__ inline cd mkcd(double r, double i) { return cd{r, i}; }
__device__ inline cd cadd(cd a, cd b) { return cd{a.re + b.re, a.im + b.im}; }
__device__ inline cd csub(cd a, cd b) { return cd{a.re - b.re, a.im - b.im}; }
__device__ inline cd cconj(cd a) { return cd{a.re, -a.im}; }
__device__ inline cd cscale(cd a, double s) { return cd{a.re * s, a.im * s}; }
// (a+bi)(c+di) = (ac - bd) + (ad + bc)i, the textbook product.
__device__ inline cd cmul(cd x, cd y)
{
    double ac = x.re * y.re, bd = x.im * y.im, ad = x.re * y.im, bc = x.im * y.re;
    return cd{ac - bd, ad + bc};
}
__device__ inline unsigned long long dabs_bits(double x);

// Complex division by R. L. Smith, "Algorithm 116: Complex division",
// CACM 5(8), 1962: divide through by the larger of |c|, |d| to avoid overflow.
// The two branches are folded into one sequence with operand selects, each
// select giving the branch's own expression (|c| >= |d|: r = d/c,
// den = d r + c, (b r + a)/den, (b - a r)/den; |c| < |d|: r = c/d,
// den = c r + d, (a r + b)/den, (b r - a)/den), so the results are the same
// bits and lanes of a warp that would take different branches no longer
// execute both.
__device__ inline cd cdiv(cd x, cd y)
{
    const double a = x.re, b = x.im, c = y.re, d = y.im;
    const bool big_c = !(dabs_bits(c) < dabs_bits(d));
    const double p = big_c ? c : d, q = big_c ? d : c;
    const double P = big_c ? a : b, Q = big_c ? b : a;
    const double r = q / p;
    const double den = q * r + p;
    const double pr = P * r;
    const double num = big_c ? (Q - pr) : (pr - Q);
    return cd{(Q * r + P) / den, num / den};
}

// Comparisons of doubles on their bit patterns (integer pipe).  IEEE doubles
// order like sign-magnitude integers, so these give the same answers as the
// floating-point comparisons for every non-NaN operand (-0 and +0 included).
__device__ inline unsigned long long dabs_bits(double x)
{
    return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}
// |x| < c for c > 0
__device__ inline bool abs_lt(double x, double c)
{
    return dabs_bits(x) < (unsigned long long)__double_as_longlong(c);
}
// |x| > |y|
__device__ inline bool abs_gt(double x, double y) { return dabs_bits(x) > dabs_bits(y); }
// x > 0
__device__ inline bool pos(double x) { return __double_as_longlong(x) > 0; }
// x < 0
__device__ inline bool neg(double x)
{
    const long long b = __double_as_longlong(x);
    return b < 0 && (b & 0x7fffffffffffffffLL) != 0;
}
// Order-preserving integer key: +x -> bits, -x -> -(magnitude bits).
__device__ inline long long dkey(double x)
{
    const long long b = __double_as_longlong(x);
    return (b >= 0) ? b : -(b & 0x7fffffffffffffffLL);
}
// a < b and a <= b (keys map -0 and +0 to the same value)
__device__ inline bool dlt(double a, double b) { return dkey(a) < dkey(b); }
__device__ inline bool dle(double a, double b) { return dkey(a) <= dkey(b); }

// The term-approximation test of make_gtable, ps2 * |v| > 1e-15 with
// |v| = hypot(re, im) (flattening.hpp:242-247).  ps2^2 (re^2 + im^2) is
// compared with the threshold first; only values within a relative 1e-9 of it
// take the reference's exact expression.
__device__ inline bool above_approx_threshold(double ps2, double re, double im)
{
    const double t = (ps2 * ps2) * (re * re + im * im);
    const double thr = kTermApproxEps * kTermApproxEps;
    if (t > thr * (1.0 + 1e-9)) return true;
    if (t < thr * (1.0 - 1e-9)) return false;
    return ps2 * hypot(re, im) > kTermApproxEps;
}

// Binary search over ascending keys (gtable.hpp:283-301 semantics).
__device__ inline int bsearch_key(const int* __restrict__ keys, int n, int key)
{
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int mk = keys[mid];
        if (mk == key) return mid;
        if (mk > key) hi = mid - 1;
        else lo = mid + 1;
    }
    return -1;
}

// Position of `key` in keys[] where keys[i] ^ x ascends (a sorted table whose
// entries were all XORed with x), -1 if absent.
__device__ inline int bsearch_key_xor(const int* __restrict__ keys, int n, int key, int x)
{
    const int target = key ^ x;
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int mk = keys[mid] ^ x;
        if (mk == target) return mid;
        if (mk > target) hi = mid - 1;
        else lo = mid + 1;
    }
    return -1;
}

// g numerator from the parent table with half storage: a key whose bit phc-1
// is set is looked up reversed and conjugated (eval_gs.hpp:94-153).
__device__ inline cd lookup_num(const int* __restrict__ keys, const cd* __restrict__ vals, int n, int enc, int phc)
{
    const int top = 1 << (phc - 1);
    const int rev = (1 << phc) - 1;
    if (enc & top) {
        const int idx = bsearch_key(keys, n, rev ^ enc);
        return idx < 0 ? mkcd(0, 0) : cconj(vals[idx]);
    }
    const int idx = bsearch_key(keys, n, enc);
    return idx < 0 ? mkcd(0, 0) : vals[idx];
}

// Central-arrangement cell count (cell_enumeration.hpp:34-44).
__host__ __device__ inline long long binom_ll(int n, int k)
{
    if (k < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    long long r = 1;
    for (int i = 0; i < k; i++) {
        r *= (n - i);
        r /= (i + 1);
    }
    return r;
}
__host__ __device__ inline int cells_central(int m, int d)
{
    if (m < d) return 1 << m;
    long long s = 0;
    for (int i = 0; i < d; i++) s += binom_ll(m - 1, i);
    return (int)(2 * s);
}
__host__ __device__ inline int half_cells_cap(int m, int d)
{
    int c = cells_central(m, d) / 2;
    return c < 1 ? 1 : c;
}

// Row-vs-row coalignment gate (cauchy_term.hpp:494-504): +1 same, -1 opposite, 0 none.
template <int D>
__device__ inline int coalign_gate(const double* r, const double* c)
{
    bool ps = true, ng = true;
#pragma unroll
    for (int l = 0; l < D; l++) {
        if (ps) ps &= abs_lt(r[l] - c[l], kCoalignEps);
        if (ng) ng &= abs_lt(r[l] + c[l], kCoalignEps);
        if (!(ps || ng)) break;
    }
    return ps ? 1 : (ng ? -1 : 0);
}

// Orientation mask of two equal arrangements: for each row, the first
// component significant in both decides (cell_enumeration.hpp:630-640).
template <int D>
__device__ inline int orientation_mask(const double* Ai, const double* Aj, int m)
{
    int s = 0;
    for (int k = 0; k < m; k++) {
        int l = 0;
        while (l < D - 1 && (abs_lt(Ai[k * D + l], kReductionEps) || abs_lt(Aj[k * D + l], kReductionEps))) l++;
        if (Ai[k * D + l] * Aj[k * D + l] < 0) s |= 1 << k;
    }
    return s;
}

// ---------------------------------------------------------------------------
// Dense D x D linear algebra in the reference's operation order
// (cauchy_linalg.hpp:1180-1390).
template <int D>
__device__ inline bool plu(double* A, int* P)
{
    for (int j = 0; j < D; j++) {
        double piv = kPluEps;
        int pi = -1;
        for (int i = j; i < D; i++)
            if (abs_gt(A[i * D + j], piv)) {
                piv = A[i * D + j];
                pi = i;
            }
        if (pi == -1) return false;
        if (pi != j)
            for (int c = 0; c < D; c++) {
                const double t = A[j * D + c];
                A[j * D + c] = A[pi * D + c];
                A[pi * D + c] = t;
            }
        P[j] = pi;
        for (int k = j + 1; k < D; k++) {
            A[k * D + j] /= A[j * D + j];
            const double t = A[k * D + j];
            for (int q = j + 1; q < D; q++) A[k * D + q] -= t * A[j * D + q];
        }
    }
    return true;
}

// Row permutation applied by the pivot list, inverted (cauchy_linalg.hpp:1258-1277).
template <int D>
__device__ inline void inverse_perm(const int* P, int* PT)
{
    int Preg[D];
    for (int i = 0; i < D; i++) Preg[i] = i;
    for (int i = 0; i < D; i++) {
        const int t = Preg[i];
        Preg[i] = Preg[P[i]];
        Preg[P[i]] = t;
    }
    for (int i = 0; i < D; i++) PT[Preg[i]] = i;
}

template <int D>
__device__ inline void lu_solve_inplace(const double* LU, double* x)
{
#pragma unroll
    for (int i = 0; i < D; i++) {
        double s = x[i];
#pragma unroll
        for (int j = 0; j < i; j++) s -= LU[i * D + j] * x[j];
        x[i] = s;
    }
#pragma unroll
    for (int i = D - 1; i >= 0; i--) {
        double s = x[i];
#pragma unroll
        for (int j = D - 1; j > i; j--) s -= LU[i * D + j] * x[j];
        x[i] = s / LU[i * D + i];
    }
}

template <int D>
__device__ inline double cond1_from_lu(const double* A, const int* P, double nrm);

// Upper bound on the 1-norm of (LU)^-1 from packed factors with partial
// pivoting: ||A^-1|| <= ||M(U)^-1|| ||L^-1|| with M(U) the comparison matrix
// of U (|u_ii| on the diagonal, -|u_ij| above) and ||L^-1||_1 <= 2^(D-1) since
// |l_ij| <= 1.  M(U)^-1 is non-negative, so its column sums are computed by a
// cancellation-free back substitution in single precision, then inflated by a
// margin that covers the rounding.  Returns +inf when it cannot bound.
template <int D>
__device__ inline float inv_norm1_bound(const double* LU)
{
    float Ua[D * D];
    for (int i = 0; i < D; i++)
        for (int j = i; j < D; j++) Ua[i * D + j] = fabsf(__double2float_ru(fabs(LU[i * D + j])));
    float best = 0.f;
    for (int k = 0; k < D; k++) {
        float x[D];
        float colsum = 0.f;
        for (int i = k; i >= 0; i--) {
            float acc = (i == k) ? 1.f : 0.f;
            for (int j = i + 1; j <= k; j++) acc += Ua[i * D + j] * x[j];
            // a lower bound of |u_ii| keeps the quotient an upper bound
            const float den = __double2float_rd(fabs(LU[i * D + i]));
            x[i] = acc / den;
            colsum += x[i];
        }
        best = fmaxf(best, colsum);
    }
    // row sums of |M(U)^-1| in 1-norm sense: column sums as computed above bound ||M(U)^-1||_1
    return best * (float)(1 << (D - 1)) * 1.0001f;
}

// 1-norm condition number through the explicit inverse; on success A holds
// the packed LU factors and P the pivots.  Returns DBL_MAX when PLU fails.
template <int D>
__device__ inline double cond1(double* A, int* P)
{
    double nrm = -1;
#pragma unroll
    for (int c = 0; c < D; c++) {
        double s = 0;
#pragma unroll
        for (int r = 0; r < D; r++) s += fabs(A[r * D + c]);
        if (dlt(nrm, s)) nrm = s;
    }
    if (!plu<D>(A, P)) return 1.79769313486231570815e+308;
    return cond1_from_lu<D>(A, P, nrm);
}

// The second half of cond1: 1-norm of the explicit inverse from the packed LU
// factors, times the 1-norm of A (cauchy_linalg.hpp:1369-1389).
template <int D>
__device__ inline double cond1_from_lu(const double* A, const int* P, double nrm)
{
    int PT[D];
    inverse_perm<D>(P, PT);
    double inrm = -1;
    (void)A;
#pragma unroll
    for (int i = 0; i < D; i++) {
        double w[D];
#pragma unroll
        for (int j = 0; j < D; j++) w[j] = (j == PT[i]) ? 1.0 : 0.0;
        lu_solve_inplace<D>(A, w);
        double s = 0;
#pragma unroll
        for (int j = 0; j < D; j++) s += fabs(w[j]);
        if (dlt(inrm, s)) inrm = s;
    }
    return nrm * inrm;
}

// cond1_from_lu(A, P, nrm) > eps, stopping at the first inverse column whose
// 1-norm s already gives nrm * s > eps: the full value is nrm times the
// largest column norm, and rounding is monotone, so that column settles the
// comparison exactly as the full computation would (the columns are solved
// in the same order and the same arithmetic).  Nearly singular subsets,
// whose every inverse column is large, then cost one solve instead of D.
template <int D>
__device__ inline bool cond1_exceeds(const double* A, const int* P, double nrm, double eps)
{
    int PT[D];
    inverse_perm<D>(P, PT);
    double inrm = -1;
#pragma unroll
    for (int i = 0; i < D; i++) {
        double w[D];
#pragma unroll
        for (int j = 0; j < D; j++) w[j] = (j == PT[i]) ? 1.0 : 0.0;
        lu_solve_inplace<D>(A, w);
        double s = 0;
#pragma unroll
        for (int j = 0; j < D; j++) s += fabs(w[j]);
        if (nrm * s > eps) return true;
        if (dlt(inrm, s)) inrm = s;
    }
    return nrm * inrm > eps;
}

template <int D>
__device__ inline void solve_lu(const double* LU, const int* P, const double* b, double* x)
{
    int PT[D];
    inverse_perm<D>(P, PT);
    for (int i = 0; i < D; i++) x[PT[i]] = b[i];
    lu_solve_inplace<D>(LU, x);
}

// ---------------------------------------------------------------------------
// Post-MU term records (structure of arrays, one slot per term; rows padded
// to the run's row capacity MC).
struct TermRecs {
    int* est;
    int* m;       // rows after MU coalignment
    int* pbc;     // rows at the MU (before MU coalignment)
    int* phc;     // rows of the parent table's arrangement
    int* z;       // index of the MU hyperplane (== pbc for the parent itself)
    int* lhp;     // enc_lhp
    int* fam;     // parent index (row of the parent list) of this term's family
    int* flags;   // kFlagNewChild | kFlagHasCmap
    unsigned* horthog;
    double* A;    // [n][MC][D]
    double* p;    // [n][MC]
    double* q;    // [n][MC]
    double* b;    // [n][D]
    double* cval;
    double* dval;
    signed char* cmap;   // [n][MC]
    signed char* csmap;  // [n][MC]
    double* ps2;         // (sum of p)^2, the term-approximation weight (flattening.hpp:103-108)
};

// Parent list at the start of a step (one slot per term, ordered by
// estimator, shape, index).
struct ParentList {
    int* est;
    int* m;          // rows (updated in place by time propagation)
    int* m_old;      // rows before time propagation (the table's bit count)
    double* A;       // [n][MC][D]
    double* p;       // [n][MC]
    double* b;       // [n][D]
    long long* tab_off;  // g-table slice in the table arena
    int* tab_cnt;
    long long* B_off;    // this step's B (then B_mu) slice in the B arena
    int* B_cnt;
    int* nkids;      // integrable children written as records
    int* nkids_all;  // integrable children (moments are taken over them even on the final MU)
    long long* kscan;  // exclusive scan of nkids
    int* bflip;        // mask the MU XORed into the parent's (ascending) B table
};

struct Tables {
    int* keys;
    cd* vals;
};

// Flat g-table evaluation of one step: per group (root list index) its cell
// count, item offset, root p-sum and kept flag; per member slot its info word,
// p-sum and kept flag; the evaluated items.
struct GFlat {
    int* gnr;
    long long* ioff;
    double* rps2;
    int* rflag;
    int* minfo;
    double* mps2;
    int* mflag;
    cd* gv;
    // groups whose root the flat pass approximated out and whose promoted
    // root the serial path found (per root list index): the members left
    // after it go through the promoted-root flat pass
    int* pr_root;          // the promoted root record
    int* pr_mb;            // its first remaining member's slot in the members list
    int* pr_mcnt;          // remaining members (0: nothing handed over)
    int* pr_cells;         // the promoted root's cell count (0 when nothing is handed over)
    int* pr_items;         // pr_mcnt * pr_cells
    long long* pr_moff;    // exclusive scans of pr_mcnt, pr_items, pr_cells
    long long* pr_ioff;
    long long* pr_coff;
    cd* pr_gv;             // the remaining members' values
};

// Per-estimator step inputs, packed by the host each step.
template <int D>
struct EstStep {
    double msmt;
    double gamma;
    double Phi[D * D];
    double H[D];
    double Bu[D];     // B @ u (control shift), zero when there is no control
    double Gt[kMaxGamma * D];  // pre-coaligned Gamma rows
    double bt[kMaxGamma];
    int gcnt;
    int has_control;
    int active;   // stepping this measurement
    int skip;     // final measurement update of this estimator: moments only
};

}  // namespace mce
