// Adjoint of the MCE step path: the gradient of sum_k w_k Re(fz_k) -- and so
// of the accumulated log-likelihood sum_k log fz_k -- with respect to the
// model's Cauchy scales and matrices (beta, gamma, p0, Phi, Gamma, H), holding
// the enumerated cell structure fixed (which cells exist, which terms merge,
// which rows coalign, which terms are approximated out).
//
// Why a linear seed suffices.  After update j every g-table is scaled by
// G_SCALE_FACTOR_j = 1/(2 pi Re fz_j) (include/cauchy_estimator.hpp:342) and
// every later table and fz is linear in the earlier tables, so
// prod_{j<=k} Re fz_j = Re U_k, the fz of update k computed without the
// scales.  Hence d(sum_{j<=k} log Re fz_j) = d Re fz_k / Re fz_k with the
// scales held constant: the log-likelihood of a run is one seed, 1/Re fz_K, on
// the last update's fz, and any sum of log fz over a range of updates is two.
//
// Layout of the computation (one run per mce_adjoint; an mce_adjoint_batch
// steps its runs with one batched handle and records and reverses them on
// several host threads, each thread with its own stream and buffers):
//  * forward: the library's GPU step path runs the updates; after each one
//    the object copies the kept terms and their g-tables (mce_dump_terms) and
//    the update's G_SCALE_FACTOR.  On the host it re-derives, per update, the
//    records of every post-MU term (time propagation, Gamma coalignment,
//    measurement update, MU coalignment: O(terms * rows * d)) and the
//    reduction groups, in the reference's arithmetic, so they are the same
//    doubles as the GPU's (checked against the dump);
//  * on the GPU, per update, one thread per (group member, cell) evaluates
//    the member's g value on the kept root's cells (make_gtable,
//    include/flattening.hpp:77-255) with its two parent-table lookups: this
//    decides which members are approximated out and checks every kept table
//    against the dumped one;
//  * reverse, on the GPU, update by update from the last: the fz seeds (one
//    thread per post-MU term: eval_g_yei, include/cauchy_term.hpp:312-401)
//    and the table adjoints (one thread per (member, cell)) give the adjoints
//    of the parent-table cells (atomic adds), and of every term's scalars
//    that enter the g values: the row scales (q, or p before coalignment
//    for the fz terms), d_val and c_val;
//  * the record chain, on the GPU: one thread per (parent, parameter
//    direction) repeats the parent's derivation in forward-mode dual numbers
//    and dots the tangents of those scalars with their adjoints.
#include "mce_device.cuh"
#include "../../include/mce_c_api.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace mce {
void report_error(const std::string& s);
}

using mce::cd;

namespace {

// ---------------------------------------------------------------------------
// Constants of the record derivation (the GPU record chain below repeats the
// derivation on dual numbers).
constexpr double kCoalignEps = 1e-8;
constexpr double kMuEps = 1e-10;
constexpr double kReductionEps = 1e-8;

// Term records of one update: a slot per term with room for MS rows (A slot
// major, its rows row-major, d wide), held in flat arrays that keep their
// capacity from update to update, so deriving a term allocates nothing.
struct RecSet {
    int MS = 0, d = 0, n = 0, cap = 0;
    std::vector<int> m;
    std::vector<unsigned> horthog;
    std::vector<double> c, dv;  // c_val, d_val
    std::vector<double> A, p, b;
    std::vector<double> q;      // row scales before normalisation (the g-table's)
    void init(int MS_, int d_)
    {
        MS = MS_;
        d = d_;
        n = 0;
    }
    void ensure(int want)
    {
        if (want <= cap) return;
        cap = std::max(want, 2 * cap);
        m.resize(cap);
        horthog.resize(cap);
        c.resize(cap);
        dv.resize(cap);
        A.resize((size_t)cap * MS * d);
        p.resize((size_t)cap * MS);
        q.resize((size_t)cap * MS);
        b.resize((size_t)cap * d);
    }
    int add()
    {
        ensure(n + 1);
        return n++;
    }
    double* Ar(int t) { return &A[(size_t)t * MS * d]; }
    const double* Ar(int t) const { return &A[(size_t)t * MS * d]; }
    double* pr(int t) { return &p[(size_t)t * MS]; }
    const double* pr(int t) const { return &p[(size_t)t * MS]; }
    double* qr(int t) { return &q[(size_t)t * MS]; }
    const double* qr(int t) const { return &q[(size_t)t * MS]; }
    double* br(int t) { return &b[(size_t)t * d]; }
    const double* br(int t) const { return &b[(size_t)t * d]; }
    void copy_from(int t, const RecSet& o, int u)
    {
        m[t] = o.m[u];
        horthog[t] = o.horthog[u];
        c[t] = o.c[u];
        dv[t] = o.dv[u];
        memcpy(Ar(t), o.Ar(u), sizeof(double) * o.m[u] * d);
        memcpy(pr(t), o.pr(u), sizeof(double) * o.m[u]);
        memcpy(qr(t), o.qr(u), sizeof(double) * o.m[u]);
        memcpy(br(t), o.br(u), sizeof(double) * d);
    }
    void swap(RecSet& o)
    {
        std::swap(MS, o.MS);
        std::swap(d, o.d);
        std::swap(n, o.n);
        std::swap(cap, o.cap);
        m.swap(o.m);
        horthog.swap(o.horthog);
        c.swap(o.c);
        dv.swap(o.dv);
        A.swap(o.A);
        p.swap(o.p);
        q.swap(o.q);
        b.swap(o.b);
    }
};

constexpr int kRowsMax = 32, kDMax = 8;

// coalignment gate on values: +1 same, -1 opposite, 0 (cauchy_term.hpp:494-504)
int gate(const double* r, const double* c, int d)
{
    bool pos = true, neg = true;
    for (int l = 0; l < d; l++) {
        if (pos) pos &= std::fabs(r[l] - c[l]) < kCoalignEps;
        if (neg) neg &= std::fabs(r[l] + c[l]) < kCoalignEps;
        if (!(pos || neg)) break;
    }
    return pos ? 1 : (neg ? -1 : 0);
}

// normalize_hps (cauchy_term.hpp:458-472) on m rows: p *= |A_i|_1,
// A_i /= |A_i|_1; q (if not null) receives the scales before normalisation.
void normalize_rows(double* A, double* p, double* q, int m, int d)
{
    if (q) memcpy(q, p, sizeof(double) * m);
    for (int i = 0; i < m; i++) {
        double n1 = 0.0;
        for (int j = 0; j < d; j++) n1 += std::fabs(A[i * d + j]);
        p[i] *= n1;
        for (int j = 0; j < d; j++) A[i * d + j] /= n1;
    }
}

// What the host keeps of one post-MU term for the GPU and the record chain.
struct TermInfo {
    int parent = -1;      // kept term of the previous update (its table), -1 at update 0
    int m_pre = 0, m = 0; // rows before and after MU coalignment
    int phc = 0, z = 0, enc_lhp = 0;
    bool new_child = false, has_cmap = false;
    unsigned horthog_pre = 0, horthog = 0;
    int cmap[32], csmap[32];
    int lp = 0, lm = 0;   // eval lookup keys (before the enc_lhp XOR), or -1 at update 0
    double y_eval = 0;    // sum of p s over the non-orthogonal rows at the root point
    double d_eval = 0, c_eval = 0;  // d_val, c_val
    unsigned sneg = 0;    // rows with a negative sign at the root point
    int shape_key = 0;
};

// One candidate of a reduction group whose table enters a kept table.
struct Member {
    int term;     // post-MU term index
    int kept;     // kept term (root's slot) this member's table goes into
    int s_fixed;  // orientation XOR from the root's cells to this member's cells
    int conj;     // the member's value enters conjugated
    int contrib;  // 1 if not approximated out (decided on the GPU)
};

// GPU view of a member: everything make_gtable needs.
struct MInfoDev {
    int m, phc, z, enc_lhp, flags, horthog, s_fixed, conj;
    int kept, parent, term;
    long long cell_off, cell_cnt;  // the root's cells in the kept table arrays
    double d, c, ps2;
    double q[32];
    signed char cmap[32], csmap[32];
};
constexpr int kMiNewChild = 1, kMiHasCmap = 2, kMiFirst = 4;

struct EvalDev {
    int parent, lp, lm, enc_lhp, phc, first;
    double y, d, c;
};

// ---------------------------------------------------------------------------
// Kernels

__device__ inline cd lookup_idx(const int* keys, const cd* vals, long long off, int n, int enc, int phc, long long* idx,
                                int* cj)
{
    const int top = 1 << (phc - 1), rev = (1 << phc) - 1;
    *cj = 0;
    int key = enc;
    if (enc & top) {
        key = rev ^ enc;
        *cj = 1;
    }
    const int i = mce::bsearch_key(keys + off, n, key);
    if (i < 0) {
        *idx = -1;
        return mce::mkcd(0, 0);
    }
    *idx = off + i;
    const cd v = vals[off + i];
    return *cj ? mce::cconj(v) : v;
}

// lookup keys of a member's cell (flattening.hpp:77-255)
__device__ inline void cell_keys(const MInfoDev& M, int be, int* lp, int* lm, double* y)
{
    int sb[32];
    double yy = 0;
    for (int k = 0; k < M.m; k++) {
        sb[k] = ((be >> k) & 1) ? -1 : 1;
        if (!((M.horthog >> k) & 1)) yy += M.q[k] * sb[k];
    }
    *y = yy;
    int a = 0, b = 0;
    if (!(M.flags & kMiNewChild)) {
        a = be & ((1 << M.phc) - 1);
        b = a;
    } else {
        int k = 0, l = 0;
        while (k < M.phc) {
            if (k == M.z) {
                b |= 1 << k;
                k++;
                if (k == M.phc) break;
            }
            const int bv = (M.flags & kMiHasCmap) ? sb[M.cmap[l]] * M.csmap[l] : sb[l];
            if (bv < 0) {
                a |= 1 << k;
                b |= 1 << k;
            }
            k++;
            l++;
        }
    }
    *lp = a;
    *lm = b;
}

// v = S (gp / (y + d + ic) - gm / (y - d + ic))
__device__ inline cd gval(cd gp, cd gm, double y, double d, double c, double S)
{
    const cd a = mce::cdiv(gp, mce::mkcd(y + d, c));
    const cd b = mce::cdiv(gm, mce::mkcd(y - d, c));
    return mce::cscale(mce::csub(a, b), S);
}

__device__ inline void atomic_add_cd(cd* p, cd v)
{
    atomicAdd(&p->re, v.re);
    atomicAdd(&p->im, v.im);
}

// forward: every (member, cell) value and the members' approximation flags
__global__ void k_adj_member_values(const MInfoDev* mi, const long long* item_off, int nmem, long long nitems,
                                    const int* kkeys, const int* pkeys, const cd* pvals, const long long* poff,
                                    const int* pcnt, double gscale, cd* vout, int* alive)
{
    for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < nitems;
         it += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = nmem - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (item_off[mid] <= it) lo = mid;
            else hi = mid - 1;
        }
        const MInfoDev& M = mi[lo];
        const long long i = it - item_off[lo];
        const int be = kkeys[M.cell_off + i] ^ M.s_fixed;
        cd v;
        if (M.flags & kMiFirst) {
            double y = 0;
            for (int k = 0; k < M.m; k++)
                if (!((M.horthog >> k) & 1)) y += M.q[k] * (((be >> k) & 1) == 0 ? 1.0 : -1.0);
            v = gval(mce::mkcd(1, 0), mce::mkcd(1, 0), y, M.d, M.c, gscale);
        } else {
            int lp, lm, cj;
            double y;
            long long ip, im;
            cell_keys(M, be, &lp, &lm, &y);
            const cd gp = lookup_idx(pkeys, pvals, poff[M.parent], pcnt[M.parent], lp ^ M.enc_lhp, M.phc, &ip, &cj);
            const cd gm = lookup_idx(pkeys, pvals, poff[M.parent], pcnt[M.parent], lm ^ M.enc_lhp, M.phc, &im, &cj);
            v = gval(gp, gm, y, M.d, M.c, gscale);
        }
        vout[it] = v;
        if (M.ps2 * hypot(v.re, v.im) > mce::kTermApproxEps) alive[lo] = 1;
    }
}

// forward check: every kept cell = its root's value plus the contributing
// members' values, in member order (flattening.hpp:259-315)
__global__ void k_adj_check_tables(const long long* kept_first_mem, const int* kept_nmem, const MInfoDev* mi,
                                   const long long* item_off, const int* contrib, const cd* vals_member,
                                   const long long* koff, const int* kcnt, const cd* kvals, int nkept,
                                   unsigned long long* max_err_bits)
{
    if (nkept == 0) return;
    const long long ncells = koff[nkept - 1] + kcnt[nkept - 1];
    for (long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x; cell < ncells;
         cell += (long long)gridDim.x * blockDim.x) {
        // the kept table holding this cell
        int lo = 0, hi = nkept - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (koff[mid] <= cell) lo = mid;
            else hi = mid - 1;
        }
        const long long i = cell - koff[lo];
        if (i >= kcnt[lo]) continue;
        cd s = mce::mkcd(0, 0);
        bool first = true;
        for (int j = 0; j < kept_nmem[lo]; j++) {
            const long long mj = kept_first_mem[lo] + j;
            if (!contrib[mj]) continue;
            cd v = vals_member[item_off[mj] + i];
            if (mi[mj].conj) v = mce::cconj(v);
            s = first ? v : mce::cadd(s, v);
            first = false;
        }
        const cd want = kvals[cell];
        const double den = fmax(hypot(want.re, want.im), 1e-300);
        const double e = hypot(s.re - want.re, s.im - want.im) / den;
        atomicMax(max_err_bits, (unsigned long long)__double_as_longlong(e));
    }
}

// reverse: table adjoints of the kept cells -> the parent-table cells and the
// members' scalars (q rows, d_val, c_val)
__global__ void k_adj_member_reverse(const MInfoDev* mi, const long long* item_off, int nmem, long long nitems,
                                     const int* contrib, const int* kkeys, const cd* kbar, const int* pkeys,
                                     const cd* pvals, const long long* poff, const int* pcnt, double gscale,
                                     cd* pbar, double* qbar, double* dbar, double* cbar)
{
    for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < nitems;
         it += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = nmem - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (item_off[mid] <= it) lo = mid;
            else hi = mid - 1;
        }
        if (!contrib[lo]) continue;
        const MInfoDev& M = mi[lo];
        const long long i = it - item_off[lo];
        cd vb = kbar[M.cell_off + i];
        if (M.conj) vb = mce::cconj(vb);
        if (vb.re == 0 && vb.im == 0) continue;
        const int be = kkeys[M.cell_off + i] ^ M.s_fixed;
        cd gp = mce::mkcd(1, 0), gm = mce::mkcd(1, 0);
        long long ip = -1, im = -1;
        int cjp = 0, cjm = 0;
        double y = 0;
        if (M.flags & kMiFirst) {
            for (int k = 0; k < M.m; k++)
                if (!((M.horthog >> k) & 1)) y += M.q[k] * (((be >> k) & 1) == 0 ? 1.0 : -1.0);
        } else {
            int lp, lm;
            cell_keys(M, be, &lp, &lm, &y);
            gp = lookup_idx(pkeys, pvals, poff[M.parent], pcnt[M.parent], lp ^ M.enc_lhp, M.phc, &ip, &cjp);
            gm = lookup_idx(pkeys, pvals, poff[M.parent], pcnt[M.parent], lm ^ M.enc_lhp, M.phc, &im, &cjm);
        }
        const cd Dp = mce::mkcd(y + M.d, M.c), Dm = mce::mkcd(y - M.d, M.c);
        const cd ip_ = mce::cdiv(mce::mkcd(1, 0), Dp), im_ = mce::cdiv(mce::mkcd(1, 0), Dm);
        // dv/dgp = S / Dp, dv/dgm = -S / Dm
        if (ip >= 0) {
            cd a = mce::cmul(mce::cconj(mce::cscale(ip_, gscale)), vb);
            atomic_add_cd(&pbar[ip], cjp ? mce::cconj(a) : a);
        }
        if (im >= 0) {
            cd a = mce::cmul(mce::cconj(mce::cscale(im_, -gscale)), vb);
            atomic_add_cd(&pbar[im], cjm ? mce::cconj(a) : a);
        }
        // dv/dy = S (-gp/Dp^2 + gm/Dm^2), dv/dd = S (-gp/Dp^2 - gm/Dm^2), dv/dc = i dv/dy
        const cd tp = mce::cmul(gp, mce::cmul(ip_, ip_)), tm = mce::cmul(gm, mce::cmul(im_, im_));
        const cd vy = mce::cscale(mce::csub(tm, tp), gscale);
        const cd vd = mce::cscale(mce::cadd(tp, tm), -gscale);
        const double yb = vb.re * vy.re + vb.im * vy.im;     // Re(conj(vb) vy)
        const double db = vb.re * vd.re + vb.im * vd.im;
        const double cb = vb.re * (-vy.im) + vb.im * vy.re;  // Re(conj(vb) i vy)
        for (int k = 0; k < M.m; k++)
            if (!((M.horthog >> k) & 1)) atomicAdd(&qbar[(size_t)lo * 32 + k], yb * (((be >> k) & 1) ? -1.0 : 1.0));
        atomicAdd(&dbar[lo], db);
        atomicAdd(&cbar[lo], cb);
    }
}

// reverse of the fz seeds: g_t = (gp/(y+d+ic) - gm/(y-d+ic)) / (2 pi), with
// adjoint w (real) per term
__global__ void k_adj_eval_reverse(const EvalDev* ev, int nt, double w, const int* pkeys, const cd* pvals,
                                   const long long* poff, const int* pcnt, cd* pbar, double* ybar, double* dbar,
                                   double* cbar)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const EvalDev& E = ev[t];
    const cd vb = mce::mkcd(w, 0);
    cd gp = mce::mkcd(1, 0), gm = mce::mkcd(1, 0);
    long long ip = -1, im = -1;
    int cjp = 0, cjm = 0;
    if (!E.first) {
        gp = lookup_idx(pkeys, pvals, poff[E.parent], pcnt[E.parent], E.lp ^ E.enc_lhp, E.phc, &ip, &cjp);
        gm = lookup_idx(pkeys, pvals, poff[E.parent], pcnt[E.parent], E.lm ^ E.enc_lhp, E.phc, &im, &cjm);
    }
    const double S = mce::kTwoPiInv;
    const cd Dp = mce::mkcd(E.y + E.d, E.c), Dm = mce::mkcd(E.y - E.d, E.c);
    const cd ip_ = mce::cdiv(mce::mkcd(1, 0), Dp), im_ = mce::cdiv(mce::mkcd(1, 0), Dm);
    if (ip >= 0) {
        cd a = mce::cmul(mce::cconj(mce::cscale(ip_, S)), vb);
        atomic_add_cd(&pbar[ip], cjp ? mce::cconj(a) : a);
    }
    if (im >= 0) {
        cd a = mce::cmul(mce::cconj(mce::cscale(im_, -S)), vb);
        atomic_add_cd(&pbar[im], cjm ? mce::cconj(a) : a);
    }
    const cd tp = mce::cmul(gp, mce::cmul(ip_, ip_)), tm = mce::cmul(gm, mce::cmul(im_, im_));
    const cd vy = mce::cscale(mce::csub(tm, tp), S);
    const cd vd = mce::cscale(mce::cadd(tp, tm), -S);
    ybar[t] = vb.re * vy.re + vb.im * vy.im;
    dbar[t] = vb.re * vd.re + vb.im * vd.im;
    cbar[t] = vb.re * (-vy.im) + vb.im * vy.re;
}

// the real part of fz from the recorded lookups (a check of the eval tape)
__global__ void k_adj_eval_fz(const EvalDev* ev, int nt, const int* pkeys, const cd* pvals, const long long* poff,
                              const int* pcnt, double* fz_re)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const EvalDev& E = ev[t];
    cd gp = mce::mkcd(1, 0), gm = mce::mkcd(1, 0);
    long long ip, im;
    int cj;
    if (!E.first) {
        gp = lookup_idx(pkeys, pvals, poff[E.parent], pcnt[E.parent], E.lp ^ E.enc_lhp, E.phc, &ip, &cj);
        gm = lookup_idx(pkeys, pvals, poff[E.parent], pcnt[E.parent], E.lm ^ E.enc_lhp, E.phc, &im, &cj);
    }
    const cd g = gval(gp, gm, E.y, E.d, E.c, mce::kTwoPiInv);
    fz_re[t] = g.re;
}

// ---------------------------------------------------------------------------
// The record chain on the GPU: one thread per (parent, parameter direction)
// re-derives the parent's post-MU terms in forward-mode dual numbers (the
// host derivation's arithmetic, so the same values and branches), dots the
// tangents of the scalars that enter the g values with their adjoints, and
// passes the tangents of the kept terms' records to the next update.

struct DD {
    double v, t;
};
__device__ inline DD dd(double v) { return DD{v, 0.0}; }
__device__ inline DD dadd(DD a, DD b) { return DD{a.v + b.v, a.t + b.t}; }
__device__ inline DD dsub(DD a, DD b) { return DD{a.v - b.v, a.t - b.t}; }
__device__ inline DD dneg(DD a) { return DD{-a.v, -a.t}; }
__device__ inline DD dmul(DD a, DD b) { return DD{a.v * b.v, a.t * b.v + a.v * b.t}; }
__device__ inline DD ddiv(DD a, DD b)
{
    const double q = a.v / b.v;
    return DD{q, (a.t - q * b.t) / b.v};
}
// a / b with rb = 1 / b.v: the value divides (the same double as the
// forward run), the tangent multiplies by the shared reciprocal (a row
// normalised by one norm divides d values by it)
__device__ inline DD ddiv_r(DD a, DD b, double rb)
{
    const double q = a.v / b.v;
    return DD{q, (a.t - q * b.t) * rb};
}
__device__ inline DD dabs(DD x) { return x.v < 0 ? dneg(x) : (x.v > 0 ? x : DD{0.0, 0.0}); }

// The record chain's limits: at most kGammaMax process-noise columns; a
// kernel instantiation per state dimension D and row capacity MR (16, or 32
// for records of 17 to 31 rows), so a thread's arrays are sized to the run.
constexpr int kGammaMax = 8;

struct ChainArgs {
    int d, pncc, p, MS, N, first, last, with_tp, sub, nP;
    double z;
    const double *beta, *gamma, *p0, *Phi, *Gamma, *H, *A0, *b0;
    // parents: kept records of the previous update (values), padded to MS rows
    const double *PA, *Pp, *Pb;
    const int* Pm;
    // tangents: [dir][slot][MS*d + MS + d]
    const double* Tin;
    double* Tout;
    int rec;  // MS*d + MS + d
    int n_next;
    const int* kid_off;  // per parent: term index of its first child
    const unsigned *sneg, *hpre;
    const double *ybar_e, *dbar_e, *cbar_e;
    const double *qbar_t, *dbar_t, *cbar_t;  // member adjoints per term
    const int* kept_of;
    double* grad;
};

__device__ inline int dgate(const DD* r, const DD* c, int d)
{
    bool pos = true, ng = true;
    for (int l = 0; l < d; l++) {
        if (pos) pos &= fabs(r[l].v - c[l].v) < kCoalignEps;
        if (ng) ng &= fabs(r[l].v + c[l].v) < kCoalignEps;
        if (!(pos || ng)) break;
    }
    return pos ? 1 : (ng ? -1 : 0);
}

template <int D, int MR>
__global__ void __launch_bounds__(128) k_adj_chain(ChainArgs a)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)a.nP * a.N) return;
    const int pi = (int)(idx % a.nP), dir = (int)(idx / a.nP);
    constexpr int d = D;
    const int offb = 0, offg = offb + a.pncc, offp = offg + a.p, offPhi = offp + d, offG = offPhi + d * d,
              offH = offG + d * a.pncc;
    auto par = [&](const double* v, int i, int off) { return DD{v[i], dir == off + i ? 1.0 : 0.0}; };
    // the parent's record; A then holds the MU's mu rows (m + 1 of them) and
    // P its rho values
    DD A[(MR + 1) * D], P[MR + 1], B[D];
    int m;
    if (a.first) {
        m = d;
        for (int i = 0; i < d * d; i++) A[i] = dd(a.A0[i]);
        for (int i = 0; i < d; i++) P[i] = par(a.p0, i, offp);
        for (int i = 0; i < d; i++) B[i] = dd(a.b0[i]);
    } else {
        m = a.Pm[pi];
        const double* tin = a.Tin + ((size_t)dir * a.nP + pi) * a.rec;
        for (int i = 0; i < m * d; i++) A[i] = DD{a.PA[(size_t)pi * a.MS * d + i], tin[i]};
        for (int i = 0; i < m; i++) P[i] = DD{a.Pp[(size_t)pi * a.MS + i], tin[a.MS * d + i]};
        for (int i = 0; i < d; i++) B[i] = DD{a.Pb[(size_t)pi * d + i], tin[a.MS * d + a.MS + i]};
    }
    if (a.with_tp) {
        // Gamma pre-coalignment
        DD Gt[kGammaMax * D], bt[kGammaMax];
        const int pncc = a.pncc;
        for (int i = 0; i < pncc; i++) {
            for (int j = 0; j < d; j++) Gt[i * d + j] = par(a.Gamma, j * pncc + i, offG);
            bt[i] = par(a.beta, i, offb);
        }
        for (int i = 0; i < pncc; i++) {
            DD nf = dd(0.0);
            for (int j = 0; j < d; j++) nf = dadd(nf, dabs(Gt[i * d + j]));
            const double rnf = 1.0 / nf.v;
            for (int j = 0; j < d; j++) Gt[i * d + j] = ddiv_r(Gt[i * d + j], nf, rnf);
            bt[i] = dmul(bt[i], nf);
        }
        bool F[kGammaMax];
        for (int i = 0; i < pncc; i++) F[i] = true;
        for (int i = 0; i < pncc - 1; i++)
            if (F[i])
                for (int j = i + 1; j < pncc; j++)
                    if (F[j] && dgate(&Gt[i * d], &Gt[j * d], d) != 0) {
                        F[j] = false;
                        bt[i] = dadd(bt[i], bt[j]);
                    }
        int cnt = 0;
        for (int i = 0; i < pncc; i++) cnt += F[i];
        if (cnt != pncc) {
            int u = 1;
            for (int j = 1; j < pncc; j++)
                if (F[j]) {
                    if (u < j) {
                        for (int l = 0; l < d; l++) Gt[u * d + l] = Gt[j * d + l];
                        bt[u] = bt[j];
                    }
                    u++;
                }
        }
        // time_prop, a row at a time
        for (int i = 0; i < m; i++) {
            DD w[D];
            for (int k = 0; k < d; k++) w[k] = A[i * d + k];
            for (int j = 0; j < d; j++) {
                DD sum = dd(0.0);
                for (int k = 0; k < d; k++) sum = dadd(sum, dmul(w[k], par(a.Phi, k + j * d, offPhi)));
                A[i * d + j] = sum;
            }
        }
        DD wb[D];
        for (int i = 0; i < d; i++) wb[i] = B[i];
        for (int i = 0; i < d; i++) {
            DD sum = dd(0.0);
            for (int j = 0; j < d; j++) sum = dadd(sum, dmul(par(a.Phi, i * d + j, offPhi), wb[j]));
            B[i] = sum;
        }
        // tp_coalign
        for (int i = 0; i < m; i++) {
            DD n1 = dd(0.0);
            for (int j = 0; j < d; j++) n1 = dadd(n1, dabs(A[i * d + j]));
            P[i] = dmul(P[i], n1);
            const double rn1 = 1.0 / n1.v;
            for (int j = 0; j < d; j++) A[i * d + j] = ddiv_r(A[i * d + j], n1, rn1);
        }
        bool Fg[kGammaMax];
        for (int j = 0; j < cnt; j++) Fg[j] = true;
        for (int j = 0; j < cnt; j++)
            for (int k = 0; k < m; k++)
                if (Fg[j] && dgate(&Gt[j * d], &A[k * d], d) != 0) {
                    Fg[j] = false;
                    P[k] = dadd(P[k], bt[j]);
                }
        for (int j = 0; j < cnt; j++)
            if (Fg[j]) {
                for (int l = 0; l < d; l++) A[m * d + l] = Gt[j * d + l];
                P[m] = bt[j];
                m++;
            }
    }
    // measurement update
    const DD* H = nullptr;
    (void)H;
    DD Hr[D];
    for (int j = 0; j < d; j++) Hr[j] = par(a.H, a.sub * d + j, offH);
    const DD gam = par(a.gamma, a.sub, offg);
    DD* mu = A;   // the rows, scaled in place
    DD* rho = P;  // rho_l from p_l, in place
    bool Fi[MR + 1];
    rho[m] = gam;
    for (int j = 0; j < d; j++) mu[m * d + j] = dd(0.0);
    Fi[m] = true;
    for (int l = 0; l < m; l++) {
        DD h = dd(0.0);
        for (int j = 0; j < d; j++) h = dadd(h, dmul(Hr[j], mu[l * d + j]));
        if (fabs(h.v) < kMuEps) {
            Fi[l] = false;  // rho_l = p_l
        } else {
            const DD r = ddiv(dd(1.0), h);
            for (int j = 0; j < d; j++) mu[l * d + j] = dmul(mu[l * d + j], r);
            rho[l] = dmul(P[l], dabs(h));
            Fi[l] = true;
        }
    }
    DD hb = dd(0.0);
    for (int j = 0; j < d; j++) hb = dadd(hb, dmul(Hr[j], B[j]));
    const DD zeta = dsub(dd(a.z), hb);
    double g = 0.0;
    int kid = 0;
    for (int tt = 0; tt <= m; tt++) {
        if (!Fi[tt]) continue;
        const int term = tt == m ? pi : a.kid_off[pi] + kid++;
        DD cA[MR * D], cp[MR], cq[MR], cb[D];
        const DD cc = zeta, cd_ = rho[tt];
        for (int j = 0; j < d; j++) cb[j] = dadd(B[j], dmul(zeta, mu[tt * d + j]));
        int l = 0;
        unsigned hof = 0;
        for (int ll = 0; ll <= m; ll++) {
            if (ll == tt) continue;
            cp[l] = rho[ll];
            if (Fi[ll])
                for (int j = 0; j < d; j++) cA[l * d + j] = dsub(mu[ll * d + j], mu[tt * d + j]);
            else {
                for (int j = 0; j < d; j++) cA[l * d + j] = mu[ll * d + j];
                hof |= 1u << l;
            }
            l++;
        }
        // the fz seed's scalars (before coalignment)
        {
            const unsigned sn = a.sneg[term], hp = a.hpre[term];
            double yt = 0;
            for (int r = 0; r < m; r++)
                if (!((hp >> r) & 1)) yt += cp[r].t * (((sn >> r) & 1) ? -1.0 : 1.0);
            g += a.ybar_e[term] * yt + a.dbar_e[term] * cd_.t + a.cbar_e[term] * cc.t;
        }
        // coalignment (the parent only normalises; nothing at the first and last update)
        int mm = m;
        unsigned horth = hof;
        for (int r = 0; r < m; r++) cq[r] = cp[r];
        if (!a.first && !a.last) {
            for (int i = 0; i < m; i++) {
                DD n1 = dd(0.0);
                for (int j = 0; j < d; j++) n1 = dadd(n1, dabs(cA[i * d + j]));
                cp[i] = dmul(cp[i], n1);
                const double rn1 = 1.0 / n1.v;
                for (int j = 0; j < d; j++) cA[i * d + j] = ddiv_r(cA[i * d + j], n1, rn1);
            }
            if (tt != m) {
                bool F[MR], hflag[MR];
                for (int j = 0; j < m; j++) {
                    F[j] = true;
                    hflag[j] = horth ? ((horth >> j) & 1) : false;
                }
                for (int j = 0; j < m - 1; j++) {
                    if (!F[j]) continue;
                    for (int k = j + 1; k < m; k++) {
                        if (!F[k]) continue;
                        const int gt = dgate(&cA[j * d], &cA[k * d], d);
                        if (gt == 1) {
                            if (horth) {
                                const bool hj = hflag[j], hk = hflag[k];
                                if (!hj && !hk) cq[j] = dadd(cq[j], cq[k]);
                                else if (hj && !hk) {
                                    cq[j] = cq[k];
                                    hflag[j] = false;
                                } else if (!hj && hk) hflag[k] = false;
                                else {
                                    hflag[k] = false;
                                    cq[j] = dadd(cq[j], cq[k]);
                                }
                            } else
                                cq[j] = dadd(cq[j], cq[k]);
                            F[k] = false;
                            cp[j] = dadd(cp[j], cp[k]);
                        } else if (gt == -1) {
                            if (horth) {
                                const bool hj = hflag[j], hk = hflag[k];
                                if (!hj && !hk) cq[j] = dsub(cq[j], cq[k]);
                                else if (hj && !hk) {
                                    cq[j] = dneg(cq[k]);
                                    hflag[j] = false;
                                } else if (!hj && hk) hflag[k] = false;
                            } else
                                cq[j] = dsub(cq[j], cq[k]);
                            F[k] = false;
                            cp[j] = dadd(cp[j], cp[k]);
                        }
                    }
                }
                int ns = 0;
                for (int i = 0; i < m; i++) ns += F[i];
                if (ns != m) {
                    int u = 1;
                    for (int j = 1; j < m; j++)
                        if (F[j]) {
                            if (u < j) {
                                for (int l2 = 0; l2 < d; l2++) cA[u * d + l2] = cA[j * d + l2];
                                cp[u] = cp[j];
                                cq[u] = cq[j];
                            }
                            u++;
                        }
                    mm = ns;
                }
            }
        }
        // the g-table's scalars (after coalignment)
        {
            const double* qb = a.qbar_t + (size_t)term * 32;
            for (int k = 0; k < mm; k++) g += qb[k] * cq[k].t;
            g += a.dbar_t[term] * cd_.t + a.cbar_t[term] * cc.t;
        }
        // a kept term hands its record's tangents to the next update
        const int slot = a.kept_of ? a.kept_of[term] : -1;
        if (slot >= 0) {
            double* tout = a.Tout + ((size_t)dir * a.n_next + slot) * a.rec;
            for (int i = 0; i < mm * d; i++) tout[i] = cA[i].t;
            for (int i = 0; i < mm; i++) tout[a.MS * d + i] = cp[i].t;
            for (int i = 0; i < d; i++) tout[a.MS * d + a.MS + i] = cb[i].t;
        }
    }
    atomicAdd(&a.grad[dir], g);
}

template <int D>
void launch_chain_d(const ChainArgs& ca, long long nthr, cudaStream_t s)
{
    const int grid = (int)((nthr + 127) / 128);
    if (ca.MS <= 16) k_adj_chain<D, 16><<<grid, 128, 0, s>>>(ca);
    else k_adj_chain<D, 32><<<grid, 128, 0, s>>>(ca);
}

// The record chain of one update: a thread per (parent, direction).
void launch_chain(const ChainArgs& ca, long long nthr, cudaStream_t s)
{
    switch (ca.d) {
    case 2: launch_chain_d<2>(ca, nthr, s); break;
    case 3: launch_chain_d<3>(ca, nthr, s); break;
    case 4: launch_chain_d<4>(ca, nthr, s); break;
    case 5: launch_chain_d<5>(ca, nthr, s); break;
    case 6: launch_chain_d<6>(ca, nthr, s); break;
    case 7: launch_chain_d<7>(ca, nthr, s); break;
    default: launch_chain_d<8>(ca, nthr, s); break;
    }
}

// ---------------------------------------------------------------------------
// Device buffers (grow-only, half again as large as asked when they grow)
// and the per-thread workspace that holds them.

template <class T>
struct Buf {
    T* ptr = nullptr;
    size_t cap = 0;
    Buf() = default;
    Buf(const Buf&) = delete;
    Buf& operator=(const Buf&) = delete;
    ~Buf()
    {
        if (ptr) cudaFree(ptr);
    }
    // s: the stream that may still read the old buffer (finished first)
    int ensure(size_t n, cudaStream_t s)
    {
        if (n <= cap) return MCE_OK;
        if (ptr) {
            cudaStreamSynchronize(s);
            cudaFree(ptr);
        }
        ptr = nullptr;
        const size_t want = std::max<size_t>(std::max<size_t>(n, 1), cap + cap / 2);
        cap = 0;
        if (cudaMalloc(&ptr, sizeof(T) * want) != cudaSuccess) {
            cudaGetLastError();
            ptr = nullptr;
            mce::report_error("adjoint: device allocation failed");
            return MCE_ERR_NOMEM;
        }
        cap = want;
        return MCE_OK;
    }
    // host -> device on stream s (the host buffer may be reused on return:
    // pageable sources are staged before the call returns)
    int upload(const T* src, size_t n, cudaStream_t s)
    {
        int st = ensure(n, s);
        if (st) return st;
        if (n && cudaMemcpyAsync(ptr, src, sizeof(T) * n, cudaMemcpyHostToDevice, s) != cudaSuccess) {
            mce::report_error("adjoint: host-to-device copy failed");
            return MCE_ERR_CUDA;
        }
        return MCE_OK;
    }
    int zero(size_t n, cudaStream_t s)
    {
        int st = ensure(std::max<size_t>(n, 1), s);
        if (st) return st;
        return cudaMemsetAsync(ptr, 0, sizeof(T) * std::max<size_t>(n, 1), s) == cudaSuccess ? MCE_OK : MCE_ERR_CUDA;
    }
    void swap(Buf& o)
    {
        std::swap(ptr, o.ptr);
        std::swap(cap, o.cap);
    }
};

// device -> host on stream s, waited for
template <class T>
int download(T* dst, const T* src, size_t n, cudaStream_t s)
{
    if (n == 0) return MCE_OK;
    if (cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        mce::report_error("adjoint: device-to-host copy failed");
        return MCE_ERR_CUDA;
    }
    return MCE_OK;
}

// Everything one host thread needs on the device to record or reverse runs,
// on its own stream, kept from run to run so that nothing is allocated once
// the sizes have settled.
struct Workspace {
    cudaStream_t s = nullptr;
    // the parent tables (keys, values, offsets, cell counts) and whose they
    // are: run `owner`'s kept tables after its update owner_u
    Buf<int> pk, pcnt;
    Buf<cd> pv;
    Buf<long long> poff;
    const void* owner = nullptr;
    int owner_u = -1;
    // the kept tables of the update being recorded or reversed
    Buf<int> dk, dcnt;
    Buf<cd> dv;
    Buf<long long> doff;
    Buf<MInfoDev> dmi;
    Buf<long long> ditem, dkfirst;
    Buf<cd> dvals, kbar, pbar;
    Buf<int> dalive, dcontrib, dknm;
    Buf<unsigned long long> derr;
    Buf<EvalDev> dev;
    Buf<double> dfz, qbar, dbar, cbar, ybar_e, dbar_e, cbar_e;
    // the record chain
    Buf<double> tin, tout, dgrad, dPA, dPp, dPb, dyb, ddb, dcb, dqt, ddt, dct;
    Buf<double> dpar[8];
    Buf<int> dPm, dkid, dkept;
    Buf<unsigned> dsn, dhp;
    int init()
    {
        if (s) return MCE_OK;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            s = nullptr;
            mce::report_error("adjoint: stream creation failed");
            return MCE_ERR_CUDA;
        }
        return MCE_OK;
    }
    ~Workspace()
    {
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }
};

// A dumped set of kept terms with their g-tables.
struct Tables {
    int nt = 0;
    std::vector<int> shape, cells;
    std::vector<double> A, p, b;  // A nt x MS x d, p nt x MS
    std::vector<int> keys;
    std::vector<cd> vals;
    std::vector<long long> off;
};

struct Update {
    bool first = false, last = false, with_tp = false;
    int sub = 0;  // measurement index within the step
    double gscale = 0, fz_raw = 0;
    std::vector<TermInfo> terms;    // post-MU terms in creation order
    std::vector<Member> members;    // contributing candidates, grouped by kept slot
    std::vector<int> kept_first, kept_n;  // per kept term: its first member and count
    std::vector<int> kept_term;     // per kept term: the post-MU term that is its record
    Tables kept;                    // the dump after this update
    std::vector<MInfoDev> mi;       // GPU view of the members
    std::vector<long long> item_off;
    // adjoints gathered by the reverse pass
    std::vector<double> qbar;       // per member: 32 rows
    std::vector<double> dbar_m, cbar_m;
    std::vector<double> ybar_e, dbar_e, cbar_e;  // per post-MU term (fz seeds)
};

}  // namespace

// ---------------------------------------------------------------------------

struct mce_adjoint {
    int d = 0, pncc = 0, p = 0, steps = 0, MS = 0;
    std::vector<double> A0, p0, b0, root, bpert;
    mce_handle* h = nullptr;
    int est = 0;          // this run's estimator in h
    bool owns_h = true;   // false for the runs of an mce_adjoint_batch
    // model and measurements of the recorded run; Phi is d x d, or with ltv
    // one d x d matrix per step (the gradient's Phi entries are then those
    // of a perturbation common to every step's Phi)
    std::vector<double> Phi, Gamma, beta, H, gamma, msmts;
    bool ltv = false;
    // measurement index of the first update (0; p - 1 for a window restarted
    // with the last measurement of its step, whose master step then jumps to
    // p): update u is measurement (u + first_sub) % p of step
    // (u + first_sub) / p, and the run has steps * p - first_sub updates
    int first_sub = 0;
    std::vector<Update> ups;
    double max_table_err = 0;
    double fz_check_err = 0;
    // wall ms: forward step path, forward tape (host records + GPU checks),
    // reverse over the tables (GPU), record chain (GPU)
    double ms[4] = {0, 0, 0, 0};
    // the records of the update being recorded: its parents (the previous
    // update's kept terms), every post-MU term, the next parents
    RecSet parents, post, next;
    std::unique_ptr<Workspace> ws;  // the single-run calls' workspace

    ~mce_adjoint()
    {
        ws.reset();
        if (h && owns_h) mce_destroy(h);
    }

    int dump(Tables& T)
    {
        T.nt = (int)mce_num_terms(h, est);
        const long long tot = mce_total_cells(h, est);
        if (T.nt < 0 || tot < 0) return MCE_ERR_ARG;
        T.shape.assign(T.nt, 0);
        T.cells.assign(T.nt, 0);
        T.A.assign((size_t)T.nt * MS * d, 0);
        T.p.assign((size_t)T.nt * MS, 0);
        T.b.assign((size_t)T.nt * d, 0);
        T.keys.assign(std::max<long long>(tot, 1), 0);
        std::vector<double> g(2 * std::max<long long>(tot, 1));
        const int st = mce_dump_terms(h, est, MS, T.shape.data(), T.A.data(), T.p.data(), T.b.data(), T.cells.data(),
                                      T.keys.data(), g.data());
        if (st < 0) return st;
        T.vals.resize(std::max<long long>(tot, 1));
        for (long long i = 0; i < tot; i++) T.vals[i] = mce::mkcd(g[2 * i], g[2 * i + 1]);
        T.off.assign(T.nt + 1, 0);
        for (int t = 0; t < T.nt; t++) T.off[t + 1] = T.off[t] + T.cells[t];
        return MCE_OK;
    }
};

namespace {

// The Phi of update u's time propagation (of its step, u / p).
const double* phi_of(const mce_adjoint& o, int u)
{
    return o.ltv ? o.Phi.data() + (size_t)((u + o.first_sub) / o.p) * o.d * o.d : o.Phi.data();
}

// Gamma pre-coalignment (cauchy_util.hpp:128-210): normalised columns as rows
int precoalign(const mce_adjoint& o, const std::vector<double>& G, const std::vector<double>& beta,
               std::vector<double>& Gt, std::vector<double>& bt)
{
    const int d = o.d, pncc = o.pncc;
    Gt.assign((size_t)pncc * d, 0.0);
    bt.assign(pncc, 0.0);
    for (int i = 0; i < pncc; i++) {
        for (int j = 0; j < d; j++) Gt[i * d + j] = G[j * pncc + i];
        bt[i] = beta[i];
    }
    for (int i = 0; i < pncc; i++) {
        double nf = 0.0;
        for (int j = 0; j < d; j++) nf += std::fabs(Gt[i * d + j]);
        for (int j = 0; j < d; j++) Gt[i * d + j] /= nf;
        bt[i] *= nf;
    }
    std::vector<char> F(pncc, 1);
    for (int i = 0; i < pncc - 1; i++)
        if (F[i])
            for (int j = i + 1; j < pncc; j++)
                if (F[j] && gate(&Gt[i * d], &Gt[j * d], d) != 0) {
                    F[j] = 0;
                    bt[i] += bt[j];
                }
    int cnt = 0;
    for (int i = 0; i < pncc; i++) cnt += F[i];
    if (cnt != pncc) {
        int u = 1;
        for (int j = 1; j < pncc; j++)
            if (F[j]) {
                if (u < j) {
                    for (int l = 0; l < d; l++) Gt[u * d + l] = Gt[j * d + l];
                    bt[u] = bt[j];
                }
                u++;
            }
    }
    return cnt;
}

// mu_coalign (cauchy_term.hpp:533-745) in place on a normalised record of m
// rows (A, p, q, its orthogonal-row mask *horthog); returns the rows left and
// fills cmap / csmap (row -> kept row, sign).
int mu_coalign_rows(double* A, double* p, double* q, unsigned* horthog, int m, int d, int* cmap, int* csmap)
{
    char F[kRowsMax], hflag[kRowsMax];
    for (int j = 0; j < m; j++) {
        F[j] = 1;
        hflag[j] = *horthog ? (char)((*horthog >> j) & 1) : 0;
        cmap[j] = 255;
        csmap[j] = 1;
    }
    const bool ho = *horthog != 0;
    int uc = 0;
    for (int j = 0; j < m - 1; j++) {
        if (!F[j]) continue;
        cmap[j] = uc;
        for (int k = j + 1; k < m; k++) {
            if (!F[k]) continue;
            const int g = gate(&A[j * d], &A[k * d], d);
            if (g == 1) {
                if (ho) {
                    const bool hj = hflag[j], hk = hflag[k];
                    if (!hj && !hk) q[j] += q[k];
                    else if (hj && !hk) {
                        q[j] = q[k];
                        hflag[j] = 0;
                    } else if (!hj && hk) hflag[k] = 0;
                    else {
                        hflag[k] = 0;
                        q[j] += q[k];
                    }
                } else
                    q[j] += q[k];
                F[k] = 0;
                p[j] += p[k];
                cmap[k] = uc;
                csmap[k] = 1;
            } else if (g == -1) {
                if (ho) {
                    const bool hj = hflag[j], hk = hflag[k];
                    if (!hj && !hk) q[j] -= q[k];
                    else if (hj && !hk) {
                        q[j] = -q[k];
                        hflag[j] = 0;
                    } else if (!hj && hk) hflag[k] = 0;
                } else
                    q[j] -= q[k];
                F[k] = 0;
                p[j] += p[k];
                cmap[k] = uc;
                csmap[k] = -1;
            }
        }
        uc++;
    }
    if (F[m - 1]) cmap[m - 1] = uc;
    int ns = 0;
    for (int i = 0; i < m; i++) ns += F[i];
    if (ns != m) {
        int u = 1;
        for (int j = 1; j < m; j++)
            if (F[j]) {
                if (u < j) {
                    for (int l2 = 0; l2 < d; l2++) A[u * d + l2] = A[j * d + l2];
                    p[u] = p[j];
                    q[u] = q[j];
                }
                u++;
            }
        if (ho) {
            unsigned nh = 0;
            int cc = 0;
            for (int j = 0; j < m; j++)
                if (F[j]) nh |= (unsigned)hflag[j] << cc++;
            *horthog = nh;
        }
    }
    return ns;
}

// One update's record derivation (the host half of step_first / step_rest,
// include/cauchy_estimator.hpp:604-832, 1179-1208): from the kept records of
// the previous update to every post-MU term's record after MU coalignment,
// in creation order (the parents' own terms, then the children: step_first
// keeps [parent, children] and step_rest lists the parents, then the
// children).  info[t] keeps what the tape needs of the record before
// coalignment (its g-value scalars, root-point signs and lookup keys).
void derive_update(const mce_adjoint& o, const Update& U, const RecSet& parents, RecSet& post,
                   std::vector<TermInfo>& info)
{
    const int d = o.d;
    const double* Phi = phi_of(o, (int)(&U - &o.ups[0]));
    std::vector<double> Gt, bt;
    int gcnt = 0;
    if (U.with_tp) gcnt = precoalign(o, o.Gamma, o.beta, Gt, bt);
    const double* H = o.H.data() + (size_t)U.sub * d;
    const double gam = o.gamma[U.sub];
    const double z = o.msmts[(size_t)(&U - &o.ups[0])];
    const int nPar = parents.n;
    post.init(o.MS, d);
    post.ensure(nPar);
    post.n = nPar;  // the parents' own terms come first, one per parent
    info.clear();
    info.resize(nPar);
    double tA[kRowsMax * kDMax], tp_[kRowsMax], tb[kDMax], w[kRowsMax * kDMax], wb[kDMax];
    double mu[(kRowsMax + 1) * kDMax], rho[kRowsMax + 1];
    int sgn[kRowsMax];
    char Fi[kRowsMax + 1];
    for (int pi = 0; pi < nPar; pi++) {
        int tm = parents.m[pi];
        memcpy(tA, parents.Ar(pi), sizeof(double) * tm * d);
        memcpy(tp_, parents.pr(pi), sizeof(double) * tm);
        memcpy(tb, parents.br(pi), sizeof(double) * d);
        const int phc = U.first ? 0 : tm;  // the parent's table is over its rows before time propagation
        if (U.with_tp) {
            // time_prop: A <- A Phi^T, b <- Phi b (cauchy_term.hpp:435-456)
            memcpy(w, tA, sizeof(double) * tm * d);
            for (int i = 0; i < tm; i++)
                for (int j = 0; j < d; j++) {
                    double s = 0.0;
                    for (int k = 0; k < d; k++) s += w[i * d + k] * Phi[k + j * d];
                    tA[i * d + j] = s;
                }
            memcpy(wb, tb, sizeof(double) * d);
            for (int i = 0; i < d; i++) {
                double s = 0.0;
                for (int j = 0; j < d; j++) s += Phi[i * d + j] * wb[j];
                tb[i] = s;
            }
            // tp_coalign (cauchy_term.hpp:475-531)
            normalize_rows(tA, tp_, nullptr, tm, d);
            char F[kRowsMax];
            for (int j = 0; j < gcnt; j++) F[j] = 1;
            for (int j = 0; j < gcnt; j++)
                for (int k = 0; k < tm; k++)
                    if (F[j] && gate(&Gt[j * d], &tA[k * d], d) != 0) {
                        F[j] = 0;
                        tp_[k] += bt[j];
                    }
            for (int j = 0; j < gcnt; j++)
                if (F[j]) {
                    for (int l = 0; l < d; l++) tA[tm * d + l] = Gt[j * d + l];
                    tp_[tm] = bt[j];
                    tm++;
                }
        }
        // msmt_update (cauchy_term.hpp:84-310)
        const int m = tm;
        for (int i = 0; i < m * d; i++) mu[i] = tA[i];
        for (int i = 0; i < m; i++) rho[i] = tp_[i];
        rho[m] = gam;
        for (int j = 0; j < d; j++) mu[m * d + j] = 0.0;
        Fi[m] = 1;
        for (int l = 0; l < m; l++) {
            double h = 0.0;
            for (int j = 0; j < d; j++) h += H[j] * mu[l * d + j];
            if (std::fabs(h) < kMuEps) {
                rho[l] = tp_[l];
                sgn[l] = 1;
                Fi[l] = 0;
            } else {
                const double r = 1.0 / h;
                for (int j = 0; j < d; j++) mu[l * d + j] *= r;
                rho[l] = tp_[l] * std::fabs(h);
                sgn[l] = h > 0 ? 1 : -1;
                Fi[l] = 1;
            }
        }
        double hb = 0.0;
        for (int j = 0; j < d; j++) hb += H[j] * tb[j];
        const double zeta = z - hb;
        int esg = 0;
        for (int l = 0; l < m; l++)
            if (sgn[l] == -1) esg |= 1 << l;
        int lhp = esg;
        if (phc < m) lhp &= (1 << phc) - 1;
        for (int tt = 0; tt <= m; tt++) {
            if (!Fi[tt]) continue;
            // the MU output, written into the term's slot
            const int slot = tt == m ? pi : post.add();
            double* cA = post.Ar(slot);
            double* cp = post.pr(slot);
            double* cq = post.qr(slot);
            double* cb = post.br(slot);
            post.m[slot] = m;
            post.c[slot] = zeta;
            post.dv[slot] = rho[tt];
            for (int j = 0; j < d; j++) cb[j] = tb[j] + zeta * mu[tt * d + j];
            int l = 0;
            unsigned hof = 0;
            for (int ll = 0; ll <= m; ll++) {
                if (ll == tt) continue;
                cp[l] = rho[ll];
                if (Fi[ll])
                    for (int j = 0; j < d; j++) cA[l * d + j] = mu[ll * d + j] - mu[tt * d + j];
                else {
                    for (int j = 0; j < d; j++) cA[l * d + j] = mu[ll * d + j];
                    hof |= 1u << l;
                }
                l++;
            }
            post.horthog[slot] = hof;
            TermInfo ti;
            ti.parent = U.first ? -1 : pi;
            ti.m_pre = m;
            ti.phc = phc;
            ti.z = tt;
            ti.enc_lhp = U.first ? 0 : lhp;
            ti.new_child = (tt != m) && !U.first;
            ti.horthog_pre = hof;
            // eval_g_yei at the root point (signs of the rows before coalignment)
            double y = 0;
            unsigned sneg = 0;
            for (int ll = 0; ll < m; ll++) {
                double s = 0.0;
                for (int j = 0; j < d; j++) s += cA[ll * d + j] * o.root[j];
                if (!(s > 0)) sneg |= 1u << ll;
            }
            if (hof) {
                for (int ll = 0; ll < m; ll++)
                    if (!(hof & (1u << ll))) y += cp[ll] * (((sneg >> ll) & 1) ? -1.0 : 1.0);
            } else {
                double zz = 0.0;
                for (int ll = 0; ll < m; ll++) zz += cp[ll] * (((sneg >> ll) & 1) ? -1.0 : 1.0);
                y = zz;
            }
            ti.y_eval = y;
            ti.sneg = sneg;
            ti.d_eval = rho[tt];
            ti.c_eval = zeta;
            if (!U.first) {
                int lp = 0, lm = 0, k = 0;
                for (int ll = 0; ll < m; ll++) {
                    if (k < phc) {
                        if (k == tt) {
                            lm |= 1 << k;
                            k++;
                            if (k == phc) continue;
                        }
                        if ((sneg >> ll) & 1) {
                            lp |= 1 << k;
                            lm |= 1 << k;
                        }
                        k++;
                    }
                }
                ti.lp = lp;
                ti.lm = lm;
            } else {
                ti.lp = ti.lm = -1;
            }
            // MU coalignment in place (the parent's own term only normalises)
            if (U.first || U.last) {
                memcpy(cq, cp, sizeof(double) * m);
                ti.m = m;
                ti.horthog = hof;
                ti.has_cmap = false;
            } else if (tt == m) {
                normalize_rows(cA, cp, cq, m, d);
                ti.m = m;
                ti.horthog = hof;
                ti.has_cmap = false;
            } else {
                normalize_rows(cA, cp, cq, m, d);
                int cmap[kRowsMax], csmap[kRowsMax];
                const int ns = mu_coalign_rows(cA, cp, cq, &post.horthog[slot], m, d, cmap, csmap);
                post.m[slot] = ns;
                ti.m = ns;
                ti.horthog = post.horthog[slot];
                ti.has_cmap = ns < m;
                for (int j = 0; j < 32; j++) {
                    ti.cmap[j] = j < m ? cmap[j] : 0;
                    ti.csmap[j] = j < m ? csmap[j] : 1;
                }
            }
            if (tt == m)
                info[pi] = ti;
            else
                info.push_back(ti);
        }
    }
}

// orientation_mask (cell_enumeration.hpp:584-625)
int orientation_mask(const double* Ai, const double* Aj, int m, int d)
{
    int s = 0;
    for (int k = 0; k < m; k++) {
        int l = 0;
        while (l < d - 1 && ((std::fabs(Ai[k * d + l]) < kReductionEps) || (std::fabs(Aj[k * d + l]) < kReductionEps))) l++;
        if (Ai[k * d + l] * Aj[k * d + l] < 0) s |= 1 << k;
    }
    return s;
}

bool same_record(const RecSet& R, int t, const Tables& T, int k, int MS, int d)
{
    const int m = R.m[t];
    if (T.shape[k] != m) return false;
    const double* A = R.Ar(t);
    const double* p = R.pr(t);
    const double* b = R.br(t);
    for (int i = 0; i < m * d; i++)
        if (T.A[(size_t)k * MS * d + i] != A[i]) return false;
    for (int i = 0; i < m; i++)
        if (T.p[(size_t)k * MS + i] != p[i]) return false;
    for (int i = 0; i < d; i++)
        if (T.b[(size_t)k * d + i] != b[i]) return false;
    return true;
}

// fast_term_reduction (term_reduction.hpp:159-276) on one shape's terms
// (indices T into R, all of m rows): F[j] = the group root of T[j]'s position
void ftr(const RecSet& R, const std::vector<int>& T, int d, std::vector<int>& F)
{
    const int n = (int)T.size();
    F.resize(n);
    for (int i = 0; i < n; i++) F[i] = i;
    if (n == 0) return;
    const int m = R.m[T[0]];
    const double ep = kReductionEps;
    std::vector<int> ord(n);
    for (int i = 0; i < n; i++) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return R.br(T[a])[0] < R.br(T[b])[0]; });
    std::vector<double> v0(n);
    for (int i = 0; i < n; i++) v0[i] = R.br(T[ord[i]])[0];
    for (int i = 0; i < n; i++) {
        if (F[i] != i) continue;
        const double* bi = R.br(T[i]);
        const double* pi_ = R.pr(T[i]);
        const double* Ai = R.Ar(T[i]);
        const int s = (int)(std::upper_bound(v0.begin(), v0.end(), bi[0] - ep) - v0.begin());
        const int e = (int)(std::upper_bound(v0.begin(), v0.end(), bi[0] + ep) - v0.begin());
        for (int w = s; w < e; w++) {
            const int j = ord[w];
            if (j <= i || F[j] != j) continue;
            const double* bj = R.br(T[j]);
            const double* pj = R.pr(T[j]);
            const double* Aj = R.Ar(T[j]);
            bool ok = true;
            for (int a = 1; a < d && ok; a++)
                if (!(bj[a] > bi[a] - ep && bj[a] <= bi[a] + ep)) ok = false;
            for (int k = 0; k < m && ok; k++)
                if (std::fabs(pj[k] - pi_[k]) > ep) ok = false;
            for (int k = 0; k < m && ok; k++) {
                const double r = Ai[k], c = Aj[k];
                if (!(std::fabs(r - c) < ep || std::fabs(r + c) < ep)) ok = false;
            }
            if (ok) F[j] = i;
        }
    }
}

MInfoDev minfo_of(const TermInfo& ti, const RecSet& R, int t, const Member& mb, const Tables& kept, bool first)
{
    MInfoDev M;
    memset(&M, 0, sizeof(M));
    const int m = R.m[t];
    M.m = m;
    M.phc = ti.phc;
    M.z = ti.z;
    M.enc_lhp = ti.enc_lhp;
    M.flags = (ti.new_child ? kMiNewChild : 0) | (ti.has_cmap ? kMiHasCmap : 0) | (first ? kMiFirst : 0);
    M.horthog = (int)R.horthog[t];
    M.s_fixed = mb.s_fixed;
    M.conj = mb.conj;
    M.kept = mb.kept;
    M.parent = ti.parent < 0 ? 0 : ti.parent;
    M.term = mb.term;
    M.cell_off = kept.off[mb.kept];
    M.cell_cnt = kept.cells[mb.kept];
    M.d = R.dv[t];
    M.c = R.c[t];
    const double* p = R.pr(t);
    const double* q = R.qr(t);
    double ps = 0;
    for (int i = 0; i < m; i++) ps += p[i];
    M.ps2 = ps * ps;
    for (int k = 0; k < m; k++) M.q[k] = q[k];
    for (int k = 0; k < 32; k++) {
        M.cmap[k] = (signed char)ti.cmap[k];
        M.csmap[k] = (signed char)ti.csmap[k];
    }
    return M;
}

int grid_of(long long n) { return (int)std::min<long long>((n + 255) / 256, 152 * 32); }

// ---------------------------------------------------------------------------
// One run's forward record and reverse, on a workspace (its stream and
// buffers).  The GPU step of each update is the caller's: one mce_step of the
// run's own handle, or one mce_batch_step for every run of a batch.

// Copies the model and measurements of a run and resets its records.
int fwd_begin(mce_adjoint* o, const double* msmts, const double* Phi, const double* Gamma, const double* beta,
              const double* H, const double* gamma, bool ltv = false)
{
    const int d = o->d, nup = o->steps * o->p - o->first_sub;
    o->msmts.assign(msmts, msmts + nup);
    o->ltv = ltv;
    o->Phi.assign(Phi, Phi + (size_t)(ltv ? o->steps : 1) * d * d);
    o->Gamma.assign(Gamma, Gamma + d * o->pncc);
    o->beta.assign(beta, beta + o->pncc);
    o->H.assign(H, H + o->p * d);
    o->gamma.assign(gamma, gamma + o->p);
    o->ups.assign(nup, Update());
    o->max_table_err = 0;
    o->fz_check_err = 0;
    o->parents.init(o->MS, d);
    o->next.init(o->MS, d);
    o->parents.add();
    o->parents.m[0] = d;
    o->parents.horthog[0] = 0;
    o->parents.c[0] = o->parents.dv[0] = 0.0;
    memcpy(o->parents.Ar(0), o->A0.data(), sizeof(double) * d * d);
    memcpy(o->parents.pr(0), o->p0.data(), sizeof(double) * d);
    memcpy(o->parents.qr(0), o->p0.data(), sizeof(double) * d);
    memcpy(o->parents.br(0), o->b0.data(), sizeof(double) * d);
    return MCE_OK;
}

// Makes W's parent tables run o's kept tables after update u (no copy when
// W recorded that update itself).
int parent_tables(mce_adjoint* o, int u, Workspace& W)
{
    if (W.owner == o && W.owner_u == u) return MCE_OK;
    const Tables& P = o->ups[u].kept;
    int st;
    if ((st = W.pk.upload(P.keys.data(), P.keys.size(), W.s))) return st;
    if ((st = W.pv.upload(P.vals.data(), P.vals.size(), W.s))) return st;
    if ((st = W.poff.upload(P.off.data(), P.off.size(), W.s))) return st;
    if ((st = W.pcnt.upload(P.cells.data(), P.cells.size(), W.s))) return st;
    W.owner = o;
    W.owner_u = u;
    return MCE_OK;
}

// Records update u of run o after the GPU step has run it: the update's fz,
// every post-MU term's record, the reduction groups and the kept tables.
int fwd_record(mce_adjoint* o, int u, Workspace& W, double* fz_raw)
{
    const int d = o->d, nup = (int)o->ups.size();
    const cudaStream_t s = W.s;
    Update& U = o->ups[u];
    U.first = u == 0;
    U.last = u == nup - 1;
    U.sub = (u + o->first_sub) % o->p;
    U.with_tp = !U.first && U.sub == 0;
    struct Lap {
        double* acc;
        std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
        ~Lap() { *acc += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count(); }
    } lap{&o->ms[1]};
    int st;
    double rfz[2], rm[16], rc[128], gs;
    st = mce_get_raw_moments(o->h, o->est, rfz, rm, rc, &gs);
    if (st < 0) return st;
    // Re fz of the update: 1/(2 pi G_SCALE_FACTOR) (the raw copy of the
    // first update is not kept by the step path)
    U.gscale = gs;
    U.fz_raw = 1.0 / (2.0 * mce::kPi * gs);
    if (fz_raw) fz_raw[u] = U.fz_raw;
    // host records
    derive_update(*o, U, o->parents, o->post, U.terms);
    const RecSet& post = o->post;
    if (!U.first && (st = parent_tables(o, u - 1, W))) return st;
    // the fz tape: recompute Re fz from the recorded lookups on the GPU
    {
        std::vector<EvalDev> ev(U.terms.size());
        for (size_t t = 0; t < U.terms.size(); t++) {
            const TermInfo& ti = U.terms[t];
            ev[t] = EvalDev{ti.parent < 0 ? 0 : ti.parent, ti.lp, ti.lm, ti.enc_lhp, ti.phc, U.first ? 1 : 0,
                            ti.y_eval, ti.d_eval, ti.c_eval};
        }
        if ((st = W.dev.upload(ev.data(), ev.size(), s))) return st;
        if ((st = W.dfz.ensure(ev.size(), s))) return st;
        if (!ev.empty())
            k_adj_eval_fz<<<grid_of((long long)ev.size()), 256, 0, s>>>(W.dev.ptr, (int)ev.size(), W.pk.ptr, W.pv.ptr,
                                                                    W.poff.ptr, W.pcnt.ptr, W.dfz.ptr);
        std::vector<double> f(ev.size());
        if ((st = download(f.data(), W.dfz.ptr, f.size(), s))) return st;
        double sum = 0;
        for (double x : f) sum += x;
        o->fz_check_err =
            std::max(o->fz_check_err, std::fabs(sum - U.fz_raw) / std::max(std::fabs(U.fz_raw), 1e-300));
    }
    if (U.last) return MCE_OK;
    if ((st = o->dump(U.kept))) return st;
    const Tables& K = U.kept;
    // reduction groups and which post-MU term each kept slot holds
    std::vector<std::vector<int>> byshape(o->MS + 1);
    for (int t = 0; t < post.n; t++) byshape[post.m[t]].push_back(t);
    U.kept_first.assign(K.nt, 0);
    U.kept_n.assign(K.nt, 0);
    U.kept_term.assign(K.nt, -1);
    U.members.clear();
    int slot = 0;
    // candidates per kept slot (in member order): (term, s_fixed, conj)
    for (int m = 0; m <= o->MS; m++) {
        if (byshape[m].empty()) continue;
        const std::vector<int>& T = byshape[m];
        std::vector<int> F;
        if (U.first) {
            F.resize(T.size());
            for (size_t i = 0; i < T.size(); i++) F[i] = (int)i;
        } else
            ftr(post, T, d, F);
        std::vector<std::vector<int>> mem(T.size());
        for (size_t j = 0; j < T.size(); j++)
            if (F[j] != (int)j) mem[F[j]].push_back((int)j);
        for (size_t j = 0; j < T.size(); j++) {
            if (F[j] != (int)j) continue;
            // which candidate (root, or the first surviving member) holds this group's kept slot
            std::vector<int> cand;
            cand.push_back((int)j);
            for (int x : mem[j]) cand.push_back(x);
            int holder = -1;
            if (slot < K.nt)
                for (size_t c = 0; c < cand.size(); c++)
                    if (same_record(post, T[cand[c]], K, slot, o->MS, d)) {
                        holder = (int)c;
                        break;
                    }
            if (holder < 0) continue;  // the whole group was approximated out
            const int root_term = T[cand[holder]];
            U.kept_term[slot] = root_term;
            U.kept_first[slot] = (int)U.members.size();
            for (size_t c = holder; c < cand.size(); c++) {
                const int term = T[cand[c]];
                Member mb;
                mb.term = term;
                mb.kept = slot;
                int sm = orientation_mask(post.Ar(root_term), post.Ar(term), m, d);
                const int top = 1 << (m - 1), rev = (1 << m) - 1;
                mb.conj = (sm & top) ? 1 : 0;
                if (sm & top) sm ^= rev;
                mb.s_fixed = c == (size_t)holder ? 0 : sm;
                if (c == (size_t)holder) mb.conj = 0;
                mb.contrib = 1;
                U.members.push_back(mb);
            }
            U.kept_n[slot] = (int)U.members.size() - U.kept_first[slot];
            slot++;
        }
    }
    if (slot != K.nt) {
        mce::report_error("adjoint: the reduction groups do not match the GPU's kept terms (update " +
                          std::to_string(u) + ")");
        return MCE_ERR_DEVICE;
    }
    // member values on the GPU: approximation flags and the table check
    const int nmem = (int)U.members.size();
    std::vector<MInfoDev> mi(nmem);
    std::vector<long long> item_off(nmem + 1, 0);
    for (int j = 0; j < nmem; j++) {
        const Member& mb = U.members[j];
        mi[j] = minfo_of(U.terms[mb.term], post, mb.term, mb, K, U.first);
        item_off[j + 1] = item_off[j] + K.cells[mb.kept];
    }
    const long long nitems = item_off[nmem];
    if ((st = W.dmi.upload(mi.data(), nmem, s))) return st;
    if ((st = W.ditem.upload(item_off.data(), nmem + 1, s))) return st;
    U.mi.swap(mi);
    U.item_off.swap(item_off);
    if ((st = W.dk.upload(K.keys.data(), K.keys.size(), s))) return st;
    if ((st = W.dv.upload(K.vals.data(), K.vals.size(), s))) return st;
    if ((st = W.doff.upload(K.off.data(), K.off.size(), s))) return st;
    if ((st = W.dcnt.upload(K.cells.data(), K.cells.size(), s))) return st;
    if ((st = W.dvals.ensure(nitems + 1, s))) return st;
    if ((st = W.dalive.zero(nmem + 1, s))) return st;
    if (nitems > 0)
        k_adj_member_values<<<grid_of(nitems), 256, 0, s>>>(W.dmi.ptr, W.ditem.ptr, nmem, nitems, W.dk.ptr, W.pk.ptr,
                                                          W.pv.ptr, W.poff.ptr, W.pcnt.ptr, U.gscale, W.dvals.ptr,
                                                          W.dalive.ptr);
    std::vector<int> alive(nmem);
    if ((st = download(alive.data(), W.dalive.ptr, nmem, s))) return st;
    for (int j = 0; j < nmem; j++) U.members[j].contrib = (U.first || alive[j]) ? 1 : 0;
    for (int k = 0; k < K.nt; k++) U.members[U.kept_first[k]].contrib = 1;  // the holder itself
    std::vector<int> contrib(nmem);
    for (int j = 0; j < nmem; j++) contrib[j] = U.members[j].contrib;
    std::vector<long long> kf(K.nt);
    for (int k = 0; k < K.nt; k++) kf[k] = U.kept_first[k];
    if ((st = W.dcontrib.upload(contrib.data(), nmem, s))) return st;
    if ((st = W.dkfirst.upload(kf.data(), K.nt, s))) return st;
    if ((st = W.dknm.upload(U.kept_n.data(), K.nt, s))) return st;
    if ((st = W.derr.zero(1, s))) return st;
    const long long ncells = K.off[K.nt];
    if (ncells > 0)
        k_adj_check_tables<<<grid_of(ncells), 256, 0, s>>>(W.dkfirst.ptr, W.dknm.ptr, W.dmi.ptr, W.ditem.ptr,
                                                         W.dcontrib.ptr, W.dvals.ptr, W.doff.ptr, W.dcnt.ptr, W.dv.ptr,
                                                         K.nt, W.derr.ptr);
    unsigned long long eb = 0;
    if ((st = download(&eb, W.derr.ptr, 1, s))) return st;
    double e;
    memcpy(&e, &eb, sizeof(e));
    o->max_table_err = std::max(o->max_table_err, e);
    // the next parents: the kept terms' records
    o->next.init(o->MS, d);
    o->next.ensure(K.nt);
    o->next.n = K.nt;
    for (int k = 0; k < K.nt; k++) o->next.copy_from(k, post, U.kept_term[k]);
    o->parents.swap(o->next);
    // the kept tables are the next update's parent tables
    W.pk.swap(W.dk);
    W.pv.swap(W.dv);
    W.poff.swap(W.doff);
    W.pcnt.swap(W.dcnt);
    W.owner = o;
    W.owner_u = u;
    if (cudaGetLastError() != cudaSuccess) return MCE_ERR_CUDA;
    return MCE_OK;
}

int num_params(const mce_adjoint* o)
{
    return o->pncc + o->p + o->d + o->d * o->d + o->d * o->pncc + o->p * o->d;
}

// The reverse of run o's recorded updates with seeds w[steps*p]: grad[num_params].
int bwd_run(mce_adjoint* o, const double* w, double* grad, Workspace& W)
{
    const int nup = (int)o->ups.size();
    const cudaStream_t s = W.s;
    int st;
    auto tb0 = std::chrono::steady_clock::now();
    // ---- reverse over the tables and the fz seeds (GPU)
    std::vector<cd> tbar;  // adjoint of the kept tables of update u (from update u+1)
    for (int u = nup - 1; u >= 0; u--) {
        Update& U = o->ups[u];
        const Tables* P = u > 0 ? &o->ups[u - 1].kept : nullptr;
        const long long npc = P ? P->off[P->nt] : 0;
        if ((st = W.pbar.zero(npc + 1, s))) return st;
        if (P && (st = parent_tables(o, u - 1, W))) return st;
        // the tables built at this update
        const int nmem = (int)U.mi.size();
        U.qbar.assign((size_t)nmem * 32, 0.0);
        U.dbar_m.assign(nmem, 0.0);
        U.cbar_m.assign(nmem, 0.0);
        if (!U.last && nmem > 0) {
            const Tables& K = U.kept;
            const long long nitems = U.item_off[nmem];
            std::vector<int> contrib(nmem);
            for (int j = 0; j < nmem; j++) contrib[j] = U.members[j].contrib;
            if ((st = W.dmi.upload(U.mi.data(), nmem, s))) return st;
            if ((st = W.ditem.upload(U.item_off.data(), nmem + 1, s))) return st;
            if ((st = W.dcontrib.upload(contrib.data(), nmem, s))) return st;
            if ((st = W.dk.upload(K.keys.data(), K.keys.size(), s))) return st;
            if (tbar.size() != K.vals.size()) tbar.assign(K.vals.size(), mce::mkcd(0, 0));
            if ((st = W.kbar.upload(tbar.data(), tbar.size(), s))) return st;
            if ((st = W.qbar.zero((size_t)nmem * 32, s))) return st;
            if ((st = W.dbar.zero(nmem, s))) return st;
            if ((st = W.cbar.zero(nmem, s))) return st;
            if (nitems > 0)
                k_adj_member_reverse<<<grid_of(nitems), 256, 0, s>>>(
                    W.dmi.ptr, W.ditem.ptr, nmem, nitems, W.dcontrib.ptr, W.dk.ptr, W.kbar.ptr, W.pk.ptr, W.pv.ptr,
                    W.poff.ptr, W.pcnt.ptr, U.gscale, W.pbar.ptr, W.qbar.ptr, W.dbar.ptr, W.cbar.ptr);
            if ((st = download(U.qbar.data(), W.qbar.ptr, (size_t)nmem * 32, s))) return st;
            if ((st = download(U.dbar_m.data(), W.dbar.ptr, nmem, s))) return st;
            if ((st = download(U.cbar_m.data(), W.cbar.ptr, nmem, s))) return st;
        }
        // the fz seed of this update
        const int nt = (int)U.terms.size();
        U.ybar_e.assign(nt, 0.0);
        U.dbar_e.assign(nt, 0.0);
        U.cbar_e.assign(nt, 0.0);
        if (w[u] != 0.0 && nt > 0) {
            std::vector<EvalDev> ev(nt);
            for (int t = 0; t < nt; t++) {
                const TermInfo& ti = U.terms[t];
                ev[t] = EvalDev{ti.parent < 0 ? 0 : ti.parent, ti.lp, ti.lm, ti.enc_lhp, ti.phc, U.first ? 1 : 0,
                                ti.y_eval, ti.d_eval, ti.c_eval};
            }
            if ((st = W.dev.upload(ev.data(), nt, s))) return st;
            if ((st = W.ybar_e.ensure(nt, s))) return st;
            if ((st = W.dbar_e.ensure(nt, s))) return st;
            if ((st = W.cbar_e.ensure(nt, s))) return st;
            k_adj_eval_reverse<<<grid_of(nt), 256, 0, s>>>(W.dev.ptr, nt, w[u], W.pk.ptr, W.pv.ptr, W.poff.ptr,
                                                            W.pcnt.ptr, W.pbar.ptr, W.ybar_e.ptr, W.dbar_e.ptr,
                                                            W.cbar_e.ptr);
            if ((st = download(U.ybar_e.data(), W.ybar_e.ptr, nt, s))) return st;
            if ((st = download(U.dbar_e.data(), W.dbar_e.ptr, nt, s))) return st;
            if ((st = download(U.cbar_e.data(), W.cbar_e.ptr, nt, s))) return st;
        }
        tbar.assign(npc, mce::mkcd(0, 0));
        if ((st = download(tbar.data(), W.pbar.ptr, npc, s))) return st;
    }
    if (cudaGetLastError() != cudaSuccess) return MCE_ERR_CUDA;
    // ---- the record chain on the GPU: a thread per (parent, direction)
    // repeats the parent's derivation on dual numbers and dots the tangents
    // of the scalars that enter the g values with their adjoints
    auto tb1 = std::chrono::steady_clock::now();
    o->ms[2] += std::chrono::duration<double, std::milli>(tb1 - tb0).count();
    const int N = num_params(o);
    const int d = o->d, MS = o->MS, rec = MS * d + MS + d;
    long long maxP = 1;
    for (int u = 0; u + 1 < nup; u++) maxP = std::max<long long>(maxP, o->ups[u].kept.nt);
    if ((st = W.tin.ensure((size_t)N * maxP * rec, s))) return st;
    if ((st = W.tout.ensure((size_t)N * maxP * rec, s))) return st;
    if ((st = W.dgrad.zero(N, s))) return st;
    const std::vector<double>* pv_[8] = {&o->beta, &o->gamma, &o->p0, &o->Phi, &o->Gamma, &o->H, &o->A0, &o->b0};
    for (int i = 0; i < 8; i++)
        if ((st = W.dpar[i].upload(pv_[i]->data(), pv_[i]->size(), s))) return st;
    for (int u = 0; u < nup; u++) {
        const Update& U = o->ups[u];
        const int nt = (int)U.terms.size();
        const int nP = u == 0 ? 1 : o->ups[u - 1].kept.nt;
        if (u > 0) {
            const Tables& K = o->ups[u - 1].kept;
            if ((st = W.dPm.upload(K.shape.data(), K.shape.size(), s))) return st;
            if ((st = W.dPA.upload(K.A.data(), K.A.size(), s))) return st;
            if ((st = W.dPp.upload(K.p.data(), K.p.size(), s))) return st;
            if ((st = W.dPb.upload(K.b.data(), K.b.size(), s))) return st;
        }
        std::vector<int> kid_off(nP, 0), nk(nP, 0);
        for (int t = nP; t < nt; t++) nk[U.terms[t].parent < 0 ? 0 : U.terms[t].parent]++;
        for (int i = 0, acc = nP; i < nP; i++) {
            kid_off[i] = acc;
            acc += nk[i];
        }
        std::vector<unsigned> sn(nt), hp(nt);
        for (int t = 0; t < nt; t++) {
            sn[t] = U.terms[t].sneg;
            hp[t] = U.terms[t].horthog_pre;
        }
        std::vector<double> qt((size_t)nt * 32, 0.0), dt(nt, 0.0), ct(nt, 0.0);
        for (size_t j = 0; j < U.members.size(); j++) {
            const Member& mb = U.members[j];
            if (!mb.contrib || U.qbar.empty()) continue;
            for (int k = 0; k < 32; k++) qt[(size_t)mb.term * 32 + k] = U.qbar[j * 32 + k];
            dt[mb.term] = U.dbar_m[j];
            ct[mb.term] = U.cbar_m[j];
        }
        std::vector<int> kept_of(nt, -1);
        const int n_next = U.last ? 0 : (int)U.kept_term.size();
        for (int k = 0; k < n_next; k++) kept_of[U.kept_term[k]] = k;
        if ((st = W.dkid.upload(kid_off.data(), nP, s))) return st;
        if ((st = W.dsn.upload(sn.data(), nt, s))) return st;
        if ((st = W.dhp.upload(hp.data(), nt, s))) return st;
        if ((st = W.dyb.upload(U.ybar_e.data(), nt, s))) return st;
        if ((st = W.ddb.upload(U.dbar_e.data(), nt, s))) return st;
        if ((st = W.dcb.upload(U.cbar_e.data(), nt, s))) return st;
        if ((st = W.dqt.upload(qt.data(), qt.size(), s))) return st;
        if ((st = W.ddt.upload(dt.data(), nt, s))) return st;
        if ((st = W.dct.upload(ct.data(), nt, s))) return st;
        if ((st = W.dkept.upload(kept_of.data(), nt, s))) return st;
        ChainArgs ca;
        ca.d = d;
        ca.pncc = o->pncc;
        ca.p = o->p;
        ca.MS = MS;
        ca.N = N;
        ca.first = U.first;
        ca.last = U.last;
        ca.with_tp = U.with_tp;
        ca.sub = U.sub;
        ca.nP = nP;
        ca.z = o->msmts[u];
        ca.beta = W.dpar[0].ptr;
        ca.gamma = W.dpar[1].ptr;
        ca.p0 = W.dpar[2].ptr;
        ca.Phi = W.dpar[3].ptr + (o->ltv ? (size_t)((u + o->first_sub) / o->p) * d * d : 0);
        ca.Gamma = W.dpar[4].ptr;
        ca.H = W.dpar[5].ptr;
        ca.A0 = W.dpar[6].ptr;
        ca.b0 = W.dpar[7].ptr;
        ca.PA = W.dPA.ptr;
        ca.Pp = W.dPp.ptr;
        ca.Pb = W.dPb.ptr;
        ca.Pm = W.dPm.ptr;
        ca.Tin = W.tin.ptr;
        ca.Tout = W.tout.ptr;
        ca.rec = rec;
        ca.n_next = n_next;
        ca.kid_off = W.dkid.ptr;
        ca.sneg = W.dsn.ptr;
        ca.hpre = W.dhp.ptr;
        ca.ybar_e = W.dyb.ptr;
        ca.dbar_e = W.ddb.ptr;
        ca.cbar_e = W.dcb.ptr;
        ca.qbar_t = W.dqt.ptr;
        ca.dbar_t = W.ddt.ptr;
        ca.cbar_t = W.dct.ptr;
        ca.kept_of = W.dkept.ptr;
        ca.grad = W.dgrad.ptr;
        const long long nthr = (long long)nP * N;
        launch_chain(ca, nthr, s);
        W.tin.swap(W.tout);
    }
    if ((st = download(grad, W.dgrad.ptr, N, s))) {
        mce::report_error("adjoint: the record chain failed on the GPU");
        return st;
    }
    o->ms[3] += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb1).count();
    return MCE_OK;
}

// Runs f(i, worker) for i in [0, n) on up to T host threads (worker 0 is the
// caller), each on device `dev`; returns the first failure's status and
// passes its message on to the calling thread.
template <class F>
int parallel_runs(int n, int T, int dev, F&& f)
{
    std::atomic<int> next{0};
    std::atomic<int> err{0};
    std::string msg;
    std::mutex mm;
    auto body = [&](int w) {
        if (w > 0) cudaSetDevice(dev);
        for (;;) {
            const int i = next++;
            if (i >= n || err.load() != 0) break;
            const int st = f(i, w);
            if (st < 0) {
                int z = 0;
                if (err.compare_exchange_strong(z, st)) {
                    std::lock_guard<std::mutex> l(mm);
                    msg = mce_last_error();
                }
            }
        }
    };
    T = std::max(1, std::min(T, n));
    std::vector<std::thread> th;
    for (int w = 1; w < T; w++) th.emplace_back(body, w);
    body(0);
    for (auto& t : th) t.join();
    if (err.load() != 0) mce::report_error(msg);
    return err.load();
}

int host_threads(int n)
{
    int T = (int)std::thread::hardware_concurrency();
    if (T <= 0) T = 1;
    return std::max(1, std::min(std::min(T, 16), n));
}

}  // namespace

// A batch of runs of one LTI model, stepped together by one batched handle.
struct mce_adjoint_batch {
    int n = 0, d = 0, pncc = 0, p = 0, dev = 0, threads = 1;
    mce_handle* h = nullptr;
    std::vector<std::unique_ptr<mce_adjoint>> runs;
    std::vector<std::unique_ptr<Workspace>> ws;
    double ms[4] = {0, 0, 0, 0};
    ~mce_adjoint_batch()
    {
        runs.clear();
        ws.clear();
        if (h) mce_destroy(h);
    }
};

extern "C" {

mce_adjoint* mce_adjoint_create(int d, int pncc, int p, int steps, const double* A0, const double* p0,
                                const double* b0, const double* root_point, const double* b_pert, int* status)
{
    auto fail = [status](int st, const std::string& msg) -> mce_adjoint* {
        mce::report_error(msg);
        if (status) *status = st;
        return nullptr;
    };
    if (d < 2 || d > 8 || pncc < 1 || pncc > kGammaMax || p < 1 || steps < 1 || !A0 || !p0 || !b0 || !root_point ||
        !b_pert)
        return fail(MCE_ERR_ARG, "mce_adjoint_create: invalid arguments (2 <= d <= 8, 1 <= pncc <= 8)");
    std::unique_ptr<mce_adjoint> o(new mce_adjoint());
    o->d = d;
    o->pncc = pncc;
    o->p = p;
    o->steps = steps;
    o->MS = (steps - 1) * pncc + d;
    if (o->MS > 31) return fail(MCE_ERR_SHAPE, "mce_adjoint_create: more than 31 hyperplanes per term");
    o->A0.assign(A0, A0 + d * d);
    o->p0.assign(p0, p0 + d);
    o->b0.assign(b0, b0 + d);
    o->root.assign(root_point, root_point + d);
    o->bpert.assign(b_pert, b_pert + o->MS);
    int st = MCE_OK;
    o->h = mce_create(A0, p0, b0, steps, d, 0, pncc, p, root_point, b_pert, &st);
    if (!o->h) {
        if (status) *status = st;
        return nullptr;
    }
    if (status) *status = MCE_OK;
    return o.release();
}

static int forward_run(mce_adjoint* o, const double* msmts, const double* Phi, const double* Gamma,
                       const double* beta, const double* H, const double* gamma, double* fz_raw, bool ltv)
{
    if (!o || !msmts || !Phi || !Gamma || !beta || !H || !gamma) return MCE_ERR_ARG;
    int st;
    if (!o->ws) o->ws.reset(new Workspace());
    if ((st = o->ws->init())) return st;
    o->ws->owner = nullptr;
    if ((st = fwd_begin(o, msmts, Phi, Gamma, beta, H, gamma, ltv))) return st;
    if ((st = mce_reset(o->h)) < 0) return st;
    const int d = o->d, nup = (int)o->ups.size();
    for (int u = 0; u < nup; u++) {
        const int sub = u % o->p;
        auto t0 = std::chrono::steady_clock::now();
        st = mce_step(o->h, msmts[u], phi_of(*o, u), Gamma, beta, H + (size_t)sub * d, gamma[sub], nullptr, nullptr);
        if (st < 0) return st;
        o->ms[0] += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if ((st = fwd_record(o, u, *o->ws, fz_raw))) return st;
    }
    return MCE_OK;
}

int mce_adjoint_forward(mce_adjoint* o, const double* msmts, const double* Phi, const double* Gamma,
                        const double* beta, const double* H, const double* gamma, double* fz_raw)
{
    return forward_run(o, msmts, Phi, Gamma, beta, H, gamma, fz_raw, false);
}

int mce_adjoint_forward_ltv(mce_adjoint* o, const double* msmts, const double* Phis, const double* Gamma,
                            const double* beta, const double* H, const double* gamma, double* fz_raw)
{
    return forward_run(o, msmts, Phis, Gamma, beta, H, gamma, fz_raw, true);
}

int mce_adjoint_check(mce_adjoint* o, double* max_table_rel_err, double* max_fz_rel_err)
{
    if (!o) return MCE_ERR_ARG;
    if (max_table_rel_err) *max_table_rel_err = o->max_table_err;
    if (max_fz_rel_err) *max_fz_rel_err = o->fz_check_err;
    return MCE_OK;
}

int mce_adjoint_timing(mce_adjoint* o, double* ms4)
{
    if (!o || !ms4) return MCE_ERR_ARG;
    for (int i = 0; i < 4; i++) ms4[i] = o->ms[i];
    return MCE_OK;
}

int mce_adjoint_num_params(mce_adjoint* o)
{
    if (!o) return MCE_ERR_ARG;
    return num_params(o);
}

int mce_adjoint_backward(mce_adjoint* o, const double* w, double* grad)
{
    if (!o || !w || !grad || o->ups.empty()) return MCE_ERR_ARG;
    int st;
    if (!o->ws) o->ws.reset(new Workspace());
    if ((st = o->ws->init())) return st;
    return bwd_run(o, w, grad, *o->ws);
}

void mce_adjoint_destroy(mce_adjoint* o) { delete o; }

mce_adjoint_batch* mce_adjoint_batch_create(int n_runs, int d, int pncc, int p, const int* steps, const double* A0,
                                            const double* p0, const double* b0, const double* root_point,
                                            const double* b_pert, int bpert_stride, int* status)
{
    auto fail = [status](int st, const std::string& msg) -> mce_adjoint_batch* {
        mce::report_error(msg);
        if (status) *status = st;
        return nullptr;
    };
    if (n_runs < 1 || d < 2 || d > 8 || pncc < 1 || pncc > kGammaMax || p < 1 || !steps || !A0 || !p0 || !b0 ||
        !root_point || !b_pert || bpert_stride < 1)
        return fail(MCE_ERR_ARG, "mce_adjoint_batch_create: invalid arguments (2 <= d <= 8, 1 <= pncc <= 8)");
    std::unique_ptr<mce_adjoint_batch> b(new mce_adjoint_batch());
    b->n = n_runs;
    b->d = d;
    b->pncc = pncc;
    b->p = p;
    for (int r = 0; r < n_runs; r++) {
        if (steps[r] < 1) return fail(MCE_ERR_ARG, "mce_adjoint_batch_create: a run of no steps");
        const int MS = (steps[r] - 1) * pncc + d;
        if (MS > 31) return fail(MCE_ERR_SHAPE, "mce_adjoint_batch_create: more than 31 hyperplanes per term");
        if (MS > bpert_stride) return fail(MCE_ERR_ARG, "mce_adjoint_batch_create: bpert_stride below a run's shape");
    }
    int st = MCE_OK;
    b->h = mce_batch_create(n_runs, d, 0, pncc, p, steps, A0, p0, b0, root_point, b_pert, bpert_stride, &st);
    if (!b->h) {
        if (status) *status = st;
        return nullptr;
    }
    cudaGetDevice(&b->dev);
    for (int r = 0; r < n_runs; r++) {
        std::unique_ptr<mce_adjoint> o(new mce_adjoint());
        o->d = d;
        o->pncc = pncc;
        o->p = p;
        o->steps = steps[r];
        o->MS = (steps[r] - 1) * pncc + d;
        o->A0.assign(A0 + (size_t)r * d * d, A0 + (size_t)(r + 1) * d * d);
        o->p0.assign(p0 + (size_t)r * d, p0 + (size_t)(r + 1) * d);
        o->b0.assign(b0 + (size_t)r * d, b0 + (size_t)(r + 1) * d);
        o->root.assign(root_point + (size_t)r * d, root_point + (size_t)(r + 1) * d);
        o->bpert.assign(b_pert + (size_t)r * bpert_stride, b_pert + (size_t)r * bpert_stride + o->MS);
        o->h = b->h;
        o->est = r;
        o->owns_h = false;
        b->runs.push_back(std::move(o));
    }
    b->threads = host_threads(n_runs);
    for (int w = 0; w < b->threads; w++) {
        b->ws.emplace_back(new Workspace());
        if ((st = b->ws.back()->init())) {
            if (status) *status = st;
            return nullptr;
        }
    }
    if (status) *status = MCE_OK;
    return b.release();
}

static int batch_forward(mce_adjoint_batch* b, const double* msmts, int max_steps, const double* Phi,
                         const double* Gamma, const double* beta, const double* H, const double* gamma, double* fz_raw,
                         bool ltv)
{
    if (!b || !msmts || !Phi || !Gamma || !beta || !H || !gamma || max_steps < 1) return MCE_ERR_ARG;
    const int n = b->n, d = b->d, p = b->p, pncc = b->pncc, stride = max_steps * p;
    int st, max_up = 0;
    // a time-varying batch carries each run's own Phi sequence, Gamma and H
    auto Gam_of = [&](int r) { return ltv ? Gamma + (size_t)r * d * pncc : Gamma; };
    auto H_of = [&](int r) { return ltv ? H + (size_t)r * p * d : H; };
    for (int r = 0; r < n; r++) {
        mce_adjoint* o = b->runs[r].get();
        if (o->steps > max_steps) return MCE_ERR_ARG;
        const double* Ph = ltv ? Phi + (size_t)r * max_steps * d * d : Phi;
        if ((st = fwd_begin(o, msmts + (size_t)r * stride, Ph, Gam_of(r), beta, H_of(r), gamma, ltv))) return st;
        max_up = std::max(max_up, (int)o->ups.size());
    }
    for (auto& w : b->ws) w->owner = nullptr;
    if (fz_raw) std::fill(fz_raw, fz_raw + (size_t)n * stride, 0.0);
    if ((st = mce_reset(b->h)) < 0) return st;
    std::vector<double> z(n), Hr((size_t)n * d), gam(n);
    // a time-varying batch is stepped with per-estimator model arrays: each
    // run's Phi of its own step and its Gamma, beta repeated
    std::vector<double> Phb, Gb, bb;
    if (ltv) {
        Phb.assign((size_t)n * d * d, 0.0);
        Gb.assign((size_t)n * d * pncc, 0.0);
        bb.assign((size_t)n * pncc, 0.0);
        for (int r = 0; r < n; r++) {
            std::copy(Gam_of(r), Gam_of(r) + d * pncc, Gb.begin() + (size_t)r * d * pncc);
            std::copy(beta, beta + pncc, bb.begin() + (size_t)r * pncc);
        }
    }
    std::vector<int> act;
    const int fsub = b->runs[0]->first_sub;
    for (int u = 0; u < max_up; u++) {
        const int sub = (u + fsub) % p;
        act.clear();
        for (int r = 0; r < n; r++) {
            const mce_adjoint* o = b->runs[r].get();
            const bool on = u < (int)o->ups.size();
            z[r] = on ? msmts[(size_t)r * stride + u] : 0.0;
            for (int j = 0; j < d; j++) Hr[(size_t)r * d + j] = H_of(r)[(size_t)sub * d + j];
            gam[r] = gamma[sub];
            if (ltv) {
                const double* Ph = phi_of(*o, on ? u : (int)o->ups.size() - 1);
                std::copy(Ph, Ph + d * d, Phb.begin() + (size_t)r * d * d);
            }
            if (on) act.push_back(r);
        }
        auto t0 = std::chrono::steady_clock::now();
        st = ltv ? mce_batch_step(b->h, z.data(), Phb.data(), Gb.data(), bb.data(), Hr.data(), gam.data(), nullptr,
                                  nullptr, 0, nullptr)
                 : mce_batch_step(b->h, z.data(), Phi, Gamma, beta, Hr.data(), gam.data(), nullptr, nullptr, 1,
                                  nullptr);
        if (st < 0) return st;
        // a restarted window's master step jumps to p after its first update
        if (u == 0 && fsub > 0 && (st = mce_set_master_step(b->h, p)) < 0) return st;
        auto t1 = std::chrono::steady_clock::now();
        st = parallel_runs((int)act.size(), b->threads, b->dev, [&](int i, int w) {
            const int r = act[i];
            return fwd_record(b->runs[r].get(), u, *b->ws[w], fz_raw ? fz_raw + (size_t)r * stride : nullptr);
        });
        if (st < 0) return st;
        auto t2 = std::chrono::steady_clock::now();
        b->ms[0] += std::chrono::duration<double, std::milli>(t1 - t0).count();
        b->ms[1] += std::chrono::duration<double, std::milli>(t2 - t1).count();
    }
    return MCE_OK;
}

int mce_adjoint_batch_forward(mce_adjoint_batch* b, const double* msmts, int max_steps, const double* Phi,
                              const double* Gamma, const double* beta, const double* H, const double* gamma,
                              double* fz_raw)
{
    return batch_forward(b, msmts, max_steps, Phi, Gamma, beta, H, gamma, fz_raw, false);
}

int mce_adjoint_batch_forward_ltv(mce_adjoint_batch* b, const double* msmts, int max_steps, const double* Phis,
                                  const double* Gamma, const double* beta, const double* H, const double* gamma,
                                  double* fz_raw)
{
    return batch_forward(b, msmts, max_steps, Phis, Gamma, beta, H, gamma, fz_raw, true);
}

int mce_adjoint_batch_backward(mce_adjoint_batch* b, const double* w, int max_steps, double* grad)
{
    if (!b || !w || !grad || max_steps < 1) return MCE_ERR_ARG;
    const int n = b->n, stride = max_steps * b->p;
    const int N = num_params(b->runs[0].get());
    for (int r = 0; r < n; r++)
        if (b->runs[r]->ups.empty() || b->runs[r]->steps > max_steps) return MCE_ERR_ARG;
    std::fill(grad, grad + (size_t)n * N, 0.0);
    auto t0 = std::chrono::steady_clock::now();
    const int st = parallel_runs(n, b->threads, b->dev, [&](int r, int wk) {
        mce_adjoint* o = b->runs[r].get();
        const double* wr = w + (size_t)r * stride;
        bool any = false;
        for (size_t u = 0; u < o->ups.size(); u++) any |= wr[u] != 0.0;
        return any ? bwd_run(o, wr, grad + (size_t)r * N, *b->ws[wk]) : MCE_OK;
    });
    b->ms[2] += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return st;
}

int mce_adjoint_batch_set_first_sub(mce_adjoint_batch* b, int first_sub)
{
    if (!b || first_sub < 0 || first_sub >= b->p) return MCE_ERR_ARG;
    for (auto& o : b->runs) {
        o->first_sub = first_sub;
        o->ups.clear();
    }
    return MCE_OK;
}

int mce_adjoint_batch_num_params(mce_adjoint_batch* b)
{
    if (!b) return MCE_ERR_ARG;
    return num_params(b->runs[0].get());
}

int mce_adjoint_batch_check(mce_adjoint_batch* b, double* max_table_rel_err, double* max_fz_rel_err)
{
    if (!b) return MCE_ERR_ARG;
    double a = 0, c = 0;
    for (auto& o : b->runs) {
        a = std::max(a, o->max_table_err);
        c = std::max(c, o->fz_check_err);
    }
    if (max_table_rel_err) *max_table_rel_err = a;
    if (max_fz_rel_err) *max_fz_rel_err = c;
    return MCE_OK;
}

int mce_adjoint_batch_timing(mce_adjoint_batch* b, double* ms4)
{
    if (!b || !ms4) return MCE_ERR_ARG;
    for (int i = 0; i < 3; i++) ms4[i] = b->ms[i];
    ms4[3] = 0;
    for (auto& o : b->runs) ms4[3] += o->ms[3];
    return MCE_OK;
}

void mce_adjoint_batch_destroy(mce_adjoint_batch* b) { delete b; }

}  // extern "C"
