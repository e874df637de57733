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
// Layout of the computation (one estimator per object):
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
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

namespace mce {
void report_error(const std::string& s);
}

using mce::cd;

namespace {

// ---------------------------------------------------------------------------
// Host scalars of the record derivation (doubles; the GPU record chain below
// repeats the derivation on dual numbers).
inline double val(double x) { return x; }
inline double absd(double x) { return std::fabs(x); }

constexpr double kCoalignEps = 1e-8;
constexpr double kMuEps = 1e-10;
constexpr double kReductionEps = 1e-8;

// A term's record at some point of an update.
template <class S>
struct Rec {
    int m = 0;
    std::vector<S> A, p, b;  // A m x d row-major
    std::vector<S> q;        // row scales before normalisation (the g-table's)
    S c = 0.0, dv = 0.0;     // c_val, d_val
    unsigned horthog = 0;
};

// coalignment gate on values: +1 same, -1 opposite, 0 (cauchy_term.hpp:494-504)
template <class S>
int gate(const S* r, const S* c, int d)
{
    bool pos = true, neg = true;
    for (int l = 0; l < d; l++) {
        if (pos) pos &= std::fabs(val(r[l]) - val(c[l])) < kCoalignEps;
        if (neg) neg &= std::fabs(val(r[l]) + val(c[l])) < kCoalignEps;
        if (!(pos || neg)) break;
    }
    return pos ? 1 : (neg ? -1 : 0);
}

// normalize_hps (cauchy_term.hpp:458-472): p *= |A_i|_1, A_i /= |A_i|_1;
// with set_q the scales before normalisation are kept in q.
template <class S>
void normalize(Rec<S>& t, int d, bool set_q)
{
    if (set_q) t.q.assign(t.p.begin(), t.p.begin() + t.m);
    for (int i = 0; i < t.m; i++) {
        S n1 = 0.0;
        for (int j = 0; j < d; j++) n1 += absd(t.A[i * d + j]);
        t.p[i] *= n1;
        for (int j = 0; j < d; j++) t.A[i * d + j] /= n1;
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
__device__ inline DD dabs(DD x) { return x.v < 0 ? dneg(x) : (x.v > 0 ? x : DD{0.0, 0.0}); }

constexpr int kRows = 16, kDim = 8;  // the step path's limits (16 hyperplanes, 8 states)

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

__global__ void __launch_bounds__(128) k_adj_chain(ChainArgs a)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)a.nP * a.N) return;
    const int pi = (int)(idx % a.nP), dir = (int)(idx / a.nP);
    const int d = a.d;
    const int offb = 0, offg = offb + a.pncc, offp = offg + a.p, offPhi = offp + d, offG = offPhi + d * d,
              offH = offG + d * a.pncc;
    auto par = [&](const double* v, int i, int off) { return DD{v[i], dir == off + i ? 1.0 : 0.0}; };
    // the parent's record
    DD A[kRows * kDim], P[kRows], B[kDim];
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
        DD Gt[kDim * kDim], bt[kDim];
        const int pncc = a.pncc;
        for (int i = 0; i < pncc; i++) {
            for (int j = 0; j < d; j++) Gt[i * d + j] = par(a.Gamma, j * pncc + i, offG);
            bt[i] = par(a.beta, i, offb);
        }
        for (int i = 0; i < pncc; i++) {
            DD nf = dd(0.0);
            for (int j = 0; j < d; j++) nf = dadd(nf, dabs(Gt[i * d + j]));
            for (int j = 0; j < d; j++) Gt[i * d + j] = ddiv(Gt[i * d + j], nf);
            bt[i] = dmul(bt[i], nf);
        }
        bool F[kDim];
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
        // time_prop
        DD w[kRows * kDim];
        for (int i = 0; i < m * d; i++) w[i] = A[i];
        for (int i = 0; i < m; i++)
            for (int j = 0; j < d; j++) {
                DD sum = dd(0.0);
                for (int k = 0; k < d; k++) sum = dadd(sum, dmul(w[i * d + k], par(a.Phi, k + j * d, offPhi)));
                A[i * d + j] = sum;
            }
        DD wb[kDim];
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
            for (int j = 0; j < d; j++) A[i * d + j] = ddiv(A[i * d + j], n1);
        }
        bool Fg[kDim];
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
    DD Hr[kDim];
    for (int j = 0; j < d; j++) Hr[j] = par(a.H, a.sub * d + j, offH);
    const DD gam = par(a.gamma, a.sub, offg);
    DD mu[(kRows + 1) * kDim], rho[kRows + 1];
    bool Fi[kRows + 1];
    for (int i = 0; i < m * d; i++) mu[i] = A[i];
    for (int i = 0; i < m; i++) rho[i] = P[i];
    rho[m] = gam;
    for (int j = 0; j < d; j++) mu[m * d + j] = dd(0.0);
    Fi[m] = true;
    for (int l = 0; l < m; l++) {
        DD h = dd(0.0);
        for (int j = 0; j < d; j++) h = dadd(h, dmul(Hr[j], mu[l * d + j]));
        if (fabs(h.v) < kMuEps) {
            rho[l] = P[l];
            Fi[l] = false;
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
        DD cA[kRows * kDim], cp[kRows], cq[kRows], cb[kDim];
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
                for (int j = 0; j < d; j++) cA[i * d + j] = ddiv(cA[i * d + j], n1);
            }
            if (tt != m) {
                bool F[kRows], hflag[kRows];
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

// ---------------------------------------------------------------------------
// Device buffers (grow-only, owned by the object)

template <class T>
struct Buf {
    T* ptr = nullptr;
    size_t cap = 0;
    ~Buf()
    {
        if (ptr) cudaFree(ptr);
    }
    int ensure(size_t n)
    {
        if (n <= cap) return MCE_OK;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
        if (cudaMalloc(&ptr, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) {
            cudaGetLastError();
            mce::report_error("adjoint: device allocation failed");
            return MCE_ERR_NOMEM;
        }
        cap = std::max<size_t>(n, 1);
        return MCE_OK;
    }
    int upload(const T* src, size_t n)
    {
        int s = ensure(n);
        if (s) return s;
        if (n && cudaMemcpy(ptr, src, sizeof(T) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
            mce::report_error("adjoint: host-to-device copy failed");
            return MCE_ERR_CUDA;
        }
        return MCE_OK;
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
    // model (LTI) and measurements of the recorded run
    std::vector<double> Phi, Gamma, beta, H, gamma, msmts;
    std::vector<Update> ups;
    double max_table_err = 0;
    double fz_check_err = 0;
    // wall ms: forward step path, forward tape (host records + GPU checks),
    // reverse over the tables (GPU), record chain (host)
    double ms[4] = {0, 0, 0, 0};

    ~mce_adjoint()
    {
        if (h) mce_destroy(h);
    }

    int dump(Tables& T)
    {
        T.nt = (int)mce_num_terms(h, 0);
        const long long tot = mce_total_cells(h, 0);
        if (T.nt < 0 || tot < 0) return MCE_ERR_ARG;
        T.shape.assign(T.nt, 0);
        T.cells.assign(T.nt, 0);
        T.A.assign((size_t)T.nt * MS * d, 0);
        T.p.assign((size_t)T.nt * MS, 0);
        T.b.assign((size_t)T.nt * d, 0);
        T.keys.assign(std::max<long long>(tot, 1), 0);
        std::vector<double> g(2 * std::max<long long>(tot, 1));
        const int st = mce_dump_terms(h, 0, MS, T.shape.data(), T.A.data(), T.p.data(), T.b.data(), T.cells.data(),
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

// Gamma pre-coalignment (cauchy_util.hpp:128-210): normalised columns as rows
template <class S>
int precoalign(const mce_adjoint& o, const std::vector<S>& G, const std::vector<S>& beta, std::vector<S>& Gt,
               std::vector<S>& bt)
{
    const int d = o.d, pncc = o.pncc;
    Gt.assign((size_t)pncc * d, 0.0);
    bt.assign(pncc, 0.0);
    for (int i = 0; i < pncc; i++) {
        for (int j = 0; j < d; j++) Gt[i * d + j] = G[j * pncc + i];
        bt[i] = beta[i];
    }
    for (int i = 0; i < pncc; i++) {
        S nf = 0.0;
        for (int j = 0; j < d; j++) nf += absd(Gt[i * d + j]);
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

// The parameters of one run, as scalars of kind S (a tangent seeded on one).
template <class S>
struct Params {
    std::vector<S> beta, gamma, p0, Phi, Gamma, H;
};

template <class S>
Params<S> make_params(const mce_adjoint& o, int dir)
{
    Params<S> P;
    int k = 0;
    auto take = [&](std::vector<S>& v, const std::vector<double>& src) {
        v.resize(src.size());
        for (size_t i = 0; i < src.size(); i++, k++) v[i] = S(src[i]);
        (void)dir;
    };
    take(P.beta, o.beta);
    take(P.gamma, o.gamma);
    take(P.p0, o.p0);
    take(P.Phi, o.Phi);
    take(P.Gamma, o.Gamma);
    take(P.H, o.H);
    return P;
}

// One update's record derivation (the host half of step_first / step_rest,
// include/cauchy_estimator.hpp:604-832, 1179-1208): from the kept records of
// the previous update to every post-MU term's record before and after MU
// coalignment.  pre[t] holds the MU output, post[t] the coalignment output.
template <class S>
void derive_update(const mce_adjoint& o, const Update& U, const Params<S>& P, const std::vector<Rec<S>>& parents,
                   std::vector<Rec<S>>& pre, std::vector<Rec<S>>& post, std::vector<TermInfo>* info)
{
    const int d = o.d;
    std::vector<S> Gt, bt;
    int gcnt = 0;
    if (U.with_tp) gcnt = precoalign(o, P.Gamma, P.beta, Gt, bt);
    const S* H = P.H.data() + (size_t)U.sub * d;
    const S gam = P.gamma[U.sub];
    const double z = o.msmts[(size_t)(&U - &o.ups[0])];
    pre.clear();
    post.clear();
    if (info) info->clear();
    std::vector<Rec<S>> kids_pre, kids_post;
    std::vector<TermInfo> kids_info;
    std::vector<Rec<S>> par_pre, par_post;
    std::vector<TermInfo> par_info;
    for (size_t pi = 0; pi < parents.size(); pi++) {
        Rec<S> t = parents[pi];
        const int phc = U.first ? 0 : t.m;  // the parent's table is over its rows before time propagation
        if (U.with_tp) {
            // time_prop: A <- A Phi^T, b <- Phi b (cauchy_term.hpp:435-456)
            std::vector<S> w(t.A.begin(), t.A.begin() + t.m * d);
            for (int i = 0; i < t.m; i++)
                for (int j = 0; j < d; j++) {
                    S s = 0.0;
                    for (int k = 0; k < d; k++) s += w[i * d + k] * P.Phi[k + j * d];
                    t.A[i * d + j] = s;
                }
            std::vector<S> wb(t.b);
            for (int i = 0; i < d; i++) {
                S s = 0.0;
                for (int j = 0; j < d; j++) s += P.Phi[i * d + j] * wb[j];
                t.b[i] = s;
            }
            // tp_coalign (cauchy_term.hpp:475-531)
            normalize(t, d, false);
            std::vector<char> F(gcnt, 1);
            for (int j = 0; j < gcnt; j++)
                for (int k = 0; k < t.m; k++)
                    if (F[j] && gate(&Gt[j * d], &t.A[k * d], d) != 0) {
                        F[j] = 0;
                        t.p[k] += bt[j];
                    }
            for (int j = 0; j < gcnt; j++)
                if (F[j]) {
                    t.A.resize((t.m + 1) * d);
                    t.p.resize(t.m + 1);
                    for (int l = 0; l < d; l++) t.A[t.m * d + l] = Gt[j * d + l];
                    t.p[t.m] = bt[j];
                    t.m++;
                }
        }
        // msmt_update (cauchy_term.hpp:84-310)
        const int m = t.m;
        std::vector<S> mu((m + 1) * d), rho(m + 1);
        std::vector<int> sgn(m);
        std::vector<char> Fi(m + 1);
        for (int i = 0; i < m * d; i++) mu[i] = t.A[i];
        for (int i = 0; i < m; i++) rho[i] = t.p[i];
        rho[m] = gam;
        for (int j = 0; j < d; j++) mu[m * d + j] = 0.0;
        Fi[m] = 1;
        for (int l = 0; l < m; l++) {
            S h = 0.0;
            for (int j = 0; j < d; j++) h += H[j] * mu[l * d + j];
            if (std::fabs(val(h)) < kMuEps) {
                rho[l] = t.p[l];
                sgn[l] = 1;
                Fi[l] = 0;
            } else {
                const S r = S(1.0) / h;
                for (int j = 0; j < d; j++) mu[l * d + j] *= r;
                rho[l] = t.p[l] * absd(h);
                sgn[l] = val(h) > 0 ? 1 : -1;
                Fi[l] = 1;
            }
        }
        S hb = 0.0;
        for (int j = 0; j < d; j++) hb += H[j] * t.b[j];
        const S zeta = S(z) - hb;
        int esg = 0;
        for (int l = 0; l < m; l++)
            if (sgn[l] == -1) esg |= 1 << l;
        int lhp = esg;
        if (phc < m) lhp &= (1 << phc) - 1;
        for (int tt = 0; tt <= m; tt++) {
            if (!Fi[tt]) continue;
            Rec<S> c;
            c.m = m;
            c.c = zeta;
            c.dv = rho[tt];
            c.b.resize(d);
            for (int j = 0; j < d; j++) c.b[j] = t.b[j] + zeta * mu[tt * d + j];
            c.A.resize(m * d);
            c.p.resize(m);
            int l = 0;
            unsigned hof = 0;
            for (int ll = 0; ll <= m; ll++) {
                if (ll == tt) continue;
                c.p[l] = rho[ll];
                if (Fi[ll])
                    for (int j = 0; j < d; j++) c.A[l * d + j] = mu[ll * d + j] - mu[tt * d + j];
                else {
                    for (int j = 0; j < d; j++) c.A[l * d + j] = mu[ll * d + j];
                    hof |= 1u << l;
                }
                l++;
            }
            c.horthog = hof;
            TermInfo ti;
            ti.parent = U.first ? -1 : (int)pi;
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
                for (int j = 0; j < d; j++) s += val(c.A[ll * d + j]) * o.root[j];
                if (!(s > 0)) sneg |= 1u << ll;
            }
            if (hof) {
                for (int ll = 0; ll < m; ll++)
                    if (!(hof & (1u << ll))) y += val(c.p[ll]) * (((sneg >> ll) & 1) ? -1.0 : 1.0);
            } else {
                double zz = 0.0;
                for (int ll = 0; ll < m; ll++) zz += val(c.p[ll]) * (((sneg >> ll) & 1) ? -1.0 : 1.0);
                y = zz;
            }
            ti.y_eval = y;
            ti.sneg = sneg;
            ti.d_eval = val(c.dv);
            ti.c_eval = val(c.c);
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
            // MU coalignment (the parent only normalises)
            Rec<S> cp = c;
            if (U.first || U.last) {
                cp.q = cp.p;
                ti.m = m;
                ti.horthog = hof;
                ti.has_cmap = false;
            } else if (tt == m) {
                normalize(cp, d, true);
                ti.m = m;
                ti.horthog = hof;
                ti.has_cmap = false;
            } else {
                // mu_coalign (cauchy_term.hpp:533-745)
                normalize(cp, d, true);
                std::vector<char> F(m, 1), hflag(m, 0);
                int cmap[32], csmap[32];
                for (int j = 0; j < m; j++) {
                    cmap[j] = 255;
                    csmap[j] = 1;
                }
                if (cp.horthog)
                    for (int j = 0; j < m; j++) hflag[j] = (cp.horthog >> j) & 1;
                int uc = 0;
                for (int j = 0; j < m - 1; j++) {
                    if (!F[j]) continue;
                    cmap[j] = uc;
                    for (int k = j + 1; k < m; k++) {
                        if (!F[k]) continue;
                        const int g = gate(&cp.A[j * d], &cp.A[k * d], d);
                        if (g == 1) {
                            if (cp.horthog) {
                                const bool hj = hflag[j], hk = hflag[k];
                                if (!hj && !hk) cp.q[j] += cp.q[k];
                                else if (hj && !hk) {
                                    cp.q[j] = cp.q[k];
                                    hflag[j] = 0;
                                } else if (!hj && hk) hflag[k] = 0;
                                else {
                                    hflag[k] = 0;
                                    cp.q[j] += cp.q[k];
                                }
                            } else
                                cp.q[j] += cp.q[k];
                            F[k] = 0;
                            cp.p[j] += cp.p[k];
                            cmap[k] = uc;
                            csmap[k] = 1;
                        } else if (g == -1) {
                            if (cp.horthog) {
                                const bool hj = hflag[j], hk = hflag[k];
                                if (!hj && !hk) cp.q[j] -= cp.q[k];
                                else if (hj && !hk) {
                                    cp.q[j] = -cp.q[k];
                                    hflag[j] = 0;
                                } else if (!hj && hk) hflag[k] = 0;
                            } else
                                cp.q[j] -= cp.q[k];
                            F[k] = 0;
                            cp.p[j] += cp.p[k];
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
                                for (int l2 = 0; l2 < d; l2++) cp.A[u * d + l2] = cp.A[j * d + l2];
                                cp.p[u] = cp.p[j];
                                cp.q[u] = cp.q[j];
                            }
                            u++;
                        }
                    if (cp.horthog) {
                        unsigned nh = 0;
                        int cc = 0;
                        for (int j = 0; j < m; j++)
                            if (F[j]) nh |= (unsigned)hflag[j] << cc++;
                        cp.horthog = nh;
                    }
                    cp.m = ns;
                    cp.A.resize(ns * d);
                    cp.p.resize(ns);
                    cp.q.resize(ns);
                }
                ti.m = cp.m;
                ti.horthog = cp.horthog;
                ti.has_cmap = ns < m;
                for (int j = 0; j < 32; j++) {
                    ti.cmap[j] = j < m ? cmap[j] : 0;
                    ti.csmap[j] = j < m ? csmap[j] : 1;
                }
            }
            if (tt == m) {
                par_pre.push_back(c);
                par_post.push_back(cp);
                par_info.push_back(ti);
            } else {
                kids_pre.push_back(c);
                kids_post.push_back(cp);
                kids_info.push_back(ti);
            }
        }
    }
    // creation order: step_first keeps [parent, children]; step_rest lists
    // the parents, then the children
    if (U.first) {
        pre = par_pre;
        post = par_post;
        if (info) *info = par_info;
    } else {
        pre = par_pre;
        post = par_post;
        if (info) *info = par_info;
    }
    pre.insert(pre.end(), kids_pre.begin(), kids_pre.end());
    post.insert(post.end(), kids_post.begin(), kids_post.end());
    if (info) info->insert(info->end(), kids_info.begin(), kids_info.end());
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

bool same_record(const Rec<double>& t, const Tables& T, int k, int MS, int d)
{
    if (T.shape[k] != t.m) return false;
    for (int i = 0; i < t.m * d; i++)
        if (T.A[(size_t)k * MS * d + i] != t.A[i]) return false;
    for (int i = 0; i < t.m; i++)
        if (T.p[(size_t)k * MS + i] != t.p[i]) return false;
    for (int i = 0; i < d; i++)
        if (T.b[(size_t)k * d + i] != t.b[i]) return false;
    return true;
}

// fast_term_reduction (term_reduction.hpp:159-276) on one shape's terms
void ftr(const std::vector<const Rec<double>*>& T, int d, std::vector<int>& F)
{
    const int n = (int)T.size();
    F.resize(n);
    for (int i = 0; i < n; i++) F[i] = i;
    if (n == 0) return;
    const int m = T[0]->m;
    const double ep = kReductionEps;
    std::vector<int> ord(n);
    for (int i = 0; i < n; i++) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return T[a]->b[0] < T[b]->b[0]; });
    std::vector<double> v0(n);
    for (int i = 0; i < n; i++) v0[i] = T[ord[i]]->b[0];
    for (int i = 0; i < n; i++) {
        if (F[i] != i) continue;
        const double* bi = T[i]->b.data();
        const int s = (int)(std::upper_bound(v0.begin(), v0.end(), bi[0] - ep) - v0.begin());
        const int e = (int)(std::upper_bound(v0.begin(), v0.end(), bi[0] + ep) - v0.begin());
        for (int w = s; w < e; w++) {
            const int j = ord[w];
            if (j <= i || F[j] != j) continue;
            const double* bj = T[j]->b.data();
            bool ok = true;
            for (int a = 1; a < d && ok; a++)
                if (!(bj[a] > bi[a] - ep && bj[a] <= bi[a] + ep)) ok = false;
            for (int k = 0; k < m && ok; k++)
                if (std::fabs(T[j]->p[k] - T[i]->p[k]) > ep) ok = false;
            for (int k = 0; k < m && ok; k++) {
                const double r = T[i]->A[k], c = T[j]->A[k];
                if (!(std::fabs(r - c) < ep || std::fabs(r + c) < ep)) ok = false;
            }
            if (ok) F[j] = i;
        }
    }
}

MInfoDev minfo_of(const TermInfo& ti, const Rec<double>& post, const Member& mb, const Tables& kept, bool first,
                  int d)
{
    MInfoDev M;
    memset(&M, 0, sizeof(M));
    M.m = post.m;
    M.phc = ti.phc;
    M.z = ti.z;
    M.enc_lhp = ti.enc_lhp;
    M.flags = (ti.new_child ? kMiNewChild : 0) | (ti.has_cmap ? kMiHasCmap : 0) | (first ? kMiFirst : 0);
    M.horthog = (int)post.horthog;
    M.s_fixed = mb.s_fixed;
    M.conj = mb.conj;
    M.kept = mb.kept;
    M.parent = ti.parent < 0 ? 0 : ti.parent;
    M.term = mb.term;
    M.cell_off = kept.off[mb.kept];
    M.cell_cnt = kept.cells[mb.kept];
    M.d = post.dv;
    M.c = post.c;
    double ps = 0;
    for (int i = 0; i < post.m; i++) ps += post.p[i];
    M.ps2 = ps * ps;
    for (int k = 0; k < post.m; k++) M.q[k] = post.q[k];
    for (int k = 0; k < 32; k++) {
        M.cmap[k] = (signed char)ti.cmap[k];
        M.csmap[k] = (signed char)ti.csmap[k];
    }
    (void)d;
    return M;
}

int grid_of(long long n) { return (int)std::min<long long>((n + 255) / 256, 152 * 32); }

}  // namespace

extern "C" {

mce_adjoint* mce_adjoint_create(int d, int pncc, int p, int steps, const double* A0, const double* p0,
                                const double* b0, const double* root_point, const double* b_pert, int* status)
{
    auto fail = [status](int st, const std::string& msg) -> mce_adjoint* {
        mce::report_error(msg);
        if (status) *status = st;
        return nullptr;
    };
    if (d < 2 || d > 8 || pncc < 1 || p < 1 || steps < 1 || !A0 || !p0 || !b0 || !root_point || !b_pert)
        return fail(MCE_ERR_ARG, "mce_adjoint_create: invalid arguments");
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

int mce_adjoint_forward(mce_adjoint* o, const double* msmts, const double* Phi, const double* Gamma,
                        const double* beta, const double* H, const double* gamma, double* fz_raw)
{
    if (!o || !msmts || !Phi || !Gamma || !beta || !H || !gamma) return MCE_ERR_ARG;
    const int d = o->d, nup = o->steps * o->p;
    o->msmts.assign(msmts, msmts + nup);
    o->Phi.assign(Phi, Phi + d * d);
    o->Gamma.assign(Gamma, Gamma + d * o->pncc);
    o->beta.assign(beta, beta + o->pncc);
    o->H.assign(H, H + o->p * d);
    o->gamma.assign(gamma, gamma + o->p);
    int st = mce_reset(o->h);
    if (st < 0) return st;
    o->ups.assign(nup, Update());
    o->max_table_err = 0;
    o->fz_check_err = 0;
    Params<double> P = make_params<double>(*o, -1);
    std::vector<Rec<double>> parents(1), pre, post;
    parents[0].m = d;
    parents[0].A = o->A0;
    parents[0].p = o->p0;
    parents[0].b = o->b0;
    const Tables* prev = nullptr;
    Buf<int> dk, pk;
    Buf<cd> dv, pv;
    Buf<long long> doff, poffb;
    Buf<int> dcnt, pcntb;
    Buf<MInfoDev> dmi;
    Buf<long long> ditem;
    Buf<cd> dvals;
    Buf<int> dalive, dcontrib;
    Buf<long long> dkfirst;
    Buf<int> dknm;
    Buf<unsigned long long> derr;
    Buf<EvalDev> dev;
    Buf<double> dfz;
    for (int u = 0; u < nup; u++) {
        Update& U = o->ups[u];
        U.first = u == 0;
        U.last = u == nup - 1;
        U.sub = u % o->p;
        U.with_tp = !U.first && (u % o->p) == 0;
        // the GPU step
        auto t0 = std::chrono::steady_clock::now();
        st = mce_step(o->h, msmts[u], Phi, Gamma, beta, H + (size_t)U.sub * d, gamma[U.sub], nullptr, nullptr);
        if (st < 0) return st;
        auto t1 = std::chrono::steady_clock::now();
        o->ms[0] += std::chrono::duration<double, std::milli>(t1 - t0).count();
        struct Lap {
            double* acc;
            std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
            ~Lap() { *acc += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count(); }
        } lap{&o->ms[1]};
        double rfz[2], rm[16], rc[128], gs;
        st = mce_get_raw_moments(o->h, 0, rfz, rm, rc, &gs);
        if (st < 0) return st;
        // Re fz of the update: 1/(2 pi G_SCALE_FACTOR) (the raw copy of the
        // first update is not kept by the step path)
        U.gscale = gs;
        U.fz_raw = 1.0 / (2.0 * mce::kPi * gs);
        if (fz_raw) fz_raw[u] = U.fz_raw;
        // host records
        derive_update(*o, U, P, parents, pre, post, &U.terms);
        // the fz tape: recompute Re fz from the recorded lookups on the GPU
        {
            std::vector<EvalDev> ev(U.terms.size());
            for (size_t t = 0; t < U.terms.size(); t++) {
                const TermInfo& ti = U.terms[t];
                ev[t] = EvalDev{ti.parent < 0 ? 0 : ti.parent, ti.lp, ti.lm, ti.enc_lhp, ti.phc, U.first ? 1 : 0,
                                ti.y_eval, val(pre[t].dv), val(pre[t].c)};
            }
            if ((st = dev.upload(ev.data(), ev.size()))) return st;
            if ((st = dfz.ensure(ev.size()))) return st;
            if (!U.first) {
                if ((st = pk.upload(prev->keys.data(), prev->keys.size()))) return st;
                if ((st = pv.upload(prev->vals.data(), prev->vals.size()))) return st;
                if ((st = poffb.upload(prev->off.data(), prev->off.size()))) return st;
                if ((st = pcntb.upload(prev->cells.data(), prev->cells.size()))) return st;
            }
            if (!ev.empty())
                k_adj_eval_fz<<<grid_of((long long)ev.size()), 256>>>(dev.ptr, (int)ev.size(), pk.ptr, pv.ptr,
                                                                  poffb.ptr, pcntb.ptr, dfz.ptr);
            std::vector<double> f(ev.size());
            if (cudaMemcpy(f.data(), dfz.ptr, sizeof(double) * f.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
                return MCE_ERR_CUDA;
            double s = 0;
            for (double x : f) s += x;
            o->fz_check_err = std::max(o->fz_check_err, std::fabs(s - U.fz_raw) / std::max(std::fabs(U.fz_raw), 1e-300));
        }
        if (U.last) break;
        if ((st = o->dump(U.kept))) return st;
        const Tables& K = U.kept;
        // reduction groups and which post-MU term each kept slot holds
        std::vector<std::vector<int>> byshape(o->MS + 1);
        for (size_t t = 0; t < post.size(); t++) byshape[post[t].m].push_back((int)t);
        U.kept_first.assign(K.nt, 0);
        U.kept_n.assign(K.nt, 0);
        U.kept_term.assign(K.nt, -1);
        int slot = 0;
        // candidates per kept slot (in member order): (term, s_fixed, conj)
        for (int m = 0; m <= o->MS; m++) {
            if (byshape[m].empty()) continue;
            std::vector<const Rec<double>*> T;
            for (int t : byshape[m]) T.push_back(&post[t]);
            std::vector<int> F;
            if (U.first) {
                F.resize(T.size());
                for (size_t i = 0; i < T.size(); i++) F[i] = (int)i;
            } else
                ftr(T, d, F);
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
                        if (same_record(*T[cand[c]], K, slot, o->MS, d)) {
                            holder = (int)c;
                            break;
                        }
                if (holder < 0) continue;  // the whole group was approximated out
                const int root_term = byshape[m][cand[holder]];
                U.kept_term[slot] = root_term;
                U.kept_first[slot] = (int)U.members.size();
                for (size_t c = holder; c < cand.size(); c++) {
                    const int term = byshape[m][cand[c]];
                    Member mb;
                    mb.term = term;
                    mb.kept = slot;
                    int s = orientation_mask(post[root_term].A.data(), post[term].A.data(), m, d);
                    const int top = 1 << (m - 1), rev = (1 << m) - 1;
                    mb.conj = (s & top) ? 1 : 0;
                    if (s & top) s ^= rev;
                    mb.s_fixed = c == (size_t)holder ? 0 : s;
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
            mi[j] = minfo_of(U.terms[mb.term], post[mb.term], mb, K, U.first, d);
            item_off[j + 1] = item_off[j] + K.cells[mb.kept];
        }
        const long long nitems = item_off[nmem];
        if ((st = dmi.upload(mi.data(), nmem))) return st;
        if ((st = ditem.upload(item_off.data(), nmem + 1))) return st;
        U.mi = mi;
        U.item_off = item_off;
        if ((st = dk.upload(K.keys.data(), K.keys.size()))) return st;
        if ((st = dv.upload(K.vals.data(), K.vals.size()))) return st;
        if ((st = doff.upload(K.off.data(), K.off.size()))) return st;
        if ((st = dcnt.upload(K.cells.data(), K.cells.size()))) return st;
        if ((st = dvals.ensure(nitems + 1))) return st;
        if ((st = dalive.ensure(nmem + 1))) return st;
        cudaMemset(dalive.ptr, 0, sizeof(int) * (nmem + 1));
        if (nitems > 0)
            k_adj_member_values<<<grid_of(nitems), 256>>>(dmi.ptr, ditem.ptr, nmem, nitems, dk.ptr, pk.ptr, pv.ptr,
                                                       poffb.ptr, pcntb.ptr, U.gscale, dvals.ptr, dalive.ptr);
        std::vector<int> alive(nmem);
        if (cudaMemcpy(alive.data(), dalive.ptr, sizeof(int) * nmem, cudaMemcpyDeviceToHost) != cudaSuccess)
            return MCE_ERR_CUDA;
        for (int j = 0; j < nmem; j++) U.members[j].contrib = (U.first || alive[j]) ? 1 : 0;
        for (int k = 0; k < K.nt; k++) U.members[U.kept_first[k]].contrib = 1;  // the holder itself
        std::vector<int> contrib(nmem);
        for (int j = 0; j < nmem; j++) contrib[j] = U.members[j].contrib;
        std::vector<long long> kf(K.nt);
        for (int k = 0; k < K.nt; k++) kf[k] = U.kept_first[k];
        if ((st = dcontrib.upload(contrib.data(), nmem))) return st;
        if ((st = dkfirst.upload(kf.data(), K.nt))) return st;
        if ((st = dknm.upload(U.kept_n.data(), K.nt))) return st;
        if ((st = derr.ensure(1))) return st;
        cudaMemset(derr.ptr, 0, sizeof(unsigned long long));
        const long long ncells = K.off[K.nt];
        if (ncells > 0)
            k_adj_check_tables<<<grid_of(ncells), 256>>>(dkfirst.ptr, dknm.ptr, dmi.ptr, ditem.ptr, dcontrib.ptr,
                                                      dvals.ptr, doff.ptr, dcnt.ptr, dv.ptr, K.nt, derr.ptr);
        unsigned long long eb = 0;
        if (cudaMemcpy(&eb, derr.ptr, sizeof(eb), cudaMemcpyDeviceToHost) != cudaSuccess) return MCE_ERR_CUDA;
        double e;
        memcpy(&e, &eb, sizeof(e));
        o->max_table_err = std::max(o->max_table_err, e);
        // the next parents: the kept terms' records
        std::vector<Rec<double>> next(K.nt);
        for (int k = 0; k < K.nt; k++) next[k] = post[U.kept_term[k]];
        parents.swap(next);
        // the kept tables become the next update's parent tables
        if ((st = pk.upload(K.keys.data(), K.keys.size()))) return st;
        if ((st = pv.upload(K.vals.data(), K.vals.size()))) return st;
        if ((st = poffb.upload(K.off.data(), K.off.size()))) return st;
        if ((st = pcntb.upload(K.cells.data(), K.cells.size()))) return st;
        prev = &U.kept;
    }
    if (cudaGetLastError() != cudaSuccess) return MCE_ERR_CUDA;
    return MCE_OK;
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
    return o->pncc + o->p + o->d + o->d * o->d + o->d * o->pncc + o->p * o->d;
}

int mce_adjoint_backward(mce_adjoint* o, const double* w, double* grad)
{
    if (!o || !w || !grad || o->ups.empty()) return MCE_ERR_ARG;
    const int nup = (int)o->ups.size();
    int st;
    auto tb0 = std::chrono::steady_clock::now();
    // ---- reverse over the tables and the fz seeds (GPU)
    Buf<int> pk, kk, dcontrib;
    Buf<cd> pv, kbar, pbar;
    Buf<long long> poff, item;
    Buf<int> pcnt;
    Buf<MInfoDev> dmi;
    Buf<double> qbar, dbar, cbar, ybar_e, dbar_e, cbar_e;
    Buf<EvalDev> dev;
    std::vector<cd> tbar;  // adjoint of the kept tables of update u (from update u+1)
    for (int u = nup - 1; u >= 0; u--) {
        Update& U = o->ups[u];
        const Tables* P = u > 0 ? &o->ups[u - 1].kept : nullptr;
        const long long npc = P ? P->off[P->nt] : 0;
        if ((st = pbar.ensure(npc + 1))) return st;
        if (cudaMemset(pbar.ptr, 0, sizeof(cd) * (npc + 1)) != cudaSuccess) return MCE_ERR_CUDA;
        if (P) {
            if ((st = pk.upload(P->keys.data(), P->keys.size()))) return st;
            if ((st = pv.upload(P->vals.data(), P->vals.size()))) return st;
            if ((st = poff.upload(P->off.data(), P->off.size()))) return st;
            if ((st = pcnt.upload(P->cells.data(), P->cells.size()))) return st;
        }
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
            if ((st = dmi.upload(U.mi.data(), nmem))) return st;
            if ((st = item.upload(U.item_off.data(), nmem + 1))) return st;
            if ((st = dcontrib.upload(contrib.data(), nmem))) return st;
            if ((st = kk.upload(K.keys.data(), K.keys.size()))) return st;
            if (tbar.size() != K.vals.size()) tbar.assign(K.vals.size(), mce::mkcd(0, 0));
            if ((st = kbar.upload(tbar.data(), tbar.size()))) return st;
            if ((st = qbar.ensure((size_t)nmem * 32))) return st;
            if ((st = dbar.ensure(nmem))) return st;
            if ((st = cbar.ensure(nmem))) return st;
            cudaMemset(qbar.ptr, 0, sizeof(double) * nmem * 32);
            cudaMemset(dbar.ptr, 0, sizeof(double) * nmem);
            cudaMemset(cbar.ptr, 0, sizeof(double) * nmem);
            if (nitems > 0)
                k_adj_member_reverse<<<grid_of(nitems), 256>>>(dmi.ptr, item.ptr, nmem, nitems, dcontrib.ptr, kk.ptr,
                                                            kbar.ptr, pk.ptr, pv.ptr, poff.ptr, pcnt.ptr, U.gscale,
                                                            pbar.ptr, qbar.ptr, dbar.ptr, cbar.ptr);
            if (cudaMemcpy(U.qbar.data(), qbar.ptr, sizeof(double) * nmem * 32, cudaMemcpyDeviceToHost) ||
                cudaMemcpy(U.dbar_m.data(), dbar.ptr, sizeof(double) * nmem, cudaMemcpyDeviceToHost) ||
                cudaMemcpy(U.cbar_m.data(), cbar.ptr, sizeof(double) * nmem, cudaMemcpyDeviceToHost))
                return MCE_ERR_CUDA;
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
            if ((st = dev.upload(ev.data(), nt))) return st;
            if ((st = ybar_e.ensure(nt))) return st;
            if ((st = dbar_e.ensure(nt))) return st;
            if ((st = cbar_e.ensure(nt))) return st;
            k_adj_eval_reverse<<<grid_of(nt), 256>>>(dev.ptr, nt, w[u], pk.ptr, pv.ptr, poff.ptr, pcnt.ptr, pbar.ptr,
                                                      ybar_e.ptr, dbar_e.ptr, cbar_e.ptr);
            if (cudaMemcpy(U.ybar_e.data(), ybar_e.ptr, sizeof(double) * nt, cudaMemcpyDeviceToHost) ||
                cudaMemcpy(U.dbar_e.data(), dbar_e.ptr, sizeof(double) * nt, cudaMemcpyDeviceToHost) ||
                cudaMemcpy(U.cbar_e.data(), cbar_e.ptr, sizeof(double) * nt, cudaMemcpyDeviceToHost))
                return MCE_ERR_CUDA;
        }
        tbar.assign(npc, mce::mkcd(0, 0));
        if (npc && cudaMemcpy(tbar.data(), pbar.ptr, sizeof(cd) * npc, cudaMemcpyDeviceToHost) != cudaSuccess)
            return MCE_ERR_CUDA;
    }
    if (cudaGetLastError() != cudaSuccess) return MCE_ERR_CUDA;
    // ---- the record chain: tangents of the scalars that enter the g values,
    // one parameter direction at a time, dotted with their adjoints
    auto tb1 = std::chrono::steady_clock::now();
    o->ms[2] += std::chrono::duration<double, std::milli>(tb1 - tb0).count();
    // ---- the record chain on the GPU: a thread per (parent, direction)
    const int N = mce_adjoint_num_params(o);
    const int d = o->d, MS = o->MS, rec = MS * d + MS + d;
    long long maxP = 1;
    for (int u = 0; u + 1 < nup; u++) maxP = std::max<long long>(maxP, o->ups[u].kept.nt);
    Buf<double> tin, tout, dgrad, dPA, dPp, dPb, dyb, ddb, dcb, dqt, ddt, dct;
    Buf<double> dpar[8];
    Buf<int> dPm, dkid, dkept;
    Buf<unsigned> dsn, dhp;
    if ((st = tin.ensure((size_t)N * maxP * rec))) return st;
    if ((st = tout.ensure((size_t)N * maxP * rec))) return st;
    if ((st = dgrad.ensure(N))) return st;
    cudaMemset(dgrad.ptr, 0, sizeof(double) * N);
    const std::vector<double>* pv_[8] = {&o->beta, &o->gamma, &o->p0, &o->Phi, &o->Gamma, &o->H, &o->A0, &o->b0};
    for (int i = 0; i < 8; i++)
        if ((st = dpar[i].upload(pv_[i]->data(), pv_[i]->size()))) return st;
    for (int u = 0; u < nup; u++) {
        const Update& U = o->ups[u];
        const int nt = (int)U.terms.size();
        const int nP = u == 0 ? 1 : o->ups[u - 1].kept.nt;
        if (u > 0) {
            const Tables& K = o->ups[u - 1].kept;
            if ((st = dPm.upload(K.shape.data(), K.shape.size()))) return st;
            if ((st = dPA.upload(K.A.data(), K.A.size()))) return st;
            if ((st = dPp.upload(K.p.data(), K.p.size()))) return st;
            if ((st = dPb.upload(K.b.data(), K.b.size()))) return st;
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
        if ((st = dkid.upload(kid_off.data(), nP))) return st;
        if ((st = dsn.upload(sn.data(), nt))) return st;
        if ((st = dhp.upload(hp.data(), nt))) return st;
        if ((st = dyb.upload(U.ybar_e.data(), nt))) return st;
        if ((st = ddb.upload(U.dbar_e.data(), nt))) return st;
        if ((st = dcb.upload(U.cbar_e.data(), nt))) return st;
        if ((st = dqt.upload(qt.data(), qt.size()))) return st;
        if ((st = ddt.upload(dt.data(), nt))) return st;
        if ((st = dct.upload(ct.data(), nt))) return st;
        if ((st = dkept.upload(kept_of.data(), nt))) return st;
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
        ca.beta = dpar[0].ptr;
        ca.gamma = dpar[1].ptr;
        ca.p0 = dpar[2].ptr;
        ca.Phi = dpar[3].ptr;
        ca.Gamma = dpar[4].ptr;
        ca.H = dpar[5].ptr;
        ca.A0 = dpar[6].ptr;
        ca.b0 = dpar[7].ptr;
        ca.PA = dPA.ptr;
        ca.Pp = dPp.ptr;
        ca.Pb = dPb.ptr;
        ca.Pm = dPm.ptr;
        ca.Tin = tin.ptr;
        ca.Tout = tout.ptr;
        ca.rec = rec;
        ca.n_next = n_next;
        ca.kid_off = dkid.ptr;
        ca.sneg = dsn.ptr;
        ca.hpre = dhp.ptr;
        ca.ybar_e = dyb.ptr;
        ca.dbar_e = ddb.ptr;
        ca.cbar_e = dcb.ptr;
        ca.qbar_t = dqt.ptr;
        ca.dbar_t = ddt.ptr;
        ca.cbar_t = dct.ptr;
        ca.kept_of = dkept.ptr;
        ca.grad = dgrad.ptr;
        const long long nthr = (long long)nP * N;
        k_adj_chain<<<(int)((nthr + 127) / 128), 128>>>(ca);
        std::swap(tin.ptr, tout.ptr);
        std::swap(tin.cap, tout.cap);
    }
    if (cudaMemcpy(grad, dgrad.ptr, sizeof(double) * N, cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        mce::report_error("adjoint: the record chain failed on the GPU");
        return MCE_ERR_CUDA;
    }
    o->ms[3] += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb1).count();
    return MCE_OK;
}

void mce_adjoint_destroy(mce_adjoint* o) { delete o; }

}  // extern "C"
