// N-D conditional pdf of one estimator at a batch of points:
// PointWiseNDimCauchyCPDF::evaluate_cpdf (include/cpdf_ndim.hpp:677-904).
//
// The characteristic function is integrated one spectral dimension at a time.
// Lowering a term of dimension ld (construct_lowered_parent_elements
// :392-443, construct_lowered_children :520-641) gives one child of
// dimension ld - 1 per hyperplane whose last component is not zero; the child
// is coaligned as an MU child is (mu_coalign, cauchy_term.hpp:533-745), its
// cells come from the parent's cells (make_lowered_child_btable,
// cell_enumeration.hpp:1121-1279) and its g-table from the parent's
// (make_gtable, flattening.hpp:77-255, G_SCALE_FACTOR 1).  After d - 1
// lowerings every term is one-dimensional and integrates in closed form
// (evaluate_1d_cf :643-666); the value is the sum / Re fz / (2 pi)^d.
//
// Each (point, term) pair lowers on its own: the reference's term reduction
// between the lowerings (fast_term_reduction + make_gtables over reduction
// groups) adds the g-tables of terms whose arrangements agree within 1e-8
// before lowering them once; lowering them separately and adding at the end
// gives the same sum up to rounding (the integral is linear in the g-table),
// and every term the reference approximates out (per child, before any
// addition) is approximated out here too.
//
// Layout, all device arrays, point-major at every level (the children of a
// parent follow one another, parents follow their point): per term m, A
// [MC][ld], p [MC], b [ld], the slice (toff, tcnt) of the level's g-table
// arena (ascending half-storage keys and their values).
#include "mce_kernels.cuh"
#include "mce_c_api.h"

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

namespace mce {

void report_error(const std::string& s);

namespace {

template <typename T>
struct NdBuf {
    T* ptr = nullptr;
    size_t cap = 0;
    NdBuf() = default;
    NdBuf(const NdBuf&) = delete;
    NdBuf& operator=(const NdBuf&) = delete;
    ~NdBuf()
    {
        if (ptr) cudaFree(ptr);
    }
    int ensure(size_t n)
    {
        if (n <= cap && ptr) return MCE_OK;
        // half again as large as the last size, so that a sequence of calls
        // growing a little at a time does not reallocate at every call
        const size_t want = std::max<size_t>(std::max(n, cap + cap / 2), 64);
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
        if (cudaMalloc(&ptr, want * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            report_error("cudaMalloc of " + std::to_string(want * sizeof(T)) + " bytes failed (N-D pdf)");
            return MCE_ERR_NOMEM;
        }
        cap = want;
        return MCE_OK;
    }
};

// One level's terms.
struct NdTerms {
    int* pt;
    int* m;
    double* A;
    double* p;
    double* b;
    long long* toff;
    int* tcnt;
};
struct NdTermBufs {
    NdBuf<int> pt, m, tcnt;
    NdBuf<double> A, p, b;
    NdBuf<long long> toff;
    int ensure(long long n, int MC, int ld)
    {
        int s = MCE_OK;
        s |= pt.ensure(n + 1);
        s |= m.ensure(n + 1);
        s |= tcnt.ensure(n + 1);
        s |= A.ensure((size_t)(n + 1) * MC * ld);
        s |= p.ensure((size_t)(n + 1) * MC);
        s |= b.ensure((size_t)(n + 1) * ld);
        s |= toff.ensure(n + 2);
        return s;
    }
    NdTerms view() { return NdTerms{pt.ptr, m.ptr, A.ptr, p.ptr, b.ptr, toff.ptr, tcnt.ptr}; }
};

// Lowered children of one level.
struct NdKids {
    int* pt;
    long long* par;   // parent (index into the parent level)
    int* m;           // rows after coalignment
    int* mpre;        // rows before (parent rows - 1)
    int* phc;         // parent rows (bits of the parent's keys)
    int* z;           // the integrated hyperplane's index in the parent
    int* lhp;         // enc_lambda_bar
    unsigned* horthog;  // rows that do not enter the integration formula
    int* hcm;         // coalignment merged rows
    double* A;        // [MC][lc]
    double* p;        // [MC]
    double* q;        // [MC]
    double* b;        // [lc]
    double* cval;
    double* dval;
    unsigned char* cmap;  // [MC]
    signed char* csmap;   // [MC]
    int* ccnt;        // cells
    int* keep;        // not approximated out
};
struct NdKidBufs {
    NdBuf<int> pt, m, mpre, phc, z, lhp, hcm, ccnt, keep;
    NdBuf<long long> par;
    NdBuf<unsigned> horthog;
    NdBuf<double> A, p, q, b, cval, dval;
    NdBuf<unsigned char> cmap;
    NdBuf<signed char> csmap;
    int ensure(long long n, int MC, int lc)
    {
        int s = MCE_OK;
        s |= pt.ensure(n + 1);
        s |= m.ensure(n + 1);
        s |= mpre.ensure(n + 1);
        s |= phc.ensure(n + 1);
        s |= z.ensure(n + 1);
        s |= lhp.ensure(n + 1);
        s |= hcm.ensure(n + 1);
        s |= ccnt.ensure(n + 1);
        s |= keep.ensure(n + 1);
        s |= par.ensure(n + 1);
        s |= horthog.ensure(n + 1);
        s |= A.ensure((size_t)(n + 1) * MC * std::max(lc, 1));
        s |= p.ensure((size_t)(n + 1) * MC);
        s |= q.ensure((size_t)(n + 1) * MC);
        s |= b.ensure((size_t)(n + 1) * std::max(lc, 1));
        s |= cval.ensure(n + 1);
        s |= dval.ensure(n + 1);
        s |= cmap.ensure((size_t)(n + 1) * MC);
        s |= csmap.ensure((size_t)(n + 1) * MC);
        return s;
    }
    NdKids view()
    {
        return NdKids{pt.ptr,   par.ptr,  m.ptr,     mpre.ptr, phc.ptr,   z.ptr,     lhp.ptr,  horthog.ptr,
                      hcm.ptr,  A.ptr,    p.ptr,     q.ptr,    b.ptr,     cval.ptr,  dval.ptr, cmap.ptr,
                      csmap.ptr, ccnt.ptr, keep.ptr};
    }
};

constexpr int kNdMaxRows = 16;  // hyperplanes per term (cell bitmaps of 2^m bits in shared memory)

inline int nd_grid(long long n, int per, int num_sms)
{
    long long g = (n + per - 1) / per;
    const long long cap = (long long)num_sms * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

// ---------------------------------------------------------------------------
// Children per (point, parent): the hyperplanes whose last component is not
// zero (|a| > MU_EPS, cpdf_ndim.hpp:370, 411), for parents of at least ld
// rows (cpdf_ndim.hpp:711-716).  Pair i is (point i / n, parent i % n) on the
// first level (nrep points), parent i afterwards.
template <int LD>
__global__ void k_nd_count(NdTerms P, long long n, long long npairs, int MC, int* cnt)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npairs;
         i += (long long)gridDim.x * blockDim.x) {
        const long long t = i % n;
        const int m = P.m[t];
        int c = 0;
        if (m >= LD) {
            const double* A = P.A + t * MC * LD;
            for (int r = 0; r < m; r++)
                if (fabs(A[r * LD + LD - 1]) > kMuEps) c++;
        }
        cnt[i] = c;
    }
}

// mu_coalign (cauchy_term.hpp:533-745) of one lowered child held by the
// calling thread: rows normalised (q = p first), coaligned rows merged with
// their p and q, the coalignment maps recorded.  Returns the new row count,
// or -1 where the reference exits (two unintegrable rows anti-coaligned).
template <int LC>
__device__ int nd_coalign(double* A, double* p, double* q, unsigned& hor, int m, unsigned char* cmap,
                          signed char* csmap)
{
    for (int i = 0; i < m; i++) {
        q[i] = p[i];
        double n1 = 0;
        for (int j = 0; j < LC; j++) n1 += fabs(A[i * LC + j]);
        p[i] *= n1;
        for (int j = 0; j < LC; j++) A[i * LC + j] /= n1;
    }
    bool F[kNdMaxRows], hf[kNdMaxRows];
    for (int j = 0; j < m; j++) {
        F[j] = true;
        hf[j] = hor ? ((hor >> j) & 1u) : false;
        cmap[j] = 255;
        csmap[j] = 1;
    }
    int uc = 0;
    for (int j = 0; j < m - 1; j++) {
        if (!F[j]) continue;
        cmap[j] = (unsigned char)uc;
        for (int k = j + 1; k < m; k++) {
            if (!F[k]) continue;
            const int g = coalign_gate<LC>(A + j * LC, A + k * LC);
            if (g == 1) {
                if (hor) {
                    const bool hj = hf[j], hk = hf[k];
                    if (!hj && !hk) q[j] += q[k];
                    else if (hj && !hk) {
                        q[j] = q[k];
                        hf[j] = false;
                    } else if (!hj && hk) hf[k] = false;
                    else {
                        hf[k] = false;
                        q[j] += q[k];
                    }
                } else
                    q[j] += q[k];
                F[k] = false;
                p[j] += p[k];
                cmap[k] = (unsigned char)uc;
                csmap[k] = 1;
            } else if (g == -1) {
                if (hor) {
                    const bool hj = hf[j], hk = hf[k];
                    if (!hj && !hk) q[j] -= q[k];
                    else if (hj && !hk) {
                        q[j] = -q[k];
                        hf[j] = false;
                    } else if (!hj && hk) hf[k] = false;
                    else return -1;
                } else
                    q[j] -= q[k];
                F[k] = false;
                p[j] += p[k];
                cmap[k] = (unsigned char)uc;
                csmap[k] = -1;
            }
        }
        uc++;
    }
    if (F[m - 1]) cmap[m - 1] = (unsigned char)uc;
    int ns = 0;
    for (int i = 0; i < m; i++) ns += F[i] ? 1 : 0;
    if (ns != m) {
        int u = 1;
        for (int j = 1; j < m; j++)
            if (F[j]) {
                if (u < j) {
                    for (int l = 0; l < LC; l++) A[u * LC + l] = A[j * LC + l];
                    p[u] = p[j];
                    q[u] = q[j];
                }
                u++;
            }
        if (hor) {
            unsigned nh = 0;
            int c = 0;
            for (int j = 0; j < m; j++)
                if (F[j]) nh |= (hf[j] ? 1u : 0u) << c++;
            hor = nh;
        }
    }
    return ns;
}

// The lowered children, coaligned, a thread per child: child c belongs to
// the pair i whose children start at coff[i] <= c, and integrates the
// (c - coff[i])-th of its parent's rows with a nonzero last component.
// x: the points [npts][D] on the first level, else null.
template <int LD>
__global__ void k_nd_lower(NdTerms P, long long n, long long npairs, const double* x, int D, const long long* coff,
                           long long nk, int MC, NdKids K, int* err)
{
    constexpr int LC = LD - 1;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nk;
         c += (long long)gridDim.x * blockDim.x) {
        long long lo = 0, hi = npairs;
        while (hi - lo > 1) {
            const long long mid = (lo + hi) >> 1;
            if (coff[mid] <= c) lo = mid;
            else hi = mid;
        }
        const long long i = lo;
        const int ord = (int)(c - coff[i]);
        const long long t = i % n;
        const int m = P.m[t];
        const int pt = x ? (int)(i / n) : P.pt[t];
        const double* A = P.A + t * MC * LD;
        const double* pp = P.p + t * MC;
        const double* bb = P.b + t * LD;
        // construct_lowered_parent_elements (cpdf_ndim.hpp:392-443)
        double Ald[kNdMaxRows];
        bool nz[kNdMaxRows];
        int lam = 0, tz = 0, k = 0;
        for (int r = 0; r < m; r++) {
            Ald[r] = -A[r * LD + LD - 1];
            nz[r] = fabs(Ald[r]) > kMuEps;
            if (nz[r]) {
                if (Ald[r] < 0) lam |= 1 << r;
                if (k++ == ord) tz = r;
            }
        }
        double mu_t[LC > 0 ? LC : 1];
        for (int j = 0; j < LC; j++) mu_t[j] = A[tz * LD + j] / Ald[tz];
        double tb;
        double* bo = K.b + c * LC;
        if (x) {
            const double* xp = x + (long long)pt * D;
            tb = bb[LC] - xp[LC];
            for (int j = 0; j < LC; j++) bo[j] = (bb[j] - xp[j]) + tb * mu_t[j];
        } else {
            tb = bb[LC];
            for (int j = 0; j < LC; j++) bo[j] = bb[j] + tb * mu_t[j];
        }
        // construct_lowered_children (cpdf_ndim.hpp:579-636): rows mu_l - mu_t
        double Ac[kNdMaxRows * (LC > 0 ? LC : 1)], pc[kNdMaxRows], qc[kNdMaxRows];
        int l_ = 0;
        unsigned unint = 0;
        for (int l = 0; l < m; l++) {
            if (l == tz) continue;
            if (nz[l]) {
                for (int j = 0; j < LC; j++) Ac[l_ * LC + j] = A[l * LD + j] / Ald[l] - mu_t[j];
                pc[l_] = pp[l] * fabs(Ald[l]);
            } else {
                for (int j = 0; j < LC; j++) Ac[l_ * LC + j] = A[l * LD + j];
                pc[l_] = pp[l];
                unint |= 1u << l_;
            }
            l_++;
        }
        const int mpre = m - 1;
        unsigned char* cm = K.cmap + c * MC;
        signed char* cs = K.csmap + c * MC;
        const int ns = nd_coalign<LC>(Ac, pc, qc, unint, mpre, cm, cs);
        if (ns < 0) {
            atomicOr(err, kErrAntiCoalignedHorthog);
            K.m[c] = 0;
            K.keep[c] = 0;
            K.ccnt[c] = 0;
            continue;
        }
        double* Ao = K.A + c * MC * LC;
        for (int q = 0; q < ns * LC; q++) Ao[q] = Ac[q];
        for (int q = 0; q < ns; q++) {
            K.p[c * MC + q] = pc[q];
            K.q[c * MC + q] = qc[q];
        }
        K.pt[c] = pt;
        K.par[c] = t;
        K.m[c] = ns;
        K.mpre[c] = mpre;
        K.phc[c] = m;
        K.z[c] = tz;
        K.lhp[c] = lam;
        K.horthog[c] = unint;
        K.hcm[c] = ns < mpre ? 1 : 0;
        K.cval[c] = tb;
        K.dval[c] = pp[tz] * fabs(Ald[tz]);
        K.keep[c] = 0;
    }
}

__device__ inline int nd_remove_bit(int b, int bit) { return ((b >> (bit + 1)) << bit) | (b & ((1 << bit) - 1)); }

// Children of at most lc rows, a thread each: no cells below lc rows (they
// evaluate to zero and are not carried, cpdf_ndim.hpp:773-776), the
// 2^lc / 2 trivial cells at lc rows (cell_enumeration.hpp:1129-1136).  The
// others are flagged for the warp-per-child enumeration.
template <int LC>
__global__ void k_nd_cells_small(NdKids K, long long nk, const long long* coff, int* keys_out, int* big)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nk;
         c += (long long)gridDim.x * blockDim.x) {
        const int m = K.m[c];
        if (!keys_out) {
            big[c] = m > LC ? 1 : 0;
            if (m <= LC) K.ccnt[c] = m < LC ? 0 : (1 << LC) / 2;
        } else if (m == LC) {
            for (int k = 0; k < (1 << LC) / 2; k++) keys_out[coff[c] + k] = k;
        }
    }
}

__global__ void k_nd_list(const int* big, const long long* bscan, long long nk, long long* list)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nk;
         c += (long long)gridDim.x * blockDim.x)
        if (big[c]) list[bscan[c]] = c;
}

// Cells of each lowered child (make_lowered_child_btable): the parent cells
// b (keys in the enc_lambda_bar frame) whose neighbour across the
// integrated hyperplane is a parent cell too, bit z removed (the last child
// keeps the smaller of the two opposite keys), projected through the
// coalignment map.  A warp per child; the parent's keys and the child's
// cells as bitmaps in shared memory.  keys_out null: counts into ccnt;
// else the ascending keys from coff[c] on.
template <int LC>
__global__ void k_nd_cells(const long long* ptoff, const int* ptcnt, const int* pkeys, NdKids K,
                           const long long* list, const long long* nlist, int MC, int MB, const long long* coff,
                           int* keys_out)
{
    extern __shared__ unsigned nd_smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwb = blockDim.x >> 5;
    // bitmaps of 2^MB bits: no parent or child has more than MB rows
    const int words = (1 << MB) > 32 ? (1 << MB) / 32 : 1;
    unsigned* PB = nd_smem + (size_t)wib * (2 * words + 32);
    unsigned* RK = PB + words;
    int* bmk = reinterpret_cast<int*>(RK + words);
    const long long nl = *nlist;
    for (long long li = (long long)blockIdx.x * nwb + wib; li < nl; li += (long long)gridDim.x * nwb) {
        const long long c = list[li];
        const int m = K.m[c];
        if (m < LC) {
            if (!keys_out && lane == 0) K.ccnt[c] = 0;
            continue;
        }
        if (m == LC) {
            const int nc = (1 << LC) / 2;
            if (!keys_out) {
                if (lane == 0) K.ccnt[c] = nc;
            } else {
                for (int k = lane; k < nc; k += 32) keys_out[coff[c] + k] = k;
            }
            continue;
        }
        const long long par = K.par[c];
        const int phc = K.phc[c], z = K.z[c];
        const int top = 1 << (phc - 1), rev = (1 << phc) - 1, mz = 1 << z;
        int lhp = K.lhp[c];
        if (lhp & top) lhp ^= rev;
        const int wp = (1 << phc) > 32 ? (1 << phc) / 32 : 1;
        const int wm = (1 << m) > 32 ? (1 << m) / 32 : 1;
        for (int k = lane; k < wp; k += 32) PB[k] = 0;
        for (int k = lane; k < wm; k += 32) RK[k] = 0;
        const bool coal = K.hcm[c] != 0;
        if (coal && lane == 0) {
            // first row of every coalignment group (cell_enumeration.hpp:1228-1240)
            const unsigned char* cm = K.cmap + c * MC;
            const int mpre = K.mpre[c];
            unsigned seen = 0;
            int cnt = 0;
            for (int j = 0; j < mpre; j++) {
                const int ci = cm[j];
                if (ci < 32 && !((seen >> ci) & 1u)) {
                    seen |= 1u << ci;
                    bmk[cnt++] = j;
                }
            }
            bmk[31] = cnt;
        }
        __syncwarp();
        const int* pk = pkeys + ptoff[par];
        const int np = ptcnt[par];
        for (int k = lane; k < np; k += 32) {
            const int key = pk[k] ^ lhp;
            if (key >= 0 && key < (1 << phc)) atomicOr(&PB[key >> 5], 1u << (key & 31));
        }
        __syncwarp();
        const bool last = z == phc - 1;
        const int ncoal = coal ? bmk[31] : 0;
        for (int k = lane; k < np; k += 32) {
            const int b = pk[k] ^ lhp;
            int bq = b ^ mz;
            if (last) bq ^= rev;
            if (bq < 0 || bq >= (1 << phc) || !((PB[bq >> 5] >> (bq & 31)) & 1u)) continue;
            int key = nd_remove_bit(b, z);
            if (last) {
                const int c2 = nd_remove_bit(bq, z);
                if (c2 < key) key = c2;
            }
            if (coal) {
                int bc = 0;
                for (int l = 0; l < ncoal; l++)
                    if (key & (1 << bmk[l])) bc |= 1 << l;
                key = bc;
            }
            if (key >= 0 && key < (1 << m)) atomicOr(&RK[key >> 5], 1u << (key & 31));
        }
        __syncwarp();
        // count, or the ascending keys
        int count = 0;
        for (int w0 = 0; w0 < wm; w0 += 32) {
            const int w = w0 + lane;
            unsigned bits = w < wm ? RK[w] : 0u;
            if ((1 << m) < 32) bits &= (1u << (1 << m)) - 1u;
            const int cc = __popc(bits);
            int pre = cc;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, pre, o);
                if (lane >= o) pre += y;
            }
            const int tot = __shfl_sync(0xffffffffu, pre, 31);
            if (keys_out) {
                int pos = count + pre - cc;
                int* out = keys_out + coff[c];
                while (bits) {
                    const int bb = __ffs(bits) - 1;
                    bits &= bits - 1;
                    out[pos++] = w * 32 + bb;
                }
            }
            count += tot;
        }
        if (!keys_out && lane == 0) K.ccnt[c] = count;
        __syncwarp();
    }
}

// g of every (child, cell) (make_gtable, flattening.hpp:128-247, the new-child
// branch) and the term-approximation test; a thread per item.
template <int LC>
__global__ void k_nd_gvals(const long long* ptoff, const int* ptcnt, const int* pkeys, const cd* pvals, NdKids K,
                           long long nk, int MC, const long long* coff, long long nitems, const int* keys, cd* vals)
{
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < nitems;
         x += (long long)gridDim.x * blockDim.x) {
        // the last child whose cells start at or before x (children without
        // cells share the next child's offset and come before it)
        long long lo = 0, hi = nk;
        while (hi - lo > 1) {
            const long long mid = (lo + hi) >> 1;
            if (coff[mid] <= x) lo = mid;
            else hi = mid;
        }
        const long long c = lo;
        const int m = K.m[c];
        const int phc = K.phc[c], z = K.z[c];
        const unsigned hor = K.horthog[c];
        const double* q = K.q + c * MC;
        const int be = keys[x];
        double ygi = 0;
        int sb[kNdMaxRows];
        for (int k = 0; k < m; k++) {
            sb[k] = ((be >> k) & 1) ? -1 : 1;
            if (!hor || !(hor & (1u << k))) ygi += q[k] * sb[k];
        }
        int lp = 0, lm = 0;
        {
            const bool coal = K.hcm[c] != 0;
            const unsigned char* cm = K.cmap + c * MC;
            const signed char* cs = K.csmap + c * MC;
            int k = 0, l = 0;
            while (k < phc) {
                if (k == z) {
                    lm |= 1 << k;
                    k++;
                    if (k == phc) break;
                }
                const int bv = coal ? sb[cm[l]] * cs[l] : sb[l];
                if (bv < 0) {
                    lp |= 1 << k;
                    lm |= 1 << k;
                }
                k++;
                l++;
            }
        }
        const long long par = K.par[c];
        const int* pk = pkeys + ptoff[par];
        const cd* pv = pvals + ptoff[par];
        const int np = ptcnt[par];
        const int lhp = K.lhp[c];
        const cd gp = lookup_num(pk, pv, np, lp ^ lhp, phc);
        const cd gm = lookup_num(pk, pv, np, lm ^ lhp, phc);
        const double cv = K.cval[c], dv = K.dval[c];
        cd v = csub(cdiv(gp, mkcd(ygi + dv, cv)), cdiv(gm, mkcd(ygi - dv, cv)));
        v = cscale(v, 1.0);
        vals[x] = v;
        double ps = 0;
        const double* p = K.p + c * MC;
        for (int k = 0; k < m; k++) ps += p[k];
        ps *= ps;
        if (above_approx_threshold(ps, v.re, v.im)) K.keep[c] = 1;
    }
}

// The children that keep a g-table become the next level's terms.
template <int LC>
__global__ void k_nd_compact(NdKids K, long long nk, int MC, const long long* kscan, const long long* coff,
                             NdTerms N)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nk;
         c += (long long)gridDim.x * blockDim.x) {
        if (!K.keep[c]) continue;
        const long long o = kscan[c];
        const int m = K.m[c];
        N.pt[o] = K.pt[c];
        N.m[o] = m;
        for (int q = 0; q < m * LC; q++) N.A[o * MC * LC + q] = K.A[c * MC * LC + q];
        for (int q = 0; q < m; q++) N.p[o * MC + q] = K.p[c * MC + q];
        for (int q = 0; q < LC; q++) N.b[o * LC + q] = K.b[c * LC + q];
        N.toff[o] = coff[c];
        N.tcnt[o] = K.ccnt[c];
    }
}

__global__ void k_nd_keep_int(const NdKids K, long long nk, int* keep_i)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nk;
         c += (long long)gridDim.x * blockDim.x)
        keep_i[c] = K.keep[c] && K.ccnt[c] > 0 ? 1 : 0;
}

// The first term of every point (terms are point-major): pstart[p] =
// lower_bound(pt, p), p = 0..npts.
__global__ void k_nd_point_starts(const int* pt, long long n, int npts, long long* pstart)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > npts) return;
    long long lo = 0, hi = n;
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (pt[mid] < p) lo = mid + 1;
        else hi = mid;
    }
    pstart[p] = lo;
}

constexpr int kNdFinalThreads = 256;
constexpr long long kNdFinalChunk = 1LL << 14;  // terms per block of the final sum

// evaluate_1d_cf (cpdf_ndim.hpp:643-666) summed over a chunk of one point's
// one-dimensional terms; block b takes chunk b - coff[p] of point p (coff:
// exclusive scan of the points' chunk counts).  Fixed-order tree sums: the
// result does not depend on the launch.
__global__ void k_nd_final_partial(NdTerms T, int MC, const int* keys, const cd* vals, const long long* pstart,
                                   const long long* coff, int npts, cd* partial)
{
    __shared__ double sre[kNdFinalThreads], sim[kNdFinalThreads];
    const long long b = blockIdx.x;
    int lo = 0, hi = npts;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (coff[mid] <= b) lo = mid;
        else hi = mid;
    }
    const int p = lo;
    const long long a = pstart[p] + (b - coff[p]) * kNdFinalChunk;
    const long long e = min(pstart[p + 1], a + kNdFinalChunk);
    cd s = mkcd(0, 0);
    for (long long i = a + threadIdx.x; i < e; i += kNdFinalThreads) {
        const bool pos_a = T.A[i * MC] > 0;  // A is [MC][1]: row 0 of term i
        const int lp = pos_a ? 1 : 0, lm = pos_a ? 0 : 1;
        const int* k = keys + T.toff[i];
        const cd* v = vals + T.toff[i];
        const int nc = T.tcnt[i];
        const cd gp = lookup_num(k, v, nc, lp, 1);
        const cd gm = lookup_num(k, v, nc, lm, 1);
        const double p0 = T.p[i * MC], b0 = T.b[i];
        s = cadd(s, csub(cdiv(gp, mkcd(p0, b0)), cdiv(gm, mkcd(-p0, b0))));
    }
    sre[threadIdx.x] = s.re;
    sim[threadIdx.x] = s.im;
    __syncthreads();
    for (int o = kNdFinalThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            sre[threadIdx.x] += sre[threadIdx.x + o];
            sim[threadIdx.x] += sim[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[b] = mkcd(sre[0], sim[0]);
}

// Each point's chunk sums in order, then / Re fz * (2 pi)^-d
// (cpdf_ndim.hpp:892-893).
__global__ void k_nd_final_combine(const cd* partial, const long long* coff, int npts, double fz, double scale,
                                   double* out)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    cd s = mkcd(0, 0);
    for (long long c = coff[p]; c < coff[p + 1]; c++) s = cadd(s, partial[c]);
    out[2 * p] = s.re / fz * scale;
    out[2 * p + 1] = s.im / fz * scale;
}

// The marginal pdf's first level (construct_lowered_marginal_parent_elements,
// cpdf_ndim.hpp:445-517): every term's A columns and b in the order
// reo (the states integrated out first, the kept states last).
struct NdReorient {
    int r[kMaxDim];
};
__global__ void k_nd_reorient(const int* m, const double* A, const double* b, long long n, int MC, int D,
                              NdReorient reo, double* Ao, double* bo)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int mt = m[t];
        const double* Ai = A + t * MC * D;
        double* Aw = Ao + t * MC * D;
        for (int i = 0; i < mt; i++)
            for (int j = 0; j < D; j++) Aw[i * D + j] = Ai[i * D + reo.r[j]];
        for (int j = 0; j < D; j++) bo[t * D + j] = b[t * D + reo.r[j]];
    }
}

// The marginal pdf's last stage (cpdf_ndim.hpp:1180-1212) summed over a
// chunk of one point's terms (ld dimensions, A [MC][ld]): each term's g value
// at the sign vector of A nu (bit k set where row k . nu < 0).  Chunks as in
// k_nd_final_partial.
__global__ void k_nd_final_marg_partial(NdTerms T, int MC, int ld, const double* nu, const int* keys, const cd* vals,
                                        const long long* pstart, const long long* coff, int npts, cd* partial)
{
    __shared__ double sre[kNdFinalThreads], sim[kNdFinalThreads];
    const long long b = blockIdx.x;
    int lo = 0, hi = npts;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (coff[mid] <= b) lo = mid;
        else hi = mid;
    }
    const int p = lo;
    const long long a = pstart[p] + (b - coff[p]) * kNdFinalChunk;
    const long long e = min(pstart[p + 1], a + kNdFinalChunk);
    cd s = mkcd(0, 0);
    for (long long i = a + threadIdx.x; i < e; i += kNdFinalThreads) {
        const int m = T.m[i];
        const double* Ai = T.A + i * MC * ld;
        int enc = 0;
        for (int k = 0; k < m; k++) {
            double w = 0.0;
            for (int j = 0; j < ld; j++) w += Ai[k * ld + j] * nu[j];
            if (neg(w)) enc |= 1 << k;
        }
        s = cadd(s, lookup_num(keys + T.toff[i], vals + T.toff[i], T.tcnt[i], enc, m));
    }
    sre[threadIdx.x] = s.re;
    sim[threadIdx.x] = s.im;
    __syncthreads();
    for (int o = kNdFinalThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            sre[threadIdx.x] += sre[threadIdx.x + o];
            sim[threadIdx.x] += sim[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[b] = mkcd(sre[0], sim[0]);
}

}  // namespace

struct NdWork {
    NdTermBufs lev[2];
    NdKidBufs kids;
    NdBuf<int> cnt, keep_i, big, keys[2];
    NdBuf<long long> blist;
    NdBuf<cd> vals[2];
    NdBuf<long long> coff, cellof, kscan, scan_tmp;
    NdBuf<double> x, out;
    NdBuf<double> rA, rb, nu;  // the marginal's reordered first level and nu_bar
    std::vector<double> h_x;
    NdBuf<int> err;
    NdBuf<long long> pstart, pcoff;
    NdBuf<cd> partial;
    std::vector<long long> h_pstart, h_pcoff;
    ScanScratch ss{};
    long long launches = 0;
    int ensure_scan(long long n)
    {
        long long need = 4, t = n;
        while (t > 1) {
            t = (t + 2047) / 2048;
            need += t + 2;
        }
        const int s = scan_tmp.ensure(need + 64);
        if (s) return s;
        ss.block_sums = scan_tmp.ptr;
        ss.cap = (long long)scan_tmp.cap;
        return MCE_OK;
    }
};

NdWork* nd_work_create() { return new NdWork(); }
void nd_work_destroy(NdWork* w) { delete w; }

namespace {

#define ND_CUDA(x)                                                                   \
    do {                                                                             \
        cudaError_t e_ = (x);                                                        \
        if (e_ != cudaSuccess) {                                                     \
            report_error(std::string("CUDA error (N-D pdf): ") + cudaGetErrorString(e_)); \
            return MCE_ERR_CUDA;                                                     \
        }                                                                            \
    } while (0)

template <int LD>
int nd_level(NdWork& w, NdTerms P, const int* pkeys, const cd* pvals, long long n, long long npairs, const double* x,
             int D, int MC, int MB, NdTermBufs& next, int kb, long long* n_next, const LaunchCfg& lc)
{
    constexpr int LC = LD - 1;
    int s;
    const int thr = 128;
    if ((s = w.cnt.ensure(npairs + 1))) return s;
    if ((s = w.coff.ensure(npairs + 2))) return s;
    if ((s = w.ensure_scan(npairs + 1))) return s;
    k_nd_count<LD><<<nd_grid(npairs, thr, lc.num_sms), thr, 0, lc.stream>>>(P, n, npairs, MC, w.cnt.ptr);
    scan_int_to_ll(w.cnt.ptr, w.coff.ptr, npairs, w.ss, lc);
    long long nk = 0;
    ND_CUDA(cudaMemcpyAsync(&nk, w.coff.ptr + npairs, sizeof(long long), cudaMemcpyDeviceToHost, lc.stream));
    ND_CUDA(cudaStreamSynchronize(lc.stream));
    w.launches += 2;
    if (nk == 0) {
        *n_next = 0;
        return MCE_OK;
    }
    if ((s = w.kids.ensure(nk, MC, LC))) return s;
    NdKids K = w.kids.view();
    k_nd_lower<LD><<<nd_grid(nk, thr, lc.num_sms), thr, 0, lc.stream>>>(P, n, npairs, x, D, w.coff.ptr, nk, MC, K,
                                                                      w.err.ptr);
    // cells: counts, offsets, keys
    const int words = (1 << MB) > 32 ? (1 << MB) / 32 : 1;
    const size_t pw = (size_t)(2 * words + 32) * 4;
    int warps = (int)(96 * 1024 / pw);
    if (warps > 4) warps = 4;
    if (warps < 1) warps = 1;
    const size_t sm = pw * warps;
    ND_CUDA(cudaFuncSetAttribute(k_nd_cells<LC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    const int cgrid = nd_grid(nk, warps, lc.num_sms);
    if ((s = w.kscan.ensure(nk + 2))) return s;
    if ((s = w.cellof.ensure(nk + 2))) return s;
    if ((s = w.big.ensure(nk + 1))) return s;
    if ((s = w.blist.ensure(nk + 1))) return s;
    if ((s = w.ensure_scan(nk + 1))) return s;
    // the children of at most lc rows a thread each; the others listed for
    // the warp-per-child enumeration (in 1-D nearly every child coaligns to
    // one row)
    k_nd_cells_small<LC><<<nd_grid(nk, thr, lc.num_sms), thr, 0, lc.stream>>>(K, nk, nullptr, nullptr, w.big.ptr);
    scan_int_to_ll(w.big.ptr, w.kscan.ptr, nk, w.ss, lc);
    k_nd_list<<<nd_grid(nk, thr, lc.num_sms), thr, 0, lc.stream>>>(w.big.ptr, w.kscan.ptr, nk, w.blist.ptr);
    const long long* nlist = w.kscan.ptr + nk;
    k_nd_cells<LC><<<cgrid, warps * 32, sm, lc.stream>>>(P.toff, P.tcnt, pkeys, K, w.blist.ptr, nlist, MC, MB,
                                                         nullptr, nullptr);
    scan_int_to_ll(K.ccnt, w.cellof.ptr, nk, w.ss, lc);
    long long ncell = 0;
    ND_CUDA(cudaMemcpyAsync(&ncell, w.cellof.ptr + nk, sizeof(long long), cudaMemcpyDeviceToHost, lc.stream));
    ND_CUDA(cudaStreamSynchronize(lc.stream));
    w.launches += 3;
    if ((s = w.keys[kb].ensure(ncell + 1))) return s;
    if ((s = w.vals[kb].ensure(ncell + 1))) return s;
    k_nd_cells_small<LC><<<nd_grid(nk, thr, lc.num_sms), thr, 0, lc.stream>>>(K, nk, w.cellof.ptr, w.keys[kb].ptr,
                                                                            nullptr);
    k_nd_cells<LC><<<cgrid, warps * 32, sm, lc.stream>>>(P.toff, P.tcnt, pkeys, K, w.blist.ptr, nlist, MC, MB,
                                                         w.cellof.ptr, w.keys[kb].ptr);
    if (ncell > 0)
        k_nd_gvals<LC><<<nd_grid(ncell, thr, lc.num_sms), thr, 0, lc.stream>>>(
            P.toff, P.tcnt, pkeys, pvals, K, nk, MC, w.cellof.ptr, ncell, w.keys[kb].ptr, w.vals[kb].ptr);
    // the kept children, compacted in order
    if ((s = w.keep_i.ensure(nk + 1))) return s;
    k_nd_keep_int<<<nd_grid(nk, thr, lc.num_sms), thr, 0, lc.stream>>>(K, nk, w.keep_i.ptr);
    scan_int_to_ll(w.keep_i.ptr, w.kscan.ptr, nk, w.ss, lc);
    long long nn = 0;
    ND_CUDA(cudaMemcpyAsync(&nn, w.kscan.ptr + nk, sizeof(long long), cudaMemcpyDeviceToHost, lc.stream));
    ND_CUDA(cudaStreamSynchronize(lc.stream));
    w.launches += 5;
    if ((s = next.ensure(nn, MC, LC))) return s;
    if (nn > 0) {
        k_nd_compact<LC><<<nd_grid(nk, thr, lc.num_sms), thr, 0, lc.stream>>>(K, nk, MC, w.kscan.ptr,
                                                                            w.cellof.ptr, next.view());
        w.launches += 1;
    }
    *n_next = nn;
    return MCE_OK;
}

int nd_level_dispatch(int LD, NdWork& w, NdTerms P, const int* pkeys, const cd* pvals, long long n,
                      long long npairs, const double* x, int D, int MC, int MB, NdTermBufs& next, int kb,
                      long long* n_next, const LaunchCfg& lc)
{
    switch (LD) {
    case 2: return nd_level<2>(w, P, pkeys, pvals, n, npairs, x, D, MC, MB, next, kb, n_next, lc);
    case 3: return nd_level<3>(w, P, pkeys, pvals, n, npairs, x, D, MC, MB, next, kb, n_next, lc);
    case 4: return nd_level<4>(w, P, pkeys, pvals, n, npairs, x, D, MC, MB, next, kb, n_next, lc);
    case 5: return nd_level<5>(w, P, pkeys, pvals, n, npairs, x, D, MC, MB, next, kb, n_next, lc);
    case 6: return nd_level<6>(w, P, pkeys, pvals, n, npairs, x, D, MC, MB, next, kb, n_next, lc);
    case 7: return nd_level<7>(w, P, pkeys, pvals, n, npairs, x, D, MC, MB, next, kb, n_next, lc);
    case 8: return nd_level<8>(w, P, pkeys, pvals, n, npairs, x, D, MC, MB, next, kb, n_next, lc);
    default: return MCE_ERR_ARG;
    }
}

}  // namespace

int nd_pdf_chunk(const NdInput& in, const double* x_host, int npts, double* out_host, NdWork& w,
                 const LaunchCfg& lc);

int nd_pdf_eval(const NdInput& in, const double* x_host, int npts, double* out_host, NdWork* w, const LaunchCfg& lc,
                long long* launches)
{
    if (!w || npts < 1 || !x_host || !out_host || in.D < 1 || in.D > kMaxDim) return MCE_ERR_ARG;
    if (in.MB > kNdMaxRows || in.MB > in.MC) {
        report_error("N-D pdf: terms of more than 16 hyperplanes are not supported");
        return MCE_ERR_SHAPE;
    }
    const int D = in.D, MC = in.MC;
    if (D == 1) {
        report_error("N-D pdf: one-dimensional estimators use the marginal 1-D pdf");
        return MCE_ERR_ARG;
    }
    if (in.nkeep < 0 || in.nkeep >= D || (in.nkeep > 0 && !in.nu_bar)) return MCE_ERR_ARG;
    // the marginal's points: the kept states' coordinates in the last nkeep
    // places of a D-vector whose other places hold 0 (b - 0 is b, so the
    // first lowering subtracts the point at the kept states only, as
    // construct_lowered_marginal_parent_elements does)
    const int xd = in.nkeep ? in.nkeep : D;
    const double* xs = x_host;
    if (in.nkeep) {
        w->h_x.assign((size_t)npts * D, 0.0);
        for (int p = 0; p < npts; p++)
            for (int i = 0; i < in.nkeep; i++) w->h_x[(size_t)p * D + D - in.nkeep + i] = x_host[(size_t)p * in.nkeep + i];
        xs = w->h_x.data();
    }
    // points in chunks: every lowering multiplies the terms by their rows
    // (at most MC, MC - 1, ...), so the first level's (point, term) pairs are
    // bounded such that the last level stays under about 2^26 children
    const int lowerings = in.nkeep ? in.nkeep : D - 1;
    double growth = 1.0;
    for (int l = 0; l < lowerings; l++) growth *= std::max(1, MC - l);
    const double budget = (double)(1LL << 26) / growth;
    const long long per = std::max<long long>(1, (long long)(budget / (double)std::max<long long>(1, in.n)));
    (void)xd;
    w->launches = 0;
    for (long long p0 = 0; p0 < npts; p0 += per) {
        const int np = (int)std::min<long long>(per, npts - p0);
        const int s = nd_pdf_chunk(in, xs + p0 * D, np, out_host + 2 * p0, *w, lc);
        if (s) return s;
    }
    if (launches) *launches += w->launches;
    return MCE_OK;
}

int nd_pdf_chunk(const NdInput& in, const double* x_host, int npts, double* out_host, NdWork& wr,
                 const LaunchCfg& lc)
{
    NdWork* w = &wr;
    const int D = in.D, MC = in.MC;
    int s;
    if ((s = w->x.ensure((size_t)npts * D))) return s;
    if ((s = w->out.ensure((size_t)2 * npts))) return s;
    if ((s = w->err.ensure(1))) return s;
    ND_CUDA(cudaMemcpyAsync(w->x.ptr, x_host, sizeof(double) * npts * D, cudaMemcpyHostToDevice, lc.stream));
    ND_CUDA(cudaMemsetAsync(w->err.ptr, 0, sizeof(int), lc.stream));
    ND_CUDA(cudaMemsetAsync(w->out.ptr, 0, sizeof(double) * 2 * npts, lc.stream));
    // level 0: the estimator's own terms and tables, shared by every point
    // (for the marginal, their A columns and b reordered)
    NdTerms P{nullptr, const_cast<int*>(in.m), const_cast<double*>(in.A), const_cast<double*>(in.p),
              const_cast<double*>(in.b), const_cast<long long*>(in.toff), const_cast<int*>(in.tcnt)};
    const int* pkeys = in.keys;
    const cd* pvals = in.vals;
    long long n = in.n;
    const int stop = in.nkeep ? D - in.nkeep : 1;  // the dimension the lowerings end at
    if (in.nkeep && n > 0) {
        if ((s = w->rA.ensure((size_t)n * MC * D))) return s;
        if ((s = w->rb.ensure((size_t)n * D))) return s;
        NdReorient reo;
        for (int j = 0; j < kMaxDim; j++) reo.r[j] = j < D ? in.reorient[j] : 0;
        k_nd_reorient<<<nd_grid(n, 128, lc.num_sms), 128, 0, lc.stream>>>(in.m, in.A, in.b, n, MC, D, reo, w->rA.ptr,
                                                                          w->rb.ptr);
        w->launches += 1;
        P.A = w->rA.ptr;
        P.b = w->rb.ptr;
    }
    int cur = 0;
    bool empty = n == 0;
    for (int ld = D; ld > stop && !empty; ld--) {
        const bool first = ld == D;
        long long nn = 0;
        NdTermBufs& next = w->lev[cur];
        s = nd_level_dispatch(ld, *w, P, pkeys, pvals, n, first ? n * npts : n, first ? w->x.ptr : nullptr, D, MC,
                              in.MB, next, cur, &nn, lc);
        if (s) return s;
        int err = 0;
        ND_CUDA(cudaMemcpyAsync(&err, w->err.ptr, sizeof(int), cudaMemcpyDeviceToHost, lc.stream));
        ND_CUDA(cudaStreamSynchronize(lc.stream));
        if (err) {
            report_error("N-D pdf: a lowered child anti-coaligns two rows that do not enter the integration "
                         "(the reference exits, cauchy_term.hpp:673-687)");
            return MCE_ERR_DEVICE;
        }
        P = next.view();
        pkeys = w->keys[cur].ptr;
        pvals = w->vals[cur].ptr;
        n = nn;
        cur ^= 1;
        if (n == 0) empty = true;
    }
    if (!empty) {
        // pow(RECIPRICAL_TWO_PI, dim) (cpdf_ndim.hpp:893), for the marginal
        // pow(RECIPRICAL_TWO_PI, num_marg_state_idxs) (:1214)
        const double sc = pow(1.0 / (2.0 * M_PI), (double)(in.nkeep ? in.nkeep : D));
        if ((s = w->pstart.ensure(npts + 1))) return s;
        if ((s = w->pcoff.ensure(npts + 1))) return s;
        k_nd_point_starts<<<(npts + 1 + 127) / 128, 128, 0, lc.stream>>>(P.pt, n, npts, w->pstart.ptr);
        w->h_pstart.resize(npts + 1);
        ND_CUDA(cudaMemcpyAsync(w->h_pstart.data(), w->pstart.ptr, sizeof(long long) * (npts + 1),
                                cudaMemcpyDeviceToHost, lc.stream));
        ND_CUDA(cudaStreamSynchronize(lc.stream));
        w->h_pcoff.assign(npts + 1, 0);
        for (int p = 0; p < npts; p++) {
            const long long cnt = w->h_pstart[p + 1] - w->h_pstart[p];
            w->h_pcoff[p + 1] = w->h_pcoff[p] + (cnt + kNdFinalChunk - 1) / kNdFinalChunk;
        }
        const long long nb = w->h_pcoff[npts];
        ND_CUDA(cudaMemcpyAsync(w->pcoff.ptr, w->h_pcoff.data(), sizeof(long long) * (npts + 1),
                                cudaMemcpyHostToDevice, lc.stream));
        if (nb > 0) {
            if ((s = w->partial.ensure(nb + 1))) return s;
            if (in.nkeep) {
                if ((s = w->nu.ensure((size_t)stop))) return s;
                ND_CUDA(cudaMemcpyAsync(w->nu.ptr, in.nu_bar, sizeof(double) * stop, cudaMemcpyHostToDevice,
                                        lc.stream));
                k_nd_final_marg_partial<<<(unsigned)nb, kNdFinalThreads, 0, lc.stream>>>(
                    P, MC, stop, w->nu.ptr, pkeys, pvals, w->pstart.ptr, w->pcoff.ptr, npts, w->partial.ptr);
            } else
                k_nd_final_partial<<<(unsigned)nb, kNdFinalThreads, 0, lc.stream>>>(P, MC, pkeys, pvals, w->pstart.ptr,
                                                                                     w->pcoff.ptr, npts, w->partial.ptr);
        }
        k_nd_final_combine<<<(npts + 127) / 128, 128, 0, lc.stream>>>(w->partial.ptr, w->pcoff.ptr, npts, in.fz, sc,
                                                                     w->out.ptr);
        w->launches += nb > 0 ? 3 : 2;
    }
    ND_CUDA(cudaMemcpyAsync(out_host, w->out.ptr, sizeof(double) * 2 * npts, cudaMemcpyDeviceToHost, lc.stream));
    ND_CUDA(cudaStreamSynchronize(lc.stream));
    return MCE_OK;
}

}  // namespace mce
