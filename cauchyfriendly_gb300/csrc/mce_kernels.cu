// sm_103a kernels of the MCE step path (FP64).  See mce_kernels.cuh for the
// launch interface and mce_device.cuh for the shared numerics.
//
// Term order inside one estimator follows the reference's serial path
// (include/cauchy_estimator.hpp:741-780): parents in (shape, index) order,
// then children in (parent, hyperplane) order.  Estimators of a batch are laid
// out one after another, so every per-estimator rule (root = lowest index in a
// reduction group, member order, next parent order) is a rule on positions.
#include "mce_kernels.cuh"
#include "mce_c_api.h"

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#ifndef MCE_ONLY_DIM
#define MCE_ONLY_DIM -1  // every dimension and the shape-agnostic kernels in one unit
#endif
#define MCE_COMMON_UNIT (MCE_ONLY_DIM <= 0)

namespace mce {

#if MCE_COMMON_UNIT
thread_local long long g_launches = 0;

namespace {
constexpr int kTuneCands[4] = {64, 128, 256, 512};
constexpr int kTuneSamples = 2;
constexpr long long kTuneMinItems = 1LL << 15;  // smaller launches keep the default size
struct TuneEntry {
    int device, kernel, D, MC, bucket;
    int next = 0;  // next measurement: candidate index * kTuneSamples + sample
    float ms[4] = {1e30f, 1e30f, 1e30f, 1e30f};  // fastest sample per candidate
    int best = -1;  // index into kTuneCands once tuned
    int pending = -1;  // candidate whose events are in flight
    cudaEvent_t e0 = nullptr, e1 = nullptr;
};
std::mutex g_tune_mu;
std::vector<TuneEntry*> g_tune;
int g_tune_enabled = -1;  // -1: read MCE_AUTOTUNE on first use

TuneEntry* tune_find(int device, int kernel, int D, int MC, int bucket)
{
    for (TuneEntry* e : g_tune)
        if (e->device == device && e->kernel == kernel && e->D == D && e->MC == MC && e->bucket == bucket) return e;
    TuneEntry* e = new TuneEntry();
    e->device = device;
    e->kernel = kernel;
    e->D = D;
    e->MC = MC;
    e->bucket = bucket;
    if (cudaEventCreate(&e->e0) != cudaSuccess || cudaEventCreate(&e->e1) != cudaSuccess) {
        cudaGetLastError();
        e->best = 1;  // no events: keep the default block size
    }
    g_tune.push_back(e);
    return e;
}

// Folds a finished measurement in; picks the winner after the last one.
void tune_collect(TuneEntry* e)
{
    if (e->pending < 0) return;
    const cudaError_t q = cudaEventQuery(e->e1);
    if (q == cudaErrorNotReady) return;
    float ms = 0;
    if (q == cudaSuccess && cudaEventElapsedTime(&ms, e->e0, e->e1) == cudaSuccess) {
        e->ms[e->pending] = std::min(e->ms[e->pending], ms);
    } else {
        cudaGetLastError();
    }
    e->pending = -1;
    if (e->next >= 4 * kTuneSamples) {
        int b = 1;
        for (int c = 0; c < 4; c++)
            if (e->ms[c] < e->ms[b]) b = c;
        e->best = b;
    }
}
}  // namespace

TuneLaunch tune_begin(int kernel, int D, int MC, long long items, int def_block, int max_block, cudaStream_t st)
{
    TuneLaunch t;
    t.block = def_block;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    if (g_tune_enabled < 0) {
        const char* v = getenv("MCE_AUTOTUNE");
        g_tune_enabled = (v && v[0] == '0') ? 0 : 1;
    }
    if (!g_tune_enabled || items < kTuneMinItems) return t;
    int bucket = 0;
    while (bucket < 62 && (1LL << (bucket + 1)) <= items) bucket++;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) {
        cudaGetLastError();
        return t;
    }
    TuneEntry* e = tune_find(device, kernel, D, MC, bucket);
    tune_collect(e);
    if (e->best >= 0) {
        t.block = std::min(kTuneCands[e->best], max_block);
        return t;
    }
    // one measurement in flight per key; launches meanwhile take the default
    if (e->pending >= 0 || e->next >= 4 * kTuneSamples) return t;
    int c = e->next / kTuneSamples;
    while (c < 4 && kTuneCands[c] > max_block) {
        e->ms[c] = 1e30f;
        e->next = (c + 1) * kTuneSamples;
        c++;
    }
    if (c >= 4) {
        e->best = 1;
        return t;
    }
    if (cudaEventRecord(e->e0, st) != cudaSuccess) {
        cudaGetLastError();
        return t;
    }
    e->next++;
    e->pending = c;
    t.block = kTuneCands[c];
    t.entry = e;
    return t;
}

void tune_end(const TuneLaunch& t, cudaStream_t st)
{
    if (!t.entry) return;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    TuneEntry* e = static_cast<TuneEntry*>(t.entry);
    if (cudaEventRecord(e->e1, st) != cudaSuccess) {
        cudaGetLastError();
        e->pending = -1;  // the sample is lost; the candidate is measured again
        e->next--;
    }
}

int tune_table(int* out, float* best_ms, int n)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    int k = 0;
    for (TuneEntry* e : g_tune) {
        tune_collect(e);
        if (e->best < 0) continue;
        if (k < n) {
            out[5 * k] = e->kernel;
            out[5 * k + 1] = e->D;
            out[5 * k + 2] = e->MC;
            out[5 * k + 3] = e->bucket;
            out[5 * k + 4] = kTuneCands[e->best];
            if (best_ms) best_ms[k] = e->ms[e->best] < 1e29f ? e->ms[e->best] : 0.0f;
        }
        k++;
    }
    return k;
}

void tune_configure(int enabled)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    for (TuneEntry* e : g_tune) {
        if (e->pending >= 0) cudaEventSynchronize(e->e1);
        if (e->e0) cudaEventDestroy(e->e0);
        if (e->e1) cudaEventDestroy(e->e1);
        delete e;
    }
    g_tune.clear();
    cudaGetLastError();
    g_tune_enabled = enabled ? 1 : 0;
}
#endif

static constexpr unsigned kFull = 0xffffffffu;

__device__ inline void set_err(int* err, int bit)
{
    if (err) atomicOr(err, bit);
}

static inline int grid_for(long long items, int per_block, int num_sms, int blocks_per_sm = 16)
{
    long long g = (items + per_block - 1) / per_block;
    long long cap = (long long)num_sms * blocks_per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

// Grid of a tuned launch: the same resident threads per SM as blocks_per_sm
// blocks of 128 threads, whatever block size the tuner chose.
static inline int tuned_grid(long long items, int block, int num_sms, int blocks_per_sm_at_128)
{
    int bps = blocks_per_sm_at_128 * 128 / block;
    if (bps > 64) bps = 64;
    if (bps < 1) bps = 1;
    return grid_for(items, block, num_sms, bps);
}

// The largest block a kernel may launch with (registers bound it).
static inline int max_block_of(const void* kern)
{
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, kern) != cudaSuccess) {
        cudaGetLastError();
        return 128;
    }
    return a.maxThreadsPerBlock;
}

// ---------------------------------------------------------------------------
// Device-wide exclusive scan (int counts -> long long offsets + total).
static constexpr int kScanThreads = 256;
static constexpr int kScanItems = 8;
static constexpr int kScanTile = kScanThreads * kScanItems;

template <typename T>
__device__ inline long long block_exclusive_scan(long long v, long long* total)
{
    __shared__ long long warp_sums[kScanThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        long long y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    if (w == 0) {
        long long s = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            long long y = __shfl_up_sync(kFull, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kScanThreads / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    long long pre = (w > 0 ? warp_sums[w - 1] : 0) + x - v;
    *total = warp_sums[kScanThreads / 32 - 1];
    __syncthreads();
    return pre;
}

template <typename TIn>
__global__ void k_scan_tiles(const TIn* in, long long* out, long long n, long long* tile_sums)
{
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    long long v[kScanItems];
    long long s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        long long idx = base + k;
        v[k] = idx < n ? (long long)in[idx] : 0;
        s += v[k];
    }
    long long tot;
    long long pre = block_exclusive_scan<long long>(s, &tot);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        long long idx = base + k;
        if (idx < n) out[idx] = pre;
        pre += v[k];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

#if MCE_COMMON_UNIT
__global__ void k_scan_add(long long* out, long long n, const long long* tile_off)
{
    const long long base = (long long)blockIdx.x * kScanTile;
    const long long add = tile_off[blockIdx.x];
    for (int k = threadIdx.x; k < kScanTile; k += blockDim.x) {
        long long idx = base + k;
        if (idx < n) out[idx] += add;
    }
}

__global__ void k_write_total(long long* out, long long n, const long long* tile_off, long long ntiles)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) out[n] = tile_off[ntiles];
}

static void scan_ll_inplace(long long* data, long long n, long long* scratch, long long scratch_cap,
                            const LaunchCfg& c);

// Exclusive scan of long long values in place, total written at data[n].
__global__ void k_copy_ll(const long long* a, long long* b, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = a[i];
}

static void scan_ll_inplace(long long* data, long long n, long long* scratch, long long scratch_cap,
                            const LaunchCfg& c)
{
    // data has n+1 slots
    const long long ntiles = (n + kScanTile - 1) / kScanTile;
    if (ntiles <= 1) {
        long long* ts = scratch;
        ++g_launches;
        k_scan_tiles<long long><<<1, kScanThreads, 0, c.stream>>>(data, data, n, ts);
        // total: the single tile sum
        ++g_launches;
        k_copy_ll<<<1, 32, 0, c.stream>>>(ts, data + n, 1);
        return;
    }
    long long* ts = scratch;  // ntiles + 1
    ++g_launches;
    k_scan_tiles<long long><<<(unsigned)ntiles, kScanThreads, 0, c.stream>>>(data, data, n, ts);
    scan_ll_inplace(ts, ntiles, scratch + ntiles + 1, scratch_cap - (ntiles + 1), c);
    ++g_launches;
    k_scan_add<<<(unsigned)ntiles, kScanThreads, 0, c.stream>>>(data, n, ts);
    ++g_launches;
    k_write_total<<<1, 32, 0, c.stream>>>(data, n, ts, ntiles);
}

void scan_int_to_ll(const int* in, long long* out, long long n, ScanScratch& s, const LaunchCfg& c)
{
    const long long ntiles = (n + kScanTile - 1) / kScanTile;
    if (n == 0) {
        cudaMemsetAsync(out, 0, sizeof(long long), c.stream);
        return;
    }
    long long* ts = s.block_sums;
    ++g_launches;
    k_scan_tiles<int><<<(unsigned)ntiles, kScanThreads, 0, c.stream>>>(in, out, n, ts);
    if (ntiles == 1) {
        ++g_launches;
        k_copy_ll<<<1, 32, 0, c.stream>>>(ts, out + n, 1);
        return;
    }
    scan_ll_inplace(ts, ntiles, s.block_sums + ntiles + 1, s.cap - (ntiles + 1), c);
    ++g_launches;
    k_scan_add<<<(unsigned)ntiles, kScanThreads, 0, c.stream>>>(out, n, ts);
    ++g_launches;
    k_write_total<<<1, 32, 0, c.stream>>>(out, n, ts, ntiles);
}

#endif  // MCE_COMMON_UNIT

// ---------------------------------------------------------------------------
// First measurement update: one thread per estimator (d+1 terms at most).

template <int D>
__global__ void k_first_count(const double* A0, const EstStep<D>* st, int E, int* cnt)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const EstStep<D>& S = st[e];
    if (!S.active) {
        cnt[e] = 0;
        return;
    }
    int c = 1;
    for (int l = 0; l < D; l++) {
        double h = 0.0;
        for (int j = 0; j < D; j++) h += S.H[j] * A0[(long long)e * D * D + l * D + j];
        if (!(fabs(h) < kMuEps)) c++;
    }
    cnt[e] = c;
}

// msmt_update with first_update=true (cauchy_term.hpp:84-310) followed by
// compute_moments (cauchy_estimator.hpp:524-602): the d+1 terms are written
// to the parent list in the reference's order and the moments are summed in
// that same order.
template <int D>
__global__ void k_first_build(const double* A0, const double* p0, const double* b0, const EstStep<D>* st,
                              const double* roots, int E, const long long* pstart, ParentList P, int MC,
                              double* cval, double* dval, unsigned* hof_out, cd* est_raw)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const EstStep<D>& S = st[e];
    if (!S.active) return;
    const double* A = A0 + (long long)e * D * D;
    const double* p = p0 + (long long)e * D;
    const double* b = b0 + (long long)e * D;
    const double* root = roots + (long long)e * D;
    double mu[(D + 1) * D];
    double rho[D + 1];
    bool Fi[D + 1];
    for (int l = 0; l < D; l++) {
        double h = 0.0;
        for (int j = 0; j < D; j++) h += S.H[j] * A[l * D + j];
        const double ah = fabs(h);
        if (ah < kMuEps) {
            for (int j = 0; j < D; j++) mu[l * D + j] = A[l * D + j];
            rho[l] = p[l];
            Fi[l] = false;
        } else {
            const double r = 1.0 / h;
            for (int j = 0; j < D; j++) mu[l * D + j] = A[l * D + j] * r;
            rho[l] = p[l] * ah;
            Fi[l] = true;
        }
    }
    for (int j = 0; j < D; j++) mu[D * D + j] = 0.0;
    rho[D] = S.gamma;
    Fi[D] = true;
    double hb = 0.0;
    for (int j = 0; j < D; j++) hb += S.H[j] * b[j];
    const double zeta = S.msmt - hb;

    cd fz = mkcd(0, 0);
    cd mean[D];
    cd cov[D * D];
    for (int j = 0; j < D; j++) mean[j] = mkcd(0, 0);
    for (int j = 0; j < D * D; j++) cov[j] = mkcd(0, 0);

    long long slot = pstart[e];
    // order: the parent (t == D) first, then the children t = 0..D-1
    for (int n = 0; n <= D; n++) {
        const int t = (n == 0) ? D : n - 1;
        if (!Fi[t]) continue;
        double* At = P.A + slot * MC * D;
        double* pt = P.p + slot * MC;
        double* bt = P.b + slot * D;
        unsigned hof = 0;
        double ty[D];
        for (int j = 0; j < D; j++) ty[j] = 0;
        double ygi = 0;
        int l = 0;
        for (int ll = 0; ll <= D; ll++) {
            if (ll == t) continue;
            double row[D];
            if (Fi[ll])
                for (int j = 0; j < D; j++) row[j] = mu[ll * D + j] - mu[t * D + j];
            else {
                for (int j = 0; j < D; j++) row[j] = mu[ll * D + j];
                hof |= 1u << l;
            }
            for (int j = 0; j < D; j++) At[l * D + j] = row[j];
            pt[l] = rho[ll];
            double s = 0.0;
            for (int j = 0; j < D; j++) s += row[j] * root[j];
            const double sg = s > 0 ? 1.0 : -1.0;
            const double sc = rho[ll] * sg;
            for (int j = 0; j < D; j++) ty[j] += sc * row[j];
            if (!(hof & (1u << l))) ygi += rho[ll] * sg;
            l++;
        }
        for (int j = 0; j < D; j++) bt[j] = b[j] + zeta * mu[t * D + j];
        P.est[slot] = e;
        P.m[slot] = D;
        P.m_old[slot] = D;
        cval[slot] = zeta;
        dval[slot] = rho[t];
        hof_out[slot] = hof;
        const cd one = mkcd(1, 0);
        cd g = csub(cdiv(one, mkcd(ygi + rho[t], zeta)), cdiv(one, mkcd(ygi - rho[t], zeta)));
        g = cscale(g, kTwoPiInv);
        fz = cadd(fz, g);
        for (int j = 0; j < D; j++) {
            const cd y = mkcd(-ty[j], bt[j]);
            const cd gy = cmul(g, y);
            mean[j] = cadd(mean[j], gy);
            for (int k = 0; k < D; k++) cov[j * D + k] = csub(cov[j * D + k], cmul(gy, mkcd(-ty[k], bt[k])));
        }
        slot++;
    }
    // compute_moments finalisation (cauchy_estimator.hpp:567-578)
    const int NM = 1 + D + D * D;
    cd* out = est_raw + (long long)e * NM;
    const cd ifz = mkcd(0, fz.re);
    cd mfin[D];
    for (int j = 0; j < D; j++) mfin[j] = cdiv(mean[j], ifz);
    out[0] = fz;
    for (int j = 0; j < D; j++) out[1 + j] = mfin[j];
    for (int j = 0; j < D; j++)
        for (int k = 0; k < D; k++)
            out[1 + D + j * D + k] = csub(cdiv(cov[j * D + k], fz), cmul(mfin[j], mfin[k]));
}

// make_gtable_first (flattening.hpp:14-67): 2^(d-1) cells with keys 0..2^(d-1)-1.
template <int D>
__global__ void k_first_tables(ParentList P, long long nP, const double* cval, const double* dval,
                               const unsigned* hof, const double* gscale, Tables T, int MC)
{
    const int cells = 1 << (D - 1);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nP * cells;
         i += (long long)gridDim.x * blockDim.x) {
        const long long t = i / cells;
        const int j = (int)(i % cells);
        const double* p = P.p + t * MC;
        const unsigned h = hof[t];
        double ygi = 0;
        for (int k = 0; k < D; k++)
            if (!(h & (1u << k))) ygi += p[k] * (((j >> k) & 1) == 0 ? 1.0 : -1.0);
        const cd one = mkcd(1, 0);
        cd v = csub(cdiv(one, mkcd(ygi + dval[t], cval[t])), cdiv(one, mkcd(ygi - dval[t], cval[t])));
        v = cscale(v, gscale[P.est[t]]);
        const long long off = t * cells;
        T.keys[off + j] = j;
        T.vals[off + j] = v;
        if (j == 0) {
            P.tab_off[t] = off;
            P.tab_cnt[t] = cells;
        }
    }
}

// ---------------------------------------------------------------------------
// Time propagation + TP coalignment (cauchy_term.hpp:435-531) and the count
// of hyperplanes the MU will integrate (cauchy_term.hpp:106-130).
template <int D>
__global__ void k_tp(ParentList P, long long nP, const EstStep<D>* st, int with_tp, int MC, int* Bcap, int* nvert,
                     int* err)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nP; i += (long long)gridDim.x * blockDim.x) {
        const int e = P.est[i];
        const EstStep<D>& S = st[e];
        int m = P.m[i];
        P.m_old[i] = m;
        double* A = P.A + i * MC * D;
        double* p = P.p + i * MC;
        double* b = P.b + i * D;
        if (with_tp) {
            // A <- A Phi^T, then normalize_hps(false): per row in registers,
            // one read and one write of the row
            for (int r = 0; r < m; r++) {
                double w[D], v[D];
                for (int k = 0; k < D; k++) w[k] = A[r * D + k];
                for (int j = 0; j < D; j++) {
                    double s = 0.0;
                    for (int k = 0; k < D; k++) s += w[k] * S.Phi[j * D + k];
                    v[j] = s;
                }
                double n1 = 0;
                for (int j = 0; j < D; j++) n1 += fabs(v[j]);
                p[r] *= n1;
                for (int j = 0; j < D; j++) A[r * D + j] = v[j] / n1;
            }
            double wb[D];
            for (int j = 0; j < D; j++) wb[j] = b[j];
            for (int r = 0; r < D; r++) {
                double s = 0.0;
                for (int j = 0; j < D; j++) s += S.Phi[r * D + j] * wb[j];
                b[r] = s;
            }
            if (S.has_control)
                for (int r = 0; r < D; r++) b[r] += 1.0 * S.Bu[r];
            bool F[kMaxGamma];
            for (int j = 0; j < S.gcnt; j++) F[j] = true;
            for (int j = 0; j < S.gcnt; j++)
                for (int k = 0; k < m; k++)
                    if (F[j] && coalign_gate<D>(S.Gt + j * D, A + k * D) != 0) {
                        F[j] = false;
                        p[k] += S.bt[j];
                    }
            for (int j = 0; j < S.gcnt; j++)
                if (F[j]) {
                    if (m >= MC) {
                        set_err(err, kErrShapeTooLarge);
                        break;
                    }
                    for (int l = 0; l < D; l++) A[m * D + l] = S.Gt[j * D + l];
                    p[m] = S.bt[j];
                    m++;
                }
            P.m[i] = m;
        }
        int cnt = 0;
        for (int l = 0; l < m; l++) {
            double h = 0.0;
            for (int j = 0; j < D; j++) h += S.H[j] * A[l * D + j];
            if (!(fabs(h) < kMuEps)) cnt++;
        }
        P.nkids_all[i] = cnt;
        P.nkids[i] = S.skip ? 0 : cnt;
        int cap;
        if (S.skip) cap = 0;
        else if (with_tp && m != P.m_old[i]) cap = m < D ? (1 << (m - 1)) : half_cells_cap(m, D);
        else cap = P.tab_cnt[i];
        Bcap[i] = cap;
        // d-subsets the TP enumeration solves (none for m <= d: the reference
        // has no subsets for m == d)
        nvert[i] = (!S.skip && with_tp && m != P.m_old[i] && m > D) ? (int)binom_ll(m, D) : 0;
    }
}

// ---------------------------------------------------------------------------
// B tables.  A parent whose arrangement grew under TP gets its cells from the
// vertex enumeration of make_time_prop_btable (cell_enumeration.hpp:676-855):
// every non-degenerate d-subset of hyperplanes (cond <= 1e12) is solved for a
// vertex of the perturbed arrangement A x = b_pert, the 2^d cells around the
// vertex are formed, those whose parent part is a parent cell are kept, and a
// sign vector is output (half storage) when its negation was found too.  The
// sets are held as shared-memory bitmaps, so the output comes out sorted and
// de-duplicated without hashing.  Other parents copy their table keys.
// The FP64 half of the enumeration, a thread per (parent, d-subset) of every
// enumerating parent (voff: exclusive subset offsets): cond(A_c) > 1e12 skips
// the subset (cell_enumeration.hpp:751-757); otherwise the vertex
// A_c v = b_pert_c and the signs of the other rows at it give the subset's
// sign vector, written to vsv (-1: skipped).  Most parents have few subsets
// (a 3-state term of 4-6 hyperplanes has 4-20), so one parent per warp would
// leave most lanes idle; here every lane solves a subset.
template <int D>
__global__ void k_build_B_vertices(ParentList P, long long nP, const long long* voff, long long nv,
                                   const double* bpert_all, int MC, const int* combo_off,
                                   const unsigned char* combos, int* vsv)
{
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < nv; x += (long long)gridDim.x * blockDim.x) {
        long long lo = 0, hi = nP;
        while (hi - lo > 1) {
            const long long mid = (lo + hi) >> 1;
            if (voff[mid] <= x) lo = mid;
            else hi = mid;
        }
        const long long i = lo;
        const int m = P.m[i];
        const double* As = P.A + i * MC * D;
        const double* bp = bpert_all + (long long)P.est[i] * MC;
        const unsigned char* c = combos + combo_off[m] + (x - voff[i]) * D;
        double Ac[D * D], bc[D], v[D];
        int Pv[D];
        for (int j = 0; j < D; j++) {
            for (int l = 0; l < D; l++) Ac[j * D + l] = As[c[j] * D + l];
            bc[j] = bp[c[j]];
        }
        int out = -1;
        // cond(A) > 1e12 skips the vertex.  A single-precision upper bound from
        // the exact LU factors settles the well-conditioned subsets; the
        // reference's explicit-inverse value is computed only when the bound is
        // not at least ten times below 1e12.
        double nrm = -1;
        for (int cc = 0; cc < D; cc++) {
            double sm = 0;
            for (int r = 0; r < D; r++) sm += fabs(Ac[r * D + cc]);
            if (dlt(nrm, sm)) nrm = sm;
        }
        if (plu<D>(Ac, Pv)) {
            const double bound = nrm * (double)inv_norm1_bound<D>(Ac);
            if ((bound <= 0.1 * kCondEps) || !cond1_exceeds<D>(Ac, Pv, nrm, kCondEps)) {
                solve_lu<D>(Ac, Pv, bc, v);
                unsigned inmask = 0;
                for (int j = 0; j < D; j++) inmask |= 1u << c[j];
                int niv = 0;
                // the m - D rows outside the subset, every lane on one of its
                // own rows per iteration (no idle lanes in the FP64 work)
                int a = 0;
                for (int q = 0; q < m - D; q++) {
                    while ((inmask >> a) & 1u) a++;
                    double s = 0.0;
                    for (int j = 0; j < D; j++) s += As[a * D + j] * v[j];
                    if (neg(s - bp[a])) niv |= 1 << a;
                    a++;
                }
                out = niv;
            }
        }
        vsv[x] = out;
    }
}

template <int D>
__global__ void k_build_B(ParentList P, long long nP, const EstStep<D>* st, int with_tp, Tables Told, int* Bkeys,
                          const double* bpert_all, int MC, const int* combo_off, const unsigned char* combos,
                          const long long* voff, const int* vsv, int* err, unsigned* gbits)
{
    extern __shared__ unsigned long long smem_u64[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwb = blockDim.x >> 5;
    const int words = (1 << MC) > 32 ? (1 << MC) / 32 : 1;
    unsigned* PB = gbits ? gbits + (size_t)((long long)blockIdx.x * nwb + wib) * 2 * words
                         : reinterpret_cast<unsigned*>(smem_u64) + (size_t)wib * 2 * words;  // parent cells
    unsigned* IS = PB + words;                                                     // cells found
    for (long long i = (long long)blockIdx.x * nwb + wib; i < nP; i += (long long)gridDim.x * nwb) {
        const int e = P.est[i];
        const EstStep<D>& S = st[e];
        if (S.skip) continue;
        const int m = P.m[i], phc = P.m_old[i];
        int* out = Bkeys + P.B_off[i];
        const int cap = (int)(P.B_off[i + 1] - P.B_off[i]);
        const int* pk = Told.keys + P.tab_off[i];
        const int pcnt = P.tab_cnt[i];
        const bool dce = with_tp && m != phc;
        if (!dce) {
            for (int k = lane; k < pcnt; k += 32)
                if (k < cap) out[k] = pk[k];
            if (lane == 0) {
                P.B_cnt[i] = pcnt <= cap ? pcnt : cap;
                if (pcnt > cap) set_err(err, kErrTableOverflow);
            }
            continue;
        }
        if (m < D) {
            const int n = 1 << (m - 1);
            for (int k = lane; k < n && k < cap; k += 32) out[k] = k;
            if (lane == 0) P.B_cnt[i] = n;
            continue;
        }
        const int mw = (1 << m) > 32 ? (1 << m) / 32 : 1;
        const int pw = (1 << phc) > 32 ? (1 << phc) / 32 : 1;
        for (int k = lane; k < mw; k += 32) IS[k] = 0;
        for (int k = lane; k < pw; k += 32) PB[k] = 0;
        __syncwarp();
        for (int k = lane; k < pcnt; k += 32) {
            const int key = pk[k];
            if (key >= 0 && key < (1 << phc)) atomicOr(&PB[key >> 5], 1u << (key & 31));
        }
        __syncwarp();
        const int gmask = (1 << phc) - 1, ptop = 1 << (phc - 1);
        const int ncomb = m > D ? (int)binom_ll(m, D) : 0;
        const unsigned char* cmb = combos + combo_off[m];
        const int* vv = vsv + voff[i];
        for (int ci = lane; ci < ncomb; ci += 32) {
            // the subset's sign vector from k_build_B_vertices, then the 2^d
            // cells around its vertex whose parent part is a parent cell
            const int niv = vv[ci];
            if (niv < 0) continue;
            const unsigned char* c = cmb + (long long)ci * D;
            for (int j = 0; j < (1 << D); j++) {
                int sv = niv;
                for (int k = 0; k < D; k++)
                    if ((j >> k) & 1) sv |= 1 << c[k];
                int psv = sv & gmask;
                if (psv & ptop) psv ^= gmask;
                if ((PB[psv >> 5] >> (psv & 31)) & 1u) atomicOr(&IS[sv >> 5], 1u << (sv & 31));
            }
        }
        __syncwarp();
        // pairs (b, ~b): output b with its top bit clear, ascending
        int count = 0;
        const int rev = (1 << m) - 1;
        if (m <= 5) {
            if (lane == 0) {
                for (int sv = 0; sv < (1 << (m - 1)); sv++) {
                    const int pr = sv ^ rev;
                    if (((IS[sv >> 5] >> (sv & 31)) & 1u) && ((IS[pr >> 5] >> (pr & 31)) & 1u)) {
                        if (count < cap) out[count] = sv;
                        count++;
                    }
                }
            }
            count = __shfl_sync(kFull, count, 0);
        } else {
            const int half = mw / 2;
            for (int w0 = 0; w0 < half; w0 += 32) {
                const int w = w0 + lane;
                unsigned bits = 0;
                if (w < half) bits = IS[w] & __brev(IS[mw - 1 - w]);
                const int c = __popc(bits);
                int pre = c;
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(kFull, pre, o);
                    if (lane >= o) pre += y;
                }
                const int tot = __shfl_sync(kFull, pre, 31);
                int pos = count + pre - c;
                while (bits) {
                    const int bt = __ffs(bits) - 1;
                    bits &= bits - 1;
                    if (pos < cap) out[pos] = w * 32 + bt;
                    pos++;
                }
                count += tot;
            }
        }
        if (lane == 0) {
            P.B_cnt[i] = count <= cap ? count : cap;
            if (count > cap) set_err(err, kErrDceOverflow);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// MU coalignment of one staged child (cauchy_term.hpp:533-745), in place on
// the lane's shared-memory rows.  Returns the new row count.
template <int D>
// The coalignment of mu_coalign after its normalize_hps(true) (the caller
// normalises the rows: the parent's record takes the same normalisation, so
// parents and children of one warp share those instructions).
__device__ inline int mu_coalign_smem(double* A, double* p, double* q, int m, unsigned& hof, signed char* cmap,
                                      signed char* csmap, int* err)
{
    unsigned F = (m >= 32) ? kFull : ((1u << m) - 1);
    unsigned hf = hof;
    for (int j = 0; j < m; j++) {
        cmap[j] = -1;  // 255 as uint8: no coalignment
        csmap[j] = 1;
    }
    int uc = 0;
    for (int j = 0; j < m - 1; j++) {
        if (!((F >> j) & 1u)) continue;
        cmap[j] = (signed char)uc;
        for (int k = j + 1; k < m; k++) {
            if (!((F >> k) & 1u)) continue;
            const int g = coalign_gate<D>(A + j * D, A + k * D);
            if (g == 0) continue;
            const bool hj = (hf >> j) & 1u, hk = (hf >> k) & 1u;
            if (g == 1) {
                if (hof) {
                    if (!hj && !hk) q[j] += q[k];
                    else if (hj && !hk) {
                        q[j] = q[k];
                        hf &= ~(1u << j);
                    } else if (!hj && hk) hf &= ~(1u << k);
                    else {
                        hf &= ~(1u << k);
                        q[j] += q[k];
                    }
                } else
                    q[j] += q[k];
                csmap[k] = 1;
            } else {
                if (hof) {
                    if (!hj && !hk) q[j] -= q[k];
                    else if (hj && !hk) {
                        q[j] = -q[k];
                        hf &= ~(1u << j);
                    } else if (!hj && hk) hf &= ~(1u << k);
                    else set_err(err, kErrAntiCoalignedHorthog);
                } else
                    q[j] -= q[k];
                csmap[k] = -1;
            }
            F &= ~(1u << k);
            p[j] += p[k];
            cmap[k] = (signed char)uc;
        }
        uc++;
    }
    if ((F >> (m - 1)) & 1u) cmap[m - 1] = (signed char)uc;
    const int ns = __popc(F);
    if (ns != m) {
        int u = 1;
        for (int j = 1; j < m; j++)
            if ((F >> j) & 1u) {
                if (u < j) {
                    for (int l = 0; l < D; l++) A[u * D + l] = A[j * D + l];
                    p[u] = p[j];
                    q[u] = q[j];
                }
                u++;
            }
        if (hof) {
            unsigned nh = 0;
            int c = 0;
            for (int j = 0; j < m; j++)
                if ((F >> j) & 1u) nh |= ((hf >> j) & 1u) << c++;
            hof = nh;
        }
    }
    return ns;
}

// Measurement update (cauchy_term.hpp:84-310) in two passes.
//
// k_mu_rows, a thread per parent: the MU rows mu_l = A_l / (H . A_l) with
// rho_l = p_l |H . A_l| (an H-orthogonal row keeps A_l and p_l and gets no
// child), the measurement row (0, gamma), zeta = z - H . b, the masks of
// integrable rows and of negative H . A_l, and the parent's B -> B_mu flip
// (cauchy_term.hpp:245-250).  Per parent the row record holds (MC + 1) x D mu
// values, MC + 1 rho values and zeta; the int record holds the integrable
// mask, enc_lhp and the flip mask.
template <int D>
__global__ void k_mu_rows(ParentList P, long long nP, const EstStep<D>* st, int* Bkeys, double* frow, int* fint,
                          int MC)
{
    const int FR = (MC + 1) * (D + 1) + 1;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nP; i += (long long)gridDim.x * blockDim.x) {
        const EstStep<D>& S = st[P.est[i]];
        const int m = P.m[i], phc = P.m_old[i];
        const double* A = P.A + i * MC * D;
        const double* p = P.p + i * MC;
        const double* b = P.b + i * D;
        double* mu = frow + i * FR;
        double* rho = mu + (MC + 1) * D;
        unsigned integ = 0;
        int esg = 0;
        for (int l = 0; l < m; l++) {
            double h = 0.0;
            for (int j = 0; j < D; j++) h += S.H[j] * A[l * D + j];
            const double ah = fabs(h);
            if (abs_lt(h, kMuEps)) {
                for (int j = 0; j < D; j++) mu[l * D + j] = A[l * D + j];
                rho[l] = p[l];
            } else {
                const double r = 1.0 / h;
                for (int j = 0; j < D; j++) mu[l * D + j] = A[l * D + j] * r;
                rho[l] = p[l] * ah;
                integ |= 1u << l;
                if (!(h > 0)) esg |= 1 << l;
            }
        }
        for (int j = 0; j < D; j++) mu[m * D + j] = 0.0;
        rho[m] = S.gamma;
        double hb = 0.0;
        for (int j = 0; j < D; j++) hb += S.H[j] * b[j];
        mu[(MC + 1) * (D + 1)] = S.msmt - hb;
        int lhp = esg;
        if (phc < m) lhp &= (1 << phc) - 1;
        const int esg_c = (esg & (1 << (m - 1))) ? (esg ^ ((1 << m) - 1)) : esg;
        fint[i * 4 + 0] = (int)integ;
        fint[i * 4 + 1] = lhp;
        fint[i * 4 + 2] = esg_c;
        P.bflip[i] = esg_c;
        if (!S.skip) {
            int* B = Bkeys + P.B_off[i];
            const int n = P.B_cnt[i];
            for (int k = 0; k < n; k++) B[k] ^= esg_c;
        }
    }
}

// k_mu_terms, a thread per post-MU term, in the moment-contribution order
// (each parent, then its children by hyperplane): the child's rows
// mu_l - mu_t (the parent's rows for the parent), the g/yei evaluation
// (cauchy_term.hpp:312-401), the moment contribution (cache_moments,
// cauchy_estimator.hpp:307), and the record with the parent's
// re-normalisation or the child's MU coalignment (cauchy_term.hpp:533-745).
// Every lane runs the same per-term code, so the FP64 work fills the warps
// whatever the families' sizes.  Each thread stages its term's rows in shared
// memory for the coalignment.
template <int D>
__global__ void __launch_bounds__(128) k_mu_terms(ParentList P, long long nP, const EstStep<D>* st,
                                                  const long long* pstart, const double* roots, Tables Told,
                                                  TermRecs R, long long nR, const long long* kall_scan,
                                                  long long nterms, const double* frow, const int* fint,
                                                  cd* contrib, int MC, int* err)
{
    extern __shared__ double smem_d[];
    constexpr int NM = 1 + D + D * D;
    const int RS = MC * D + 2 * MC;
    const int FR = (MC + 1) * (D + 1) + 1;
    double* At = smem_d + (size_t)threadIdx.x * RS;
    double* pt = At + MC * D;
    double* qt = pt + MC;
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < nterms;
         x += (long long)gridDim.x * blockDim.x) {
        // threads [0, nP) take the parents, the rest the children in order,
        // so a warp runs either the parent path or the coalignment of children
        long long i;
        int ford;  // 0: the parent, c + 1: child c
        if (x < nP) {
            i = x;
            ford = 0;
        } else {
            // the family of child cidx: the last parent i with kall_scan[i] <= cidx
            const long long cidx = x - nP;
            long long lo = 0, hi = nP;
            while (hi - lo > 1) {
                const long long mid = (lo + hi) >> 1;
                if (kall_scan[mid] <= cidx) lo = mid;
                else hi = mid;
            }
            i = lo;
            ford = (int)(cidx - kall_scan[i]) + 1;
        }
        // the term's position in the reference's order (parent, then its children)
        const long long xo = i + kall_scan[i] + ford;
        const int e = P.est[i];
        const EstStep<D>& S = st[e];
        const int m = P.m[i], phc = P.m_old[i];
        const double* mu = frow + i * FR;
        const double* rho = mu + (MC + 1) * D;
        const double zeta = mu[(MC + 1) * (D + 1)];
        const unsigned integ_mask = (unsigned)fint[i * 4 + 0];
        const int lhp = fint[i * 4 + 1];
        const double* b = P.b + i * D;
        const double* root = roots + (long long)e * D;
        int t = m;
        if (ford > 0) {
            unsigned msk = integ_mask;
            for (int c = 1; c < ford; c++) msk &= msk - 1;
            t = __ffs(msk) - 1;
        }
        double bt[D], ty[D];
        for (int j = 0; j < D; j++) {
            bt[j] = b[j] + zeta * mu[t * D + j];
            ty[j] = 0;
        }
        unsigned hof = 0;
        int sneg = 0;
        double ygi = 0;
        // the m rows other than t (the parent: rows 0..m-1; child t: the
        // other MU rows and the measurement row m), one per iteration on
        // every lane
        for (int l = 0; l < m; l++) {
            const int ll = l < t ? l : l + 1;
            const bool fi = (ll < m) ? ((integ_mask >> ll) & 1u) : true;
            double row[D];
            if (fi)
                for (int j = 0; j < D; j++) row[j] = mu[ll * D + j] - mu[t * D + j];
            else {
                for (int j = 0; j < D; j++) row[j] = mu[ll * D + j];
                hof |= 1u << l;
            }
            const double pl = rho[ll];
            double s = 0.0;
            for (int j = 0; j < D; j++) s += row[j] * root[j];
            const bool sgp = pos(s);
            if (!sgp) sneg |= 1 << l;
            const double sc = sgp ? pl : -pl;  // p_l * sign, exact
            for (int j = 0; j < D; j++) ty[j] += sc * row[j];
            if (!(hof & (1u << l))) ygi += sc;
            for (int j = 0; j < D; j++) At[l * D + j] = row[j];
            pt[l] = pl;
        }
        // lambda keys into the parent table (cauchy_term.hpp:357-381)
        int lp = 0, lm = 0, k = 0;
        for (int l2 = 0; l2 < m; l2++) {
            if (k < phc) {
                if (k == t) {
                    lm |= 1 << k;
                    k++;
                    if (k == phc) continue;
                }
                if ((sneg >> l2) & 1) {
                    lp |= 1 << k;
                    lm |= 1 << k;
                }
                k++;
            }
        }
        const int* pk = Told.keys + P.tab_off[i];
        const cd* pv = Told.vals + P.tab_off[i];
        const int pcnt = P.tab_cnt[i];
        const cd gp = lookup_num(pk, pv, pcnt, lp ^ lhp, phc);
        const cd gm = lookup_num(pk, pv, pcnt, lm ^ lhp, phc);
        const double dv = rho[t];
        cd g = csub(cdiv(gp, mkcd(ygi + dv, zeta)), cdiv(gm, mkcd(ygi - dv, zeta)));
        g = cscale(g, kTwoPiInv);
        cd* cs = contrib + xo * NM;
        cs[0] = g;
        for (int j = 0; j < D; j++) {
            const cd y = mkcd(-ty[j], bt[j]);
            const cd gy = cmul(g, y);
            cs[1 + j] = gy;
            for (int kk = 0; kk < D; kk++) cs[1 + D + j * D + kk] = cmul(gy, mkcd(-ty[kk], bt[kk]));
        }
        const long long pslot = i + P.kscan[pstart[e]];            // parent's record
        const long long cslot0 = pstart[e + 1] + P.kscan[i];       // first child's record
        if (S.skip) {
            // a final MU keeps no records; mark the parent's slot empty
            if (t == m && pslot < nR) R.est[pslot] = -1;
            continue;
        }
        const long long slot = (t == m) ? pslot : cslot0 + (ford - 1);
        if (slot >= nR) {
            set_err(err, kErrRecordOverflow);
            continue;
        }
        int mfin = m;
        int flags = (t == m) ? 0 : kFlagNewChild;
        // normalize_hps(true) (cauchy_term.hpp:458-472): q keeps the
        // un-normalised scales; the parent stops there, a child is coaligned
        for (int r = 0; r < m; r++) {
            qt[r] = pt[r];
            double n1 = 0;
            for (int j = 0; j < D; j++) n1 += fabs(At[r * D + j]);
            pt[r] *= n1;
            for (int j = 0; j < D; j++) At[r * D + j] /= n1;
        }
        if (t != m) {
            mfin = mu_coalign_smem<D>(At, pt, qt, m, hof, R.cmap + slot * MC, R.csmap + slot * MC, err);
            if (mfin != m) flags |= kFlagHasCmap;
        }
        for (int j = 0; j < D; j++) R.b[slot * D + j] = bt[j];
        R.est[slot] = e;
        R.m[slot] = mfin;
        R.pbc[slot] = m;
        R.phc[slot] = phc;
        R.z[slot] = t;
        R.lhp[slot] = lhp;
        R.fam[slot] = (int)i;
        R.horthog[slot] = hof;
        R.cval[slot] = zeta;
        R.dval[slot] = dv;
        R.flags[slot] = flags;
        // rows of a family whose records do not all fit are dropped, as before
        if (pslot < nR && cslot0 + __popc(integ_mask) <= nR) {
            double* Ao = R.A + slot * MC * D;
            for (int q = 0; q < mfin * D; q++) Ao[q] = At[q];
            double ps = 0;
            for (int q = 0; q < mfin; q++) {
                R.p[slot * MC + q] = pt[q];
                R.q[slot * MC + q] = qt[q];
                ps += pt[q];
            }
            R.ps2[slot] = ps * ps;  // (sum of p)^2 in row order
        }
    }
}

// Per-estimator moment sums, then finalize_cached_moments
// (cauchy_estimator.hpp:340-357).  The reference accumulates fz, the mean and
// the covariance in one sequential pass over the terms (parents in order, each
// followed by its children); the same chain is summed here, so the moments
// come out bit-identical to the serial reference.
//
// The chains are independent per moment component: one warp per (estimator,
// 32 components), each lane adding its component over the estimator's rows in
// order.  A chain is a run of dependent additions, so the rows are streamed
// into a shared-memory ring by cp.async ahead of the adder: with one active
// estimator of 10^6 terms the chain runs at the FP64 add rate instead of
// waiting on DRAM once every few rows.  Each lane copies and reads only its
// own column, so its own cp.async.wait_group is the only synchronisation.
constexpr int kMomStages = 3, kMomRows = 64;

__device__ inline void cp_async8(double* smem_dst, const double* gmem_src)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem_src) : "memory");
}
__device__ inline void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ inline void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <int D>
__global__ void __launch_bounds__(32) k_moments_chain(const cd* contrib, const long long* pstart,
                                                      const long long* kall_scan, int E, const int* order,
                                                      const EstStep<D>* st, double* tot)
{
    constexpr int NM = 1 + D + D * D;
    constexpr int ND = 2 * NM;              // doubles per term
    constexpr int NS = (ND + 31) / 32;      // 32-component slices
    __shared__ double ring[kMomStages][kMomRows][32];
    const int lane = threadIdx.x;
    const int eb = blockIdx.x / NS, slice = blockIdx.x - eb * NS;
    if (eb >= E) return;
    // blocks start in launch order: the longest chains go first
    const int e = order ? order[eb] : eb;
    if (!st[e].active) return;
    const long long a = pstart[e] + kall_scan[pstart[e]];
    const long long n = pstart[e + 1] + kall_scan[pstart[e + 1]] - a;
    const int comp = slice * 32 + lane;
    const bool valid = comp < ND;
    const double* col = reinterpret_cast<const double*>(contrib) + a * ND + comp;
    const long long nchunks = (n + kMomRows - 1) / kMomRows;
    // chunk k of this lane's column into ring slot k % kMomStages (one commit group per chunk)
    auto issue = [&](long long k) {
        if (valid && k < nchunks) {
            const long long r0 = k * kMomRows;
            const int cnt = n - r0 < kMomRows ? (int)(n - r0) : kMomRows;
            double(*slot)[32] = ring[k % kMomStages];
            const double* src = col + r0 * ND;
            if (cnt == kMomRows) {
#pragma unroll
                for (int r = 0; r < kMomRows; r++) cp_async8(&slot[r][lane], src + r * ND);
            } else
                for (int r = 0; r < cnt; r++) cp_async8(&slot[r][lane], src + r * ND);
        }
        cp_async_commit();
    };
    for (int k = 0; k < kMomStages - 1; k++) issue(k);
    double sum = 0.0;
    for (long long k = 0; k < nchunks; k++) {
        cp_async_wait<kMomStages - 2>();  // chunk k has landed
        // refill the slot of chunk k - 1, whose values were added last iteration
        issue(k + kMomStages - 1);
        if (valid) {
            const long long r0 = k * kMomRows;
            const double(*slot)[32] = ring[k % kMomStages];
            if (n - r0 >= kMomRows) {
                // all loads first, then the dependent additions back to back
                double v[kMomRows];
#pragma unroll
                for (int r = 0; r < kMomRows; r++) v[r] = slot[r][lane];
#pragma unroll
                for (int r = 0; r < kMomRows; r++) sum += v[r];
            } else {
                const int cnt = (int)(n - r0);
                for (int r = 0; r < cnt; r++) sum += slot[r][lane];
            }
        }
    }
    cp_async_wait<0>();
    if (valid) tot[(long long)e * ND + comp] = sum;
}

// finalize_cached_moments (cauchy_estimator.hpp:340-357) from the chain totals.
template <int D>
__global__ void k_moments_final(const double* tot, int E, const EstStep<D>* st, cd* est_raw, double* gscale)
{
    constexpr int NM = 1 + D + D * D;
    constexpr int ND = 2 * NM;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E || !st[e].active) return;
    const double* t = tot + (long long)e * ND;
    const cd fz = mkcd(t[0], t[1]);
    gscale[e] = kTwoPiInv / fz.re;
    const cd ifz = mkcd(0, fz.re);
    cd* out = est_raw + (long long)e * NM;
    out[0] = fz;
    cd mfin[D];
    for (int j = 0; j < D; j++) {
        mfin[j] = cdiv(mkcd(t[2 * (1 + j)], t[2 * (1 + j) + 1]), ifz);
        out[1 + j] = mfin[j];
    }
    // the covariance is accumulated as cov -= (g y_j) y_k, i.e. minus the chain
    for (int j = 0; j < D; j++)
        for (int k = 0; k < D; k++) {
            const int q = 2 * (1 + D + j * D + k);
            const cd cv = mkcd(-t[q], -t[q + 1]);
            out[1 + D + j * D + k] = csub(cdiv(cv, fz), cmul(mfin[j], mfin[k]));
        }
}

// ---------------------------------------------------------------------------
// Fast term reduction.  The reference sorts b along each axis and, for each
// not-yet-reduced term i in index order, takes every later unreduced term j
// with qp-eps < b_j <= qp+eps on all axes (qp = b_i), |p_j - p_i| <= eps and
// the hyperplane test, and reduces it into i (term_reduction.hpp:159-276).
// Here candidates come from a grid over all coordinates of b with cells of
// width 64 eps, keyed by (estimator, shape, cell): a near pair is at most one
// cell apart per axis, and a term only probes the neighbour cell on an axis
// when its +-3 eps window crosses the cell boundary (about 1.2 probes per term
// in three dimensions).  Cells are counting-sorted into contiguous buckets
// that carry b inline, so candidate scans read contiguous memory.  The greedy
// index-order resolution of the reference is reproduced by ftr_resolve.
constexpr double kCellWidth = 64.0 * kReductionEps;
constexpr double kProbeHalfWidth = 3.0 * kReductionEps;

__device__ inline unsigned long long mix64(unsigned long long x)
{
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}
__device__ inline long long cell_of(double v)
{
    // only a bucketing device: the same rounding on every side keeps it consistent
    double q = floor(v * (1.0 / kCellWidth));
    if (!(q > -4.0e18)) q = -4.0e18;  // also catches NaN
    if (q > 4.0e18) q = 4.0e18;
    return (long long)q;
}
template <int D>
__device__ inline long long cell_slot(int e, int m, const long long* c, long long hmask)
{
    unsigned long long h = mix64(((unsigned long long)e << 8) ^ (unsigned long long)m);
    for (int a = 0; a < D; a++) h = mix64(h ^ ((unsigned long long)c[a] * 0x9e3779b97f4a7c15ull));
    return (long long)(h & (unsigned long long)hmask);
}

// A bucket entry: the term, its (estimator, shape) and the integer keys of
// its b window (b - eps, b + eps], computed once per term instead of once
// per candidate test.
template <int D>
struct CellEntry {
    int idx;
    int est_m;  // est << 5 | m
    long long lo[D], hi[D];
};

template <int D>
__global__ void k_ftr_count_cells(TermRecs R, long long nR, long long hmask, int* slot_of, int* bcount)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < nR; j += (long long)gridDim.x * blockDim.x) {
        const int e = R.est[j];
        if (e < 0) {
            slot_of[j] = -1;
            continue;
        }
        long long c[D];
        for (int a = 0; a < D; a++) c[a] = cell_of(R.b[j * D + a]);
        const int s = (int)cell_slot<D>(e, R.m[j], c, hmask);
        slot_of[j] = s;
        atomicAdd(&bcount[s], 1);
    }
}

template <int D>
__global__ void k_ftr_scatter(TermRecs R, long long nR, const int* slot_of, const long long* boff, int* bfill,
                              CellEntry<D>* ent)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < nR; j += (long long)gridDim.x * blockDim.x) {
        const int s = slot_of[j];
        if (s < 0) continue;
        const long long pos = boff[s] + atomicAdd(&bfill[s], 1);
        CellEntry<D> c;
        c.idx = (int)j;
        c.est_m = (R.est[j] << 5) | R.m[j];
        for (int a = 0; a < D; a++) {
            const double b = R.b[j * D + a];
            c.lo[a] = dkey(b - kReductionEps);
            c.hi[a] = dkey(b + kReductionEps);
        }
        ent[pos] = c;
    }
}

template <int D>
__device__ inline bool ftr_near_pm(const TermRecs& R, long long i, long long j, int m, int MC)
{
    const double* pi = R.p + i * MC;
    const double* pj = R.p + j * MC;
    for (int k = 0; k < m; k++)
        if (!abs_lt(pj[k] - pi[k], kReductionEps) && dabs_bits(pj[k] - pi[k]) != dabs_bits(kReductionEps))
            return false;  // |p_j - p_i| > eps
    // the reference compares Ai[k] with Aj[k] for k < m inside its per-component
    // loop (term_reduction.hpp:237-244), i.e. the first m entries of row-major A
    const double* Ai = R.A + i * MC * D;
    const double* Aj = R.A + j * MC * D;
    for (int k = 0; k < m; k++) {
        const double r = Ai[k], c = Aj[k];
        if (!(abs_lt(r - c, kReductionEps) || abs_lt(r + c, kReductionEps))) return false;
    }
    return true;
}

// Buckets in ascending term order: every entry ranks itself inside its bucket.
template <int D>
__global__ void k_ftr_sort_buckets(const CellEntry<D>* in, long long n, const int* slot_of, const long long* boff,
                                   CellEntry<D>* out)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const CellEntry<D> me = in[k];
        const int s = slot_of[me.idx];
        const long long a = boff[s], bnd = boff[s + 1];
        long long rank = 0;
        for (long long q = a; q < bnd; q++) rank += in[q].idx < me.idx;
        out[a + rank] = me;
    }
}

// One round of the greedy term reduction (term_reduction.hpp:186-270): a term
// whose smallest not-yet-reduced near predecessor is a root joins it; a term
// with no such predecessor is a root; otherwise it waits for the next round.
// Near predecessors are found by scanning the sorted buckets of the cells
// around b in ascending index, stopping at the first one that is not a member.
// Members and non-near entries stay what they are, so a term that must wait
// resumes each bucket at the entry that stopped it (resume[j][q] for its q-th
// distinct bucket), and later rounds run over the worklist of waiting terms.

// One resolution round over the records (wl_in null, the first round) or
// the worklist wl_in[0..*n_in): each record still undecided looks for its
// nearest near predecessor in its cell buckets; it becomes a member of a
// root, a root, or waits for the next round (wl_out).  A decision is only
// taken on predecessors that are decided, so the result does not depend on
// the order the threads run in.
template <int D>
__device__ __forceinline__ void ftr_round(const TermRecs& R, long long nR, const CellEntry<D>* ent,
                                          const long long* boff, long long hmask, int MC, int* status, int* owner,
                                          const int* wl_in, const int* n_in, int* wl_out, int* n_out, int* resume,
                                          long long tid, long long nth)
{
    const long long n = wl_in ? (long long)*(volatile const int*)n_in : nR;
    for (long long w = tid; w < n; w += nth) {
        // records, states and resume points written in earlier rounds are read
        // through L2 (a persistent launch does not refresh an SM's L1)
        const long long j = wl_in ? (long long)__ldcg(wl_in + w) : w;
        if (__ldcg(status + j) != 0) continue;
        const int e = R.est[j];
        const int m = R.m[j];
        const int em = (e << 5) | m;
        double bj[D];
        long long kj[D], lo[D], nc[D];
        int nprobe = 1;
        for (int a = 0; a < D; a++) {
            bj[a] = R.b[j * D + a];
            kj[a] = dkey(bj[a]);
            lo[a] = cell_of(bj[a] - kProbeHalfWidth);
            const long long hi = cell_of(bj[a] + kProbeHalfWidth);
            nc[a] = hi - lo[a] + 1;
            if (nc[a] < 1) nc[a] = 1;
            if (nc[a] > 2) nc[a] = 2;
            nprobe *= (int)nc[a];
        }
        int best = INT_MAX, minu = INT_MAX;
        long long seen[1 << (D < 5 ? D : 5)];
        int nseen = 0;
        for (int pr = 0; pr < nprobe; pr++) {
            long long c[D];
            int rem = pr;
            for (int a = 0; a < D; a++) {
                c[a] = lo[a] + (rem % nc[a]);
                rem /= (int)nc[a];
            }
            const long long s = cell_slot<D>(e, m, c, hmask);
            bool dup = false;
            for (int q = 0; q < nseen; q++) dup |= seen[q] == s;
            if (dup) continue;
            const int q = nseen;
            if (nseen < (1 << (D < 5 ? D : 5))) seen[nseen++] = s;
            const long long kb = boff[s], ke = boff[s + 1];
            long long k = kb + ((wl_in && q < kFtrResume) ? __ldcg(resume + j * kFtrResume + q) : 0);
            for (; k < ke; k++) {
                const CellEntry<D>& ce = ent[k];
                if (ce.idx >= j) break;  // ascending: no predecessors beyond
                if (ce.est_m != em) continue;
                bool ok = true;
                for (int a = 0; a < D && ok; a++)
                    if (!(ce.lo[a] < kj[a] && kj[a] <= ce.hi[a])) ok = false;
                if (!ok || !ftr_near_pm<D>(R, ce.idx, j, m, MC)) continue;
                const int st = ((volatile int*)status)[ce.idx];
                if (st == 2) continue;  // a member: look further
                if (st == 1) best = ce.idx < best ? ce.idx : best;
                else minu = ce.idx < minu ? ce.idx : minu;
                break;  // the first non-member near predecessor of this bucket decides it
            }
            if (q < kFtrResume) resume[j * kFtrResume + q] = (int)(k - kb);
        }
        if (best < minu) {
            owner[j] = best;
            ((volatile int*)status)[j] = 2;
        } else if (minu == INT_MAX) {
            owner[j] = (int)j;
            ((volatile int*)status)[j] = 1;
        } else
            wl_out[atomicAdd(n_out, 1)] = (int)j;
    }
}

template <int D>
__global__ void k_ftr_resolve_scan(TermRecs R, long long nR, const CellEntry<D>* ent, const long long* boff,
                                   long long hmask, int MC, int* status, int* owner, const int* wl_in, const int* n_in,
                                   int* wl_out, int* n_out, int* resume)
{
    ftr_round<D>(R, nR, ent, boff, hmask, MC, status, owner, wl_in, n_in, wl_out, n_out, resume,
                 blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
}

// Grid-wide barrier of a cooperative launch with a bounded wait: bar[0]
// counts the blocks arrived, bar[1] is the generation.  Returns false (for
// every thread of the block) when the wait ran past spin_limit polls; the
// caller then stops.
__device__ inline bool grid_barrier(unsigned* bar, long long spin_limit)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned gen = *(volatile unsigned*)(bar + 1);
        __threadfence();
        const unsigned arrived = atomicAdd(bar, 1u) + 1;
        if (arrived == gridDim.x) {
            *(volatile unsigned*)bar = 0;
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long it = 0;
            while (*(volatile unsigned*)(bar + 1) == gen) {
                if (++it > spin_limit) {
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// The resolution rounds from first_round on in one persistent cooperative
// launch over a device worklist: round r reads the worklist and count of
// round r - 1, writes its own, and the grid synchronises between rounds; the
// loop ends when a round leaves nothing undecided.  After max_rounds rounds, or a barrier wait past
// its limit, it stops with kErrResolveStalled.  Round r's count is
// cnt[r % 3]; cnt[(r + 1) % 3], which no thread touches in round r, is
// cleared then for round r + 1.
template <int D>
__global__ void __launch_bounds__(128) k_ftr_resolve_all(TermRecs R, long long nR, const CellEntry<D>* ent,
                                                         const long long* boff, long long hmask, int MC, int* status,
                                                         int* owner, int* wl0, int* wl1, int* cnt, int* resume,
                                                         unsigned* bar, int first_round, int max_rounds, int* err)
{
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nth = (long long)gridDim.x * blockDim.x;
    for (int r = first_round;; r++) {
        if (r >= max_rounds) {
            if (tid == 0) atomicOr(err, kErrResolveStalled);
            break;
        }
        int* wl_out = (r & 1) ? wl1 : wl0;
        const int* wl_in = r ? ((r & 1) ? wl0 : wl1) : nullptr;
        int* n_out = cnt + r % 3;
        const int* n_in = r ? cnt + (r + 2) % 3 : nullptr;
        if (tid == 0) cnt[(r + 1) % 3] = 0;
        ftr_round<D>(R, nR, ent, boff, hmask, MC, status, owner, wl_in, n_in, wl_out, n_out, resume, tid, nth);
        if (!grid_barrier(bar, 1LL << 26)) {
            if (threadIdx.x == 0) atomicOr(err, kErrResolveStalled);
            break;
        }
        if (*(volatile int*)n_out == 0) break;
    }
}

// The resolution rounds after the first as a loop that runs on the device
// inside a CUDA graph: a WHILE conditional node whose body is one round over
// the previous round's worklist (k_ftr_graph_round) followed by a one-thread
// kernel (k_ftr_graph_next) that advances the round, clears the next round's
// count and sets the loop condition from the worklist just produced, so the
// host neither launches nor waits for the rounds.  The graph is built once per
// engine; its kernels read their pointers from a device argument block that
// the host rewrites before each launch.  Round r reads worklist (r - 1) & 1
// and count cnt[(r - 1) % 8] and writes worklist r & 1 and cnt[r % 8], as the
// batched rounds do.  After max_rounds rounds the loop stops with
// kErrResolveStalled.
template <int D>
struct FtrLoopArgs {
    TermRecs R;
    long long nR;
    const CellEntry<D>* ent;
    const long long* boff;
    long long hmask;
    int MC;
    int* status;
    int* owner;
    int* wl0;
    int* wl1;
    int* cnt;
    int* resume;
    int* err;
    int round;       // the round the body runs next (the device advances it)
    int max_rounds;
};

template <int D>
__global__ void __launch_bounds__(128) k_ftr_graph_round(const FtrLoopArgs<D>* a)
{
    const int r = *(volatile const int*)&a->round;
    const TermRecs R = a->R;
    const int* wl_in = ((r - 1) & 1) ? a->wl1 : a->wl0;
    int* wl_out = (r & 1) ? a->wl1 : a->wl0;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nth = (long long)gridDim.x * blockDim.x;
    ftr_round<D>(R, a->nR, a->ent, a->boff, a->hmask, a->MC, a->status, a->owner, wl_in, a->cnt + (r - 1) % 8, wl_out,
                 a->cnt + r % 8, a->resume, tid, nth);
}

template <int D>
__global__ void k_ftr_graph_next(FtrLoopArgs<D>* a, cudaGraphConditionalHandle h)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int r = a->round;
    const int n = *(volatile int*)(a->cnt + r % 8);
    a->cnt[(r + 1) % 8] = 0;
    a->round = r + 1;
    unsigned more = n > 0 ? 1u : 0u;
    if (more && r + 1 >= a->max_rounds) {
        atomicOr(a->err, kErrResolveStalled);
        more = 0u;
    }
    cudaGraphSetConditional(h, more);
}

#if MCE_COMMON_UNIT
__global__ void k_group_count(const int* status, const int* owner, long long nR, int* gcnt)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < nR; j += (long long)gridDim.x * blockDim.x)
        if (status[j] == 2) atomicAdd(&gcnt[owner[j]], 1);
}

__global__ void k_group_fill(const int* status, const int* owner, long long nR, const long long* goff, int* gfill,
                             int* members)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < nR; j += (long long)gridDim.x * blockDim.x)
        if (status[j] == 2) {
            const int r = owner[j];
            const int k = atomicAdd(&gfill[r], 1);
            members[goff[r] + k] = (int)j;
        }
}

// Member lists in ascending index order (the forward flag array's order,
// cauchy_util.hpp:387-410): one warp per group ranks each member by counting
// smaller ones.
__global__ void k_group_sort(const int* gcnt, const long long* goff, long long nR, const int* members_in,
                             int* members_out)
{
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwb = blockDim.x >> 5;
    for (long long r = (long long)blockIdx.x * nwb + wib; r < nR; r += (long long)gridDim.x * nwb) {
        const int n = gcnt[r];
        if (n == 0) continue;
        const int* a = members_in + goff[r];
        int* o = members_out + goff[r];
        for (int x = lane; x < n; x += 32) {
            const int v = a[x];
            int rank = 0;
            for (int y = 0; y < n; y++) rank += a[y] < v;
            o[rank] = v;
        }
    }
}

__global__ void k_roots_flags(const int* status, const int* m, long long nR, int D, int* is_root, int* cap)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < nR; j += (long long)gridDim.x * blockDim.x) {
        const bool r = status[j] == 1;
        is_root[j] = r ? 1 : 0;
        cap[j] = r ? half_cells_cap(m[j], D) : 0;
    }
}

__global__ void k_roots_list(const int* is_root, const long long* rscan, long long nR, int* list)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < nR; j += (long long)gridDim.x * blockDim.x)
        if (is_root[j]) list[rscan[j]] = (int)j;
}

#endif  // MCE_COMMON_UNIT

// ---------------------------------------------------------------------------
// g-table construction per reduction group (flattening.hpp:77-568).

struct GCtx {
    TermRecs R;
    ParentList P;
    Tables Told;
    const int* Bkeys;
    int MC;
    unsigned* gbits;  // global bitmap regions (see LaunchCfg), or null: shared memory
    int capR;         // cells of a group's list and scratch (LaunchCfg::cells_cap)
};

// One cell of make_gtable (flattening.hpp:105-224) for record s at `key`.
template <int D>
__device__ inline cd g_cell(const GCtx& c, long long s, int key, double gscale)
{
    const TermRecs& R = c.R;
    const int MC = c.MC;
    const int m = R.m[s], phc = R.phc[s], flags = R.flags[s];
    const unsigned hof = R.horthog[s];
    const double* q = R.q + s * MC;
    double ygi = 0;
    for (int k = 0; k < m; k++)
        if (!(hof & (1u << k))) ygi += ((key >> k) & 1) ? -q[k] : q[k];  // q_k * s_k, exact
    int lp = 0, lm = 0;
    if (!(flags & kFlagNewChild)) {
        lp = key & ((1 << phc) - 1);
        lm = lp;
    } else {
        const int z = R.z[s];
        const signed char* cmap = R.cmap + s * MC;
        const signed char* csmap = R.csmap + s * MC;
        const bool hc = flags & kFlagHasCmap;
        int k = 0, l = 0;
        while (k < phc) {
            if (k == z) {
                lm |= 1 << k;
                k++;
                if (k == phc) break;
            }
            int neg;
            if (hc) {
                const int ci = (unsigned char)cmap[l];
                const int bv = (((key >> ci) & 1) ? -1 : 1) * (int)csmap[l];
                neg = bv < 0;
            } else
                neg = (key >> l) & 1;
            if (neg) {
                lp |= 1 << k;
                lm |= 1 << k;
            }
            k++;
            l++;
        }
    }
    const int fam = R.fam[s];
    const int* pk = c.Told.keys + c.P.tab_off[fam];
    const cd* pv = c.Told.vals + c.P.tab_off[fam];
    const int pcnt = c.P.tab_cnt[fam];
    const int lhp = R.lhp[s];
    const cd gp = lookup_num(pk, pv, pcnt, lp ^ lhp, phc);
    const cd gm = lookup_num(pk, pv, pcnt, lm ^ lhp, phc);
    const double dv = R.dval[s], cv = R.cval[s];
    cd v = csub(cdiv(gp, mkcd(ygi + dv, cv)), cdiv(gm, mkcd(ygi - dv, cv)));
    return cscale(v, gscale);
}

__device__ inline bool bm_get(const unsigned* bm, int k) { return (bm[k >> 5] >> (k & 31)) & 1u; }

// Extracts the set bits of a 2^m-bit bitmap in ascending order into out[]; returns the count.
__device__ inline int bm_extract(const unsigned* bm, int m, int* out, int cap, int lane)
{
    const int nb = 1 << m;
    const int words = nb > 32 ? nb / 32 : 1;
    int count = 0;
    for (int w0 = 0; w0 < words; w0 += 32) {
        const int w = w0 + lane;
        unsigned bits = w < words ? bm[w] : 0u;
        if (nb < 32) bits &= (1u << nb) - 1;
        const int c = __popc(bits);
        int pre = c;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(kFull, pre, o);
            if (lane >= o) pre += y;
        }
        const int tot = __shfl_sync(kFull, pre, 31);
        int pos = count + pre - c;
        while (bits) {
            const int b = __ffs(bits) - 1;
            bits &= bits - 1;
            if (pos < cap) out[pos] = w * 32 + b;
            pos++;
        }
        count += tot;
    }
    return count;
}


// Root cells of a new child: make_new_child_btable (cell_enumeration.hpp:206-371)
// into the bitmap RK (2^m bits).  PB receives the parent's B_mu as a bitmap.
template <int D>
__device__ inline void new_child_cells(const GCtx& c, long long s, unsigned* RK, unsigned* PB, int* bmk, int lane)
{
    const TermRecs& R = c.R;
    const int m = R.m[s];
    const int words_m = (1 << m) > 32 ? (1 << m) / 32 : 1;
    for (int k = lane; k < words_m; k += 32) RK[k] = 0;
    if (m <= D) {
        __syncwarp();
        for (int k = lane; k < (1 << (m - 1)); k += 32) atomicOr(&RK[k >> 5], 1u << (k & 31));
        __syncwarp();
        return;
    }
    const int fam = R.fam[s];
    const int* Bmu = c.Bkeys + c.P.B_off[fam];
    const int nB = c.P.B_cnt[fam];
    const int pbc = R.pbc[s], z = R.z[s];
    const int words_p = (1 << pbc) > 32 ? (1 << pbc) / 32 : 1;
    for (int k = lane; k < words_p; k += 32) PB[k] = 0;
    const bool coal = m < pbc;
    if (coal && lane == 0) {
        // first original row of every coaligned group (cell_enumeration.hpp:318-331)
        unsigned seen = 0;
        int cnt = 0;
        const signed char* cmap = R.cmap + s * c.MC;
        for (int j = 0; j < pbc; j++) {
            const int ci = (unsigned char)cmap[j];
            if (ci < 32 && !((seen >> ci) & 1u)) {
                seen |= 1u << ci;
                bmk[cnt++] = j;
            }
        }
        bmk[31] = cnt;
    }
    __syncwarp();
    for (int k = lane; k < nB; k += 32) {
        const int key = Bmu[k];
        if (key >= 0 && key < (1 << pbc)) atomicOr(&PB[key >> 5], 1u << (key & 31));
    }
    __syncwarp();
    const int ncoal = coal ? bmk[31] : 0;
    const int mz = 1 << z, hb = 1 << (pbc - 1), rev = (1 << pbc) - 1;
    for (int k = lane; k < nB; k += 32) {
        const int b = Bmu[k];
        int bq = b ^ mz;
        if (bq & hb) bq ^= rev;
        if (bq < 0 || bq >= (1 << pbc) || !bm_get(PB, bq)) continue;
        const int zb = (b & mz) >> z;
        const int c1 = ((b >> (z + 1)) << z) | (b & (mz - 1)) | (zb << (pbc - 1));
        const int c2 = c1 ^ hb;
        int out[2] = {(c1 & hb) ? (c1 ^ rev) : c1, (c2 & hb) ? (c2 ^ rev) : c2};
        for (int u = 0; u < 2; u++) {
            int key = out[u];
            if (coal) {
                int bc = 0;
                for (int l = 0; l < ncoal; l++)
                    if (key & (1 << bmk[l])) bc |= 1 << l;
                key = bc;
            }
            if (key >= 0 && key < (1 << m)) atomicOr(&RK[key >> 5], 1u << (key & 31));
        }
    }
    __syncwarp();
}

template <int D>
__device__ inline void own_cells(const GCtx& c, long long s, unsigned* bm, int lane)
{
    const int m = c.R.m[s];
    const int words_m = (1 << m) > 32 ? (1 << m) / 32 : 1;
    for (int k = lane; k < words_m; k += 32) bm[k] = 0;
    __syncwarp();
    const int fam = c.R.fam[s];
    const int* B = c.Bkeys + c.P.B_off[fam];
    const int n = c.P.B_cnt[fam];
    for (int k = lane; k < n; k += 32) {
        const int key = B[k];
        if (key >= 0 && key < (1 << m)) atomicOr(&bm[key >> 5], 1u << (key & 31));
    }
    __syncwarp();
}

// ---------------------------------------------------------------------------
// Flat g-table evaluation.  make_gtables (flattening.hpp:318-568) spends its
// FP64 work in one cell evaluation per (term, cell) of every reduction group:
// the root's cells, then each member's cells in the root's orientation.  Most
// groups are small (a 3-state term of 4-6 hyperplanes has 7-16 cells, a group
// holds one to three terms), so evaluating them a group per warp leaves most
// lanes idle through every FP64 instruction.  Instead:
//   k_gtable_prep  (a warp per group)  the root's cells into its output keys,
//                  each member's orientation and mode, the p sums;
//   k_gtable_eval  (a thread per (term, cell) of every group)  g_cell, and
//                  the term-approximation flags;
//   k_gtable       (a warp per group)  the sums in member order; a group whose
//                  root is approximated out takes the serial path, which
//                  re-derives everything in the reference's order.
// Member info word: bits 0-15 the orientation mask relative to the root,
// bit 30 the own-table mode.
constexpr int kInfoOwn = 1 << 30;
constexpr int kFlatMaxCells = 64;

template <int D>
__global__ void k_gtable_prep(GCtx c, const int* roots_list, long long nroots, const int* gcnt, const long long* goff,
                              const int* members, const long long* toff, Tables Tnew, int* gnr, int* gitems,
                              int* gcells, int* minfo, double* rps2, double* mps2, int* rflag, int* mflag,
                              int* need, int* over)
{
    extern __shared__ unsigned smem_g[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwb = blockDim.x >> 5;
    const int MC = c.MC;
    const int words = (1 << MC) > 32 ? (1 << MC) / 32 : 1;
    const int capMC = c.capR;
    const size_t pw = (size_t)(2 * words + 32 + capMC);
    unsigned* PB = c.gbits ? c.gbits + (size_t)((long long)blockIdx.x * nwb + wib) * pw : smem_g + (size_t)wib * pw;
    unsigned* RK = PB + words;
    int* bmk = reinterpret_cast<int*>(RK + words);
    int* RKL = bmk + 32;
    const TermRecs& R = c.R;
    for (long long ri = (long long)blockIdx.x * nwb + wib; ri < nroots; ri += (long long)gridDim.x * nwb) {
        const long long r = roots_list[ri];
        const int m = R.m[r];
        const int cap = (int)(toff[r + 1] - toff[r]);
        int* okeys = Tnew.keys + toff[r];
        if (R.flags[r] & kFlagNewChild) new_child_cells<D>(c, r, RK, PB, bmk, lane);
        else own_cells<D>(c, r, RK, lane);
        int nR = bm_extract(RK, m, RKL, capMC, lane);
        __syncwarp();
        if (nR > cap || nR > capMC) {
            // more cells than a central arrangement in general position can
            // have: the caller re-sizes this root's slot and runs again
            if (lane == 0) {
                need[r] = nR;
                atomicOr(over, 1);
                atomicMax(over + 1, nR);
            }
            nR = cap < capMC ? cap : capMC;
        }
        for (int k = lane; k < nR; k += 32) okeys[k] = RKL[k];
        const int nmem = gcnt[r];
        // groups of many cells fill warps on their own: they stay on the
        // serial path, which keeps the items buffer small
        const bool flat = nR > 0 && nR <= kFlatMaxCells;
        if (lane == 0) {
            gnr[ri] = nR;
            gitems[ri] = flat ? (1 + nmem) * nR : 0;
            gcells[ri] = flat ? nR : 0;
            rps2[ri] = R.ps2[r];
            rflag[ri] = 0;
        }
        const long long mb = goff[r];
        for (int j = lane; j < nmem; j += 32) {
            const long long cm = members[mb + j];
            const bool own = !(R.flags[cm] & kFlagNewChild) && c.P.B_cnt[R.fam[cm]] == nR;
            const int sig = orientation_mask<D>(R.A + r * MC * D, R.A + cm * MC * D, m);
            minfo[mb + j] = sig | (own ? kInfoOwn : 0);
            mps2[mb + j] = R.ps2[cm];
            mflag[mb + j] = 0;
        }
        __syncwarp();
    }
}

// Items of each group laid out root cells first, then each member's: item
// (j, k) of group ri is ioff[ri] + j * nR + k.  The key of a member's item is
// its k-th own-table key (own mode, make_gtable over the member's B) or the
// root's k-th cell in the member's orientation.
template <int D>
__global__ void k_gtable_eval(GCtx c, const int* roots_list, long long nroots, const long long* ioff, long long nitems,
                              const int* gnr, const long long* goff, const int* members, const int* minfo,
                              const double* rps2, const double* mps2, const double* gscale_e, const long long* toff,
                              Tables Tnew, cd* gv, int* rflag, int* mflag)
{
    const TermRecs& R = c.R;
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < nitems;
         x += (long long)gridDim.x * blockDim.x) {
        // the group: the last ri with ioff[ri] <= x
        long long lo = 0, hi = nroots;
        while (hi - lo > 1) {
            const long long mid = (lo + hi) >> 1;
            if (ioff[mid] <= x) lo = mid;
            else hi = mid;
        }
        const long long ri = lo;
        const long long r = roots_list[ri];
        const int nR = gnr[ri];
        const long long loc = x - ioff[ri];
        const int j = (int)(loc / nR), k = (int)(loc - (long long)j * nR);
        const int* okeys = Tnew.keys + toff[r];
        long long s;
        int key;
        double ps2;
        int* flag;
        if (j == 0) {
            s = r;
            key = okeys[k];
            ps2 = rps2[ri];
            flag = rflag + ri;
        } else {
            const long long mi = goff[r] + j - 1;
            s = members[mi];
            const int info = minfo[mi];
            if (info & kInfoOwn) {
                key = c.Bkeys[c.P.B_off[R.fam[s]] + k];
            } else {
                const int m = R.m[r];
                const int top = 1 << (m - 1), rev = (1 << m) - 1;
                const int sig = info & 0xffff;
                key = okeys[k] ^ ((sig & top) ? (sig ^ rev) : sig);
            }
            ps2 = mps2[mi];
            flag = mflag + mi;
        }
        const cd v = g_cell<D>(c, s, key, gscale_e[R.est[r]]);
        gv[x] = v;
        if (above_approx_threshold(ps2, v.re, v.im)) *flag = 1;
    }
}

// The sums of kept groups, a thread per root cell (coff: the flat groups'
// exclusive cell offsets): the root's value plus each member that is not
// approximated out, in member order (flattening.hpp:493-552), from the
// evaluated items.  A member's value for root cell bi is at the root cell
// bj ^ sigf, bj the canonical form of bi ^ sig (own mode: at bj in the
// member's own table).
template <int D>
__global__ void k_gtable_combine(GCtx c, const int* roots_list, long long nroots, const long long* coff,
                                 long long ncells, const int* gcnt, const long long* goff, const int* members,
                                 const long long* toff, Tables Tnew, int* tcnt, int* alive, int* src, const int* rflag,
                                 const long long* ioff, const int* gnr, const int* minfo, const int* mflag,
                                 const cd* gv)
{
    const TermRecs& R = c.R;
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < ncells;
         x += (long long)gridDim.x * blockDim.x) {
        long long lo = 0, hi = nroots;
        while (hi - lo > 1) {
            const long long mid = (lo + hi) >> 1;
            if (coff[mid] <= x) lo = mid;
            else hi = mid;
        }
        const long long ri = lo;
        if (!rflag[ri]) continue;  // the serial path takes this group
        const long long r = roots_list[ri];
        const int m = R.m[r];
        const int top = 1 << (m - 1), rev = (1 << m) - 1;
        const int nR = gnr[ri];
        const int k = (int)(x - coff[ri]);
        const long long base = ioff[ri];
        const int* okeys = Tnew.keys + toff[r];
        const int nmem = gcnt[r];
        const long long mb = goff[r];
        const int bi = okeys[k];
        cd acc = gv[base + k];
        for (int j = 0; j < nmem; j++) {
            if (!mflag[mb + j]) continue;
            const int info = minfo[mb + j];
            const int sig = info & 0xffff;
            const int sigf = (sig & top) ? (sig ^ rev) : sig;
            const int t = bi ^ sig;
            const bool cj = t & top;
            const int bj = cj ? (t ^ rev) : t;
            int idx;
            if (info & kInfoOwn) {
                if (bj < 0 || bj >= (1 << m)) continue;
                // the member's table is its family's B_mu: ascending before
                // the MU's XOR, so search through the XOR
                const int fam = R.fam[members[mb + j]];
                idx = bsearch_key_xor(c.Bkeys + c.P.B_off[fam], c.P.B_cnt[fam], bj, c.P.bflip[fam]);
            } else {
                idx = (bj == (bi ^ sigf)) ? k : bsearch_key(okeys, nR, bj ^ sigf);
            }
            if (idx < 0) continue;
            const cd v = gv[base + (long long)(j + 1) * nR + idx];
            acc = cadd(acc, cj ? cconj(v) : v);
        }
        Tnew.vals[toff[r] + k] = acc;
        if (k == 0) {
            alive[r] = 1;
            tcnt[r] = nR;
            src[r] = (int)r;
        }
    }
}

template <int D>
__global__ void k_gtable(GCtx c, const int* roots_list, long long nroots, const int* gcnt, const long long* goff,
                         const int* members, const double* gscale_e, const long long* toff, Tables Tnew, int* tcnt,
                         int* alive, int* src, cd* scratch, long long scratch_per_warp, const int* rflag,
                         const int* gnr, int* pr_root, int* pr_mb, int* pr_mcnt, int* pr_cells, int* pr_items,
                         int* err)
{
    extern __shared__ unsigned smem_g[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwb = blockDim.x >> 5;
    const int MC = c.MC;
    const int words = (1 << MC) > 32 ? (1 << MC) / 32 : 1;
    const int capMC = c.capR;
    const size_t pw = (size_t)(3 * words + 32 + capMC);
    unsigned* PB = c.gbits ? c.gbits + (size_t)((long long)blockIdx.x * nwb + wib) * pw : smem_g + (size_t)wib * pw;
    unsigned* RK = PB + words;
    unsigned* OK = RK + words;
    int* bmk = reinterpret_cast<int*>(OK + words);
    int* RKL = bmk + 32;
    const long long gw = (long long)blockIdx.x * nwb + wib;
    cd* scr = scratch + gw * scratch_per_warp;
    const TermRecs& R = c.R;
    for (long long ri = gw; ri < nroots; ri += (long long)gridDim.x * nwb) {
        if (rflag[ri]) continue;  // kept root: k_gtable_combine
        // the root is approximated out (or has no cells): the serial path
        const long long r = roots_list[ri];
        // a group of at most kFlatMaxCells cells had its root evaluated by the
        // flat pass, so its root is known to be approximated out; alone, the
        // group simply dies
        const bool root_out = gnr[ri] <= kFlatMaxCells;
        if (root_out && gcnt[r] == 0) {
            if (lane == 0) {
                alive[r] = 0;
                tcnt[r] = 0;
            }
            continue;
        }
        const int m = R.m[r];
        const int e = R.est[r];
        const double gs = gscale_e[e];
        const int top = 1 << (m - 1), rev = (1 << m) - 1;
        const long long out_off = toff[r];
        const int cap = (int)(toff[r + 1] - toff[r]);
        int* okeys = Tnew.keys + out_off;
        cd* ovals = Tnew.vals + out_off;
        // ---- root cells
        if (R.flags[r] & kFlagNewChild) new_child_cells<D>(c, r, RK, PB, bmk, lane);
        else own_cells<D>(c, r, RK, lane);
        int nR = bm_extract(RK, m, RKL, capMC, lane);
        __syncwarp();
        if (nR > cap || nR > capMC) {
            if (lane == 0) set_err(err, kErrRootCellsOverflow);
            nR = cap < capMC ? cap : capMC;
        }
        long long root = r;
        // ---- root values and the term-approximation test (flattening.hpp:242-247),
        // unless the flat pass already found the root approximated out
        bool negl = true;
        if (!root_out) {
            const double ps2 = R.ps2[root];
            for (int k = lane; k < nR; k += 32) {
                const cd v = g_cell<D>(c, root, RKL[k], gs);
                okeys[k] = RKL[k];
                ovals[k] = v;
                if (above_approx_threshold(ps2, v.re, v.im)) negl = false;
            }
            negl = __all_sync(kFull, negl);
        }
        const int nmem = gcnt[r];
        const int* mem = members + goff[r];
        int kidx = 0;
        if (negl) {
            // the root is approximated out: the first member that is not
            // becomes the root, with the group's cells carried along
            // (flattening.hpp:412-489)
            root = -1;
            long long alfr = r;
            while (kidx < nmem) {
                const long long cm = mem[kidx++];
                if (R.flags[cm] & kFlagNewChild) {
                    int sg = 0;
                    if (lane == 0) {
                        sg = orientation_mask<D>(R.A + alfr * MC * D, R.A + cm * MC * D, m);
                        if (sg & top) sg ^= rev;
                    }
                    sg = __shfl_sync(kFull, sg, 0);
                    // re-orient the group's cell list into RK and re-sort
                    for (int k = lane; k < words; k += 32) RK[k] = 0;
                    __syncwarp();
                    for (int k = lane; k < nR; k += 32) {
                        const int key = RKL[k] ^ sg;
                        if (key >= 0 && key < (1 << m)) atomicOr(&RK[key >> 5], 1u << (key & 31));
                    }
                    __syncwarp();
                    nR = bm_extract(RK, m, RKL, capMC, lane);
                } else {
                    own_cells<D>(c, cm, RK, lane);
                    nR = bm_extract(RK, m, RKL, capMC, lane);
                }
                __syncwarp();
                if (nR > cap) {
                    if (lane == 0) set_err(err, kErrMemberCellsOverflow);
                    nR = cap;
                }
                const double ps2c = R.ps2[cm];
                bool ng = true;
                for (int k = lane; k < nR; k += 32) {
                    const cd v = g_cell<D>(c, cm, RKL[k], gs);
                    okeys[k] = RKL[k];
                    ovals[k] = v;
                    if (above_approx_threshold(ps2c, v.re, v.im)) ng = false;
                }
                ng = __all_sync(kFull, ng);
                if (!ng) {
                    root = cm;
                    break;
                }
                alfr = cm;
            }
        }
        if (root < 0) {
            if (lane == 0) {
                alive[r] = 0;
                tcnt[r] = 0;
            }
            __syncwarp();
            continue;
        }
        // RK holds the root's cells as a bitmap, RKL as a sorted list.
        // A group of at most kFlatMaxCells cells hands the members left to the
        // promoted-root flat pass (k_gtable_prom_*), which computes what the
        // loop below would, relative to the same root and cells.
        if (root != r && nR <= kFlatMaxCells && kidx < nmem) {
            if (lane == 0) {
                pr_root[ri] = (int)root;
                pr_mb[ri] = (int)(goff[r] + kidx);
                pr_mcnt[ri] = nmem - kidx;
                pr_cells[ri] = nR;
                pr_items[ri] = nR * (nmem - kidx);
                alive[r] = 1;
                tcnt[r] = nR;
                src[r] = (int)root;
            }
            __syncwarp();
            continue;
        }
        // ---- members: make_gtable + add_gtables (flattening.hpp:493-552)
        for (; kidx < nmem; kidx++) {
            const long long cm = mem[kidx];
            const bool newc = R.flags[cm] & kFlagNewChild;
            bool own = false;
            if (!newc) own = c.P.B_cnt[R.fam[cm]] == nR;
            int sig = 0;
            if (lane == 0) sig = orientation_mask<D>(R.A + root * MC * D, R.A + cm * MC * D, m);
            sig = __shfl_sync(kFull, sig, 0);
            const int sigf = (sig & top) ? (sig ^ rev) : sig;
            const double ps2c = R.ps2[cm];
            bool ng = true;
            if (!own) {
                for (int k = lane; k < nR; k += 32) {
                    const cd v = g_cell<D>(c, cm, RKL[k] ^ sigf, gs);
                    scr[k] = v;
                    if (above_approx_threshold(ps2c, v.re, v.im)) ng = false;
                }
                ng = __all_sync(kFull, ng);
                if (!ng)
                    for (int k = lane; k < nR; k += 32) {
                        const int bi = RKL[k];
                        const int t = bi ^ sig;
                        const bool cj = t & top;
                        const int bj = cj ? (t ^ rev) : t;
                        cd v;
                        if (bj == (bi ^ sigf)) v = scr[k];
                        else if (bm_get(RK, bj ^ sigf)) v = g_cell<D>(c, cm, bj, gs);
                        else continue;
                        const cd a = ovals[k];
                        ovals[k] = cadd(a, cj ? cconj(v) : v);
                    }
            } else {
                own_cells<D>(c, cm, OK, lane);
                const int fam = R.fam[cm];
                const int* B = c.Bkeys + c.P.B_off[fam];
                const int n = c.P.B_cnt[fam];
                for (int k = lane; k < n; k += 32) {
                    const cd v = g_cell<D>(c, cm, B[k], gs);
                    if (above_approx_threshold(ps2c, v.re, v.im)) ng = false;
                }
                ng = __all_sync(kFull, ng);
                if (!ng)
                    for (int k = lane; k < nR; k += 32) {
                        const int bi = RKL[k];
                        const int t = bi ^ sig;
                        const bool cj = t & top;
                        const int bj = cj ? (t ^ rev) : t;
                        if (bj < 0 || bj >= (1 << m) || !bm_get(OK, bj)) continue;
                        const cd v = g_cell<D>(c, cm, bj, gs);
                        const cd a = ovals[k];
                        ovals[k] = cadd(a, cj ? cconj(v) : v);
                    }
            }
            __syncwarp();
        }
        if (lane == 0) {
            alive[r] = 1;
            tcnt[r] = nR;
            src[r] = (int)root;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Promoted-root flat pass: the members left after a promotion, against the
// promoted root and its cells (already in the output table), in three flat
// steps like the first pass: member info (orientation relative to the
// promoted root and the own-table mode), a thread per (member, cell) value
// with the term-approximation flag, and a thread per root cell summing the
// kept members in order (flattening.hpp:493-552).
__device__ inline long long last_le(const long long* off, long long n, long long x)
{
    long long lo = 0, hi = n;
    while (hi - lo > 1) {
        const long long mid = (lo + hi) >> 1;
        if (off[mid] <= x) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <int D>
__global__ void k_gtable_prom_prep(GCtx c, long long nroots, long long nmem_total, const int* members, GFlat f)
{
    const TermRecs& R = c.R;
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < nmem_total;
         x += (long long)gridDim.x * blockDim.x) {
        const long long ri = last_le(f.pr_moff, nroots, x);
        const long long root = f.pr_root[ri];
        const int nR = f.pr_cells[ri];
        const long long mi = f.pr_mb[ri] + (x - f.pr_moff[ri]);
        const long long cm = members[mi];
        const int m = R.m[root];
        const bool own = !(R.flags[cm] & kFlagNewChild) && c.P.B_cnt[R.fam[cm]] == nR;
        const int sig = orientation_mask<D>(R.A + root * c.MC * D, R.A + cm * c.MC * D, m);
        f.minfo[mi] = sig | (own ? kInfoOwn : 0);
        f.mflag[mi] = 0;
    }
}

template <int D>
__global__ void k_gtable_prom_eval(GCtx c, const int* roots_list, long long nroots, long long nitems,
                                   const int* members, const double* gscale_e, const long long* toff, Tables Tnew,
                                   GFlat f)
{
    const TermRecs& R = c.R;
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < nitems;
         x += (long long)gridDim.x * blockDim.x) {
        const long long ri = last_le(f.pr_ioff, nroots, x);
        const long long r = roots_list[ri];
        const int nR = f.pr_cells[ri];
        const long long loc = x - f.pr_ioff[ri];
        const int jj = (int)(loc / nR), k = (int)(loc - (long long)jj * nR);
        const long long mi = f.pr_mb[ri] + jj;
        const long long s = members[mi];
        const int info = f.minfo[mi];
        int key;
        if (info & kInfoOwn) {
            key = c.Bkeys[c.P.B_off[R.fam[s]] + k];
        } else {
            const int m = R.m[r];
            const int top = 1 << (m - 1), rev = (1 << m) - 1;
            const int sig = info & 0xffff;
            key = Tnew.keys[toff[r] + k] ^ ((sig & top) ? (sig ^ rev) : sig);
        }
        const cd v = g_cell<D>(c, s, key, gscale_e[R.est[r]]);
        f.pr_gv[x] = v;
        if (above_approx_threshold(R.ps2[s], v.re, v.im)) f.mflag[mi] = 1;
    }
}

template <int D>
__global__ void k_gtable_prom_combine(GCtx c, const int* roots_list, long long nroots, long long ncells,
                                      const int* members, const long long* toff, Tables Tnew, GFlat f)
{
    const TermRecs& R = c.R;
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < ncells;
         x += (long long)gridDim.x * blockDim.x) {
        const long long ri = last_le(f.pr_coff, nroots, x);
        const long long r = roots_list[ri];
        const int m = R.m[r];
        const int top = 1 << (m - 1), rev = (1 << m) - 1;
        const int nR = f.pr_cells[ri];
        const int k = (int)(x - f.pr_coff[ri]);
        const long long base = f.pr_ioff[ri];
        const int* okeys = Tnew.keys + toff[r];
        const int nm = f.pr_mcnt[ri];
        const long long mb = f.pr_mb[ri];
        const int bi = okeys[k];
        cd acc = Tnew.vals[toff[r] + k];  // the promoted root's value
        for (int jj = 0; jj < nm; jj++) {
            if (!f.mflag[mb + jj]) continue;
            const int info = f.minfo[mb + jj];
            const int sig = info & 0xffff;
            const int sigf = (sig & top) ? (sig ^ rev) : sig;
            const int t = bi ^ sig;
            const bool cj = t & top;
            const int bj = cj ? (t ^ rev) : t;
            int idx;
            if (info & kInfoOwn) {
                if (bj < 0 || bj >= (1 << m)) continue;
                const int fam = R.fam[members[mb + jj]];
                idx = bsearch_key_xor(c.Bkeys + c.P.B_off[fam], c.P.B_cnt[fam], bj, c.P.bflip[fam]);
            } else {
                idx = (bj == (bi ^ sigf)) ? k : bsearch_key(okeys, nR, bj ^ sigf);
            }
            if (idx < 0) continue;
            const cd v = f.pr_gv[base + (long long)jj * nR + idx];
            acc = cadd(acc, cj ? cconj(v) : v);
        }
        Tnew.vals[toff[r] + k] = acc;
    }
}

// ---------------------------------------------------------------------------
// Next parent list: per estimator, surviving roots bucketed by shape in
// position order (cauchy_estimator.hpp:1059-1101 keeps roots in index order
// within each shape; shapes ascend).

#if MCE_COMMON_UNIT
// Stable partition of the surviving records by (estimator, shape).  Each
// estimator's record range is cut into tiles of kPartTile records; a block
// counts a tile's records per shape, a thread per (estimator, shape) scans
// the counts over the estimator's tiles (its totals are the shape histogram),
// and a block per tile ranks its records in order.  One estimator of 10^7
// records thus spreads over thousands of blocks instead of one.
constexpr int kPartTile = 4096;

__global__ void k_ptile_count(const long long* rbase, int E, int* ntile)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x)
        ntile[e] = (int)((rbase[e + 1] - rbase[e] + kPartTile - 1) / kPartTile);
}

// the estimator of tile t: the last e with tstart[e] <= t
__device__ inline int tile_est(const long long* tstart, int E, long long t)
{
    int lo = 0, hi = E;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (tstart[mid] <= t) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void k_ptile_hist(const int* alive, const int* m, const long long* rbase, int E, int MCp,
                             const long long* tstart, int* C)
{
    __shared__ int cnt[33];
    const long long NT = tstart[E];
    for (long long t = blockIdx.x; t < NT; t += gridDim.x) {
        if (threadIdx.x < MCp) cnt[threadIdx.x] = 0;
        __syncthreads();
        const int e = tile_est(tstart, E, t);
        const long long a = rbase[e] + (t - tstart[e]) * kPartTile;
        const long long b = a + kPartTile < rbase[e + 1] ? a + kPartTile : rbase[e + 1];
        for (long long j = a + threadIdx.x; j < b; j += blockDim.x)
            if (alive[j]) atomicAdd(&cnt[m[j]], 1);
        __syncthreads();
        if (threadIdx.x < MCp) C[t * MCp + threadIdx.x] = cnt[threadIdx.x];
        __syncthreads();
    }
}

// per (estimator, shape): tile counts -> exclusive prefix over the
// estimator's tiles, the total into the shape histogram
__global__ void k_ptile_scan(int E, int MCp, const long long* tstart, int* C, int* hist)
{
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < (long long)E * MCp;
         x += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(x / MCp), sh = (int)(x - (long long)e * MCp);
        int run = 0;
        for (long long t = tstart[e]; t < tstart[e + 1]; t++) {
            const int c = C[t * MCp + sh];
            C[t * MCp + sh] = run;
            run += c;
        }
        hist[x] = run;
    }
}

// a block per tile: each surviving record's slot, bucket start + records of
// its shape in earlier tiles + earlier ones in this tile
__global__ void k_ptile_rank(const int* alive, const int* m, const long long* rbase, int E, int MCp,
                             const long long* tstart, const int* P, const long long* bucket_off, int* new_slot)
{
    __shared__ long long running[33];
    __shared__ int wcnt[8][33];
    __shared__ int total[33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long long NT = tstart[E];
    for (long long t = blockIdx.x; t < NT; t += gridDim.x) {
        const int e = tile_est(tstart, E, t);
        if (threadIdx.x < MCp)
            running[threadIdx.x] = bucket_off[(long long)e * MCp + threadIdx.x] + P[t * MCp + threadIdx.x];
        for (int k = threadIdx.x; k < 8 * 33; k += blockDim.x) wcnt[k / 33][k % 33] = 0;
        __syncthreads();
        const long long a = rbase[e] + (t - tstart[e]) * kPartTile;
        const long long bnd = a + kPartTile < rbase[e + 1] ? a + kPartTile : rbase[e + 1];
        for (long long base = a; base < bnd; base += blockDim.x) {
            const long long j = base + threadIdx.x;
            const int key = (j < bnd && alive[j]) ? m[j] : -1;
            const unsigned mask = __match_any_sync(kFull, key);
            const int rank = __popc(mask & ((1u << lane) - 1));
            const int leader = __ffs(mask) - 1;
            if (key >= 0 && lane == leader) wcnt[w][key] = __popc(mask);
            __syncthreads();
            if (threadIdx.x < MCp) {
                int acc = 0;
                for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) {
                    const int c = wcnt[ww][threadIdx.x];
                    wcnt[ww][threadIdx.x] = acc;
                    acc += c;
                }
                total[threadIdx.x] = acc;
            }
            __syncthreads();
            if (key >= 0) new_slot[j] = (int)(running[key] + wcnt[w][key] + rank);
            __syncthreads();
            if (threadIdx.x < MCp) {
                running[threadIdx.x] += total[threadIdx.x];
                for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) wcnt[ww][threadIdx.x] = 0;
            }
            __syncthreads();
        }
    }
}

#endif  // MCE_COMMON_UNIT

template <int D>
__global__ void k_compact(TermRecs R, const int* alive, const int* src, long long nR, const int* new_slot,
                          const long long* toff, const int* tcnt, ParentList Pn, int MC)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < nR; j += (long long)gridDim.x * blockDim.x) {
        if (!alive[j]) continue;
        const long long s = src[j];
        const long long o = new_slot[j];
        const int m = R.m[s];
        Pn.est[o] = R.est[s];
        Pn.m[o] = m;
        for (int k = 0; k < m * D; k++) Pn.A[o * MC * D + k] = R.A[s * MC * D + k];
        for (int k = 0; k < m; k++) Pn.p[o * MC + k] = R.p[s * MC + k];
        for (int k = 0; k < D; k++) Pn.b[o * D + k] = R.b[s * D + k];
        Pn.tab_off[o] = toff[j];
        Pn.tab_cnt[o] = tcnt[j];
    }
}

#if MCE_COMMON_UNIT
__global__ void k_rbase(const long long* pstart, const long long* kscan, int E, long long* rbase)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e <= E; e += gridDim.x * blockDim.x)
        rbase[e] = pstart[e] + kscan[pstart[e]];
}

#endif  // MCE_COMMON_UNIT

// ---------------------------------------------------------------------------
// Launchers

template <int D>
void Kernels<D>::first_count(const double* A0, const EstStep<D>* st, int E, int* cnt, const LaunchCfg& c)
{
    ++g_launches;
    k_first_count<D><<<(E + 127) / 128, 128, 0, c.stream>>>(A0, st, E, cnt);
}

template <int D>
void Kernels<D>::first_build(const double* A0, const double* p0, const double* b0, const EstStep<D>* st,
                             const double* roots, int E, const long long* pstart, ParentList P, int MC, cd* est_raw,
                             const LaunchCfg& c)
{
    // c_val, d_val and the H-orthogonal flags of the first terms ride in
    // spare parent-list arrays until the first tables are built.
    ++g_launches;
    k_first_build<D><<<(E + 63) / 64, 64, 0, c.stream>>>(A0, p0, b0, st, roots, E, pstart, P, MC,
                                                         reinterpret_cast<double*>(P.kscan),
                                                         reinterpret_cast<double*>(P.B_off),
                                                         reinterpret_cast<unsigned*>(P.nkids), est_raw);
}

template <int D>
void Kernels<D>::first_tables(ParentList P, long long nP, const double* cval, const double* dval, const unsigned* hof,
                              const double* gscale, Tables T, int MC, const LaunchCfg& c)
{
    const long long n = nP << (D - 1);
    ++g_launches;
    k_first_tables<D><<<grid_for(n, 256, c.num_sms), 256, 0, c.stream>>>(P, nP, cval, dval, hof, gscale, T, MC);
}

template <int D>
void Kernels<D>::tp(ParentList P, long long nP, const EstStep<D>* st, int with_tp, int MC, int* Bcap, int* nvert,
                    int* err, const LaunchCfg& c)
{
    if (nP == 0) return;
    ++g_launches;
    static const int mb = max_block_of((const void*)k_tp<D>);
    const TuneLaunch t = tune_begin(TK_TP, D, MC, nP, 128, mb, c.stream);
    k_tp<D><<<tuned_grid(nP, t.block, c.num_sms, 16), t.block, 0, c.stream>>>(P, nP, st, with_tp, MC, Bcap, nvert,
                                                                             err);
    tune_end(t, c.stream);
}

static inline size_t build_B_smem_per_warp(int MC, int D)
{
    (void)D;
    const int words = (1 << MC) > 32 ? (1 << MC) / 32 : 1;
    return (size_t)2 * words * 4;
}

template <int D>
void Kernels<D>::build_B(ParentList P, long long nP, const EstStep<D>* st, int with_tp, Tables Told, int* Bkeys,
                         long long Bcap_total, const double* bpert, int MC, const int* combo_off,
                         const unsigned char* combos, const long long* voff, long long nv, int* vsv, int* err,
                         const LaunchCfg& c)
{
    (void)Bcap_total;
    if (nP == 0) return;
    if (nv > 0) {
        ++g_launches;
        static const int mb = max_block_of((const void*)k_build_B_vertices<D>);
        const TuneLaunch t = tune_begin(TK_BUILD_B_VERTICES, D, MC, nv, 128, mb, c.stream);
        k_build_B_vertices<D><<<tuned_grid(nv, t.block, c.num_sms, 16), t.block, 0, c.stream>>>(
            P, nP, voff, nv, bpert, MC, combo_off, combos, vsv);
        tune_end(t, c.stream);
    }
    const bool global_bits = MC > kSmemBitmapRows && c.gbits;
    const size_t pw = build_B_smem_per_warp(MC, D);
    int warps = global_bits ? 4 : (int)(96 * 1024 / pw);
    if (warps > 8) warps = 8;
    if (warps < 1) warps = 1;
    const size_t sm = global_bits ? 0 : pw * warps;
    int grid = grid_for(nP, warps, c.num_sms, 8);
    if (global_bits && (long long)grid * warps > c.gbits_warps) grid = (int)(c.gbits_warps / warps);
    if (!global_bits) cudaFuncSetAttribute(k_build_B<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    ++g_launches;
    k_build_B<D><<<grid, warps * 32, sm, c.stream>>>(P, nP, st, with_tp, Told, Bkeys, bpert, MC, combo_off, combos,
                                                     voff, vsv, err, global_bits ? c.gbits : nullptr);
}

template <int D>
void Kernels<D>::mu(ParentList P, long long nP, const EstStep<D>* st, const long long* pstart, const double* roots,
                    Tables Told, int* Bkeys, TermRecs R, long long nR, const long long* kall_scan, long long nterms,
                    double* frow, int* fint, cd* contrib, int MC, int* err, const LaunchCfg& c)
{
    if (nP == 0) return;
    ++g_launches;
    {
        static const int mb = max_block_of((const void*)k_mu_rows<D>);
        const TuneLaunch t = tune_begin(TK_MU_ROWS, D, MC, nP, 128, mb, c.stream);
        k_mu_rows<D><<<tuned_grid(nP, t.block, c.num_sms, 16), t.block, 0, c.stream>>>(P, nP, st, Bkeys, frow, fint,
                                                                                      MC);
        tune_end(t, c.stream);
    }
    if (nterms == 0) return;
    // each thread stages one term's rows (MC x D, p, q) in shared memory
    const size_t rs = (size_t)(MC * D + 2 * MC) * sizeof(double);
    int threads = (int)(96 * 1024 / rs) / 32 * 32;
    if (threads > 128) threads = 128;
    if (threads < 32) threads = 32;
    const size_t sm = rs * threads;
    cudaFuncSetAttribute(k_mu_terms<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    ++g_launches;
    k_mu_terms<D><<<grid_for(nterms, threads, c.num_sms, 16), threads, sm, c.stream>>>(
        P, nP, st, pstart, roots, Told, R, nR, kall_scan, nterms, frow, fint, contrib, MC, err);
}

template <int D>
void Kernels<D>::moments(const cd* contrib, const long long* pstart, const long long* kall_scan, int E,
                         const int* order, const EstStep<D>* st, double* tot, cd* est_raw, double* gscale,
                         const LaunchCfg& c)
{
    constexpr int NS = (2 * (1 + D + D * D) + 31) / 32;
    g_launches += 2;
    k_moments_chain<D><<<(unsigned)E * NS, 32, 0, c.stream>>>(contrib, pstart, kall_scan, E, order, st, tot);
    k_moments_final<D><<<(E + 127) / 128, 128, 0, c.stream>>>(tot, E, st, est_raw, gscale);
}

template <int D>
void Kernels<D>::ftr_cells(TermRecs R, long long nR, long long hmask, int* slot_of, int* bcount, const LaunchCfg& c)
{
    if (nR == 0) return;
    ++g_launches;
    k_ftr_count_cells<D><<<grid_for(nR, 256, c.num_sms), 256, 0, c.stream>>>(R, nR, hmask, slot_of, bcount);
}

template <int D>
void Kernels<D>::ftr_scatter(TermRecs R, long long nR, const int* slot_of, const long long* boff, int* bfill,
                             void* ent, const LaunchCfg& c)
{
    if (nR == 0) return;
    ++g_launches;
    k_ftr_scatter<D><<<grid_for(nR, 256, c.num_sms), 256, 0, c.stream>>>(R, nR, slot_of, boff, bfill,
                                                                         static_cast<CellEntry<D>*>(ent));
}

template <int D>
size_t Kernels<D>::cell_entry_bytes()
{
    return sizeof(CellEntry<D>);
}

template <int D>
void Kernels<D>::ftr_sort(const void* in, long long n, const int* slot_of, const long long* boff, void* out,
                          const LaunchCfg& c)
{
    if (n == 0) return;
    ++g_launches;
    k_ftr_sort_buckets<D><<<grid_for(n, 256, c.num_sms), 256, 0, c.stream>>>(
        static_cast<const CellEntry<D>*>(in), n, slot_of, boff, static_cast<CellEntry<D>*>(out));
}

template <int D>
void Kernels<D>::ftr_resolve(TermRecs R, long long nR, const void* ent, const long long* boff, long long hmask,
                             int MC, int* status, int* owner, const int* wl_in, const int* n_in, long long n_bound,
                             int* wl_out, int* n_out, int* resume, const LaunchCfg& c)
{
    const long long n = wl_in ? n_bound : nR;
    if (n == 0) return;
    ++g_launches;
    static const int mb = max_block_of((const void*)k_ftr_resolve_scan<D>);
    const TuneLaunch t = tune_begin(TK_FTR_RESOLVE, D, MC, n, 128, mb, c.stream);
    k_ftr_resolve_scan<D><<<tuned_grid(n, t.block, c.num_sms, 16), t.block, 0, c.stream>>>(
        R, nR, static_cast<const CellEntry<D>*>(ent), boff, hmask, MC, status, owner, wl_in, n_in, wl_out, n_out,
        resume);
    tune_end(t, c.stream);
}

template <int D>
int Kernels<D>::ftr_resolve_all(TermRecs R, long long nR, const void* ent, const long long* boff, long long hmask,
                                int MC, int* status, int* owner, int* wl0, int* wl1, int* cnt, int* resume,
                                unsigned* bar, int first_round, int max_rounds, int* err, const LaunchCfg& c)
{
    if (nR == 0) return MCE_OK;
    // blocks that fit on the GPU at once (half of them: other streams' kernels
    // may hold part of the SMs while this one waits at its barriers; one block
    // per SM measured slower, 28.7 against 20.8 ms of term reduction per pass)
    static int bps = -1;
    if (bps < 0) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_ftr_resolve_all<D>, 128, 0) != cudaSuccess) {
            cudaGetLastError();
            b = 0;
        }
        bps = b;
    }
    if (bps <= 0) return MCE_ERR_CUDA;
    long long grid = (long long)std::max(1, bps / 2) * c.num_sms;
    const long long need = (nR + 127) / 128;
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    const CellEntry<D>* e = static_cast<const CellEntry<D>*>(ent);
    void* args[] = {&R,    &nR,     &e,   &boff,   &hmask, &MC,          &status,     &owner,
                    &wl0,  &wl1,    &cnt, &resume, &bar,   &first_round, &max_rounds, &err};
    const cudaError_t st = cudaLaunchCooperativeKernel((const void*)k_ftr_resolve_all<D>, dim3((unsigned)grid),
                                                       dim3(128), args, 0, c.stream);
    if (st != cudaSuccess) {
        cudaGetLastError();
        return MCE_ERR_CUDA;
    }
    ++g_launches;
    return MCE_OK;
}

template <int D>
struct FtrGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    FtrLoopArgs<D>* dargs = nullptr;
    int* hround = nullptr;  // page-locked copy of the round counter after a launch
    FtrLoopArgs<D> hargs;
    bool pending = false;
    ~FtrGraph()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (dargs) cudaFree(dargs);
        if (hround) cudaFreeHost(hround);
    }
};

template <int D>
int Kernels<D>::ftr_graph_create(void** out, const LaunchCfg& c)
{
    *out = nullptr;
    std::unique_ptr<FtrGraph<D>> g(new FtrGraph<D>());
    auto fail = [&]() {
        cudaGetLastError();
        return MCE_ERR_CUDA;
    };
    if (cudaMalloc(&g->dargs, sizeof(FtrLoopArgs<D>)) != cudaSuccess) return fail();
    if (cudaMallocHost(&g->hround, sizeof(int)) != cudaSuccess) {
        g->hround = nullptr;
        return fail();
    }
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_ftr_graph_round<D>, 128, 0) != cudaSuccess || bps < 1)
        return fail();
    if (cudaGraphCreate(&g->graph, 0) != cudaSuccess) return fail();
    cudaGraphConditionalHandle h;
    if (cudaGraphConditionalHandleCreate(&h, g->graph, 1, cudaGraphCondAssignDefault) != cudaSuccess) return fail();
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cond;
    if (cudaGraphAddNode(&cond, g->graph, nullptr, nullptr, 0, &cp) != cudaSuccess) return fail();
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    FtrLoopArgs<D>* a = g->dargs;
    void* rargs[] = {&a};
    cudaKernelNodeParams kr;
    memset(&kr, 0, sizeof(kr));
    kr.func = (void*)k_ftr_graph_round<D>;
    kr.gridDim = dim3((unsigned)(bps * c.num_sms));
    kr.blockDim = dim3(128);
    kr.kernelParams = rargs;
    cudaGraphNode_t nround, nnext;
    if (cudaGraphAddKernelNode(&nround, body, nullptr, 0, &kr) != cudaSuccess) return fail();
    void* nargs[] = {&a, &h};
    cudaKernelNodeParams kn;
    memset(&kn, 0, sizeof(kn));
    kn.func = (void*)k_ftr_graph_next<D>;
    kn.gridDim = dim3(1);
    kn.blockDim = dim3(32);
    kn.kernelParams = nargs;
    if (cudaGraphAddKernelNode(&nnext, body, &nround, 1, &kn) != cudaSuccess) return fail();
    if (cudaGraphInstantiate(&g->exec, g->graph, 0) != cudaSuccess) {
        g->exec = nullptr;
        return fail();
    }
    *out = g.release();
    return MCE_OK;
}

template <int D>
int Kernels<D>::ftr_graph_launch(void* gv, TermRecs R, long long nR, const void* ent, const long long* boff,
                                 long long hmask, int MC, int* status, int* owner, int* wl0, int* wl1, int* cnt,
                                 int* resume, int max_rounds, int* err, const LaunchCfg& c)
{
    FtrGraph<D>* g = static_cast<FtrGraph<D>*>(gv);
    FtrLoopArgs<D>& h = g->hargs;
    h.R = R;
    h.nR = nR;
    h.ent = static_cast<const CellEntry<D>*>(ent);
    h.boff = boff;
    h.hmask = hmask;
    h.MC = MC;
    h.status = status;
    h.owner = owner;
    h.wl0 = wl0;
    h.wl1 = wl1;
    h.cnt = cnt;
    h.resume = resume;
    h.err = err;
    h.round = 1;
    h.max_rounds = max_rounds;
    // (a pageable source: staged before the call returns)
    if (cudaMemcpyAsync(g->dargs, &h, sizeof(h), cudaMemcpyHostToDevice, c.stream) != cudaSuccess ||
        cudaGraphLaunch(g->exec, c.stream) != cudaSuccess ||
        cudaMemcpyAsync(g->hround, &g->dargs->round, sizeof(int), cudaMemcpyDeviceToHost, c.stream) != cudaSuccess) {
        cudaGetLastError();
        return MCE_ERR_CUDA;
    }
    g->pending = true;
    return MCE_OK;
}

template <int D>
void Kernels<D>::ftr_graph_collect(void* gv)
{
    FtrGraph<D>* g = static_cast<FtrGraph<D>*>(gv);
    if (!g || !g->pending) return;
    g->pending = false;
    g_launches += 2LL * std::max(0, *g->hround - 1);  // a round and its loop step per iteration
}

template <int D>
void Kernels<D>::ftr_graph_destroy(void* gv)
{
    delete static_cast<FtrGraph<D>*>(gv);
}

static inline size_t gtable_smem_per_warp(int MC, int capR)
{
    const int words = (1 << MC) > 32 ? (1 << MC) / 32 : 1;
    return (size_t)(3 * words + 32 + capR) * 4;
}

template <int D>
void Kernels<D>::gtable(TermRecs R, const int* roots_list, long long nroots, const int* gcnt, const long long* goff,
                        const int* members, ParentList P, Tables Told, const int* Bkeys, const double* gscale,
                        const long long* toff, Tables Tnew, int* tcnt, int* alive, int* src, cd* scratch,
                        long long scratch_per_warp, const GFlat& f, int MC, int* err, const LaunchCfg& c,
                        long long max_warps)
{
    if (nroots == 0) return;
    const bool global_bits = MC > kSmemBitmapRows && c.gbits;
    GCtx ctx{R, P, Told, Bkeys, MC, global_bits ? c.gbits : nullptr, cells_cap_of(c, MC, D)};
    const size_t pw = gtable_smem_per_warp(MC, ctx.capR);
    int warps = global_bits ? 4 : (int)(96 * 1024 / pw);
    if (warps > 4) warps = 4;
    if (warps < 1) warps = 1;
    const size_t sm = global_bits ? 0 : pw * warps;
    if (!global_bits) cudaFuncSetAttribute(k_gtable<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    int grid = grid_for(nroots, warps, c.num_sms, 16);
    if (global_bits && (long long)grid * warps > c.gbits_warps) grid = (int)(c.gbits_warps / warps);
    // a scratch region sized for max_warps warps (the caller guarantees
    // max_warps >= 4 >= warps): the warps stride over the roots, so fewer of
    // them give the same tables
    if (max_warps > 0 && (long long)grid * warps > max_warps) grid = (int)(max_warps / warps);
    ++g_launches;
    k_gtable<D><<<grid, warps * 32, sm, c.stream>>>(ctx, roots_list, nroots, gcnt, goff, members, gscale, toff, Tnew,
                                                    tcnt, alive, src, scratch, scratch_per_warp, f.rflag, f.gnr,
                                                    f.pr_root, f.pr_mb, f.pr_mcnt, f.pr_cells, f.pr_items, err);
}

template <int D>
void Kernels<D>::gtable_promoted(TermRecs R, const int* roots_list, long long nroots, long long nmem, long long nitems,
                                 long long ncells, const int* members, ParentList P, Tables Told, const int* Bkeys,
                                 const double* gscale, const long long* toff, Tables Tnew, const GFlat& f, int MC,
                                 const LaunchCfg& c)
{
    if (nitems == 0) return;
    GCtx ctx{R, P, Told, Bkeys, MC, nullptr, cells_cap_of(c, MC, D)};
    g_launches += 3;
    k_gtable_prom_prep<D><<<grid_for(nmem, 128, c.num_sms, 8), 128, 0, c.stream>>>(ctx, nroots, nmem, members, f);
    static const int mb = max_block_of((const void*)k_gtable_prom_eval<D>);
    const TuneLaunch t = tune_begin(TK_GTABLE_PROM_EVAL, D, MC, nitems, 128, mb, c.stream);
    k_gtable_prom_eval<D><<<tuned_grid(nitems, t.block, c.num_sms, 16), t.block, 0, c.stream>>>(
        ctx, roots_list, nroots, nitems, members, gscale, toff, Tnew, f);
    tune_end(t, c.stream);
    k_gtable_prom_combine<D><<<grid_for(ncells, 128, c.num_sms, 8), 128, 0, c.stream>>>(
        ctx, roots_list, nroots, ncells, members, toff, Tnew, f);
}

template <int D>
void Kernels<D>::gtable_prep(TermRecs R, const int* roots_list, long long nroots, const int* gcnt,
                             const long long* goff, const int* members, ParentList P, Tables Told, const int* Bkeys,
                             const long long* toff, Tables Tnew, const GFlat& f, int* gitems, int* gcells, int MC,
                             int* need, int* over, const LaunchCfg& c)
{
    if (nroots == 0) return;
    const bool global_bits = MC > kSmemBitmapRows && c.gbits;
    GCtx ctx{R, P, Told, Bkeys, MC, global_bits ? c.gbits : nullptr, cells_cap_of(c, MC, D)};
    const int words = (1 << MC) > 32 ? (1 << MC) / 32 : 1;
    const size_t pw = (size_t)(2 * words + 32 + ctx.capR) * 4;
    int warps = global_bits ? 4 : (int)(96 * 1024 / pw);
    if (warps > 4) warps = 4;
    if (warps < 1) warps = 1;
    const size_t sm = global_bits ? 0 : pw * warps;
    if (!global_bits) cudaFuncSetAttribute(k_gtable_prep<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    int grid = grid_for(nroots, warps, c.num_sms, 16);
    if (global_bits && (long long)grid * warps > c.gbits_warps) grid = (int)(c.gbits_warps / warps);
    ++g_launches;
    k_gtable_prep<D><<<grid, warps * 32, sm, c.stream>>>(
        ctx, roots_list, nroots, gcnt, goff, members, toff, Tnew, f.gnr, gitems, gcells, f.minfo, f.rps2, f.mps2,
        f.rflag, f.mflag, need, over);
}

template <int D>
void Kernels<D>::gtable_combine(TermRecs R, const int* roots_list, long long nroots, const long long* coff,
                                long long ncells, const int* gcnt, const long long* goff, const int* members,
                                ParentList P, Tables Told, const int* Bkeys, const long long* toff, Tables Tnew,
                                int* tcnt, int* alive, int* src, const GFlat& f, int MC, const LaunchCfg& c)
{
    if (ncells == 0) return;
    GCtx ctx{R, P, Told, Bkeys, MC, nullptr, cells_cap_of(c, MC, D)};
    ++g_launches;
    static const int mb = max_block_of((const void*)k_gtable_combine<D>);
    const TuneLaunch t = tune_begin(TK_GTABLE_COMBINE, D, MC, ncells, 128, mb, c.stream);
    k_gtable_combine<D><<<tuned_grid(ncells, t.block, c.num_sms, 16), t.block, 0, c.stream>>>(
        ctx, roots_list, nroots, coff, ncells, gcnt, goff, members, toff, Tnew, tcnt, alive, src, f.rflag, f.ioff,
        f.gnr, f.minfo, f.mflag, f.gv);
    tune_end(t, c.stream);
}

template <int D>
void Kernels<D>::gtable_eval(TermRecs R, const int* roots_list, long long nroots, long long nitems,
                             const long long* goff, const int* members, ParentList P, Tables Told, const int* Bkeys,
                             const double* gscale, const long long* toff, Tables Tnew, const GFlat& f, int MC,
                             const LaunchCfg& c)
{
    if (nitems == 0) return;
    GCtx ctx{R, P, Told, Bkeys, MC, nullptr, cells_cap_of(c, MC, D)};
    ++g_launches;
    static const int mb = max_block_of((const void*)k_gtable_eval<D>);
    const TuneLaunch t = tune_begin(TK_GTABLE_EVAL, D, MC, nitems, 128, mb, c.stream);
    k_gtable_eval<D><<<tuned_grid(nitems, t.block, c.num_sms, 16), t.block, 0, c.stream>>>(
        ctx, roots_list, nroots, f.ioff, nitems, f.gnr, goff, members, f.minfo, f.rps2, f.mps2, gscale, toff, Tnew,
        f.gv, f.rflag, f.mflag);
    tune_end(t, c.stream);
}

template <int D>
void Kernels<D>::compact(TermRecs R, const int* alive, const int* src, long long nR, const int* new_slot,
                         const long long* toff, const int* tcnt, ParentList Pn, int MC, const LaunchCfg& c)
{
    if (nR == 0) return;
    ++g_launches;
    static const int mb = max_block_of((const void*)k_compact<D>);
    const TuneLaunch t = tune_begin(TK_COMPACT, D, MC, nR, 256, mb, c.stream);
    k_compact<D><<<tuned_grid(nR, t.block, c.num_sms, 32), t.block, 0, c.stream>>>(R, alive, src, nR, new_slot, toff,
                                                                                 tcnt, Pn, MC);
    tune_end(t, c.stream);
}

// ---------------------------------------------------------------------------
// Marginal 1-D conditional pdf over the current terms
// (PointWiseNDimCauchyCPDF::evaluate_1D_marginal_cpdf, cpdf_ndim.hpp:1233-1352).
// k_cpdf1d_terms: per term, p_cc = sum_j p_j |A_j,marg|, the two sign
// encodings (a row with |A_j,marg| <= 1e-15 takes the sign of A_j . bar_nu),
// the two g numerators and the cache entry (a, b, w, s).  Each term's record
// is 8 doubles: g_lhs, g_rhs, p_cc, s, a, b.
template <int D>
__global__ void k_cpdf1d_terms(ParentList P, long long a, long long n, int marg, const double* bar_nu, Tables T,
                               int MC, double* tt)
{
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
        const long long i = a + j;
        const int m = P.m[i];
        const double* A = P.A + i * MC * D;
        const double* p = P.p + i * MC;
        double p_cc = 0;
        int lhs = 0, rhs = 0;
        for (int l = 0; l < m; l++) {
            const double acj = A[l * D + marg];
            const double fa = fabs(acj);
            p_cc += p[l] * fa;
            bool left;
            if (fa > 1e-15) {
                left = acj > 0;
            } else {
                double ip = 0.0;
                for (int k = 0; k < D; k++) ip += A[l * D + k] * bar_nu[k];
                left = ip > 0;
            }
            if (left) lhs |= 1 << l;
            else rhs |= 1 << l;
        }
        const int* keys = T.keys + P.tab_off[i];
        const cd* vals = T.vals + P.tab_off[i];
        const int cnt = P.tab_cnt[i];
        const cd gl = lookup_num(keys, vals, cnt, lhs, m);
        const cd gr = lookup_num(keys, vals, cnt, rhs, m);
        const double s = P.b[i * D + marg];
        double* o = tt + j * 8;
        o[0] = gl.re;
        o[1] = gl.im;
        o[2] = gr.re;
        o[3] = gr.im;
        o[4] = p_cc;
        o[5] = s;
        o[6] = gr.im / kPi;
        o[7] = (gr.re * p_cc - gr.im * s) / kPi;
    }
}

template <int D>
void Kernels<D>::cpdf1d_terms(ParentList P, long long a, long long n, int marg, const double* bar_nu, Tables T, int MC,
                              double* tt, const LaunchCfg& c)
{
    if (n == 0) return;
    ++g_launches;
    k_cpdf1d_terms<D><<<grid_for(n, 128, c.num_sms, 16), 128, 0, c.stream>>>(P, a, n, marg, bar_nu, T, MC, tt);
}

// Extended-mode helpers (cauchy_estimator.hpp:1312-1394) over the terms of
// one estimator: b +/- v (shift_cf_by_bias, finalize_extended_moments) and
// time_prop (cauchy_term.hpp:435-456: A <- A Phi^T, b <- Phi b, b += B u).
template <int D>
__global__ void k_shift_b(ParentList P, long long a, long long n, const double* v, int sub)
{
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
        double* b = P.b + (a + j) * D;
        for (int k = 0; k < D; k++) b[k] = sub ? b[k] - v[k] : b[k] + v[k];
    }
}

template <int D>
__global__ void k_det_tp(ParentList P, long long a, long long n, const double* Phi, const double* Bu, int MC)
{
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
        const long long i = a + j;
        const int m = P.m[i];
        double* A = P.A + i * MC * D;
        for (int r = 0; r < m; r++) {
            double w[D];
            for (int k = 0; k < D; k++) w[k] = A[r * D + k];
            for (int c = 0; c < D; c++) {
                double s = 0.0;
                for (int k = 0; k < D; k++) s += w[k] * Phi[c * D + k];
                A[r * D + c] = s;
            }
        }
        double* b = P.b + i * D;
        double wb[D];
        for (int k = 0; k < D; k++) wb[k] = b[k];
        for (int r = 0; r < D; r++) {
            double s = 0.0;
            for (int k = 0; k < D; k++) s += Phi[r * D + k] * wb[k];
            b[r] = s;
        }
        if (Bu)
            for (int r = 0; r < D; r++) b[r] += 1.0 * Bu[r];
    }
}

template <int D>
void Kernels<D>::shift_b(ParentList P, long long a, long long n, const double* v, int sub, const LaunchCfg& c)
{
    if (n == 0) return;
    ++g_launches;
    k_shift_b<D><<<grid_for(n, 128, c.num_sms, 16), 128, 0, c.stream>>>(P, a, n, v, sub);
}

template <int D>
void Kernels<D>::det_tp(ParentList P, long long a, long long n, const double* Phi, const double* Bu, int MC,
                        const LaunchCfg& c)
{
    if (n == 0) return;
    ++g_launches;
    k_det_tp<D><<<grid_for(n, 128, c.num_sms, 16), 128, 0, c.stream>>>(P, a, n, Phi, Bu, MC);
}

// ---------------------------------------------------------------------------
// Marginal 2-D conditional pdf over the current terms
// (PointWiseNDimCauchyCPDF::evaluate_2D_marginal_cpdf, cpdf_ndim.hpp:1356-1455).
// k_cpdf2d_terms, a thread per term: the two marginal columns of A
// normalised, zero rows marked and coaligned rows merged
// (marg2d_remove_zeros_and_coalign, :42-140); the 2m cell-wall angles sorted
// (:143-174); per half-plane cell its sign vector at the mid angle (:177-202),
// its parent-table key (zero rows take the sign of A_j . bar_nu), g value and
// the real parts of gamma1, gamma2 (:1551-1600).  This is the reference's
// per-term cache (Cached2DCPDFTerm); its exact first evaluation uses the same
// sines, cosines and gammas, so every grid point is summed from the cache.
// Record per term (cpdf2d_stride doubles): m, b1, b2, sin[MC+1], cos[MC+1],
// g1r[MC], g2r[MC], g[MC] (re, im).

template <int D>
__global__ void k_cpdf2d_terms(ParentList P, long long a, long long n, int i1, int i2, const double* bar_nu, Tables T,
                               int MC, double* tt)
{
    const int RT = cpdf2d_stride(MC);
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const long long i = a + q;
        const int m = P.m[i];
        const double* At = P.A + i * MC * D;
        double A[2 * kMaxRows], p[kMaxRows], A2[2 * kMaxRows], p2[kMaxRows];
        int cmap[kMaxRows], csmap[kMaxRows], fidx[kMaxRows];
        unsigned F = 0;
        for (int r = 0; r < m; r++) {
            A[2 * r] = At[r * D + i1];
            A[2 * r + 1] = At[r * D + i2];
            p[r] = P.p[i * MC + r];
            F |= 1u << r;
        }
        for (int r = 0; r < m; r++) {
            const double f0 = fabs(A[2 * r]), f1 = fabs(A[2 * r + 1]);
            if (f0 < kMuEps && f1 < kMuEps) {
                cmap[r] = csmap[r] = fidx[r] = 32;
                F &= ~(1u << r);
                continue;
            }
            const double s = f0 + f1;
            A[2 * r] /= s;
            A[2 * r + 1] /= s;
            p[r] *= s;
        }
        int mn = 0;
        for (int r = 0; r < m; r++) {
            if (!((F >> r) & 1u)) continue;
            cmap[r] = mn;
            csmap[r] = 1;
            fidx[r] = r;
            p2[mn] = p[r];
            for (int j = r + 1; j < m; j++) {
                if (!((F >> j) & 1u)) continue;
                if (fabs(A[2 * r] - A[2 * j]) < kCoalignEps && fabs(A[2 * r + 1] - A[2 * j + 1]) < kCoalignEps) {
                    cmap[j] = mn;
                    csmap[j] = 1;
                    F &= ~(1u << j);
                    fidx[j] = r;
                    p2[mn] += p[j];
                    continue;
                }
                if (fabs(A[2 * r] + A[2 * j]) < kCoalignEps && fabs(A[2 * r + 1] + A[2 * j + 1]) < kCoalignEps) {
                    cmap[j] = mn;
                    csmap[j] = -1;
                    F &= ~(1u << j);
                    fidx[j] = r;
                    p2[mn] += p[j];
                }
            }
            mn++;
        }
        {
            int u = 0;
            for (int r = 0; r < m; r++)
                if (mn == m || fidx[r] == r) {
                    A2[2 * u] = A[2 * r];
                    A2[2 * u + 1] = A[2 * r + 1];
                    u++;
                }
        }
        double th[2 * kMaxRows];
        for (int r = 0; r < mn; r++) {
            const double a0 = A2[2 * r], a1 = A2[2 * r + 1];
            double pt0, pt1;
            if (fabs(a0) < fabs(a1)) {
                pt0 = 1;
                pt1 = -a0 / a1;
            } else {
                pt0 = -a1 / a0;
                pt1 = 1;
            }
            double t1 = atan2(pt1, pt0);
            if (t1 < 0) t1 += kPi;
            th[2 * r] = t1;
            th[2 * r + 1] = t1 + kPi;
        }
        for (int x = 1; x < 2 * mn; x++) {  // ascending (the reference's qsort of distinct angles)
            const double v = th[x];
            int y = x - 1;
            while (y >= 0 && th[y] > v) {
                th[y + 1] = th[y];
                y--;
            }
            th[y + 1] = v;
        }
        double* o = tt + q * RT;
        double* os = o + 3;
        double* oc = os + (MC + 1);
        double* o1 = oc + (MC + 1);
        double* o2 = o1 + MC;
        double* og = o2 + MC;
        o[0] = mn;
        o[1] = P.b[i * D + i1];
        o[2] = P.b[i * D + i2];
        const int* keys = T.keys + P.tab_off[i];
        const cd* vals = T.vals + P.tab_off[i];
        const int cnt = P.tab_cnt[i];
        for (int c = 0; c < mn; c++) {
            const double tm = (th[c + 1] + th[c]) / 2.0;
            const double ct = cos(tm), st = sin(tm);
            unsigned neg = 0;  // sv[j] = -1
            for (int j = 0; j < mn; j++)
                if (!(A2[2 * j] * ct + A2[2 * j + 1] * st > 0)) neg |= 1u << j;
            int enc = 0;
            if (mn == m) {
                enc = (int)neg;
            } else {
                for (int j = 0; j < m; j++) {
                    if (cmap[j] == 32) {
                        double ip = 0.0;
                        for (int l = 0; l < D; l++) ip += At[j * D + l] * bar_nu[l];
                        if (ip < 0) enc |= 1 << j;
                    } else {
                        const bool sneg = (neg >> cmap[j]) & 1u;
                        if (sneg != (csmap[j] < 0)) enc |= 1 << j;
                    }
                }
            }
            const cd g = lookup_num(keys, vals, cnt, enc, m);
            double g1r = 0, g2r = 0;
            for (int j = 0; j < mn; j++) {
                const double sv = ((neg >> j) & 1u) ? -1.0 : 1.0;
                g1r -= (A2[2 * j] * p2[j]) * sv;
                g2r -= (A2[2 * j + 1] * p2[j]) * sv;
            }
            os[c] = sin(th[c]);
            oc[c] = cos(th[c]);
            o1[c] = g1r;
            o2[c] = g2r;
            og[2 * c] = g.re;
            og[2 * c + 1] = g.im;
        }
        os[mn] = mn > 0 ? sin(th[mn]) : 0.0;
        oc[mn] = mn > 0 ? cos(th[mn]) : 0.0;
    }
}

template <int D>
void Kernels<D>::cpdf2d_terms(ParentList P, long long a, long long n, int i1, int i2, const double* bar_nu, Tables T,
                              int MC, double* tt, const LaunchCfg& c)
{
    if (n == 0) return;
    ++g_launches;
    k_cpdf2d_terms<D><<<grid_for(n, 128, c.num_sms, 16), 128, 0, c.stream>>>(P, a, n, i1, i2, bar_nu, T, MC, tt);
}

// ---------------------------------------------------------------------------
// Relative-then-transformed 2-D system (cauchy_prediction.hpp), a thread per
// (primary term, secondary term) pair:
//   A_rel = [-A_prim; A_sec], p_rel = [p_prim; p_sec], b_rel = b_sec - b_prim
//   (:573-584); A_2d = A_rel Trel^T, b_2d = Trel b_rel (:587-588);
//   marg2d_remove_zeros_and_coalign (cpdf_ndim.hpp:42-138);
//   eval_rel_sys_moments_for_term (:207-285) on the normalised rows;
//   cache_rel_marg2d_term_for_cpdf (:306-443): the 2m sorted cell-wall angles,
//   per cell the sign vector at its mid angle (flipped for the second half of
//   a full solve), the product of the two parent-table values and the real
//   parts of gamma1, gamma2;
//   approx_out_rel_marg2d_term_for_cpdf (:445-470).
// Zero rows (both projected components below MU_EPS) take the sign of the
// full-dimensional row against bar_nu_full.
template <int D>
__global__ void __launch_bounds__(128) k_rel2d_pairs(Rel2DArgs a)
{
    const int RT = rel2d_stride(a.CC);
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < a.npairs;
         x += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = a.nblk;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (a.blk[mid].off <= x) lo = mid;
            else hi = mid;
        }
        const Rel2DBlock B = a.blk[lo];
        const long long loc = x - B.off;
        const long long tp = loc / B.sc;
        const long long ts = loc - tp * B.sc;
        const long long ip = a.idxP[B.po + tp], is = a.idxS[B.so + ts];
        const int mp = a.P.m[ip], ms = a.S.m[is], mps = mp + ms;
        if (mp < 1 || ms < 1 || mps > kMaxRows || mps * (1 + a.full) > a.CC) {
            // cannot happen for terms within their estimators' max shapes
            // (the host checks those); an empty, dropped term keeps it in bounds
            a.tt[x * RT] = 0;
            a.keep[x] = 0;
            if (a.moments)
                for (int k = 0; k < 14; k++) a.mrows[x * 14 + k] = 0;
            continue;
        }
        const double* Ap = a.P.A + ip * a.MCp * D;
        const double* As = a.S.A + is * a.MCs * D;
        double b2[2];
        {
            double br[D];
            for (int i = 0; i < D; i++) br[i] = a.S.b[is * D + i] - a.P.b[ip * D + i];
            for (int r = 0; r < 2; r++) {
                double s = 0.0;
                for (int j = 0; j < D; j++) s += a.Trel[r * D + j] * br[j];
                b2[r] = s;
            }
        }
        double A2[2 * kMaxRows], pr[kMaxRows], Ac[2 * kMaxRows], pc[kMaxRows];
        signed char cmap[kMaxRows], csmap[kMaxRows], fidx[kMaxRows];
        for (int i = 0; i < mps; i++) {
            const double* row = i < mp ? Ap + i * D : As + (i - mp) * D;
            const double sg = i < mp ? -1.0 : 1.0;
            for (int j = 0; j < 2; j++) {
                double s = 0.0;
                for (int k = 0; k < D; k++) s += (row[k] * sg) * a.Trel[j * D + k];
                A2[2 * i + j] = s;
            }
            pr[i] = i < mp ? a.P.p[ip * a.MCp + i] : a.S.p[is * a.MCs + (i - mp)];
        }
        // zero rows: normalisation skipped, sign from the full row
        unsigned zmask = 0, zneg = 0, zpos = 0, F = 0;
        for (int i = 0; i < mps; i++) {
            const double f0 = fabs(A2[2 * i]), f1 = fabs(A2[2 * i + 1]);
            if (f0 < kMuEps && f1 < kMuEps) {
                cmap[i] = csmap[i] = fidx[i] = 32;
                zmask |= 1u << i;
                const double* row = i < mp ? Ap + i * D : As + (i - mp) * D;
                const double sg = i < mp ? -1.0 : 1.0;
                double v = 0.0;
                for (int l = 0; l < D; l++) v += (row[l] * sg) * a.nu_full[l];
                if (v < 0) zneg |= 1u << i;
                if (v > 0) zpos |= 1u << i;
                continue;
            }
            F |= 1u << i;
            const double s = f0 + f1;
            A2[2 * i] /= s;
            A2[2 * i + 1] /= s;
            pr[i] *= s;
        }
        int mn = 0;
        for (int i = 0; i < mps; i++) {
            if (!((F >> i) & 1u)) continue;
            cmap[i] = (signed char)mn;
            csmap[i] = 1;
            fidx[i] = (signed char)i;
            pc[mn] = pr[i];
            for (int j = i + 1; j < mps; j++) {
                if (!((F >> j) & 1u)) continue;
                if (fabs(A2[2 * i] - A2[2 * j]) < kCoalignEps && fabs(A2[2 * i + 1] - A2[2 * j + 1]) < kCoalignEps) {
                    cmap[j] = (signed char)mn;
                    csmap[j] = 1;
                    F &= ~(1u << j);
                    fidx[j] = (signed char)i;
                    pc[mn] += pr[j];
                    continue;
                }
                if (fabs(A2[2 * i] + A2[2 * j]) < kCoalignEps && fabs(A2[2 * i + 1] + A2[2 * j + 1]) < kCoalignEps) {
                    cmap[j] = (signed char)mn;
                    csmap[j] = -1;
                    F &= ~(1u << j);
                    fidx[j] = (signed char)i;
                    pc[mn] += pr[j];
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
        const int* kp = a.TP.keys + a.P.tab_off[ip];
        const cd* vp = a.TP.vals + a.P.tab_off[ip];
        const int np_ = a.P.tab_cnt[ip];
        const int* ks = a.TS.keys + a.S.tab_off[is];
        const cd* vs = a.TS.vals + a.S.tab_off[is];
        const int ns_ = a.S.tab_cnt[is];
        const int maskp = (1 << mp) - 1;
        if (a.moments) {
            double nu[2];
            for (int r = 0; r < 2; r++) {
                double s = 0.0;
                for (int j = 0; j < D; j++) s += a.Trel[r * D + j] * a.nu_full[j];
                nu[r] = s;
            }
            double ty0 = 0, ty1 = 0;
            int enc = 0;
            for (int i = 0; i < mps; i++) {
                double v;
                if ((zmask >> i) & 1u) v = ((zneg >> i) & 1u) ? -1.0 : (((zpos >> i) & 1u) ? 1.0 : 0.0);  // its sign
                else v = A2[2 * i] * nu[0] + A2[2 * i + 1] * nu[1];
                const double sgn = (double)((v > 0) - (v < 0));
                const double sc = pr[i] * sgn;
                ty0 += sc * A2[2 * i];
                ty1 += sc * A2[2 * i + 1];
                if (v < 0) enc |= 1 << i;
            }
            const cd g = cmul(lookup_num(kp, vp, np_, enc & maskp, mp), lookup_num(ks, vs, ns_, enc >> mp, ms));
            const cd y[2] = {mkcd(-ty0, b2[0]), mkcd(-ty1, b2[1])};
            double* mr = a.mrows + x * 14;
            mr[0] = g.re;
            mr[1] = g.im;
            for (int j = 0; j < 2; j++) {
                const cd gy = cmul(g, y[j]);
                mr[2 + 2 * j] = gy.re;
                mr[3 + 2 * j] = gy.im;
                for (int k = 0; k < 2; k++) {
                    const cd t = cmul(gy, y[k]);
                    mr[6 + 2 * (2 * j + k)] = -t.re;
                    mr[7 + 2 * (2 * j + k)] = -t.im;
                }
            }
        }
        double th[2 * kMaxRows + 1];
        for (int r = 0; r < mn; r++) {
            const double a0 = Ac[2 * r], a1 = Ac[2 * r + 1];
            double pt0, pt1;
            if (fabs(a0) < fabs(a1)) {
                pt0 = 1;
                pt1 = -a0 / a1;
            } else {
                pt0 = -a1 / a0;
                pt1 = 1;
            }
            double t1 = atan2(pt1, pt0);
            if (t1 < 0) t1 += kPi;
            th[2 * r] = t1;
            th[2 * r + 1] = t1 + kPi;
        }
        for (int u = 1; u < 2 * mn; u++) {  // ascending (the reference's qsort of distinct angles)
            const double v = th[u];
            int w = u - 1;
            while (w >= 0 && th[w] > v) {
                th[w + 1] = th[w];
                w--;
            }
            th[w + 1] = v;
        }
        if (a.full && mn > 0) th[2 * mn] = th[0] + 2 * kPi;
        const int cells = mn * (1 + a.full);
        double* o = a.tt + x * RT;
        double* os = o + 3;
        double* oc = os + (a.CC + 1);
        double* o1 = oc + (a.CC + 1);
        double* o2 = o1 + a.CC;
        double* og = o2 + a.CC;
        o[0] = mn;
        o[1] = b2[0];
        o[2] = b2[1];
        const unsigned allm = mn >= 32 ? 0xffffffffu : ((1u << mn) - 1u);
        for (int c = 0; c < cells; c++) {
            const int h = c < mn ? c : c - mn;
            const double tm = (th[h + 1] + th[h]) / 2.0;
            double st, ct;
            sincos(tm, &st, &ct);
            unsigned neg = 0;  // sv[j] = -1
            for (int j = 0; j < mn; j++)
                if (!(Ac[2 * j] * ct + Ac[2 * j + 1] * st > 0)) neg |= 1u << j;
            if (c >= mn) neg ^= allm;
            int enc = (int)zneg;
            for (int j = 0; j < mps; j++) {
                if ((zmask >> j) & 1u) continue;
                const bool sneg = (neg >> cmap[j]) & 1u;
                if (sneg != (csmap[j] < 0)) enc |= 1 << j;
            }
            const cd g = cmul(lookup_num(kp, vp, np_, enc & maskp, mp), lookup_num(ks, vs, ns_, enc >> mp, ms));
            double g1r = 0, g2r = 0;
            for (int j = 0; j < mn; j++) {
                const double sv = ((neg >> j) & 1u) ? -1.0 : 1.0;
                g1r -= (Ac[2 * j] * pc[j]) * sv;
                g2r -= (Ac[2 * j + 1] * pc[j]) * sv;
            }
            sincos(th[c], os + c, oc + c);
            o1[c] = g1r;
            o2[c] = g2r;
            og[2 * c] = g.re;
            og[2 * c + 1] = g.im;
        }
        if (cells > 0) sincos(th[cells], os + cells, oc + cells);
        else os[0] = oc[0] = 0.0;
        int keep = 1;
        if (a.approx) {
            double total = 0;
            bool den_small = false;
            for (int i = 0; i < mn; i++) {
                const double a1 = o1[i], a2 = o2[i], c1 = oc[i], s1 = os[i], c2 = oc[i + 1], s2 = os[i + 1];
                const double den1 = a1 * (a1 * c1 + a2 * s1);
                const double den2 = a1 * (a1 * c2 + a2 * s2);
                if (fabs(den1) < 1e-14 || fabs(den2) < 1e-14) {
                    den_small = true;
                    break;
                }
                const double gr = hypot(og[2 * i], og[2 * i + 1]);
                total += fabs((gr * s2) / den2) + fabs((gr * s1) / den1);
            }
            if (!den_small) {
                total *= (2 * a.approx_nf);
                if (fabs(total) < a.eps) keep = 0;
            }
        }
        a.keep[x] = keep;
    }
}

// compute_moments(false) (cauchy_estimator.hpp:524-602), the moments of the
// reduced terms after the table build when print_basic_info is set: a thread
// per term, eval_g_yei_after_ftr (cauchy_term.hpp:403-433) -- the rows' signs
// at the root point (0 counts as negative), the term's table value there,
// yei = -sum p_l s_l A_l + i b -- into a moment row laid out as k_mu_terms
// writes them (g, g y_j, g y_j y_k), for the same chain and finalisation.
template <int D>
__global__ void k_post_ftr_terms(ParentList P, long long nP, const double* roots, Tables T, int MC, cd* contrib)
{
    constexpr int NM = 1 + D + D * D;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nP;
         i += (long long)gridDim.x * blockDim.x) {
        const int e = P.est[i];
        const int m = P.m[i];
        const double* A = P.A + i * MC * D;
        const double* p = P.p + i * MC;
        const double* root = roots + (long long)e * D;
        int enc = 0;
        double ty[D];
        for (int j = 0; j < D; j++) ty[j] = 0;
        for (int l = 0; l < m; l++) {
            double s = 0.0;
            for (int j = 0; j < D; j++) s += A[l * D + j] * root[j];
            const bool sp = s > 0;
            const double sc = sp ? p[l] : -p[l];  // p_l * sign, exact
            for (int j = 0; j < D; j++) ty[j] += sc * A[l * D + j];
            if (!sp) enc |= 1 << l;
        }
        const cd g = lookup_num(T.keys + P.tab_off[i], T.vals + P.tab_off[i], P.tab_cnt[i], enc, m);
        cd* cs = contrib + i * NM;
        cs[0] = g;
        for (int j = 0; j < D; j++) {
            const cd gy = cmul(g, mkcd(-ty[j], P.b[i * D + j]));
            cs[1 + j] = gy;
            for (int k = 0; k < D; k++) cs[1 + D + j * D + k] = cmul(gy, mkcd(-ty[k], P.b[i * D + k]));
        }
    }
}

template <int D>
void Kernels<D>::post_ftr_terms(ParentList P, long long nP, const double* roots, Tables T, int MC, cd* contrib,
                                const LaunchCfg& c)
{
    if (nP == 0) return;
    ++g_launches;
    k_post_ftr_terms<D><<<grid_for(nP, 128, c.num_sms, 16), 128, 0, c.stream>>>(P, nP, roots, T, MC, contrib);
}

template <int D>
void Kernels<D>::rel2d_pairs(const Rel2DArgs& a, const LaunchCfg& c)
{
    if (a.npairs == 0) return;
    ++g_launches;
    k_rel2d_pairs<D><<<grid_for(a.npairs, 128, c.num_sms, 16), 128, 0, c.stream>>>(a);
}

#if MCE_COMMON_UNIT
// One thread per point, the terms summed in order.  Points below `exact`
// take the complex formula (fx * 1/(2 pi) / fz), the others the cached one
// (fx / fz).
__global__ void k_cpdf1d_points(const double* tt, long long n, const double* xs, int npts, int exact, double fz,
                                double* ys)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= npts) return;
    const double x = xs[q];
    double fx = 0;
    if (q < exact) {
        for (long long j = 0; j < n; j++) {
            const double* t = tt + j * 8;
            const double b_c = t[5] - x;
            const cd g = csub(cdiv(mkcd(t[0], t[1]), mkcd(t[4], b_c)), cdiv(mkcd(t[2], t[3]), mkcd(-t[4], b_c)));
            fx += g.re;
        }
        ys[q] = fx * kTwoPiInv / fz;
    } else {
        for (long long j = 0; j < n; j++) {
            const double* t = tt + j * 8;
            const double w2 = t[4] * t[4];
            double xms = x - t[5];
            xms *= xms;
            fx += (t[6] * x + t[7]) / (w2 + xms);
        }
        ys[q] = fx / fz;
    }
}

// One cell's integral (marg2d_eval_term_for_cpdf / marg2d_cached_eval_term_for_cpdf,
// cpdf_ndim.hpp:1602-1640, 1710-1740): the fast form, or, with gamma1 ~ 0,
// the form that also handles gamma2 ~ 0; both ~ 0 is the reference's exit,
// reported here through *bad.
__device__ inline double marg2d_cell(double s1, double c1, double s2, double c2, double g1r, double g1i, double g2r,
                                     double g2i, bool check, cd g, int* bad)
{
    cd gamma1 = mkcd(g1r, g1i), gamma2 = mkcd(g2r, g2i);
    bool fast = true;
    if (check && fabs(g1r) < 1e-8) {
        fast = false;
        if (fabs(g2r) < 1e-8 && fabs(g2i) < 1e-8) {
            *bad = 1;
            return 0.0;
        }
    }
    cd cell;
    if (fast) {
        gamma2 = cmul(gamma2, gamma1);
        gamma1 = cmul(gamma1, gamma1);
        const cd lo = cdiv(mkcd(s1, 0), cadd(cscale(gamma1, c1), cscale(gamma2, s1)));
        const cd hi = cdiv(mkcd(s2, 0), cadd(cscale(gamma1, c2), cscale(gamma2, s2)));
        cell = cmul(csub(hi, lo), g);
    } else {
        const cd lo = cdiv(csub(cscale(gamma1, s1), cscale(gamma2, c1)), cadd(cscale(gamma1, c1), cscale(gamma2, s1)));
        const cd hi = cdiv(csub(cscale(gamma1, s2), cscale(gamma2, c2)), cadd(cscale(gamma1, c2), cscale(gamma2, s2)));
        cell = csub(hi, lo);
        gamma1 = cmul(gamma1, gamma1);
        gamma2 = cmul(gamma2, gamma2);
        cell = cmul(cell, cdiv(g, cadd(gamma1, gamma2)));
    }
    return cell.re;
}

// A thread per grid point; terms and their cells summed in order, then
// 2 fx / (2 pi)^2 / fz (cpdf_ndim.hpp:1447).
__global__ void k_cpdf2d_points(const double* tt, long long n, int MC, const double* xs, const double* ys, int npts,
                                double fz, double* zs, int* bad)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= npts) return;
    const int RT = cpdf2d_stride(MC);
    const double x1 = xs[q], x2 = ys[q];
    double fx = 0;
    int b = 0;
    for (long long j = 0; j < n; j++) {
        const double* o = tt + j * RT;
        const int mn = (int)o[0];
        const double* os = o + 3;
        const double* oc = os + (MC + 1);
        const double* o1 = oc + (MC + 1);
        const double* o2 = o1 + MC;
        const double* og = o2 + MC;
        const double g1i = o[1] - x1, g2i = o[2] - x2;
        const bool check = fabs(g1i) < 1e-8;
        double t = 0;
        for (int c = 0; c < mn; c++)
            t += marg2d_cell(os[c], oc[c], os[c + 1], oc[c + 1], o1[c], g1i, o2[c], g2i, check,
                             mkcd(og[2 * c], og[2 * c + 1]), &b);
        fx += t;
    }
    zs[q] = 2 * fx * kTwoPiInv * kTwoPiInv / fz;
    if (b) atomicOr(bad, 1);
}

void cpdf2d_points(const double* tt, long long n, int MC, const double* xs, const double* ys, int npts, double fz,
                   double* zs, int* bad, const LaunchCfg& c)
{
    if (npts <= 0) return;
    ++g_launches;
    k_cpdf2d_points<<<(npts + 63) / 64, 64, 0, c.stream>>>(tt, n, MC, xs, ys, npts, fz, zs, bad);
}

void cpdf1d_points(const double* tt, long long n, const double* xs, int npts, int exact, double fz, double* ys,
                   const LaunchCfg& c)
{
    if (npts <= 0) return;
    ++g_launches;
    k_cpdf1d_points<<<(npts + 63) / 64, 64, 0, c.stream>>>(tt, n, xs, npts, exact, fz, ys);
}

// Relative 2-D pdf (eval_marg2d_relative_and_transformed_cpdf,
// cauchy_prediction.hpp:973-1073): a thread per (grid point, chunk of pairs),
// the chunk's kept terms and their cells summed in order; the integral of a
// cell is the marginal 2-D one.
__global__ void k_rel2d_points(const double* tt, const long long* kidx, long long nk, int CC, int full,
                               long long chunk, const double* xs, const double* ys, int npts, double* part, int* bad)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= npts) return;
    const long long j0 = (long long)blockIdx.y * chunk;
    const long long j1 = j0 + chunk < nk ? j0 + chunk : nk;
    const int RT = rel2d_stride(CC);
    const double x1 = xs[q], x2 = ys[q];
    double fx = 0;
    int b = 0;
    for (long long j = j0; j < j1; j++) {
        const double* o = tt + kidx[j] * RT;
        const int cells = (int)o[0] * (1 + full);
        const double* os = o + 3;
        const double* oc = os + (CC + 1);
        const double* o1 = oc + (CC + 1);
        const double* o2 = o1 + CC;
        const double* og = o2 + CC;
        const double g1i = o[1] - x1, g2i = o[2] - x2;
        const bool check = fabs(g1i) < 1e-8;
        double t = 0;
        for (int c = 0; c < cells; c++)
            t += marg2d_cell(os[c], oc[c], os[c + 1], oc[c + 1], o1[c], g1i, o2[c], g2i, check,
                             mkcd(og[2 * c], og[2 * c + 1]), &b);
        fx += t;
    }
    part[(long long)blockIdx.y * npts + q] = fx;
    if (b) atomicOr(bad, 1);
}

__global__ void k_rel2d_finish(const double* part, int nch, int npts, int full, double nf_prim, double nf_sec,
                               double* zs)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= npts) return;
    double fx = 0;
    for (int ch = 0; ch < nch; ch++) fx += part[(long long)ch * npts + q];
    zs[q] = ((double)(2 - full)) * fx * kTwoPiInv * kTwoPiInv / (nf_prim * nf_sec);
}

void rel2d_points(const double* tt, const long long* kidx, long long nk, int CC, int full, long long chunk,
                  int nch, const double* xs, const double* ys, int npts, double* part, int* bad, const LaunchCfg& c)
{
    if (npts <= 0) return;
    ++g_launches;
    k_rel2d_points<<<dim3((npts + 63) / 64, nch), 64, 0, c.stream>>>(tt, kidx, nk, CC, full, chunk, xs, ys, npts,
                                                                      part, bad);
}

// kidx[kpos[j]] = j for every kept pair j (kpos: exclusive scan of keep)
__global__ void k_rel2d_compact(const int* keep, const long long* kpos, long long n, long long* kidx)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x)
        if (keep[j]) kidx[kpos[j]] = j;
}

void rel2d_compact(const int* keep, const long long* kpos, long long n, long long* kidx, const LaunchCfg& c)
{
    if (n <= 0) return;
    ++g_launches;
    k_rel2d_compact<<<grid_for(n, 256, c.num_sms, 8), 256, 0, c.stream>>>(keep, kpos, n, kidx);
}

void rel2d_finish(const double* part, int nch, int npts, int full, double nf_prim, double nf_sec, double* zs,
                  const LaunchCfg& c)
{
    if (npts <= 0) return;
    ++g_launches;
    k_rel2d_finish<<<(npts + 127) / 128, 128, 0, c.stream>>>(part, nch, npts, full, nf_prim, nf_sec, zs);
}

// Relative moments: a thread per (chunk, column) sums its chunk of pairs in
// order, then one thread per column sums the chunks in order and thread 0
// applies finalize_rel_sys_moments (cauchy_prediction.hpp:288-303).
__global__ void k_rel2d_msum(const double* mrows, long long n, long long chunk, int nch, double* part)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nch * 14) return;
    const long long ch = t / 14;
    const int col = (int)(t - ch * 14);
    const long long j0 = ch * chunk, j1 = j0 + chunk < n ? j0 + chunk : n;
    double acc = 0;
    for (long long j = j0; j < j1; j++) acc += mrows[j * 14 + col];
    part[ch * 14 + col] = acc;
}

__global__ void k_rel2d_mfinal(const double* part, int nch, double* out)
{
    __shared__ double s[14];
    const int col = threadIdx.x;
    if (col < 14) {
        double acc = 0;
        for (int ch = 0; ch < nch; ch++) acc += part[(long long)ch * 14 + col];
        s[col] = acc;
    }
    __syncthreads();
    if (col != 0) return;
    const cd fz = mkcd(s[0], s[1]);
    const cd ifz = mkcd(0, fz.re);
    cd mean[2];
    for (int i = 0; i < 2; i++) mean[i] = cdiv(mkcd(s[2 + 2 * i], s[3 + 2 * i]), ifz);
    out[0] = fz.re;
    out[1] = fz.im;
    for (int i = 0; i < 2; i++) {
        out[2 + 2 * i] = mean[i].re;
        out[3 + 2 * i] = mean[i].im;
    }
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) {
            const int k = 2 * i + j;
            const cd v = csub(cdiv(mkcd(s[6 + 2 * k], s[7 + 2 * k]), fz), cmul(mean[i], mean[j]));
            out[6 + 2 * k] = v.re;
            out[7 + 2 * k] = v.im;
        }
}

void rel2d_moments(const double* mrows, long long n, long long chunk, double* part, double* out, const LaunchCfg& c)
{
    const long long nch = n > 0 ? (n + chunk - 1) / chunk : 0;
    g_launches += 2;
    if (nch > 0)
        k_rel2d_msum<<<(unsigned)((nch * 14 + 127) / 128), 128, 0, c.stream>>>(mrows, n, chunk, (int)nch, part);
    k_rel2d_mfinal<<<1, 32, 0, c.stream>>>(part, (int)nch, out);
}
#endif  // MCE_COMMON_UNIT

#if MCE_COMMON_UNIT
void group_count(const int* status, const int* owner, long long nR, int* gcnt, const LaunchCfg& c)
{
    if (nR == 0) return;
    ++g_launches;
    k_group_count<<<grid_for(nR, 256, c.num_sms), 256, 0, c.stream>>>(status, owner, nR, gcnt);
}
void group_fill(const int* status, const int* owner, long long nR, const long long* goff, int* gfill, int* members,
                const LaunchCfg& c)
{
    if (nR == 0) return;
    ++g_launches;
    k_group_fill<<<grid_for(nR, 256, c.num_sms), 256, 0, c.stream>>>(status, owner, nR, goff, gfill, members);
}
void group_sort(const int* gcnt, const long long* goff, long long nR, const int* members_in, int* members_out,
                const LaunchCfg& c)
{
    if (nR == 0) return;
    ++g_launches;
    k_group_sort<<<grid_for(nR, 8, c.num_sms), 256, 0, c.stream>>>(gcnt, goff, nR, members_in, members_out);
}
void roots_flags(const int* status, const int* m, long long nR, int D, int* is_root, int* cap, const LaunchCfg& c)
{
    if (nR == 0) return;
    ++g_launches;
    k_roots_flags<<<grid_for(nR, 256, c.num_sms), 256, 0, c.stream>>>(status, m, nR, D, is_root, cap);
}
void roots_list(const int* is_root, const long long* rscan, long long nR, int* list, const LaunchCfg& c)
{
    if (nR == 0) return;
    ++g_launches;
    k_roots_list<<<grid_for(nR, 256, c.num_sms), 256, 0, c.stream>>>(is_root, rscan, nR, list);
}
long long partition_tiles_cap(long long nR, int E) { return nR / kPartTile + E + 1; }

void partition_tiles(const int* alive, const int* m, const long long* rbase, int E, int MCp, long long nR,
                     int* ntile, long long* tstart, int* C, int* hist, ScanScratch& ss, const LaunchCfg& c)
{
    if (E <= 0) return;
    const long long cap = partition_tiles_cap(nR, E);
    const int g = (int)(cap < (long long)c.num_sms * 16 ? cap : (long long)c.num_sms * 16);
    g_launches += 3;
    k_ptile_count<<<(E + 255) / 256, 256, 0, c.stream>>>(rbase, E, ntile);
    scan_int_to_ll(ntile, tstart, E, ss, c);
    k_ptile_hist<<<g, 256, 0, c.stream>>>(alive, m, rbase, E, MCp, tstart, C);
    k_ptile_scan<<<grid_for((long long)E * MCp, 256, c.num_sms), 256, 0, c.stream>>>(E, MCp, tstart, C, hist);
}

void partition_rank(const int* alive, const int* m, const long long* rbase, int E, int MCp, long long nR,
                    const long long* tstart, const int* P, const long long* bucket_off, int* new_slot,
                    const LaunchCfg& c)
{
    if (E <= 0) return;
    const long long cap = partition_tiles_cap(nR, E);
    const int g = (int)(cap < (long long)c.num_sms * 16 ? cap : (long long)c.num_sms * 16);
    ++g_launches;
    k_ptile_rank<<<g, 256, 0, c.stream>>>(alive, m, rbase, E, MCp, tstart, P, bucket_off, new_slot);
}
void rbase_kernel(const long long* pstart, const long long* kscan, int E, long long* rbase, const LaunchCfg& c)
{
    ++g_launches;
    k_rbase<<<(E + 1 + 255) / 256, 256, 0, c.stream>>>(pstart, kscan, E, rbase);
}

#endif  // MCE_COMMON_UNIT

#if MCE_ONLY_DIM > 0
template struct Kernels<MCE_ONLY_DIM>;
#elif MCE_ONLY_DIM < 0
template struct Kernels<1>;
template struct Kernels<2>;
template struct Kernels<3>;
template struct Kernels<4>;
template struct Kernels<5>;
template struct Kernels<6>;
template struct Kernels<7>;
template struct Kernels<8>;
#endif

}  // namespace mce
