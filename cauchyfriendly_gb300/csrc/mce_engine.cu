// Host engine of the MCE step path and the C ABI declared in include/mce_c_api.h.
//
// One engine owns a batch of independent estimators that step in lock-step
// (a single estimator is a batch of one).  All term state stays in device
// arenas that only grow; a step issues the kernel sequence of
// mce_kernels.cu on one stream and synchronises only where the host must
// size the next allocation or read the moments the API returns.
//
// Host-side work per step is limited to per-estimator scalars: packing each
// estimator's (Phi, Gamma, beta, H, gamma, B u) and pre-coaligning Gamma
// (cauchy_util.hpp:128-210), and the numeric checks of the returned moments
// (cauchy_estimator.hpp:359-461), both O(d^3) per estimator.
#include "mce_kernels.cuh"
#include "../../include/mce_c_api.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#ifndef MCE_ONLY_DIM
#define MCE_ONLY_DIM -1  // every dimension and the C ABI in one unit
#endif

namespace mce {

extern thread_local std::string g_last_error;
// Set by mce_batch_step_noalloc for the duration of its step: a DevBuf that
// would have to grow fails with MCE_ERR_NOMEM instead of calling cudaMalloc.
extern thread_local bool g_device_alloc_forbidden;
#if MCE_ONLY_DIM <= 0
thread_local std::string g_last_error;
thread_local bool g_device_alloc_forbidden = false;
#endif

static void set_error(const std::string& s) { g_last_error = s; }

#define MCE_CUDA(call)                                                                     \
    do {                                                                                   \
        cudaError_t _e = (call);                                                           \
        if (_e != cudaSuccess) {                                                           \
            set_error(std::string(#call) + ": " + cudaGetErrorString(_e));                 \
            return MCE_ERR_CUDA;                                                           \
        }                                                                                  \
    } while (0)

// Grow-only device buffer.
template <typename T>
struct DevBuf {
    T* ptr = nullptr;
    size_t cap = 0;
    ~DevBuf() { release(); }
    void release()
    {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
    }
    int ensure(size_t n)
    {
        if (n <= cap && ptr) return MCE_OK;
        if (g_device_alloc_forbidden) {
            set_error("mce_batch_step_noalloc: a device buffer of the handle is too small for this step (" +
                      std::to_string(n * sizeof(T)) + " bytes needed, " + std::to_string(cap * sizeof(T)) +
                      " held) and this call may not allocate; the handle must be reset");
            return MCE_ERR_NOMEM;
        }
        size_t want = std::max<size_t>(n, cap + cap / 2);
        want = std::max<size_t>(want, 64);
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&ptr, want * sizeof(T));
        if (e != cudaSuccess) {
            cudaGetLastError();
            set_error("cudaMalloc of " + std::to_string(want * sizeof(T)) + " bytes failed: " + cudaGetErrorString(e));
            return MCE_ERR_NOMEM;
        }
        cap = want;
        return MCE_OK;
    }
};

// Page-locked host buffer: device-to-host copies into it are asynchronous, so
// the host goes on queueing work while they wait on the stream.
template <typename T>
struct PinnedBuf {
    T* ptr = nullptr;
    size_t cap = 0;
    ~PinnedBuf()
    {
        if (ptr) cudaFreeHost(ptr);
    }
    int ensure(size_t n)
    {
        if (n <= cap && ptr) return MCE_OK;
        if (ptr) cudaFreeHost(ptr);
        ptr = nullptr;
        cap = 0;
        cudaError_t e = cudaMallocHost(&ptr, std::max<size_t>(n, 1) * sizeof(T));
        if (e != cudaSuccess) {
            cudaGetLastError();
            set_error(std::string("cudaMallocHost failed: ") + cudaGetErrorString(e));
            return MCE_ERR_NOMEM;
        }
        cap = std::max<size_t>(n, 1);
        return MCE_OK;
    }
    T* data() { return ptr; }
    T& operator[](size_t i) { return ptr[i]; }
};

// Numeric checks of one estimator's raw moments (cauchy_estimator.hpp:359-461,
// covariance_checker cauchy_util.hpp:1882-2004).
enum {
    E_FZ_NEG = 9, E_FZ_UNST = 8, E_MEAN_DNE = 7, E_MEAN_NF = 6, E_MEAN_F = 5, E_MEAN_ANY = 4,
    E_COV_DNE = 3, E_COV_NF = 2, E_COV_F = 1, E_COV_ANY = 0
};

static void jacobi_eigvals(const double* S, double* ev, int n)
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
                const double apq = a[p * n + q];
                if (apq == 0) continue;
                const double th = (a[q * n + q] - a[p * n + p]) / (2 * apq);
                const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1));
                const double c = 1 / sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; k++) {
                    const double akp = a[k * n + p], akq = a[k * n + q];
                    a[k * n + p] = c * akp - s * akq;
                    a[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    const double apk = a[p * n + k], aqk = a[q * n + k];
                    a[p * n + k] = c * apk - s * aqk;
                    a[q * n + k] = s * apk + c * aqk;
                }
            }
    }
    for (int i = 0; i < n; i++) ev[i] = a[i * n + i];
}

static int cov_flags(const double* cre, const double* cim, int d)
{
    int f = 0;
    double ev[kMaxDim];
    jacobi_eigvals(cre, ev, d);
    for (int i = 0; i < d; i++)
        if (ev[i] < -1e-5) f |= 1;
    for (int i = 0; i < d - 1; i++) {
        const double sii = sqrt(cre[i * d + i]);
        for (int j = i + 1; j < d; j++) {
            const double sjj = sqrt(cre[j * d + j]);
            if (fabs(cre[i * d + j] / (sii * sjj)) > 1) f |= 2;
        }
    }
    for (int i = 0; i < d; i++)
        for (int j = i; j < d; j++)
            if (fabs(cim[i * d + j]) / (fabs(cre[i * d + j]) + 1e-15) > 10) f |= 4;
    for (int i = 0; i < d * d; i++)
        if (fabs(cim[i]) > 2000) f |= 8;
    return f;
}

// Host threads for the per-estimator host work of a step (input packing and
// the moment checks of finalize/moments_numerical_check), which is
// independent per estimator: run(n, f) calls f(a, b) on contiguous chunks
// covering [0, n) and returns when all are done.  Chunks are claimed
// dynamically (the calling thread takes part), so a worker that wakes late
// only finds fewer chunks left; a claim names the job's generation, so a late
// worker never takes a chunk of a later job.
class HostPool {
public:
    explicit HostPool(int workers)
    {
        for (int i = 0; i < workers; i++) th_.emplace_back([this] { loop(); });
    }
    ~HostPool()
    {
        {
            std::lock_guard<std::mutex> l(m_);
            stop_ = true;
        }
        cv_.notify_all();
        for (std::thread& t : th_) t.join();
    }
    void run(int n, const std::function<void(int, int)>& f)
    {
        const int parts = (int)th_.size() + 1;
        int chunk = n / (4 * parts);
        if (chunk < 32) chunk = 32;
        const int nch = (n + chunk - 1) / chunk;
        unsigned long long g;
        {
            std::lock_guard<std::mutex> l(m_);
            g = ++gen_;
            job_ = &f;
            n_ = n;
            chunk_ = chunk;
            nch_ = nch;
            done_.store(0);
            claim_.store(g << 32);
        }
        cv_.notify_all();
        work(g, &f, n, chunk, nch);
        while (done_.load() < nch) std::this_thread::yield();
    }

private:
    void work(unsigned long long g, const std::function<void(int, int)>* f, int n, int chunk, int nch)
    {
        for (;;) {
            unsigned long long w = claim_.load();
            int c;
            do {
                if ((w >> 32) != g) return;
                c = (int)(w & 0xffffffffull);
                if (c >= nch) return;
            } while (!claim_.compare_exchange_weak(w, w + 1));
            const int a = c * chunk, b = a + chunk < n ? a + chunk : n;
            (*f)(a, b);
            done_.fetch_add(1);
        }
    }
    void loop()
    {
        unsigned long long seen = 0;
        for (;;) {
            unsigned long long g;
            const std::function<void(int, int)>* f;
            int n, chunk, nch;
            {
                std::unique_lock<std::mutex> l(m_);
                cv_.wait(l, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = g = gen_;
                f = job_;
                n = n_;
                chunk = chunk_;
                nch = nch_;
            }
            work(g, f, n, chunk, nch);
        }
    }
    std::vector<std::thread> th_;
    std::mutex m_;
    std::condition_variable cv_;
    const std::function<void(int, int)>* job_ = nullptr;
    int n_ = 0, chunk_ = 1, nch_ = 0;
    unsigned long long gen_ = 0;
    std::atomic<unsigned long long> claim_{0};
    std::atomic<int> done_{0};
    bool stop_ = false;
};

enum KernelGroup {
    KID_FIRST = 0, KID_TP, KID_BUILD_B, KID_MU, KID_MOMENTS, KID_FTR, KID_GROUPS, KID_GTABLE, KID_PARTITION,
    KID_SCAN, KID_WAIT, KID_COUNT
};
// "wait": the engine's stream waiting for the side stream's moment chains
static const char* kKernelGroupNames[KID_COUNT] = {
    "first_step", "tp", "build_B", "mu", "moments", "ftr", "groups", "gtable", "partition", "scan", "wait"};

struct EstHost {
    int steps = 0;          // estimation steps
    int num_updates = 0;    // p * steps
    int max_shape = 0;
    std::vector<double> A0, p0, b0;
    int errors = 0;
    // reported moments (after checks) and the last good ones
    double fz[2] = {0, 0}, last_fz[2] = {0, 0};
    std::vector<double> mean, cov, last_mean, last_cov;  // interleaved complex
    // raw moments of the last update
    double raw_fz[2] = {0, 0};
    std::vector<double> raw_mean, raw_cov;
    double gscale = 0;
    long long nt = 1;
    std::vector<int> tps;
    int win_num = 0;
    // the constructor's print_basic_info: the moments reported after each
    // table build are those of compute_moments(false)
    bool print_basic_info = false;
};

class EngineBase {
public:
    virtual ~EngineBase() {}
    virtual int step(const double* msmt, const double* Phi, const double* Gamma, const double* beta,
                     const double* H, const double* gamma, const double* B, const double* u, int shared,
                     int* err_out) = 0;
    virtual int dump_terms(int est, int max_shape, int* shape, double* A, double* p, double* b, int* cells,
                           int* keys, double* g) = 0;
    virtual long long total_cells(int est) = 0;
    virtual int reset() = 0;
    // Frees the buffers that grow with the term count (only between a reset
    // or creation and the next step) when they hold at least min_bytes;
    // returns the bytes released.
    virtual long long trim(long long min_bytes) = 0;
    // copies estimator e's start statistics to the device, where the next
    // first update reads them
    virtual int upload_start(int e) = 0;
    // every current term of estimator e: b += v (sub = 0) or b -= v (sub = 1)
    virtual int shift_terms_b(int e, const double* v, int sub) = 0;
    // every current term of estimator e: time_prop with Phi and B u (Bu may be null)
    virtual int time_prop_terms(int e, const double* Phi, const double* Bu) = 0;
    virtual int cpdf_2d_grid(int est, int i1, int i2, const double* bar_nu, double lx, double hx, double rx,
                             double ly, double hy, double ry, int reset_cache, int max_points, double* xs,
                             double* ys, double* zs) = 0;
    virtual int cpdf_1d_grid(int est, int marg, const double* bar_nu, double low, double high, double res,
                             int max_points, double* xs, double* ys) = 0;
    // PointWiseNDimCauchyCPDF::evaluate_cpdf at npts points (csrc/mce_ndpdf.cu)
    virtual int cpdf_nd(int est, const double* x, int npts, double* out) = 0;
    virtual int cpdf_marginal(int est, const int* idx, int nm, const double* nu_bar, const double* x, int npts,
                              double* out) = 0;
    // waits for the work the engine queued (after a step that stopped early)
    virtual void drain() = 0;
    // Estimator e's current terms for the relative system: the device lists,
    // the term indices grouped by shape (ascending, positions in order) and
    // the reported fz.  Refused before the first and after the last update.
    struct TermsView {
        ParentList P;
        Tables T;
        int MC = 0;
        std::vector<long long> idx;
        std::vector<int> shape_off, shape_cnt;  // per shape 0..MC
        double fz = 0;
    };
    virtual int terms_view(int e, TermsView* v) = 0;
    // launches the pair kernel of this engine's state dimension
    virtual void rel2d_pairs(const Rel2DArgs& a, cudaStream_t st) = 0;

    int E = 0, d = 0, cmcc = 0, pncc = 0, p = 0, MC = 0;
    // the device the handle's streams and buffers live on
    int device = 0;
    // When set (only by mce_batch_step_noalloc), the g-table kernel takes its
    // per-warp scratch from this caller-owned region instead of the handle's
    // own buffer, with as many warps as fit in it.
    void* fixed_gtable_scratch = nullptr;
    size_t fixed_gtable_scratch_bytes = 0;
    // bytes of g-table scratch one warp needs: half the cells of a full-shape term
    size_t gtable_scratch_bytes_per_warp() const { return sizeof(cd) * (size_t)half_cells_cap(MC, d); }
    int master_step = 0;
    int device_errors = 0;
    // host wall time of the steps (ms): whole step, input packing, moment checks
    double host_ms[3] = {0, 0, 0};
    // per-estimator host work, split over host threads for large batches
    std::unique_ptr<HostPool> pool;
    void for_estimators(const std::function<void(int, int)>& f)
    {
        if (E >= 256 && !pool) {
            const unsigned hw = std::thread::hardware_concurrency();
            const int workers = (int)std::min<unsigned>(hw > 1 ? hw - 1 : 0, 15);
            if (workers > 0) pool.reset(new HostPool(workers));
        }
        if (pool && E >= 256) pool->run(E, f);
        else f(0, E);
    }
    long long post_mu_terms = 0;
    double last_ms = 0;
    // profiling: per-kernel-group device time (CUDA events on the engine's
    // stream), launch counts and algorithmic bytes / FP64 flops
    int prof_mode = 0;
    double device_ms_total = 0;
    long long launches = 0;
    double kms[KID_COUNT] = {0};
    long long klaunch[KID_COUNT] = {0};
    double kbytes[KID_COUNT] = {0};
    double kflops[KID_COUNT] = {0};
    void clear_prof()
    {
        device_ms_total = 0;
        host_ms[0] = host_ms[1] = host_ms[2] = 0;
        launches = 0;
        for (int k = 0; k < KID_COUNT; k++) {
            kms[k] = 0;
            klaunch[k] = 0;
            kbytes[k] = 0;
            kflops[k] = 0;
        }
    }
    std::vector<EstHost> est;
    std::vector<double> roots, bpert;  // E*d, E*MC
};

template <int D>
class Engine : public EngineBase {
public:
    LaunchCfg lc{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // the moment chains run on a side stream, overlapping the term reduction
    cudaStream_t mstream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // per-estimator device inputs
    DevBuf<double> dA0, dp0, db0, droots, dbpert;
    DevBuf<EstStep<D>> dsteps;
    std::vector<EstStep<D>> hsteps;
    DevBuf<long long> dpstart;
    std::vector<long long> hpstart;  // E+1
    std::vector<int> h_order;       // moment-chain launch order
    DevBuf<int> ftr_cnt;            // worklist lengths of the resolution rounds
    static constexpr int kFtrFirstBatch = 4, kFtrBatch = 2, kFtrCntSlots = 8, kFtrMaxRounds = 100000;
    // How the resolution rounds after the first run: 0 queued in batches, the
    // host reading the worklist length once per batch; 1 one persistent
    // cooperative launch; 2 a device-side loop in a CUDA graph.  Chosen with
    // MCE_FTR_ROUNDS=batched|persistent|graph (MCE_FTR_PERSISTENT=1 is
    // persistent).
    static int ftr_rounds_mode()
    {
        static const int mode = [] {
            const char* p = getenv("MCE_FTR_PERSISTENT");
            if (p && p[0] == '1') return 1;
            const char* v = getenv("MCE_FTR_ROUNDS");
            if (v && !strcmp(v, "batched")) return 0;
            if (v && !strcmp(v, "persistent")) return 1;
            if (v && !strcmp(v, "graph")) return 2;
            return 0;
        }();
        return mode;
    }
    void* ftr_graph = nullptr;  // the rounds' CUDA graph (mode 2), built on first use
    DevBuf<int> d_order;
    // combos per shape (lexicographic d-subsets)
    DevBuf<int> dcombo_off;
    DevBuf<unsigned char> dcombos;
    // parent lists (double-buffered) and tables
    struct PBufs {
        DevBuf<int> est, m, m_old, tab_cnt, B_cnt, nkids, nkids_all, bflip;
        DevBuf<double> A, p, b;
        DevBuf<long long> tab_off, B_off, kscan;
        int ensure(long long n, int MC)
        {
            int s = MCE_OK;
            s |= est.ensure(n + 1);
            s |= m.ensure(n + 1);
            s |= m_old.ensure(n + 1);
            s |= tab_cnt.ensure(n + 1);
            s |= B_cnt.ensure(n + 1);
            s |= nkids.ensure(n + 1);
            s |= nkids_all.ensure(n + 1);
            s |= bflip.ensure(n + 1);
            s |= A.ensure((n + 1) * MC * D);
            s |= p.ensure((n + 1) * MC);
            s |= b.ensure((n + 1) * D);
            s |= tab_off.ensure(n + 1);
            s |= B_off.ensure(n + 1);
            s |= kscan.ensure(n + 1);
            return s;
        }
        ParentList view()
        {
            ParentList P;
            P.est = est.ptr;
            P.m = m.ptr;
            P.m_old = m_old.ptr;
            P.A = A.ptr;
            P.p = p.ptr;
            P.b = b.ptr;
            P.tab_off = tab_off.ptr;
            P.tab_cnt = tab_cnt.ptr;
            P.B_off = B_off.ptr;
            P.B_cnt = B_cnt.ptr;
            P.nkids = nkids.ptr;
            P.nkids_all = nkids_all.ptr;
            P.kscan = kscan.ptr;
            P.bflip = bflip.ptr;
            return P;
        }
    } Pb[2];
    int cur = 0;
    long long nP = 0;
    struct TBufs {
        DevBuf<int> keys;
        DevBuf<cd> vals;
    } Tb[2];
    // per-step buffers
    DevBuf<int> Bcap, Bkeys;
    DevBuf<long long> kall_scan;
    struct RBufs {
        DevBuf<int> est, m, pbc, phc, z, lhp, fam, flags;
        DevBuf<unsigned> horthog;
        DevBuf<double> A, p, q, b, cval, dval, ps2;
        DevBuf<signed char> cmap, csmap;
        int ensure(long long n, int MC)
        {
            int s = MCE_OK;
            s |= est.ensure(n + 1);
            s |= m.ensure(n + 1);
            s |= ps2.ensure(n + 1);
            s |= pbc.ensure(n + 1);
            s |= phc.ensure(n + 1);
            s |= z.ensure(n + 1);
            s |= lhp.ensure(n + 1);
            s |= fam.ensure(n + 1);
            s |= flags.ensure(n + 1);
            s |= horthog.ensure(n + 1);
            s |= A.ensure((n + 1) * MC * D);
            s |= p.ensure((n + 1) * MC);
            s |= q.ensure((n + 1) * MC);
            s |= b.ensure((n + 1) * D);
            s |= cval.ensure(n + 1);
            s |= dval.ensure(n + 1);
            s |= cmap.ensure((n + 1) * MC);
            s |= csmap.ensure((n + 1) * MC);
            return s;
        }
        TermRecs view()
        {
            TermRecs R;
            R.est = est.ptr;
            R.m = m.ptr;
            R.pbc = pbc.ptr;
            R.phc = phc.ptr;
            R.z = z.ptr;
            R.lhp = lhp.ptr;
            R.fam = fam.ptr;
            R.flags = flags.ptr;
            R.horthog = horthog.ptr;
            R.A = A.ptr;
            R.p = p.ptr;
            R.q = q.ptr;
            R.b = b.ptr;
            R.cval = cval.ptr;
            R.dval = dval.ptr;
            R.ps2 = ps2.ptr;
            R.cmap = cmap.ptr;
            R.csmap = csmap.ptr;
            return R;
        }
    } Rb;
    DevBuf<cd> fam_mom, est_raw, scratch, g_vals, pr_gv;
    // post-FTR moments (print_basic_info): rows, chain totals, results
    DevBuf<cd> pf_rows, pf_raw;
    DevBuf<double> pf_tot, pf_gscale;
    DevBuf<long long> pf_zero;
    std::vector<cd> h_pf_raw;
    std::vector<double> h_pf_gscale;
    bool have_post = false;
    DevBuf<int> pr_root, pr_mb, pr_mcnt, pr_cells, pr_items;
    DevBuf<long long> pr_moff, pr_ioff, pr_coff;
    DevBuf<int> ftr_wl[2], ftr_resume;
    DevBuf<int> g_nr, g_items, g_cells, g_rflag, g_minfo, g_mflag, nvert, vsv;
    DevBuf<long long> g_ioff, g_coff, voff;
    DevBuf<double> g_rps2, g_mps2;
    DevBuf<double> gscale, mom_tot, mu_rows;
    DevBuf<int> mu_ints;
    DevBuf<long long> goff, toff, rscan, bucket_off, rbase, scan_tmp, kall_est, ptile_start;
    DevBuf<int> status, owner, gcnt, gfill, members, members_tmp, is_root, cap, roots_list, alive, src,
        tcnt, hist, new_slot, counters, first_cnt, bcount, bfill, slot_of, ptile_n, ptile_c;
    DevBuf<long long> boff;
    DevBuf<unsigned char> cell_ent, cell_ent2;
    // number of bucket entries (valid records), known after the bucket scan
    long long nvalid_entries(long long H) { return read_ll(boff.ptr + H); }
    // raw moments and G_SCALE_FACTOR per estimator, read back asynchronously
    // at the join and used after the step's final synchronisation
    PinnedBuf<cd> h_raw;
    PinnedBuf<double> h_gscale;
    std::vector<int> h_hist;
    ScanScratch ss{};
    // profiling events
    std::vector<cudaEvent_t> evpool;
    struct PEv {
        int id, a, b;
        long long launches;
    };
    std::vector<PEv> pevs;
    int ev_used = 0, p_id = 0, p_a = 0;
    long long p_l0 = 0;
    DevBuf<double> alg;  // [KID_COUNT][2] bytes, flops
    DevBuf<unsigned> gbits;  // cell bitmaps of terms above kSmemBitmapRows hyperplanes
    DevBuf<int> g_over;      // g-table preparation: a root above its slot, the largest count

    // profiling brackets on the engine's stream (or on st when given)
    void pbeg(int id, cudaStream_t st = nullptr)
    {
        p_l0 = g_launches;
        p_id = id;
        if (!prof_mode) return;
        if (ev_used + 2 > (int)evpool.size()) {
            for (int k = 0; k < 256; k++) {
                cudaEvent_t ev;
                if (cudaEventCreate(&ev) != cudaSuccess) return;
                evpool.push_back(ev);
            }
        }
        p_a = ev_used++;
        cudaEventRecord(evpool[p_a], st ? st : lc.stream);
    }
    void pend(cudaStream_t st = nullptr)
    {
        const long long nl = g_launches - p_l0;
        launches += nl;
        if (!prof_mode || p_a >= ev_used) return;
        const int b_ = ev_used++;
        cudaEventRecord(evpool[b_], st ? st : lc.stream);
        pevs.push_back(PEv{p_id, p_a, b_, nl});
    }
    void collect_prof()
    {
        for (const PEv& pe : pevs) {
            float ms = 0;
            if (cudaEventElapsedTime(&ms, evpool[pe.a], evpool[pe.b]) == cudaSuccess) kms[pe.id] += ms;
            klaunch[pe.id] += pe.launches;
        }
        pevs.clear();
        ev_used = 0;
    }
    void alg_stats(bool with_tp, long long nR, bool tables_built);

    int init(int E_, int cmcc_, int pncc_, int p_, const int* steps, const double* A0, const double* p0,
             const double* b0, const double* root, const double* bp, int bp_stride)
    {
        E = E_;
        d = D;
        cmcc = cmcc_;
        pncc = pncc_;
        p = p_;
        if (pncc > kMaxGamma || pncc < 0 || cmcc < 0 || p < 1) {
            set_error("unsupported pncc/cmcc/p");
            return MCE_ERR_ARG;
        }
        est.resize(E);
        MC = 1;
        for (int e = 0; e < E; e++) {
            EstHost& h = est[e];
            h.steps = steps[e];
            if (h.steps < 1) {
                set_error("steps must be >= 1");
                return MCE_ERR_ARG;
            }
            h.num_updates = p * h.steps;
            h.max_shape = D > 1 ? (h.steps - 1) * pncc + D : D + pncc;
            MC = std::max(MC, h.max_shape);
            h.A0.assign(A0 + (size_t)e * D * D, A0 + (size_t)(e + 1) * D * D);
            h.p0.assign(p0 + (size_t)e * D, p0 + (size_t)(e + 1) * D);
            h.b0.assign(b0 + (size_t)e * D, b0 + (size_t)(e + 1) * D);
            h.mean.assign(2 * D, 0);
            h.cov.assign(2 * D * D, 0);
            h.last_mean = h.mean;
            h.last_cov = h.cov;
            h.raw_mean = h.mean;
            h.raw_cov = h.cov;
        }
        if (MC > kMaxRows) {
            set_error("max shape exceeds 31 hyperplanes (cauchy_estimator.hpp:231-235)");
            return MCE_ERR_SHAPE;
        }
        // cell bitmaps hold 2^MC bits per warp: in shared memory up to 16
        // hyperplanes, in a global buffer above (its size, warps x 3 x 2^MC bits,
        // bounds the build at 24)
        if (MC > kMaxBitmapRows) {
            set_error("this build supports up to " + std::to_string(kMaxBitmapRows) + " hyperplanes per term");
            return MCE_ERR_SHAPE;
        }
        if (bp && bp_stride < MC) {
            for (int e = 0; e < E; e++)
                if (bp_stride < est[e].max_shape) {
                    set_error("b_pert stride smaller than an estimator's max shape");
                    return MCE_ERR_ARG;
                }
        }
        roots.assign((size_t)E * D, 0);
        bpert.assign((size_t)E * MC, 0);
        for (int e = 0; e < E; e++) {
            if (root) memcpy(&roots[(size_t)e * D], root + (size_t)e * D, D * sizeof(double));
            if (bp) memcpy(&bpert[(size_t)e * MC], bp + (size_t)e * bp_stride, est[e].max_shape * sizeof(double));
        }
        int dev = 0;
        MCE_CUDA(cudaGetDevice(&dev));
        device = dev;
        MCE_CUDA(cudaDeviceGetAttribute(&lc.num_sms, cudaDevAttrMultiProcessorCount, dev));
        MCE_CUDA(cudaStreamCreateWithFlags(&lc.stream, cudaStreamNonBlocking));
        MCE_CUDA(cudaEventCreate(&ev0));
        MCE_CUDA(cudaEventCreate(&ev1));
        MCE_CUDA(cudaStreamCreateWithFlags(&mstream, cudaStreamNonBlocking));
        MCE_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
        MCE_CUDA(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
        int s = MCE_OK;
        // profiling counters, sized here so no later step has to allocate them
        s |= alg.ensure(2 * KID_COUNT);
        s |= g_over.ensure(2);
        if (MC > kSmemBitmapRows) {
            // a region per warp for the bitmap kernels (8 warps per SM)
            const long long warps = (long long)lc.num_sms * 8;
            s |= gbits.ensure((size_t)(warps * gtable_bitmap_words(MC, D)));
            lc.gbits = gbits.ptr;
            lc.gbits_warps = warps;
        }
        s |= dA0.ensure((size_t)E * D * D);
        s |= dp0.ensure((size_t)E * D);
        s |= db0.ensure((size_t)E * D);
        s |= droots.ensure((size_t)E * D);
        s |= dbpert.ensure((size_t)E * MC);
        s |= dsteps.ensure(E);
        s |= dpstart.ensure(E + 1);
        s |= est_raw.ensure((size_t)E * (1 + D + D * D));
        s |= mom_tot.ensure((size_t)E * 2 * (1 + D + D * D));
        s |= gscale.ensure(E);
        s |= counters.ensure(8);
        s |= first_cnt.ensure(E + 1);
        s |= scan_tmp.ensure(1 << 16);
        s |= h_raw.ensure((size_t)E * (1 + D + D * D));
        s |= h_gscale.ensure(E);
        if (s) return MCE_ERR_NOMEM;
        ss.block_sums = scan_tmp.ptr;
        ss.cap = (long long)scan_tmp.cap;
        MCE_CUDA(cudaMemcpy(droots.ptr, roots.data(), roots.size() * sizeof(double), cudaMemcpyHostToDevice));
        MCE_CUDA(cudaMemcpy(dbpert.ptr, bpert.data(), bpert.size() * sizeof(double), cudaMemcpyHostToDevice));
        // combination tables
        std::vector<int> off(MC + 2, 0);
        std::vector<unsigned char> cmb;
        for (int m = 0; m <= MC; m++) {
            off[m] = (int)cmb.size();
            if (m > D) {
                std::vector<int> c(D);
                for (int i = 0; i < D; i++) c[i] = i;
                while (true) {
                    for (int i = 0; i < D; i++) cmb.push_back((unsigned char)c[i]);
                    int i = D - 1;
                    while (i >= 0 && c[i] == m - D + i) i--;
                    if (i < 0) break;
                    c[i]++;
                    for (int j = i + 1; j < D; j++) c[j] = c[j - 1] + 1;
                }
            }
        }
        off[MC + 1] = (int)cmb.size();
        if (cmb.empty()) cmb.push_back(0);
        s |= dcombo_off.ensure(off.size());
        s |= dcombos.ensure(cmb.size());
        if (s) return MCE_ERR_NOMEM;
        MCE_CUDA(cudaMemcpy(dcombo_off.ptr, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice));
        MCE_CUDA(cudaMemcpy(dcombos.ptr, cmb.data(), cmb.size(), cudaMemcpyHostToDevice));
        hsteps.resize(E);
        return reset();
    }

    ~Engine() override
    {
        if (lc.stream) cudaStreamSynchronize(lc.stream);
        if (ftr_graph) Kernels<D>::ftr_graph_destroy(ftr_graph);
        if (ndw) nd_work_destroy(ndw);
        if (mstream) cudaStreamSynchronize(mstream);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (mstream) cudaStreamDestroy(mstream);
        for (cudaEvent_t ev : evpool) cudaEventDestroy(ev);
        if (lc.stream) cudaStreamDestroy(lc.stream);
    }

    void drain() override
    {
        if (lc.stream) cudaStreamSynchronize(lc.stream);
        if (mstream) cudaStreamSynchronize(mstream);
    }

    int upload_start(int e) override
    {
        MCE_CUDA(cudaMemcpy(dA0.ptr + (size_t)e * D * D, est[e].A0.data(), D * D * sizeof(double),
                            cudaMemcpyHostToDevice));
        MCE_CUDA(cudaMemcpy(dp0.ptr + (size_t)e * D, est[e].p0.data(), D * sizeof(double), cudaMemcpyHostToDevice));
        MCE_CUDA(cudaMemcpy(db0.ptr + (size_t)e * D, est[e].b0.data(), D * sizeof(double), cudaMemcpyHostToDevice));
        return MCE_OK;
    }

    int reset() override
    {
        std::vector<double> A0((size_t)E * D * D), p0((size_t)E * D), b0((size_t)E * D);
        for (int e = 0; e < E; e++) {
            memcpy(&A0[(size_t)e * D * D], est[e].A0.data(), D * D * sizeof(double));
            memcpy(&p0[(size_t)e * D], est[e].p0.data(), D * sizeof(double));
            memcpy(&b0[(size_t)e * D], est[e].b0.data(), D * sizeof(double));
            est[e].errors = 0;
            est[e].nt = 1;
            est[e].tps.assign(MC + 1, 0);
            est[e].tps[D] = 1;
        }
        MCE_CUDA(cudaMemcpy(dA0.ptr, A0.data(), A0.size() * sizeof(double), cudaMemcpyHostToDevice));
        MCE_CUDA(cudaMemcpy(dp0.ptr, p0.data(), p0.size() * sizeof(double), cudaMemcpyHostToDevice));
        MCE_CUDA(cudaMemcpy(db0.ptr, b0.data(), b0.size() * sizeof(double), cudaMemcpyHostToDevice));
        master_step = 0;
        nP = 0;
        post_mu_terms = 0;
        cpdf_step.assign(cpdf_step.size(), -1);  // the pdf caches belong to the old terms
        cpdf2_step.assign(cpdf2_step.size(), -1);
        device_errors = 0;
        MCE_CUDA(cudaMemset(counters.ptr, 0, 8 * sizeof(int)));
        return MCE_OK;
    }

    long long trim(long long min_bytes) override
    {
        if (master_step != 0) return MCE_ERR_ARG;
        if (min_bytes > 0 && trim_pass(false) < min_bytes) return 0;
        return trim_pass(true);
    }
    // the bytes the term-sized buffers hold; released when `release`
    long long trim_pass(bool release)
    {
        long long freed = 0;
        auto rel = [&freed, release](auto& buf) {
            freed += (long long)(buf.cap * sizeof(*buf.ptr));
            if (release) buf.release();
        };
        for (auto& P : Pb) {
            rel(P.est), rel(P.m), rel(P.m_old), rel(P.tab_cnt), rel(P.B_cnt), rel(P.nkids), rel(P.nkids_all);
            rel(P.bflip), rel(P.A), rel(P.p), rel(P.b), rel(P.tab_off), rel(P.B_off), rel(P.kscan);
        }
        for (auto& T : Tb) rel(T.keys), rel(T.vals);
        rel(Rb.est), rel(Rb.m), rel(Rb.pbc), rel(Rb.phc), rel(Rb.z), rel(Rb.lhp), rel(Rb.fam), rel(Rb.flags);
        rel(Rb.horthog), rel(Rb.A), rel(Rb.p), rel(Rb.q), rel(Rb.b), rel(Rb.cval), rel(Rb.dval), rel(Rb.ps2);
        rel(Rb.cmap), rel(Rb.csmap);
        rel(Bcap), rel(Bkeys), rel(kall_scan), rel(nvert), rel(voff), rel(vsv), rel(fam_mom), rel(mu_rows);
        rel(mu_ints), rel(bcount), rel(bfill), rel(boff), rel(slot_of), rel(cell_ent), rel(cell_ent2), rel(status);
        rel(owner), rel(ftr_wl[0]), rel(ftr_wl[1]), rel(ftr_resume), rel(gcnt), rel(gfill), rel(goff), rel(members);
        rel(members_tmp), rel(is_root), rel(cap), rel(rscan), rel(toff), rel(roots_list), rel(alive), rel(src);
        rel(tcnt), rel(g_nr), rel(g_items), rel(g_cells), rel(g_ioff), rel(g_coff), rel(g_rps2), rel(g_rflag);
        rel(g_minfo), rel(g_mps2), rel(g_mflag), rel(pr_root), rel(pr_mb), rel(pr_mcnt), rel(pr_cells);
        rel(pr_items), rel(pr_moff), rel(pr_ioff), rel(pr_coff), rel(pr_gv), rel(g_vals), rel(new_slot);
        rel(ptile_c), rel(pf_rows), rel(pf_zero);
        return freed;
    }

    // Packs one estimator's step parameters; Gamma pre-coalignment follows
    // precoalign_Gamma_beta (cauchy_util.hpp:128-210).
    void pack(int e, double msmt, const double* Phi, const double* Gamma, const double* beta, const double* H,
              double gamma, const double* B, const double* u, bool active, bool skip)
    {
        EstStep<D>& S = hsteps[e];
        memset(&S, 0, sizeof(S));
        S.msmt = msmt;
        S.gamma = gamma;
        S.active = active ? 1 : 0;
        S.skip = skip ? 1 : 0;
        memcpy(S.Phi, Phi, sizeof(double) * D * D);
        memcpy(S.H, H, sizeof(double) * D);
        if (cmcc > 0 && B && u) {
            for (int i = 0; i < D; i++) {
                double s = 0.0;
                for (int j = 0; j < cmcc; j++) s += B[i * cmcc + j] * u[j];
                S.Bu[i] = s;
            }
            S.has_control = 1;
        }
        const int n = pncc;
        for (int i = 0; i < n; i++) {
            for (int j = 0; j < D; j++) S.Gt[i * D + j] = Gamma[j * n + i];
            S.bt[i] = beta[i];
        }
        for (int i = 0; i < n; i++) {
            double nf = 0;
            for (int j = 0; j < D; j++) nf += fabs(S.Gt[i * D + j]);
            for (int j = 0; j < D; j++) S.Gt[i * D + j] /= nf;
            S.bt[i] *= nf;
        }
        bool F[kMaxGamma];
        for (int i = 0; i < n; i++) F[i] = true;
        for (int i = 0; i < n - 1; i++)
            if (F[i])
                for (int j = i + 1; j < n; j++)
                    if (F[j]) {
                        bool pos = true, neg = true;
                        for (int l = 0; l < D; l++) {
                            const double r = S.Gt[i * D + l], c = S.Gt[j * D + l];
                            if (pos) pos &= fabs(r - c) < kCoalignEps;
                            if (neg) neg &= fabs(r + c) < kCoalignEps;
                            if (!(pos || neg)) break;
                        }
                        if (pos || neg) {
                            F[j] = false;
                            S.bt[i] += S.bt[j];
                        }
                    }
        int cnt = 0;
        for (int i = 0; i < n; i++) cnt += F[i];
        if (cnt != n) {
            int uq = 1;
            for (int j = 1; j < n; j++)
                if (F[j]) {
                    if (uq < j) {
                        for (int l = 0; l < D; l++) S.Gt[uq * D + l] = S.Gt[j * D + l];
                        S.bt[uq] = S.bt[j];
                    }
                    uq++;
                }
        }
        S.gcnt = cnt;
    }

    int sync_and_check()
    {
        MCE_CUDA(cudaGetLastError());
        MCE_CUDA(cudaStreamSynchronize(lc.stream));
        if (ftr_graph) Kernels<D>::ftr_graph_collect(ftr_graph);
        int err = 0;
        MCE_CUDA(cudaMemcpy(&err, counters.ptr, sizeof(int), cudaMemcpyDeviceToHost));
        if (err) {
            device_errors |= err;
            set_error("device error bits " + std::to_string(err));
            return MCE_ERR_DEVICE;
        }
        return MCE_OK;
    }

    long long read_ll(const long long* p_)
    {
        long long v = 0;
        cudaMemcpyAsync(&v, p_, sizeof(long long), cudaMemcpyDeviceToHost, lc.stream);
        cudaStreamSynchronize(lc.stream);
        return v;
    }

    int step(const double* msmt, const double* Phi, const double* Gamma, const double* beta, const double* H,
             const double* gamma, const double* B, const double* u, int shared, int* err_out) override
    {
        using clk = std::chrono::steady_clock;
        const auto t0 = clk::now();
        const int ms = master_step;
        const int sub = ms % p;
        const bool with_tp = sub == 0;
        bool any_active = false;
        for (int e = 0; e < E; e++) {
            const EstHost& h = est[e];
            const bool done = ms >= h.num_updates;
            const bool blocked = (h.errors >> E_FZ_NEG) & 1;
            any_active |= !done && !blocked;
        }
        for_estimators([&](int a, int b) {
            for (int e = a; e < b; e++) {
                const EstHost& h = est[e];
                const bool done = ms >= h.num_updates;
                const bool blocked = (h.errors >> E_FZ_NEG) & 1;
                const bool active = !done && !blocked;
                const bool skip = active && ms == h.num_updates - 1;
                const size_t oe = shared ? 0 : (size_t)e;
                pack(e, msmt[e], Phi + oe * D * D, Gamma + oe * D * pncc, beta + oe * pncc, H + (size_t)e * D,
                     gamma[e], B ? B + oe * D * cmcc : nullptr, u ? u + (size_t)e * cmcc : nullptr, active, skip);
            }
        });
        bool any_done_past = true;
        for (int e = 0; e < E; e++)
            if (ms < est[e].num_updates) any_done_past = false;
        if (any_done_past) {
            set_error("master_step == num_estimation_steps: the estimator must be reset");
            return MCE_ERR_DONE;
        }
        MCE_CUDA(cudaMemcpyAsync(dsteps.ptr, hsteps.data(), sizeof(EstStep<D>) * E, cudaMemcpyHostToDevice,
                                 lc.stream));
        const auto t1 = clk::now();
        have_post = false;
        MCE_CUDA(cudaEventRecord(ev0, lc.stream));
        int rc = any_active ? (ms == 0 ? step_first() : step_main(with_tp)) : MCE_OK;
        if (rc != MCE_OK) return rc;
        MCE_CUDA(cudaEventRecord(ev1, lc.stream));
        rc = sync_and_check();
        if (rc != MCE_OK) return rc;
        float msf = 0;
        cudaEventElapsedTime(&msf, ev0, ev1);
        last_ms = msf;
        device_ms_total += msf;
        collect_prof();
        // moments of every active estimator
        const auto t2 = clk::now();
        finish_moments(ms);
        const auto t3 = clk::now();
        host_ms[0] += std::chrono::duration<double, std::milli>(t3 - t0).count();
        host_ms[1] += std::chrono::duration<double, std::milli>(t1 - t0).count();
        host_ms[2] += std::chrono::duration<double, std::milli>(t3 - t2).count();
        master_step++;
        if (err_out)
            for (int e = 0; e < E; e++) err_out[e] = est[e].errors;
        return MCE_OK;
    }

    void finish_moments(int ms)
    {
        for_estimators([&](int a, int b) { finish_moments_range(ms, a, b); });
    }

    void finish_moments_range(int ms, int a, int b)
    {
        const int NM = 1 + D + D * D;
        for (int e = a; e < b; e++) {
            const EstStep<D>& S = hsteps[e];
            if (!S.active) continue;
            EstHost& h = est[e];
            const cd* r = &h_raw[(size_t)e * NM];
            h.raw_fz[0] = r[0].re;
            h.raw_fz[1] = r[0].im;
            for (int j = 0; j < D; j++) {
                h.raw_mean[2 * j] = r[1 + j].re;
                h.raw_mean[2 * j + 1] = r[1 + j].im;
            }
            for (int j = 0; j < D * D; j++) {
                h.raw_cov[2 * j] = r[1 + D + j].re;
                h.raw_cov[2 * j + 1] = r[1 + D + j].im;
            }
            h.gscale = h_gscale[e];
            h.fz[0] = h.raw_fz[0];
            h.fz[1] = h.raw_fz[1];
            h.mean = h.raw_mean;
            h.cov = h.raw_cov;
            const bool post = have_post && h.print_basic_info;
            if (ms == 0) {
                // step_first reports through compute_moments without the checks
                if (post) post_ftr_report(h, e);
                else {
                    h.fz[0] = 1;
                    h.fz[1] = 0;
                }
                h.last_mean = h.mean;
                h.last_cov = h.cov;
                h.last_fz[0] = h.fz[0];
                h.last_fz[1] = h.fz[1];
                continue;
            }
            numeric_check(h, ms);
            if (!S.skip) {
                // after the tables are rebuilt fz is set to 1, or, with
                // print_basic_info, compute_moments(false) replaces fz, the
                // moments and G_SCALE_FACTOR (cauchy_estimator.hpp:1166-1177)
                if (post) post_ftr_report(h, e);
                else {
                    h.fz[0] = 1;
                    h.fz[1] = 0;
                }
            }
        }
    }

    void post_ftr_report(EstHost& h, int e)
    {
        const int NM = 1 + D + D * D;
        const cd* r = &h_pf_raw[(size_t)e * NM];
        h.fz[0] = r[0].re;
        h.fz[1] = r[0].im;
        for (int j = 0; j < D; j++) {
            h.mean[2 * j] = r[1 + j].re;
            h.mean[2 * j + 1] = r[1 + j].im;
        }
        for (int j = 0; j < D * D; j++) {
            h.cov[2 * j] = r[1 + D + j].re;
            h.cov[2 * j + 1] = r[1 + D + j].im;
        }
        h.gscale = h_pf_gscale[e];
    }

    void numeric_check(EstHost& h, int ms)
    {
        const int ph = ms % p;
        const bool first = ph == 0, not_last = ph != p - 1, last = ph == p - 1;
        if (first) {
            h.errors |= (1 << E_MEAN_DNE) | (1 << E_COV_DNE);
            h.errors &= ~((1 << E_MEAN_F) | (1 << E_MEAN_NF) | (1 << E_COV_NF) | (1 << E_COV_F));
        }
        int ne = 0;
        if (h.fz[0] <= 0) ne |= 1 << E_FZ_NEG;
        if (fabs(h.fz[1] / (1e-15 + h.fz[0])) > 1e-3) ne |= 1 << E_FZ_UNST;
        bool mean_ok = true;
        for (int i = 0; i < D; i++) {
            const double re = fabs(h.mean[2 * i]), im = fabs(h.mean[2 * i + 1]);
            if (im / (1e-15 + re) > 1e-1 || im > 0.001) {
                ne |= 1 << E_MEAN_ANY;
                if (not_last) ne |= 1 << E_MEAN_NF;
                if (last) ne |= 1 << E_MEAN_F;
                mean_ok = false;
            }
        }
        double cre[kMaxDim * kMaxDim], cim[kMaxDim * kMaxDim];
        for (int i = 0; i < D * D; i++) {
            cre[i] = h.cov[2 * i];
            cim[i] = h.cov[2 * i + 1];
        }
        bool cov_ok = true;
        if (cov_flags(cre, cim, D)) {
            ne |= 1 << E_COV_ANY;
            if (not_last) ne |= 1 << E_COV_NF;
            if (last) ne |= 1 << E_COV_F;
            cov_ok = false;
        }
        h.errors |= ne;
        if (mean_ok) h.errors &= ~(1 << E_MEAN_DNE);
        if (cov_ok) h.errors &= ~(1 << E_COV_DNE);
        if (mean_ok) h.last_mean = h.mean;
        else h.mean = h.last_mean;
        if (cov_ok) h.last_cov = h.cov;
        else h.cov = h.last_cov;
        if (!mean_ok && !cov_ok) {
            h.fz[0] = h.last_fz[0];
            h.fz[1] = h.last_fz[1];
        } else {
            h.last_fz[0] = h.fz[0];
            h.last_fz[1] = h.fz[1];
        }
    }

    // the engine's stream waits for the side stream's moments; then the
    // raw moments and G_SCALE_FACTOR are copied to the host
    int join_moments()
    {
        pbeg(KID_WAIT);
        MCE_CUDA(cudaStreamWaitEvent(lc.stream, ev_join, 0));
        pend();
        return read_moments();
    }

    int read_moments()
    {
        const int NM = 1 + D + D * D;
        MCE_CUDA(cudaMemcpyAsync(h_raw.data(), est_raw.ptr, sizeof(cd) * E * NM, cudaMemcpyDeviceToHost, lc.stream));
        MCE_CUDA(cudaMemcpyAsync(h_gscale.data(), gscale.ptr, sizeof(double) * E, cudaMemcpyDeviceToHost, lc.stream));
        return MCE_OK;
    }

    int step_first()
    {
        int s = first_cnt.ensure(E + 1);
        if (s) return s;
        pbeg(KID_FIRST);
        Kernels<D>::first_count(dA0.ptr, dsteps.ptr, E, first_cnt.ptr, lc);
        pend();
        std::vector<int> cnt(E);
        MCE_CUDA(cudaMemcpyAsync(cnt.data(), first_cnt.ptr, sizeof(int) * E, cudaMemcpyDeviceToHost, lc.stream));
        MCE_CUDA(cudaStreamSynchronize(lc.stream));
        hpstart.assign(E + 1, 0);
        for (int e = 0; e < E; e++) hpstart[e + 1] = hpstart[e] + cnt[e];
        nP = hpstart[E];
        PBufs& P = Pb[cur];
        if ((s = P.ensure(nP, MC))) return s;
        if ((s = Tb[cur].keys.ensure(nP << (D - 1)))) return s;
        if ((s = Tb[cur].vals.ensure(nP << (D - 1)))) return s;
        MCE_CUDA(cudaMemcpyAsync(dpstart.ptr, hpstart.data(), sizeof(long long) * (E + 1), cudaMemcpyHostToDevice,
                                 lc.stream));
        ParentList PV = P.view();
        pbeg(KID_FIRST);
        Kernels<D>::first_build(dA0.ptr, dp0.ptr, db0.ptr, dsteps.ptr, droots.ptr, E, dpstart.ptr, PV, MC,
                                est_raw.ptr, lc);
        // G_SCALE_FACTOR per estimator from the first moments
        k_gscale_from_raw(E);
        Kernels<D>::first_tables(PV, nP, reinterpret_cast<double*>(PV.kscan), reinterpret_cast<double*>(PV.B_off),
                                 reinterpret_cast<unsigned*>(PV.nkids), gscale.ptr, Tables{Tb[cur].keys.ptr,
                                 Tb[cur].vals.ptr}, MC, lc);
        pend();
        read_moments();
        for (int e = 0; e < E; e++) {
            est[e].nt = cnt[e];
            est[e].tps.assign(MC + 1, 0);
            est[e].tps[D] = cnt[e];
            post_mu_terms += cnt[e];
        }
        return post_ftr_moments(true);
    }

    void k_gscale_from_raw(int E_);

    int step_main(bool with_tp)
    {
        int s;
        PBufs& P = Pb[cur];
        PBufs& Pn = Pb[cur ^ 1];
        ParentList PV = P.view();
        Tables Told{Tb[cur].keys.ptr, Tb[cur].vals.ptr};
        int* err = counters.ptr;
        // a step that ended early on an error may have left moments running
        MCE_CUDA(cudaStreamWaitEvent(lc.stream, ev_join, 0));
        if ((s = Bcap.ensure(nP + 1))) return s;
        if ((s = nvert.ensure(nP + 1))) return s;
        if ((s = voff.ensure(nP + 2))) return s;
        if ((s = kall_scan.ensure(nP + 2))) return s;

        if ((s = ensure_scan_scratch(nP + 1))) return s;
        pbeg(KID_TP);
        Kernels<D>::tp(PV, nP, dsteps.ptr, with_tp ? 1 : 0, MC, Bcap.ptr, nvert.ptr, err, lc);
        pend();
        pbeg(KID_SCAN);
        scan_int_to_ll(PV.nkids, PV.kscan, nP, ss, lc);
        scan_int_to_ll(Bcap.ptr, PV.B_off, nP, ss, lc);
        scan_int_to_ll(PV.nkids_all, kall_scan.ptr, nP, ss, lc);
        scan_int_to_ll(nvert.ptr, voff.ptr, nP, ss, lc);
        pend();
        long long tot[4] = {0, 0, 0, 0};
        MCE_CUDA(cudaMemcpyAsync(&tot[0], PV.kscan + nP, sizeof(long long), cudaMemcpyDeviceToHost, lc.stream));
        MCE_CUDA(cudaMemcpyAsync(&tot[1], PV.B_off + nP, sizeof(long long), cudaMemcpyDeviceToHost, lc.stream));
        MCE_CUDA(cudaMemcpyAsync(&tot[2], kall_scan.ptr + nP, sizeof(long long), cudaMemcpyDeviceToHost, lc.stream));
        MCE_CUDA(cudaMemcpyAsync(&tot[3], voff.ptr + nP, sizeof(long long), cudaMemcpyDeviceToHost, lc.stream));
        // per-estimator post-MU counts for the un-reduced final MU
        std::vector<long long> kall_at(E + 1, 0);
        MCE_CUDA(cudaStreamSynchronize(lc.stream));
        const long long K = tot[0], Btot = tot[1], Kall = tot[2], Nvert = tot[3];
        const long long nR = nP + K;
        post_mu_terms += nP + Kall;
        if ((s = fam_mom.ensure((size_t)(nP + Kall + 1) * (1 + D + D * D)))) return s;
        if ((s = Bkeys.ensure(Btot + 1))) return s;
        if ((s = vsv.ensure(Nvert + 1))) return s;
        if ((s = Rb.ensure(nR, MC))) return s;
        pbeg(KID_BUILD_B);
        Kernels<D>::build_B(PV, nP, dsteps.ptr, with_tp ? 1 : 0, Told, Bkeys.ptr, Btot, dbpert.ptr, MC,
                            dcombo_off.ptr, dcombos.ptr, voff.ptr, Nvert, vsv.ptr, err, lc);
        pend();
        TermRecs R = Rb.view();
        if ((s = mu_rows.ensure((size_t)(nP + 1) * ((MC + 1) * (D + 1) + 1)))) return s;
        if ((s = mu_ints.ensure((size_t)(nP + 1) * 4))) return s;
        pbeg(KID_MU);
        Kernels<D>::mu(PV, nP, dsteps.ptr, dpstart.ptr, droots.ptr, Told, Bkeys.ptr, R, nR, kall_scan.ptr, nP + Kall,
                       mu_rows.ptr, mu_ints.ptr, fam_mom.ptr, MC, err, lc);
        pend();
        // the moment chains (and G_SCALE_FACTOR) on the side stream: the term
        // reduction below does not read them; the g-table evaluation does, so
        // the engine's stream waits for them before it (join_moments)
        // a chain's length follows its estimator's parent count: chains
        // start longest first, so that the longest does not wait for a
        // later wave of blocks
        const int* order = nullptr;
        if (E > 1) {
            h_order.resize(E);
            for (int e = 0; e < E; e++) h_order[e] = e;
            std::stable_sort(h_order.begin(), h_order.end(), [&](int x, int y) {
                return hpstart[x + 1] - hpstart[x] > hpstart[y + 1] - hpstart[y];
            });
            if ((s = d_order.ensure(E))) return s;
            MCE_CUDA(cudaMemcpyAsync(d_order.ptr, h_order.data(), sizeof(int) * E, cudaMemcpyHostToDevice,
                                     lc.stream));
            order = d_order.ptr;
        }
        MCE_CUDA(cudaEventRecord(ev_fork, lc.stream));
        MCE_CUDA(cudaStreamWaitEvent(mstream, ev_fork, 0));
        {
            LaunchCfg lcm = lc;
            lcm.stream = mstream;
            pbeg(KID_MOMENTS, mstream);
            Kernels<D>::moments(fam_mom.ptr, dpstart.ptr, kall_scan.ptr, E, order, dsteps.ptr, mom_tot.ptr,
                                est_raw.ptr, gscale.ptr, lcm);
            pend(mstream);
        }
        MCE_CUDA(cudaEventRecord(ev_join, mstream));
        // terms after the MU per estimator (un-reduced count, cauchy_estimator.hpp:749-751, 806-812)
        if ((s = kall_est.ensure(E + 2))) return s;
        pbeg(KID_SCAN);
        k_gather_bounds(kall_scan.ptr, E);
        pend();
        MCE_CUDA(cudaMemcpyAsync(kall_at.data(), kall_est.ptr, sizeof(long long) * (E + 1), cudaMemcpyDeviceToHost,
                                 lc.stream));
        // shapes of the final-MU estimators (terms_per_shape of the parents' shapes)
        std::vector<int> skip_hist;
        bool any_skip = false, any_keep = false;
        for (int e = 0; e < E; e++) {
            if (hsteps[e].active && hsteps[e].skip) any_skip = true;
            if (hsteps[e].active && !hsteps[e].skip) any_keep = true;
        }
        const int MCp = MC + 1;
        if (any_skip) {
            if ((s = hist.ensure((size_t)E * MCp))) return s;
            if (!any_keep) {
                // every estimator ends its step here: the step waits for its
                // moment chains in any case, so the wait is taken (and timed)
                // before the shape histogram rather than behind it
                pbeg(KID_WAIT);
                MCE_CUDA(cudaStreamWaitEvent(lc.stream, ev_join, 0));
                pend();
            }
            MCE_CUDA(cudaMemsetAsync(hist.ptr, 0, sizeof(int) * E * MCp, lc.stream));
            pbeg(KID_PARTITION);
            k_skip_hist(PV, nP, MCp);
            pend();
            skip_hist.resize((size_t)E * MCp);
            MCE_CUDA(cudaMemcpyAsync(skip_hist.data(), hist.ptr, sizeof(int) * E * MCp, cudaMemcpyDeviceToHost,
                                     lc.stream));
        }
        MCE_CUDA(cudaStreamSynchronize(lc.stream));
        for (int e = 0; e < E; e++) {
            if (!hsteps[e].active) continue;
            if (hsteps[e].skip) {
                est[e].nt = (hpstart[e + 1] - hpstart[e]) + (kall_at[e + 1] - kall_at[e]);
                est[e].tps.assign(MCp, 0);
                for (int m = 0; m < MCp; m++) est[e].tps[m] = skip_hist[(size_t)e * MCp + m];
            }
        }
        if (prof_mode >= 2) alg_stats(with_tp, nR, false);
        if (!any_keep || nR == 0) {
            // every estimator that stepped has now finished
            if ((s = join_moments())) return s;
            nP = 0;
            std::vector<long long> z(E + 1, 0);
            hpstart = z;
            return MCE_OK;
        }
        // ---- fast term reduction
        long long H = 1;
        while (H < nR) H <<= 1;
        if ((s = bcount.ensure(H + 1))) return s;
        if ((s = bfill.ensure(H + 1))) return s;
        if ((s = boff.ensure(H + 2))) return s;
        if ((s = slot_of.ensure(nR + 1))) return s;
        if ((s = cell_ent.ensure((nR + 1) * Kernels<D>::cell_entry_bytes()))) return s;
        if ((s = cell_ent2.ensure((nR + 1) * Kernels<D>::cell_entry_bytes()))) return s;
        if ((s = status.ensure(nR + 1))) return s;
        if ((s = owner.ensure(nR + 1))) return s;
        if ((s = ensure_scan_scratch(std::max(nR, H) + 1))) return s;
        MCE_CUDA(cudaMemsetAsync(bcount.ptr, 0, sizeof(int) * H, lc.stream));
        MCE_CUDA(cudaMemsetAsync(bfill.ptr, 0, sizeof(int) * H, lc.stream));
        pbeg(KID_FTR);
        Kernels<D>::ftr_cells(R, nR, H - 1, slot_of.ptr, bcount.ptr, lc);
        pend();
        pbeg(KID_SCAN);
        scan_int_to_ll(bcount.ptr, boff.ptr, H, ss, lc);
        pend();
        const long long nent = nvalid_entries(H);  // bucket entries = valid records
        pbeg(KID_FTR);
        Kernels<D>::ftr_scatter(R, nR, slot_of.ptr, boff.ptr, bfill.ptr, cell_ent.ptr, lc);
        // sort each bucket by term index
        Kernels<D>::ftr_sort(cell_ent.ptr, nent, slot_of.ptr, boff.ptr, cell_ent2.ptr, lc);
        k_status_init(R, nR);
        pend();
        if ((s = ftr_wl[0].ensure(nR + 1))) return s;
        if ((s = ftr_wl[1].ensure(nR + 1))) return s;
        if ((s = ftr_resume.ensure((size_t)(nR + 1) * kFtrResume))) return s;
        // resolution rounds, queued kFtrBatch at a time (the first batch
        // kFtrFirstBatch): a round reads the previous round's worklist length
        // on the device, a round after the last is empty, and the host reads
        // the count once per batch
        if ((s = ftr_cnt.ensure(kFtrCntSlots))) return s;
        // the first round over every record as an ordinary (full-occupancy)
        // launch; the rounds after it as ftr_rounds_mode() says: queued in
        // batches, the host reading the worklist length once per batch; in one
        // persistent cooperative launch over the device worklists; or as a
        // device-side loop in a CUDA graph (neither of the last two has a host
        // round trip).  The no-allocation step runs the batched rounds.
        MCE_CUDA(cudaMemsetAsync(ftr_cnt.ptr, 0, sizeof(int) * kFtrCntSlots, lc.stream));
        pbeg(KID_FTR);
        Kernels<D>::ftr_resolve(R, nR, cell_ent2.ptr, boff.ptr, H - 1, MC, status.ptr, owner.ptr, nullptr, nullptr,
                                nR, ftr_wl[0].ptr, ftr_cnt.ptr, ftr_resume.ptr, lc);
        const int fmode = ftr_rounds_mode();
        int pst = MCE_ERR_ARG;
        if (fmode == 1)
            pst = Kernels<D>::ftr_resolve_all(R, nR, cell_ent2.ptr, boff.ptr, H - 1, MC, status.ptr, owner.ptr,
                                              ftr_wl[0].ptr, ftr_wl[1].ptr, ftr_cnt.ptr, ftr_resume.ptr,
                                              reinterpret_cast<unsigned*>(ftr_cnt.ptr + 4), 1, kFtrMaxRounds, err,
                                              lc);
        else if (fmode == 2 && !g_device_alloc_forbidden) {
            if (!ftr_graph && Kernels<D>::ftr_graph_create(&ftr_graph, lc) != MCE_OK) {
                set_error("the CUDA graph of the term reduction's rounds could not be built");
                return MCE_ERR_CUDA;
            }
            pst = Kernels<D>::ftr_graph_launch(ftr_graph, R, nR, cell_ent2.ptr, boff.ptr, H - 1, MC, status.ptr,
                                               owner.ptr, ftr_wl[0].ptr, ftr_wl[1].ptr, ftr_cnt.ptr, ftr_resume.ptr,
                                               kFtrMaxRounds, err, lc);
            if (pst != MCE_OK) {
                set_error("launching the CUDA graph of the term reduction's rounds failed");
                return MCE_ERR_CUDA;
            }
        }
        pend();
        int unk = 0;
        long long bound = nR;
        for (int round = 1; pst != MCE_OK;) {
            // the rounds after the first queued in batches (round r counts
            // into ftr_cnt[r % 8])
            const int K = round == 1 ? kFtrFirstBatch - 1 : kFtrBatch;
            pbeg(KID_FTR);
            for (int q = 0; q < K; q++, round++) {
                int* n_out = ftr_cnt.ptr + round % kFtrCntSlots;
                MCE_CUDA(cudaMemsetAsync(n_out, 0, sizeof(int), lc.stream));
                Kernels<D>::ftr_resolve(R, nR, cell_ent2.ptr, boff.ptr, H - 1, MC, status.ptr, owner.ptr,
                                        round ? ftr_wl[(round - 1) & 1].ptr : nullptr,
                                        round ? ftr_cnt.ptr + (round - 1) % kFtrCntSlots : nullptr, bound,
                                        ftr_wl[round & 1].ptr, n_out, ftr_resume.ptr, lc);
            }
            pend();
            MCE_CUDA(cudaMemcpyAsync(&unk, ftr_cnt.ptr + (round - 1) % kFtrCntSlots, sizeof(int),
                                     cudaMemcpyDeviceToHost, lc.stream));
            MCE_CUDA(cudaStreamSynchronize(lc.stream));
            if (unk == 0) break;
            bound = unk;
            if (round > 100000) {
                set_error("term reduction did not converge");
                device_errors |= kErrResolveStalled;
                return MCE_ERR_DEVICE;
            }
        }
        // ---- reduction groups
        if ((s = gcnt.ensure(nR + 1))) return s;
        if ((s = gfill.ensure(nR + 1))) return s;
        if ((s = goff.ensure(nR + 2))) return s;
        MCE_CUDA(cudaMemsetAsync(gcnt.ptr, 0, sizeof(int) * (nR + 1), lc.stream));
        MCE_CUDA(cudaMemsetAsync(gfill.ptr, 0, sizeof(int) * (nR + 1), lc.stream));
        pbeg(KID_GROUPS);
        group_count(status.ptr, owner.ptr, nR, gcnt.ptr, lc);
        scan_int_to_ll(gcnt.ptr, goff.ptr, nR, ss, lc);
        pend();
        // each record is a member of at most one group: nR bounds the
        // members, so their buffers are sized without reading the count back
        const long long nmembers = nR;
        if ((s = members.ensure(nmembers + 1))) return s;
        if ((s = members_tmp.ensure(nmembers + 1))) return s;
        pbeg(KID_GROUPS);
        group_fill(status.ptr, owner.ptr, nR, goff.ptr, gfill.ptr, members_tmp.ptr, lc);
        group_sort(gcnt.ptr, goff.ptr, nR, members_tmp.ptr, members.ptr, lc);
        pend();
        if ((s = is_root.ensure(nR + 1))) return s;
        if ((s = cap.ensure(nR + 1))) return s;
        if ((s = rscan.ensure(nR + 2))) return s;
        if ((s = toff.ensure(nR + 2))) return s;
        pbeg(KID_GROUPS);
        roots_flags(status.ptr, Rb.m.ptr, nR, D, is_root.ptr, cap.ptr, lc);
        scan_int_to_ll(is_root.ptr, rscan.ptr, nR, ss, lc);
        scan_int_to_ll(cap.ptr, toff.ptr, nR, ss, lc);
        pend();
        long long t2[2];
        MCE_CUDA(cudaMemcpyAsync(&t2[0], rscan.ptr + nR, sizeof(long long), cudaMemcpyDeviceToHost, lc.stream));
        MCE_CUDA(cudaMemcpyAsync(&t2[1], toff.ptr + nR, sizeof(long long), cudaMemcpyDeviceToHost, lc.stream));
        MCE_CUDA(cudaStreamSynchronize(lc.stream));
        const long long nroots = t2[0], ttot = t2[1];
        if ((s = roots_list.ensure(nroots + 1))) return s;
        pbeg(KID_GROUPS);
        mce::roots_list(is_root.ptr, rscan.ptr, nR, roots_list.ptr, lc);
        pend();
        TBufs& Tn = Tb[cur ^ 1];
        if ((s = Tn.keys.ensure(ttot + 1))) return s;
        if ((s = Tn.vals.ensure(ttot + 1))) return s;
        if ((s = alive.ensure(nR + 1))) return s;
        if ((s = src.ensure(nR + 1))) return s;
        if ((s = tcnt.ensure(nR + 1))) return s;
        MCE_CUDA(cudaMemsetAsync(alive.ptr, 0, sizeof(int) * (nR + 1), lc.stream));
        // cells a group may hold: a central arrangement in general position
        // has at most half_cells_cap(m, d) half-cells; nearly degenerate
        // arrangements can yield more, found by the preparation below
        int capR = half_cells_cap(MC, D);
        lc.cells_cap = capR;
        // flat evaluation: cells and orientations, item offsets, the items
        if ((s = g_nr.ensure(nroots + 1))) return s;
        if ((s = g_items.ensure(nroots + 1))) return s;
        if ((s = g_cells.ensure(nroots + 1))) return s;
        if ((s = g_ioff.ensure(nroots + 2))) return s;
        if ((s = g_coff.ensure(nroots + 2))) return s;
        if ((s = g_rps2.ensure(nroots + 1))) return s;
        if ((s = g_rflag.ensure(nroots + 1))) return s;
        if ((s = g_minfo.ensure(nmembers + 1))) return s;
        if ((s = g_mps2.ensure(nmembers + 1))) return s;
        if ((s = g_mflag.ensure(nmembers + 1))) return s;
        if ((s = ensure_scan_scratch(nroots + 1))) return s;
        if ((s = pr_root.ensure(nroots + 1))) return s;
        if ((s = pr_mb.ensure(nroots + 1))) return s;
        if ((s = pr_mcnt.ensure(nroots + 1))) return s;
        if ((s = pr_cells.ensure(nroots + 1))) return s;
        if ((s = pr_items.ensure(nroots + 1))) return s;
        if ((s = pr_moff.ensure(nroots + 2))) return s;
        if ((s = pr_ioff.ensure(nroots + 2))) return s;
        if ((s = pr_coff.ensure(nroots + 2))) return s;
        GFlat gf{g_nr.ptr,    g_ioff.ptr,    g_rps2.ptr,    g_rflag.ptr,  g_minfo.ptr,  g_mps2.ptr,
                 g_mflag.ptr, nullptr,       pr_root.ptr,   pr_mb.ptr,    pr_mcnt.ptr,  pr_cells.ptr,
                 pr_items.ptr, pr_moff.ptr,  pr_ioff.ptr,   pr_coff.ptr,  nullptr};
        Tables Tnv{Tn.keys.ptr, Tn.vals.ptr};
        long long gt[2] = {0, 0};
        for (int attempt = 0;; attempt++) {
            MCE_CUDA(cudaMemsetAsync(g_over.ptr, 0, 2 * sizeof(int), lc.stream));
            pbeg(KID_GTABLE);
            Kernels<D>::gtable_prep(R, roots_list.ptr, nroots, gcnt.ptr, goff.ptr, members.ptr, PV, Told, Bkeys.ptr,
                                    toff.ptr, Tnv, gf, g_items.ptr, g_cells.ptr, MC, cap.ptr, g_over.ptr, lc);
            scan_int_to_ll(g_items.ptr, g_ioff.ptr, nroots, ss, lc);
            scan_int_to_ll(g_cells.ptr, g_coff.ptr, nroots, ss, lc);
            pend();
            int ov[2] = {0, 0};
            if (nroots > 0) {
                MCE_CUDA(cudaMemcpyAsync(&gt[0], g_ioff.ptr + nroots, sizeof(long long), cudaMemcpyDeviceToHost,
                                         lc.stream));
                MCE_CUDA(cudaMemcpyAsync(&gt[1], g_coff.ptr + nroots, sizeof(long long), cudaMemcpyDeviceToHost,
                                         lc.stream));
                MCE_CUDA(cudaMemcpyAsync(ov, g_over.ptr, 2 * sizeof(int), cudaMemcpyDeviceToHost, lc.stream));
                MCE_CUDA(cudaStreamSynchronize(lc.stream));
            }
            if (!ov[0]) break;
            if (attempt > 0) {
                device_errors |= kErrRootCellsOverflow;
                set_error("g-table preparation: a root's cells still exceed its re-sized slot");
                return MCE_ERR_DEVICE;
            }
            // roots with more cells than the general-position count: their
            // slots (cap[r] now holds their counts) and the cells capacity grow
            if (ov[1] > capR) capR = ov[1];
            lc.cells_cap = capR;
            scan_int_to_ll(cap.ptr, toff.ptr, nR, ss, lc);
            long long tt = 0;
            MCE_CUDA(cudaMemcpyAsync(&tt, toff.ptr + nR, sizeof(long long), cudaMemcpyDeviceToHost, lc.stream));
            MCE_CUDA(cudaStreamSynchronize(lc.stream));
            if ((s = Tn.keys.ensure(tt + 1))) return s;
            if ((s = Tn.vals.ensure(tt + 1))) return s;
            Tnv = Tables{Tn.keys.ptr, Tn.vals.ptr};
            if (MC > kSmemBitmapRows && lc.gbits) {
                if ((s = gbits.ensure((size_t)(lc.gbits_warps * gtable_bitmap_words(MC, D, capR))))) return s;
                lc.gbits = gbits.ptr;
            }
        }
        cd* gscr = nullptr;
        long long gscr_warps = 0;  // 0: the handle's buffer holds a warp slot for every launched warp
        if (fixed_gtable_scratch) {
            gscr = static_cast<cd*>(fixed_gtable_scratch);
            gscr_warps = (long long)(fixed_gtable_scratch_bytes / (sizeof(cd) * capR));
            if (gscr_warps < 4) {
                set_error("the fixed g-table scratch holds fewer than 4 warps' cells for this step");
                return MCE_ERR_NOMEM;
            }
        } else {
            const long long max_warps = (long long)lc.num_sms * 16 * 4;
            if ((s = scratch.ensure((size_t)max_warps * capR))) return s;
            gscr = scratch.ptr;
        }
        const long long nitems = gt[0], ncells = gt[1];
        if ((s = g_vals.ensure(nitems + 1))) return s;
        gf.gv = g_vals.ptr;
        if ((s = join_moments())) return s;
        pbeg(KID_GTABLE);
        Kernels<D>::gtable_eval(R, roots_list.ptr, nroots, nitems, goff.ptr, members.ptr, PV, Told, Bkeys.ptr,
                                gscale.ptr, toff.ptr, Tnv, gf, MC, lc);
        Kernels<D>::gtable_combine(R, roots_list.ptr, nroots, g_coff.ptr, ncells, gcnt.ptr, goff.ptr, members.ptr, PV,
                                   Told, Bkeys.ptr, toff.ptr, Tnv, tcnt.ptr, alive.ptr, src.ptr, gf, MC, lc);
        MCE_CUDA(cudaMemsetAsync(pr_mcnt.ptr, 0, sizeof(int) * (nroots + 1), lc.stream));
        MCE_CUDA(cudaMemsetAsync(pr_cells.ptr, 0, sizeof(int) * (nroots + 1), lc.stream));
        MCE_CUDA(cudaMemsetAsync(pr_items.ptr, 0, sizeof(int) * (nroots + 1), lc.stream));
        Kernels<D>::gtable(R, roots_list.ptr, nroots, gcnt.ptr, goff.ptr, members.ptr, PV, Told, Bkeys.ptr, gscale.ptr,
                           toff.ptr, Tnv, tcnt.ptr, alive.ptr, src.ptr, gscr, capR, gf, MC, err, lc, gscr_warps);
        // members left after promotions: the promoted-root flat pass
        scan_int_to_ll(pr_mcnt.ptr, pr_moff.ptr, nroots, ss, lc);
        scan_int_to_ll(pr_items.ptr, pr_ioff.ptr, nroots, ss, lc);
        scan_int_to_ll(pr_cells.ptr, pr_coff.ptr, nroots, ss, lc);
        pend();
        long long pt[3] = {0, 0, 0};
        if (nroots > 0) {
            MCE_CUDA(cudaMemcpyAsync(&pt[0], pr_moff.ptr + nroots, sizeof(long long), cudaMemcpyDeviceToHost,
                                     lc.stream));
            MCE_CUDA(cudaMemcpyAsync(&pt[1], pr_ioff.ptr + nroots, sizeof(long long), cudaMemcpyDeviceToHost,
                                     lc.stream));
            MCE_CUDA(cudaMemcpyAsync(&pt[2], pr_coff.ptr + nroots, sizeof(long long), cudaMemcpyDeviceToHost,
                                     lc.stream));
            MCE_CUDA(cudaStreamSynchronize(lc.stream));
        }
        if (pt[1] > 0) {
            if ((s = pr_gv.ensure(pt[1] + 1))) return s;
            gf.pr_gv = pr_gv.ptr;
            pbeg(KID_GTABLE);
            Kernels<D>::gtable_promoted(R, roots_list.ptr, nroots, pt[0], pt[1], pt[2], members.ptr, PV, Told,
                                        Bkeys.ptr, gscale.ptr, toff.ptr, Tnv, gf, MC, lc);
            pend();
        }
        if (prof_mode >= 2) alg_stats(with_tp, nR, true);
        // ---- next parent list
        if ((s = hist.ensure((size_t)E * MCp))) return s;
        if ((s = bucket_off.ensure((size_t)E * MCp + 2))) return s;
        if ((s = new_slot.ensure(nR + 1))) return s;
        if ((s = rbase.ensure(E + 2))) return s;
        if ((s = ptile_n.ensure(E + 1))) return s;
        if ((s = ptile_start.ensure(E + 2))) return s;
        if ((s = ptile_c.ensure((size_t)partition_tiles_cap(nR, E) * MCp + 1))) return s;
        if ((s = ensure_scan_scratch((long long)E * MCp + 1))) return s;
        pbeg(KID_PARTITION);
        rbase_kernel(dpstart.ptr, PV.kscan, E, rbase.ptr, lc);
        partition_tiles(alive.ptr, Rb.m.ptr, rbase.ptr, E, MCp, nR, ptile_n.ptr, ptile_start.ptr, ptile_c.ptr,
                        hist.ptr, ss, lc);
        scan_int_to_ll(hist.ptr, bucket_off.ptr, (long long)E * MCp, ss, lc);
        partition_rank(alive.ptr, Rb.m.ptr, rbase.ptr, E, MCp, nR, ptile_start.ptr, ptile_c.ptr, bucket_off.ptr,
                       new_slot.ptr, lc);
        pend();
        h_hist.resize((size_t)E * MCp);
        MCE_CUDA(cudaMemcpyAsync(h_hist.data(), hist.ptr, sizeof(int) * E * MCp, cudaMemcpyDeviceToHost, lc.stream));
        MCE_CUDA(cudaStreamSynchronize(lc.stream));
        std::vector<long long> np(E + 1, 0);
        for (int e = 0; e < E; e++) {
            long long c = 0;
            for (int m = 0; m < MCp; m++) c += h_hist[(size_t)e * MCp + m];
            np[e + 1] = np[e] + c;
        }
        const long long nPn = np[E];
        if ((s = Pn.ensure(nPn, MC))) return s;
        ParentList PnV = Pn.view();
        pbeg(KID_PARTITION);
        Kernels<D>::compact(R, alive.ptr, src.ptr, nR, new_slot.ptr, toff.ptr, tcnt.ptr, PnV, MC, lc);
        pend();
        for (int e = 0; e < E; e++) {
            if (!hsteps[e].active || hsteps[e].skip) continue;
            est[e].nt = np[e + 1] - np[e];
            est[e].tps.assign(MCp, 0);
            for (int m = 0; m < MCp; m++) est[e].tps[m] = h_hist[(size_t)e * MCp + m];
        }
        hpstart = np;
        MCE_CUDA(cudaMemcpyAsync(dpstart.ptr, hpstart.data(), sizeof(long long) * (E + 1), cudaMemcpyHostToDevice,
                                 lc.stream));
        nP = nPn;
        cur ^= 1;
        return post_ftr_moments(false);
    }

    // compute_moments(false) for the estimators that set print_basic_info
    // (cauchy_estimator.hpp:1166-1177, 1197-1203) over the current terms
    int post_ftr_moments(bool first)
    {
        have_post = false;
        bool any = false;
        for (int e = 0; e < E; e++)
            if (est[e].print_basic_info && hsteps[e].active && (first || !hsteps[e].skip)) any = true;
        if (!any) return MCE_OK;
        constexpr int NM = 1 + D + D * D;
        int s;
        if ((s = pf_rows.ensure((size_t)(nP + 1) * NM))) return s;
        if ((s = pf_zero.ensure(nP + 2))) return s;
        if ((s = pf_tot.ensure((size_t)E * 2 * NM))) return s;
        if ((s = pf_raw.ensure((size_t)E * NM))) return s;
        if ((s = pf_gscale.ensure(E))) return s;
        MCE_CUDA(cudaMemsetAsync(pf_zero.ptr, 0, sizeof(long long) * (nP + 2), lc.stream));
        Kernels<D>::post_ftr_terms(Pb[cur].view(), nP, droots.ptr, Tables{Tb[cur].keys.ptr, Tb[cur].vals.ptr}, MC,
                                   pf_rows.ptr, lc);
        Kernels<D>::moments(pf_rows.ptr, dpstart.ptr, pf_zero.ptr, E, nullptr, dsteps.ptr, pf_tot.ptr, pf_raw.ptr,
                            pf_gscale.ptr, lc);
        h_pf_raw.resize((size_t)E * NM);
        h_pf_gscale.resize(E);
        MCE_CUDA(cudaMemcpyAsync(h_pf_raw.data(), pf_raw.ptr, sizeof(cd) * E * NM, cudaMemcpyDeviceToHost,
                                 lc.stream));
        MCE_CUDA(cudaMemcpyAsync(h_pf_gscale.data(), pf_gscale.ptr, sizeof(double) * E, cudaMemcpyDeviceToHost,
                                 lc.stream));
        MCE_CUDA(cudaStreamSynchronize(lc.stream));
        have_post = true;
        return MCE_OK;
    }

    int ensure_scan_scratch(long long n)
    {
        long long need = 4;
        long long t = n;
        while (t > 1) {
            t = (t + 2047) / 2048;
            need += t + 2;
        }
        int s = scan_tmp.ensure(need + 64);
        if (s) return s;
        ss.block_sums = scan_tmp.ptr;
        ss.cap = (long long)scan_tmp.cap;
        return MCE_OK;
    }

    void k_skip_hist(ParentList PV, long long n, int MCp);
    void k_gather_bounds(const long long* scan, int E_);
    void k_status_init(TermRecs R, long long nR);

    // ---- extended-mode helpers (cauchy_estimator.hpp:1312-1394)
    DevBuf<double> ext_buf;

    int shift_terms_b(int e, const double* v, int sub) override
    {
        if (e < 0 || e >= E || !v) return MCE_ERR_ARG;
        int s;
        if ((s = ext_buf.ensure(D))) return s;
        MCE_CUDA(cudaMemcpyAsync(ext_buf.ptr, v, sizeof(double) * D, cudaMemcpyHostToDevice, lc.stream));
        const long long a = hpstart.empty() ? 0 : hpstart[e], n = hpstart.empty() ? 0 : hpstart[e + 1] - a;
        Kernels<D>::shift_b(Pb[cur].view(), a, n, ext_buf.ptr, sub, lc);
        MCE_CUDA(cudaStreamSynchronize(lc.stream));
        return MCE_OK;
    }

    int time_prop_terms(int e, const double* Phi, const double* Bu) override
    {
        if (e < 0 || e >= E || !Phi) return MCE_ERR_ARG;
        int s;
        if ((s = ext_buf.ensure(D * D + D))) return s;
        MCE_CUDA(cudaMemcpyAsync(ext_buf.ptr, Phi, sizeof(double) * D * D, cudaMemcpyHostToDevice, lc.stream));
        if (Bu)
            MCE_CUDA(cudaMemcpyAsync(ext_buf.ptr + D * D, Bu, sizeof(double) * D, cudaMemcpyHostToDevice, lc.stream));
        const long long a = hpstart.empty() ? 0 : hpstart[e], n = hpstart.empty() ? 0 : hpstart[e + 1] - a;
        Kernels<D>::det_tp(Pb[cur].view(), a, n, ext_buf.ptr, Bu ? ext_buf.ptr + D * D : nullptr, MC, lc);
        MCE_CUDA(cudaStreamSynchronize(lc.stream));
        return MCE_OK;
    }

    // ---- marginal 2-D pdf: CauchyCPDFGridDispatcher2D (cpdf_ndim.hpp:1774-1919)
    // over PointWiseNDimCauchyCPDF::evaluate_2D_marginal_cpdf (:1356-1455), with
    // the reference's per-term cache kept on the device, keyed by (master step,
    // the two indices) and, as for the 1-D pdf, the term count
    std::vector<int> cpdf2_step, cpdf2_i1, cpdf2_i2;
    std::vector<long long> cpdf2_n;
    std::vector<std::unique_ptr<DevBuf<double>>> cpdf2_tt;
    DevBuf<double> cpdf2_x, cpdf2_y, cpdf2_z;

    int cpdf_2d_grid(int e, int i1, int i2, const double* bar_nu, double lx, double hx, double rx, double ly,
                     double hy, double ry, int reset_cache, int max_points, double* xs, double* ys,
                     double* zs) override
    {
        if (e < 0 || e >= E || i1 < 0 || i1 >= i2 || i2 >= D || !bar_nu) return MCE_ERR_ARG;
        if (!(hx > lx) || !(rx > 0) || !(hy > ly) || !(ry > 0)) return MCE_ERR_ARG;
        const double sx = (hx - lx + rx - 1e-15) / rx, sy = (hy - ly + ry - 1e-15) / ry;
        if (!(sx < 1e6) || !(sy < 1e6)) {
            set_error("cpdf grid: too many points");
            return MCE_ERR_ARG;
        }
        const int nx = (int)sx + 1, ny = (int)sy + 1;  // reset_grid, cpdf_ndim.hpp:1816-1845
        if ((long long)nx * ny > 100000000LL) {
            set_error("cpdf grid: too many points");
            return MCE_ERR_ARG;
        }
        const int npts = nx * ny;
        if (!xs || !ys || !zs) return npts;
        if (npts > max_points) {
            set_error("cpdf grid: " + std::to_string(npts) + " points do not fit in " + std::to_string(max_points));
            return MCE_ERR_ARG;
        }
        if (master_step < 1) {
            set_error("cpdf: the estimator has not been stepped");
            return MCE_ERR_ARG;
        }
        if (master_step >= est[e].num_updates) {
            set_error("cpdf: the last step keeps no g-tables");
            return MCE_ERR_DONE;
        }
        for (int i = 0; i < ny; i++) {
            double y = ly + i * ry;
            if (y > hy) y = hy;
            for (int j = 0; j < nx; j++) {
                double x = lx + j * rx;
                if (x > hx) x = hx;
                xs[i * nx + j] = x;
                ys[i * nx + j] = y;
            }
        }
        if ((int)cpdf2_step.size() != E) {
            cpdf2_step.assign(E, -1);
            cpdf2_i1.assign(E, -1);
            cpdf2_i2.assign(E, -1);
            cpdf2_n.assign(E, -1);
            cpdf2_tt.clear();
            cpdf2_tt.resize(E);
        }
        const long long a = hpstart[e], n = hpstart[e + 1] - a;
        int s;
        if (cpdf2_step[e] != master_step || cpdf2_i1[e] != i1 || cpdf2_i2[e] != i2 || cpdf2_n[e] != n) {
            if (!cpdf2_tt[e]) cpdf2_tt[e].reset(new DevBuf<double>());
            if ((s = cpdf2_tt[e]->ensure((size_t)(n + 1) * cpdf2d_stride(MC)))) return s;
            if ((s = cpdf_nu.ensure(D))) return s;
            MCE_CUDA(cudaMemcpyAsync(cpdf_nu.ptr, bar_nu, sizeof(double) * D, cudaMemcpyHostToDevice, lc.stream));
            Kernels<D>::cpdf2d_terms(Pb[cur].view(), a, n, i1, i2, cpdf_nu.ptr,
                                     Tables{Tb[cur].keys.ptr, Tb[cur].vals.ptr}, MC, cpdf2_tt[e]->ptr, lc);
            cpdf2_step[e] = master_step;
            cpdf2_i1[e] = i1;
            cpdf2_i2[e] = i2;
            cpdf2_n[e] = n;
        }
        if ((s = cpdf2_x.ensure(npts))) return s;
        if ((s = cpdf2_y.ensure(npts))) return s;
        if ((s = cpdf2_z.ensure(npts))) return s;
        MCE_CUDA(cudaMemcpyAsync(cpdf2_x.ptr, xs, sizeof(double) * npts, cudaMemcpyHostToDevice, lc.stream));
        MCE_CUDA(cudaMemcpyAsync(cpdf2_y.ptr, ys, sizeof(double) * npts, cudaMemcpyHostToDevice, lc.stream));
        MCE_CUDA(cudaMemsetAsync(counters.ptr + 7, 0, sizeof(int), lc.stream));
        cpdf2d_points(cpdf2_tt[e]->ptr, n, MC, cpdf2_x.ptr, cpdf2_y.ptr, npts, est[e].fz[0], cpdf2_z.ptr,
                      counters.ptr + 7, lc);
        int bad = 0;
        MCE_CUDA(cudaMemcpyAsync(zs, cpdf2_z.ptr, sizeof(double) * npts, cudaMemcpyDeviceToHost, lc.stream));
        MCE_CUDA(cudaMemcpyAsync(&bad, counters.ptr + 7, sizeof(int), cudaMemcpyDeviceToHost, lc.stream));
        MCE_CUDA(cudaStreamSynchronize(lc.stream));
        // the cache survives unless the caller drops it (pycauchy.hpp:856-859)
        if (reset_cache) cpdf2_step[e] = -1;
        if (bad) {
            set_error("cpdf: a cell with gamma1 = gamma2 = 0 (the reference exits here)");
            return MCE_ERR_DEVICE;
        }
        return npts;
    }

    int terms_view(int e, TermsView* v) override
    {
        if (e < 0 || e >= E || !v) return MCE_ERR_ARG;
        if (master_step < 1) {
            set_error("relative system: the estimator has not been stepped");
            return MCE_ERR_ARG;
        }
        if (master_step >= est[e].num_updates) {
            set_error("relative system: the last step keeps no g-tables");
            return MCE_ERR_DONE;
        }
        drain();
        const long long a = hpstart[e], n = hpstart[e + 1] - a;
        std::vector<int> hm((size_t)n + 1);
        if (n > 0)
            MCE_CUDA(cudaMemcpyAsync(hm.data(), Pb[cur].m.ptr + a, sizeof(int) * n, cudaMemcpyDeviceToHost,
                                     lc.stream));
        MCE_CUDA(cudaStreamSynchronize(lc.stream));
        v->P = Pb[cur].view();
        v->T = Tables{Tb[cur].keys.ptr, Tb[cur].vals.ptr};
        v->MC = MC;
        v->fz = est[e].fz[0];
        v->shape_cnt.assign(MC + 1, 0);
        v->shape_off.assign(MC + 2, 0);
        for (long long i = 0; i < n; i++) {
            if (hm[i] < 0 || hm[i] > MC) {
                set_error("relative system: a term shape out of range");
                return MCE_ERR_DEVICE;
            }
            v->shape_cnt[hm[i]]++;
        }
        for (int m = 0; m <= MC; m++) v->shape_off[m + 1] = v->shape_off[m] + v->shape_cnt[m];
        v->idx.assign((size_t)n, 0);
        std::vector<int> fill(MC + 1, 0);
        for (long long i = 0; i < n; i++) v->idx[v->shape_off[hm[i]] + fill[hm[i]]++] = a + i;
        return MCE_OK;
    }

    // ---- N-D conditional pdf at points (PointWiseNDimCauchyCPDF::evaluate_cpdf,
    // cpdf_ndim.hpp:677-904): the estimator's terms and tables as they are
    NdWork* ndw = nullptr;
    int cpdf_nd(int e, const double* x, int npts, double* out) override
    {
        return cpdf_points(e, nullptr, 0, nullptr, x, npts, out);
    }

    // PointWiseNDimCauchyCPDF::evaluate_marginal_cpdf (cpdf_ndim.hpp:918-1230):
    // the marginal pdf of the states idx[0..nm) (ascending, 0 < nm < d) at
    // npts points x[npts][nm], the terms left after nm lowerings looked up
    // at nu_bar[d - nm]
    int cpdf_marginal(int e, const int* idx, int nm, const double* nu_bar, const double* x, int npts,
                      double* out) override
    {
        if (!idx || !nu_bar || nm < 1 || nm >= D) {
            set_error("marginal pdf: 0 < number of states < d, and nu_bar, are required");
            return MCE_ERR_ARG;
        }
        for (int i = 0; i < nm; i++)
            if (idx[i] < 0 || idx[i] >= D || (i > 0 && idx[i] <= idx[i - 1])) {
                set_error("marginal pdf: the state indices must ascend within [0, d)");
                return MCE_ERR_ARG;
            }
        return cpdf_points(e, idx, nm, nu_bar, x, npts, out);
    }

    int cpdf_points(int e, const int* idx, int nm, const double* nu_bar, const double* x, int npts, double* out)
    {
        if (e < 0 || e >= E || !x || !out || npts < 1) return MCE_ERR_ARG;
        // the largest shape the estimator's terms have now (the handle's
        // capacity MC may be larger)
        int MB = 0;
        for (int m = 0; m < (int)est[e].tps.size(); m++)
            if (est[e].tps[m] > 0) MB = m;
        if (MB > 16) {
            set_error("N-D pdf: terms of more than 16 hyperplanes are not supported");
            return MCE_ERR_SHAPE;
        }
        if (master_step < 1) {
            set_error("N-D pdf: the estimator has not been stepped");
            return MCE_ERR_ARG;
        }
        if (master_step >= est[e].num_updates) {
            set_error("N-D pdf: the last step keeps no g-tables");
            return MCE_ERR_DONE;
        }
        if (est[e].errors) {
            set_error("N-D pdf: the last step reported moment errors (the reference asserts "
                      "numeric_moment_errors == 0, cpdf_ndim.hpp:680)");
            return MCE_ERR_ARG;
        }
        drain();
        if (!ndw) ndw = nd_work_create();
        const long long a = hpstart[e];
        PBufs& P = Pb[cur];
        NdInput in;
        in.D = D;
        in.MC = MC;
        in.MB = std::max(MB, 1);
        in.n = hpstart[e + 1] - a;
        in.m = P.m.ptr + a;
        in.A = P.A.ptr + a * MC * D;
        in.p = P.p.ptr + a * MC;
        in.b = P.b.ptr + a * D;
        in.toff = P.tab_off.ptr + a;
        in.tcnt = P.tab_cnt.ptr + a;
        in.keys = Tb[cur].keys.ptr;
        in.vals = Tb[cur].vals.ptr;
        in.fz = est[e].fz[0];
        if (nm > 0) {
            // the states integrated out first, the kept states last
            // (evaluate_marginal_cpdf, cpdf_ndim.hpp:950-968)
            bool kept[kMaxDim] = {false};
            for (int i = 0; i < nm; i++) {
                in.reorient[D - nm + i] = idx[i];
                kept[idx[i]] = true;
            }
            for (int i = 0, c = 0; i < D; i++)
                if (!kept[i]) in.reorient[c++] = i;
            in.nkeep = nm;
            in.nu_bar = nu_bar;
        }
        return nd_pdf_eval(in, x, npts, out, ndw, lc, &launches);
    }

    void rel2d_pairs(const Rel2DArgs& a, cudaStream_t st) override
    {
        LaunchCfg c = lc;
        c.stream = st;
        Kernels<D>::rel2d_pairs(a, c);
    }

    // ---- marginal 1-D pdf: CauchyCPDFGridDispatcher1D (cpdf_ndim.hpp:2017-2139)
    // over PointWiseNDimCauchyCPDF::evaluate_1D_marginal_cpdf (:1233-1352),
    // with the reference's per-estimator cache of per-term constants, kept on
    // the device and keyed by (master step, marginal index)
    std::vector<int> cpdf_step, cpdf_marg;
    std::vector<long long> cpdf_n;
    std::vector<std::unique_ptr<DevBuf<double>>> cpdf_tt;
    DevBuf<double> cpdf_nu, cpdf_x, cpdf_y;

    int cpdf_1d_grid(int e, int marg, const double* bar_nu, double low, double high, double res, int max_points,
                     double* xs, double* ys) override
    {
        if (e < 0 || e >= E || marg < 0 || marg >= D || !bar_nu) return MCE_ERR_ARG;
        if (!(high > low) || !(res > 0)) return MCE_ERR_ARG;
        const double span = (high - low + res - 1e-15) / res;
        if (!(span < 1e8)) {
            set_error("cpdf grid: too many points");
            return MCE_ERR_ARG;
        }
        const int npts = (int)span + 1;  // reset_grid, cpdf_ndim.hpp:2055-2072
        if (!xs || !ys) return npts;
        if (npts > max_points) {
            set_error("cpdf grid: " + std::to_string(npts) + " points do not fit in " + std::to_string(max_points));
            return MCE_ERR_ARG;
        }
        if (master_step < 1) {
            set_error("cpdf: the estimator has not been stepped");
            return MCE_ERR_ARG;
        }
        if (master_step >= est[e].num_updates) {
            // evaluate_point_grid refuses the last step: its g-tables are skipped
            set_error("cpdf: the last step keeps no g-tables");
            return MCE_ERR_DONE;
        }
        for (int i = 0; i < npts; i++) {
            double x = low + i * res;
            if (x > high) x = high;
            xs[i] = x;
        }
        if ((int)cpdf_step.size() != E) {
            cpdf_step.assign(E, -1);
            cpdf_marg.assign(E, -1);
            cpdf_n.assign(E, -1);
            cpdf_tt.clear();
            cpdf_tt.resize(E);
        }
        const long long a = hpstart[e], n = hpstart[e + 1] - a;
        int exact = 0, s;
        // the cache also keys on the term count: a reset cannot leave one
        // whose size differs from the terms (the reference would read past it)
        if (cpdf_step[e] != master_step || cpdf_marg[e] != marg || cpdf_n[e] != n) {
            // the first evaluation at this step and index: the exact formula at
            // the first point, and the per-term constants cached
            if (!cpdf_tt[e]) cpdf_tt[e].reset(new DevBuf<double>());
            if ((s = cpdf_tt[e]->ensure((size_t)(n + 1) * 8))) return s;
            if ((s = cpdf_nu.ensure(D))) return s;
            MCE_CUDA(cudaMemcpyAsync(cpdf_nu.ptr, bar_nu, sizeof(double) * D, cudaMemcpyHostToDevice, lc.stream));
            Kernels<D>::cpdf1d_terms(Pb[cur].view(), a, n, marg, cpdf_nu.ptr,
                                     Tables{Tb[cur].keys.ptr, Tb[cur].vals.ptr}, MC, cpdf_tt[e]->ptr, lc);
            cpdf_step[e] = master_step;
            cpdf_marg[e] = marg;
            cpdf_n[e] = n;
            exact = 1;
        }
        if ((s = cpdf_x.ensure(npts))) return s;
        if ((s = cpdf_y.ensure(npts))) return s;
        MCE_CUDA(cudaMemcpyAsync(cpdf_x.ptr, xs, sizeof(double) * npts, cudaMemcpyHostToDevice, lc.stream));
        cpdf1d_points(cpdf_tt[e]->ptr, n, cpdf_x.ptr, npts, exact, est[e].fz[0], cpdf_y.ptr, lc);
        MCE_CUDA(cudaMemcpyAsync(ys, cpdf_y.ptr, sizeof(double) * npts, cudaMemcpyDeviceToHost, lc.stream));
        MCE_CUDA(cudaStreamSynchronize(lc.stream));
        return npts;
    }

    long long total_cells(int e) override
    {
        if (e < 0 || e >= E || nP == 0) return 0;
        const long long a = hpstart[e], bnd = hpstart[e + 1];
        std::vector<int> c(bnd - a);
        if (bnd > a)
            cudaMemcpy(c.data(), Pb[cur].tab_cnt.ptr + a, sizeof(int) * (bnd - a), cudaMemcpyDeviceToHost);
        long long t = 0;
        for (int x : c) t += x;
        return t;
    }

    int dump_terms(int e, int max_shape, int* shape, double* A, double* p_, double* b, int* cells, int* keys,
                   double* g) override
    {
        if (e < 0 || e >= E) return MCE_ERR_ARG;
        if (nP == 0) return MCE_OK;
        const long long a = hpstart[e], bnd = hpstart[e + 1], n = bnd - a;
        PBufs& P = Pb[cur];
        std::vector<int> m(n), tc(n);
        std::vector<double> hA(n * MC * D), hp(n * MC), hb(n * D);
        std::vector<long long> to(n);
        MCE_CUDA(cudaMemcpy(m.data(), P.m.ptr + a, sizeof(int) * n, cudaMemcpyDeviceToHost));
        MCE_CUDA(cudaMemcpy(tc.data(), P.tab_cnt.ptr + a, sizeof(int) * n, cudaMemcpyDeviceToHost));
        MCE_CUDA(cudaMemcpy(to.data(), P.tab_off.ptr + a, sizeof(long long) * n, cudaMemcpyDeviceToHost));
        MCE_CUDA(cudaMemcpy(hA.data(), P.A.ptr + a * MC * D, sizeof(double) * n * MC * D, cudaMemcpyDeviceToHost));
        MCE_CUDA(cudaMemcpy(hp.data(), P.p.ptr + a * MC, sizeof(double) * n * MC, cudaMemcpyDeviceToHost));
        MCE_CUDA(cudaMemcpy(hb.data(), P.b.ptr + a * D, sizeof(double) * n * D, cudaMemcpyDeviceToHost));
        // the estimator's tables in one copy: the span its slices cover
        long long lo = -1, hi = -1;
        for (long long t = 0; t < n; t++)
            if (tc[t] > 0) {
                lo = lo < 0 ? to[t] : std::min(lo, to[t]);
                hi = std::max(hi, to[t] + tc[t]);
            }
        std::vector<int> span_k(lo < 0 ? 0 : hi - lo);
        std::vector<cd> span_v(lo < 0 ? 0 : hi - lo);
        if (lo >= 0) {
            MCE_CUDA(cudaMemcpy(span_k.data(), Tb[cur].keys.ptr + lo, sizeof(int) * (hi - lo), cudaMemcpyDeviceToHost));
            MCE_CUDA(cudaMemcpy(span_v.data(), Tb[cur].vals.ptr + lo, sizeof(cd) * (hi - lo), cudaMemcpyDeviceToHost));
        }
        long long c = 0;
        for (long long t = 0; t < n; t++) {
            shape[t] = m[t];
            for (int k = 0; k < max_shape * D; k++) A[t * max_shape * D + k] = 0;
            for (int k = 0; k < max_shape; k++) p_[t * max_shape + k] = 0;
            for (int k = 0; k < m[t] * D && k < max_shape * D; k++) A[t * max_shape * D + k] = hA[t * MC * D + k];
            for (int k = 0; k < m[t] && k < max_shape; k++) p_[t * max_shape + k] = hp[t * MC + k];
            for (int k = 0; k < D; k++) b[t * D + k] = hb[t * D + k];
            cells[t] = tc[t];
            for (int k = 0; k < tc[t]; k++) {
                keys[c] = span_k[to[t] - lo + k];
                g[2 * c] = span_v[to[t] - lo + k].re;
                g[2 * c + 1] = span_v[to[t] - lo + k].im;
                c++;
            }
        }
        return MCE_OK;
    }
};

static __global__ void k_gscale_kernel(const cd* est_raw, int NM, int E, double* gscale)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < E) gscale[e] = kTwoPiInv / est_raw[(long long)e * NM].re;
}

template <int D>
void Engine<D>::k_gscale_from_raw(int E_)
{
    ++g_launches;
    k_gscale_kernel<<<(E_ + 127) / 128, 128, 0, lc.stream>>>(est_raw.ptr, 1 + D + D * D, E_, gscale.ptr);
}

template <int D>
__global__ void k_skip_hist_kernel(ParentList P, long long n, const EstStep<D>* st, int MCp, int* hist)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int e = P.est[i];
        if (!st[e].skip) continue;
        atomicAdd(&hist[(long long)e * MCp + P.m[i]], 1 + P.nkids_all[i]);
    }
}

template <int D>
void Engine<D>::k_skip_hist(ParentList PV, long long n, int MCp)
{
    if (n == 0) return;
    ++g_launches;
    k_skip_hist_kernel<D><<<(int)std::min<long long>((n + 255) / 256, lc.num_sms * 16), 256, 0, lc.stream>>>(
        PV, n, dsteps.ptr, MCp, hist.ptr);
}

static __global__ void k_gather_kernel(const long long* scan, const long long* pstart, int E, long long* out)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e <= E; e += gridDim.x * blockDim.x) out[e] = scan[pstart[e]];
}

template <int D>
void Engine<D>::k_gather_bounds(const long long* scan, int E_)
{
    ++g_launches;
    k_gather_kernel<<<(E_ + 256) / 256, 256, 0, lc.stream>>>(scan, dpstart.ptr, E_, kall_est.ptr);
}

// Algorithmic traffic and FP64 work per kernel group (profiling mode 2).
// Bytes count the data a kernel must move at least once (term records, table
// cells, two parent-table lookups of one key and one complex value per g
// evaluation); flops count FP64 operations of the formulas evaluated, with a
// complex division as 11 and a complex product as 6.
__device__ inline void acc_stat(double* alg, int kid, double bytes, double flops)
{
    atomicAdd(&alg[2 * kid], bytes);
    atomicAdd(&alg[2 * kid + 1], flops);
}

template <int D>
static __global__ void k_alg_parents(ParentList P, long long nP, const EstStep<D>* st, int with_tp,
                                     const long long* kall_scan, double* alg)
{
    constexpr int NM = 1 + D + D * D;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nP; i += (long long)gridDim.x * blockDim.x) {
        const EstStep<D>& S = st[P.est[i]];
        const double m = P.m[i], phc = P.m_old[i], Cp = P.tab_cnt[i];
        const double CB = S.skip ? 0.0 : (double)P.B_cnt[i];
        const double K = (double)P.nkids_all[i];
        const bool dce = with_tp && P.m[i] != P.m_old[i];
        double f = 2 * m * D;
        if (with_tp) f += 2 * phc * D * D + 2.0 * D * D + phc * (2 * D + 1);
        acc_stat(alg, KID_TP, 8 * (phc * D + phc + D) + 8 * (m * D + m + D) + 16, f);
        if (!S.skip) {
            if (dce && P.m[i] > D) {
                const double nc = (double)binom_ll(P.m[i], D);
                acc_stat(alg, KID_BUILD_B, 8 * m * D + 4 * Cp + 4 * CB,
                         nc * ((2.0 / 3.0) * D * D * D + 2.0 * D * D * D + 2.0 * D * D + 2 * (m - D) * D));
            } else
                acc_stat(alg, KID_BUILD_B, 8 * Cp, 0);
        }
        const double T = 1 + K;
        double b = 8 * (m * D + m + D) + T * 2 * 20 + T * NM * 16;
        double fl = m * (3 * D + 2) + T * (m * D + 4 * m * D + 8 * D + 14.0 * D * D + 22);
        if (!S.skip) {
            b += T * (8 * (m * D + 2 * m + D + 2) + 36 + 2 * m) + 8 * CB;
            fl += K * (m * m * D + 3 * m * D);
        }
        acc_stat(alg, KID_MU, b, fl);
        acc_stat(alg, KID_MOMENTS, T * NM * 16, T * 2 * NM);
    }
}

template <int D>
static __global__ void k_alg_roots(TermRecs R, long long nR, const int* status, const int* gcnt, const int* alive,
                                   const int* tcnt, double* alg)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < nR; j += (long long)gridDim.x * blockDim.x) {
        if (R.est[j] < 0) continue;
        const double m = R.m[j];
        acc_stat(alg, KID_FTR, 8 * D + 16 * m + 16, 2 * D);
        if (status[j] != 1) continue;
        const double g = gcnt[j];
        const double cells = alive[j] ? (double)tcnt[j] : 0.0;
        acc_stat(alg, KID_GTABLE,
                 (1 + g) * (8 * (m * D + 2 * m + D + 2) + 24) + cells * (1 + g) * 40 + cells * 20 + g * cells * 32,
                 (1 + g) * cells * (2 * m + 22) + g * cells * 2);
        if (alive[j]) acc_stat(alg, KID_PARTITION, 2 * (8 * (m * D + m + D) + 16), 0);
    }
}

template <int D>
void Engine<D>::alg_stats(bool with_tp, long long nR, bool tables_built)
{
    if (alg.ensure(2 * KID_COUNT)) return;
    cudaMemsetAsync(alg.ptr, 0, sizeof(double) * 2 * KID_COUNT, lc.stream);
    if (!tables_built) {
        if (nP > 0)
            k_alg_parents<D><<<(int)std::min<long long>((nP + 255) / 256, lc.num_sms * 8), 256, 0, lc.stream>>>(
                Pb[cur].view(), nP, dsteps.ptr, with_tp ? 1 : 0, kall_scan.ptr, alg.ptr);
    } else if (nR > 0) {
        k_alg_roots<D><<<(int)std::min<long long>((nR + 255) / 256, lc.num_sms * 8), 256, 0, lc.stream>>>(
            Rb.view(), nR, status.ptr, gcnt.ptr, alive.ptr, tcnt.ptr, alg.ptr);
    }
    double h[2 * KID_COUNT];
    cudaMemcpyAsync(h, alg.ptr, sizeof(h), cudaMemcpyDeviceToHost, lc.stream);
    cudaStreamSynchronize(lc.stream);
    for (int k = 0; k < KID_COUNT; k++) {
        kbytes[k] += h[2 * k];
        kflops[k] += h[2 * k + 1];
    }
}

static __global__ void k_status_init_kernel(const int* est, long long n, int* status)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x)
        status[j] = est[j] < 0 ? -1 : 0;
}

template <int D>
void Engine<D>::k_status_init(TermRecs R, long long nR)
{
    if (nR == 0) return;
    ++g_launches;
    k_status_init_kernel<<<(int)std::min<long long>((nR + 255) / 256, lc.num_sms * 16), 256, 0, lc.stream>>>(
        R.est, nR, status.ptr);
}

// Per-dimension factories: each dimension's engine lives in its own unit.
#define MCE_DECLARE_DIM(D)                                                                                     \
    EngineBase* make_engine_##D();                                                                            \
    int init_engine_##D(EngineBase* b, int E, int cmcc, int pncc, int p, const int* steps, const double* A0,   \
                        const double* p0, const double* b0, const double* root, const double* bp, int bps);
#define MCE_DEFINE_DIM(D)                                                                                      \
    EngineBase* make_engine_##D() { return new Engine<D>(); }                                                  \
    int init_engine_##D(EngineBase* b, int E, int cmcc, int pncc, int p, const int* steps, const double* A0,   \
                        const double* p0, const double* b0, const double* root, const double* bp, int bps)      \
    {                                                                                                          \
        return static_cast<Engine<D>*>(b)->init(E, cmcc, pncc, p, steps, A0, p0, b0, root, bp, bps);          \
    }
MCE_DECLARE_DIM(1)
MCE_DECLARE_DIM(2)
MCE_DECLARE_DIM(3)
MCE_DECLARE_DIM(4)
MCE_DECLARE_DIM(5)
MCE_DECLARE_DIM(6)
MCE_DECLARE_DIM(7)
MCE_DECLARE_DIM(8)
#if MCE_ONLY_DIM == 1 || MCE_ONLY_DIM < 0
MCE_DEFINE_DIM(1)
#endif
#if MCE_ONLY_DIM == 2 || MCE_ONLY_DIM < 0
MCE_DEFINE_DIM(2)
#endif
#if MCE_ONLY_DIM == 3 || MCE_ONLY_DIM < 0
MCE_DEFINE_DIM(3)
#endif
#if MCE_ONLY_DIM == 4 || MCE_ONLY_DIM < 0
MCE_DEFINE_DIM(4)
#endif
#if MCE_ONLY_DIM == 5 || MCE_ONLY_DIM < 0
MCE_DEFINE_DIM(5)
#endif
#if MCE_ONLY_DIM == 6 || MCE_ONLY_DIM < 0
MCE_DEFINE_DIM(6)
#endif
#if MCE_ONLY_DIM == 7 || MCE_ONLY_DIM < 0
MCE_DEFINE_DIM(7)
#endif
#if MCE_ONLY_DIM == 8 || MCE_ONLY_DIM < 0
MCE_DEFINE_DIM(8)
#endif

}  // namespace mce

#if MCE_ONLY_DIM <= 0
using namespace mce;

struct mce_handle {
    EngineBase* eng;
};

// Relative-then-transformed 2-D system of two estimators: the pair cache and
// the buffers of its grid evaluations, on a stream of its own (either
// estimator may be stepped or destroyed while it lives).
struct mce_rel2d {
    cudaStream_t stream = nullptr;
    LaunchCfg lc{};
    int full = 0, CC = 0;
    long long npairs = 0, nkept = 0;
    DevBuf<double> tt, mrows, mpart, mout, trel, nu, part, xs, ys, zs;
    DevBuf<int> keep, bad;
    DevBuf<long long> idxP, idxS, kpos, kidx, scan_tmp;
    DevBuf<Rel2DBlock> blk;
    // device time of the last pair pass, moment sum and grid (CUDA events on the stream)
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    double ms[3] = {0, 0, 0};
    long long launches = 0;  // kernels launched by the construction and the grids
    ~mce_rel2d()
    {
        if (stream) {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    }
    double elapsed(int k)
    {
        float t = 0;
        if (cudaEventElapsedTime(&t, ev[2 * k], ev[2 * k + 1]) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        return t;
    }
};

namespace {

// get_marg2d_relative_and_transformed_cpdf (cauchy_prediction.hpp:653-971)
int rel2d_build(mce_rel2d* r, EngineBase& P, int ep, EngineBase& S, int es, const double* Trel,
                const double* bar_nu_full, int full, int approx, double eps, double* moments, long long* counts)
{
    const int d = P.d;
    const long long l0 = g_launches;
    if (S.d != d) {
        set_error("relative system: the estimators' state dimensions differ");
        return MCE_ERR_ARG;
    }
    if (P.est[ep].max_shape + S.est[es].max_shape > kMaxRows) {
        set_error("relative system: the two estimators' hyperplanes exceed 31 (cauchy_prediction.hpp:695)");
        return MCE_ERR_SHAPE;
    }
    EngineBase::TermsView vp, vs;
    int s;
    if ((s = P.terms_view(ep, &vp))) return s;
    if ((s = S.terms_view(es, &vs))) return s;
    int dev = 0;
    MCE_CUDA(cudaGetDevice(&dev));
    MCE_CUDA(cudaDeviceGetAttribute(&r->lc.num_sms, cudaDevAttrMultiProcessorCount, dev));
    MCE_CUDA(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking));
    for (cudaEvent_t& e : r->ev) MCE_CUDA(cudaEventCreate(&e));
    r->lc.stream = r->stream;
    r->full = full ? 1 : 0;
    r->CC = (P.est[ep].max_shape + S.est[es].max_shape) * (1 + r->full);
    // pair blocks: primary shape, secondary shape (cauchy_prediction.hpp:789-800)
    std::vector<Rel2DBlock> blks;
    long long off = 0;
    for (int mp = 1; mp <= vp.MC; mp++)
        for (int ms = 1; ms <= vs.MC; ms++) {
            if (!vp.shape_cnt[mp] || !vs.shape_cnt[ms]) continue;
            blks.push_back(Rel2DBlock{off, vp.shape_off[mp], vp.shape_cnt[mp], vs.shape_off[ms], vs.shape_cnt[ms]});
            off += (long long)vp.shape_cnt[mp] * vs.shape_cnt[ms];
        }
    r->npairs = off;
    const int RT = rel2d_stride(r->CC);
    const bool mom = moments != nullptr;
    if ((s = r->tt.ensure((size_t)(off + 1) * RT))) return s;
    if ((s = r->keep.ensure(off + 1))) return s;
    if (mom && (s = r->mrows.ensure((size_t)(off + 1) * 14))) return s;
    if ((s = r->idxP.ensure(vp.idx.size() + 1))) return s;
    if ((s = r->idxS.ensure(vs.idx.size() + 1))) return s;
    if ((s = r->blk.ensure(blks.size() + 1))) return s;
    if ((s = r->trel.ensure(2 * d))) return s;
    if ((s = r->nu.ensure(d))) return s;
    cudaStream_t st = r->stream;
    if (!vp.idx.empty())
        MCE_CUDA(cudaMemcpyAsync(r->idxP.ptr, vp.idx.data(), sizeof(long long) * vp.idx.size(), cudaMemcpyHostToDevice,
                                 st));
    if (!vs.idx.empty())
        MCE_CUDA(cudaMemcpyAsync(r->idxS.ptr, vs.idx.data(), sizeof(long long) * vs.idx.size(), cudaMemcpyHostToDevice,
                                 st));
    if (!blks.empty())
        MCE_CUDA(cudaMemcpyAsync(r->blk.ptr, blks.data(), sizeof(Rel2DBlock) * blks.size(), cudaMemcpyHostToDevice,
                                 st));
    MCE_CUDA(cudaMemcpyAsync(r->trel.ptr, Trel, sizeof(double) * 2 * d, cudaMemcpyHostToDevice, st));
    MCE_CUDA(cudaMemcpyAsync(r->nu.ptr, bar_nu_full, sizeof(double) * d, cudaMemcpyHostToDevice, st));
    Rel2DArgs a;
    a.P = vp.P;
    a.S = vs.P;
    a.TP = vp.T;
    a.TS = vs.T;
    a.MCp = vp.MC;
    a.MCs = vs.MC;
    a.idxP = r->idxP.ptr;
    a.idxS = r->idxS.ptr;
    a.blk = r->blk.ptr;
    a.nblk = (int)blks.size();
    a.npairs = off;
    a.Trel = r->trel.ptr;
    a.nu_full = r->nu.ptr;
    a.full = r->full;
    a.approx = approx ? 1 : 0;
    a.moments = mom ? 1 : 0;
    a.eps = eps;
    // approx_norm_factor (cauchy_prediction.hpp:679)
    a.approx_nf = kTwoPiInv * kTwoPiInv / vp.fz / vs.fz;
    a.CC = r->CC;
    a.tt = r->tt.ptr;
    a.keep = r->keep.ptr;
    a.mrows = mom ? r->mrows.ptr : nullptr;
    MCE_CUDA(cudaEventRecord(r->ev[0], st));
    P.rel2d_pairs(a, st);
    MCE_CUDA(cudaEventRecord(r->ev[1], st));
    MCE_CUDA(cudaGetLastError());
    MCE_CUDA(cudaEventRecord(r->ev[2], st));
    // the kept pairs in order, for the grid's even chunks
    {
        long long need = 4, t = off;
        while (t > 1) {
            t = (t + 2047) / 2048;
            need += t + 2;
        }
        if ((s = r->scan_tmp.ensure(need + 64))) return s;
        if ((s = r->kpos.ensure(off + 2))) return s;
        if ((s = r->kidx.ensure(off + 1))) return s;
        ScanScratch ss{r->scan_tmp.ptr, (long long)r->scan_tmp.cap};
        scan_int_to_ll(r->keep.ptr, r->kpos.ptr, off, ss, r->lc);
        rel2d_compact(r->keep.ptr, r->kpos.ptr, off, r->kidx.ptr, r->lc);
    }
    if (mom) {
        const long long chunk = 65536;
        const long long nch = (off + chunk - 1) / chunk;
        if ((s = r->mpart.ensure((size_t)(nch + 1) * 14))) return s;
        if ((s = r->mout.ensure(14))) return s;
        rel2d_moments(r->mrows.ptr, off, chunk, r->mpart.ptr, r->mout.ptr, r->lc);
        MCE_CUDA(cudaGetLastError());
    }
    MCE_CUDA(cudaEventRecord(r->ev[3], st));
    if (mom) MCE_CUDA(cudaMemcpyAsync(moments, r->mout.ptr, sizeof(double) * 14, cudaMemcpyDeviceToHost, st));
    long long kept = 0;
    MCE_CUDA(cudaMemcpyAsync(&kept, r->kpos.ptr + off, sizeof(long long), cudaMemcpyDeviceToHost, st));
    MCE_CUDA(cudaStreamSynchronize(st));
    r->nkept = kept;
    r->launches += g_launches - l0;
    r->ms[0] = r->elapsed(0);
    r->ms[1] = r->elapsed(1);
    if (counts) {
        counts[0] = off;
        counts[1] = off - kept;
    }
    return MCE_OK;
}

// grid_eval_marg2d_relative_and_transformed_cpdf (cauchy_prediction.hpp:1091-1186)
int rel2d_grid(mce_rel2d* r, double xlow, double xhigh, double dx, double ylow, double yhigh, double dy,
               double nf_prim, double nf_sec, int max_points, double* x, double* y, double* z)
{
    if (!(xhigh > xlow) || !(yhigh > ylow) || !(dx > 0) || !(dy > 0)) return MCE_ERR_ARG;
    const double sx = ceil((xhigh - xlow) / dx + 1), sy = ceil((yhigh - ylow) / dy + 1);
    if (!(sx < 1e8) || !(sy < 1e8) || sx * sy > 1e8) {
        set_error("relative pdf grid: too many points");
        return MCE_ERR_ARG;
    }
    const int nx = (int)sx, ny = (int)sy;
    if (nx <= 1 || ny <= 1) {
        set_error("relative pdf grid: fewer than two points on an axis");
        return MCE_ERR_ARG;
    }
    const int npts = nx * ny;
    if (!x || !y || !z) return npts;
    if (npts > max_points) {
        set_error("relative pdf grid: " + std::to_string(npts) + " points do not fit in " +
                  std::to_string(max_points));
        return MCE_ERR_ARG;
    }
    for (int i = 0; i < nx; i++) {
        const double xv = i == nx - 1 ? xhigh : xlow + dx * i;
        for (int j = 0; j < ny; j++) {
            x[i * ny + j] = xv;
            y[i * ny + j] = j == ny - 1 ? yhigh : ylow + dy * j;
        }
    }
    // enough (point, chunk) threads for two full waves, chunks of at least 32
    // kept terms; one chunk keeps the reference's summation order exactly
    const long long nk = r->nkept;
    long long nch = ((long long)r->lc.num_sms * 2048 * 2 + npts - 1) / npts;
    const long long maxch = (nk + 31) / 32;
    if (nch > maxch) nch = maxch;
    if (nch < 1) nch = 1;
    if (nch > 65535) nch = 65535;
    long long chunk = nk > 0 ? (nk + nch - 1) / nch : 1;
    nch = nk > 0 ? (nk + chunk - 1) / chunk : 1;
    int s;
    if ((s = r->xs.ensure(npts))) return s;
    if ((s = r->ys.ensure(npts))) return s;
    if ((s = r->zs.ensure(npts))) return s;
    if ((s = r->part.ensure((size_t)nch * npts))) return s;
    if ((s = r->bad.ensure(1))) return s;
    cudaStream_t st = r->stream;
    MCE_CUDA(cudaMemcpyAsync(r->xs.ptr, x, sizeof(double) * npts, cudaMemcpyHostToDevice, st));
    MCE_CUDA(cudaMemcpyAsync(r->ys.ptr, y, sizeof(double) * npts, cudaMemcpyHostToDevice, st));
    MCE_CUDA(cudaMemsetAsync(r->bad.ptr, 0, sizeof(int), st));
    MCE_CUDA(cudaEventRecord(r->ev[4], st));
    r->launches += 2;
    rel2d_points(r->tt.ptr, r->kidx.ptr, nk, r->CC, r->full, chunk, (int)nch, r->xs.ptr, r->ys.ptr, npts,
                 r->part.ptr, r->bad.ptr, r->lc);
    rel2d_finish(r->part.ptr, (int)nch, npts, r->full, nf_prim, nf_sec, r->zs.ptr, r->lc);
    MCE_CUDA(cudaEventRecord(r->ev[5], st));
    MCE_CUDA(cudaGetLastError());
    int bad = 0;
    MCE_CUDA(cudaMemcpyAsync(z, r->zs.ptr, sizeof(double) * npts, cudaMemcpyDeviceToHost, st));
    MCE_CUDA(cudaMemcpyAsync(&bad, r->bad.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
    MCE_CUDA(cudaStreamSynchronize(st));
    r->ms[2] = r->elapsed(2);
    if (bad) {
        set_error("relative pdf: a cell with gamma1 = gamma2 = 0 (the reference exits here)");
        return MCE_ERR_DEVICE;
    }
    return npts;
}

}  // namespace

extern "C" {

const char* mce_last_error(void) { return g_last_error.c_str(); }

static std::atomic<int> g_ref_num_cpus{8};

int mce_set_reference_num_cpus(int num_cpus)
{
    if (num_cpus < 1) return MCE_ERR_ARG;
    return g_ref_num_cpus.exchange(num_cpus);
}

int mce_draw_reference_constants(long long seed, int d, int max_shape, int num_cpus, double* root_point,
                                 double* b_pert)
{
    if (num_cpus == 0) num_cpus = g_ref_num_cpus.load();
    if (d < 1 || max_shape < 1 || num_cpus < 1 || !root_point || !b_pert) return MCE_ERR_ARG;
    if (seed >= 0) srand((unsigned)seed);
    auto u = []() { return ((double)rand() + 1.0) / ((double)RAND_MAX + 1.0); };
    for (int i = 0; i < d; i++) root_point[i] = 1.0 + u();
    for (int h = 0; h < num_cpus; h++)
        for (int i = 0; i < max_shape; i++) {
            const double v = 2 * u() - 1;
            if (h == 0) b_pert[i] = v;
        }
    return MCE_OK;
}

mce_handle* mce_batch_create(int n_est, int d, int cmcc, int pncc, int p, const int* steps, const double* A0,
                             const double* p0, const double* b0, const double* root_point, const double* b_pert,
                             int bpert_stride, int* status)
{
    int st = MCE_OK;
    mce_handle* h = nullptr;
    if (n_est < 1 || d < 1 || d > kMaxDim || !steps || !A0 || !p0 || !b0) {
        set_error("invalid arguments to mce_batch_create");
        if (status) *status = MCE_ERR_ARG;
        return nullptr;
    }
    std::vector<double> roots, bps;
    int stride = bpert_stride;
    if (!root_point || !b_pert) {
        // draw as the reference constructor does, estimator after estimator
        int msmax = 1;
        for (int e = 0; e < n_est; e++) msmax = std::max(msmax, d > 1 ? (steps[e] - 1) * pncc + d : d + pncc);
        roots.resize((size_t)n_est * d);
        bps.assign((size_t)n_est * msmax, 0);
        for (int e = 0; e < n_est; e++) {
            const int ms = d > 1 ? (steps[e] - 1) * pncc + d : d + pncc;
            mce_draw_reference_constants(-1, d, ms, 0, &roots[(size_t)e * d], &bps[(size_t)e * msmax]);
        }
        if (root_point) memcpy(roots.data(), root_point, sizeof(double) * n_est * d);
        if (b_pert) {
            for (int e = 0; e < n_est; e++)
                memcpy(&bps[(size_t)e * msmax], b_pert + (size_t)e * bpert_stride,
                       sizeof(double) * std::min(bpert_stride, msmax));
        }
        root_point = roots.data();
        b_pert = bps.data();
        stride = msmax;
    }
    EngineBase* eng = nullptr;
#define MCE_CASE(D)                                                                                    \
    case D:                                                                                            \
        eng = make_engine_##D();                                                                       \
        st = init_engine_##D(eng, n_est, cmcc, pncc, p, steps, A0, p0, b0, root_point, b_pert, stride); \
        break;
    switch (d) {
        MCE_CASE(1) MCE_CASE(2) MCE_CASE(3) MCE_CASE(4) MCE_CASE(5) MCE_CASE(6) MCE_CASE(7) MCE_CASE(8)
    }
#undef MCE_CASE
    if (st != MCE_OK) {
        delete eng;
        if (status) *status = st;
        return nullptr;
    }
    h = new mce_handle{eng};
    if (status) *status = MCE_OK;
    return h;
}

int mce_batch_step(mce_handle* h, const double* msmt, const double* Phi, const double* Gamma, const double* beta,
                   const double* H, const double* gamma, const double* B, const double* u, int shared_model,
                   int* err_out)
{
    if (!h || !msmt || !Phi || !H || !gamma) return MCE_ERR_ARG;
    if (h->eng->pncc > 0 && (!Gamma || !beta)) return MCE_ERR_ARG;
    static const double zero[kMaxGamma * kMaxDim] = {0};
    const int E = h->eng->E, d = h->eng->d;
    if (shared_model) {
        // one model for every estimator: H and gamma are expanded per estimator
        std::vector<double> Hs((size_t)E * d), gs(E);
        for (int e = 0; e < E; e++) {
            memcpy(&Hs[(size_t)e * d], H, sizeof(double) * d);
            gs[e] = gamma[0];
        }
        return h->eng->step(msmt, Phi, Gamma ? Gamma : zero, beta ? beta : zero, Hs.data(), gs.data(), B, u, 1,
                            err_out);
    }
    return h->eng->step(msmt, Phi, Gamma ? Gamma : zero, beta ? beta : zero, H, gamma, B, u, 0, err_out);
}

int mce_batch_run(mce_handle* h, const double* msmts, int max_steps, const double* Phi, const double* Gamma,
                  const double* beta, const double* H, const double* gamma, const double* B, const double* u,
                  int shared_model, double* fz, double* mean, double* cov, int* err, long long* nt)
{
    if (!h || !msmts || max_steps < 1) return MCE_ERR_ARG;
    EngineBase* g = h->eng;
    const int E = g->E, d = g->d, p = g->p;
    int max_updates = 0;
    for (auto& e : g->est) max_updates = std::max(max_updates, e.num_updates);
    std::vector<double> z(E), gam(E), Hrow((size_t)E * d);
    for (int k = 0; k < max_updates; k++) {
        const int step = k / p, j = k % p;
        for (int e = 0; e < E; e++) {
            z[e] = (step < max_steps) ? msmts[((size_t)e * max_steps + step) * p + j] : 0.0;
            const size_t oe = shared_model ? 0 : (size_t)e;
            gam[e] = gamma[oe * p + j];
            memcpy(&Hrow[(size_t)e * d], H + (oe * p + j) * d, sizeof(double) * d);
        }
        const double* uk = u ? u + (size_t)k * E * g->cmcc : nullptr;
        static const double zero[kMaxGamma * kMaxDim] = {0};
        int rc = g->step(z.data(), Phi, Gamma ? Gamma : zero, beta ? beta : zero, Hrow.data(), gam.data(), B, uk,
                         shared_model ? 1 : 0, nullptr);
        if (rc != MCE_OK) return rc;
        for (int e = 0; e < E; e++) {
            const EstHost& s = g->est[e];
            const size_t o = (size_t)e * max_updates + k;
            if (fz) {
                fz[2 * o] = s.fz[0];
                fz[2 * o + 1] = s.fz[1];
            }
            if (mean) memcpy(mean + o * 2 * d, s.mean.data(), sizeof(double) * 2 * d);
            if (cov) memcpy(cov + o * 2 * d * d, s.cov.data(), sizeof(double) * 2 * d * d);
            if (err) err[o] = s.errors;
            if (nt) nt[o] = s.nt;
        }
    }
    return MCE_OK;
}

mce_handle* mce_create(const double* A0, const double* p0, const double* b0, int steps, int d, int cmcc, int pncc,
                       int p, const double* root_point, const double* b_pert, int* status)
{
    const int ms = d > 1 ? (steps - 1) * pncc + d : d + pncc;
    return mce_batch_create(1, d, cmcc, pncc, p, &steps, A0, p0, b0, root_point, b_pert, ms, status);
}

int mce_step(mce_handle* h, double msmt, const double* Phi, const double* Gamma, const double* beta, const double* H,
             double gamma, const double* B, const double* u)
{
    int err = 0;
    int rc = mce_batch_step(h, &msmt, Phi, Gamma, beta, H, &gamma, B, u, 1, &err);
    return rc == MCE_OK ? err : rc;
}

static bool bad(mce_handle* h, int e) { return !h || e < 0 || e >= h->eng->E; }

int mce_get_moments(mce_handle* h, int e, double* fz, double* mean, double* cov)
{
    if (bad(h, e)) return MCE_ERR_ARG;
    const EstHost& s = h->eng->est[e];
    if (fz) {
        fz[0] = s.fz[0];
        fz[1] = s.fz[1];
    }
    if (mean) memcpy(mean, s.mean.data(), sizeof(double) * s.mean.size());
    if (cov) memcpy(cov, s.cov.data(), sizeof(double) * s.cov.size());
    return MCE_OK;
}

int mce_get_raw_moments(mce_handle* h, int e, double* fz, double* mean, double* cov, double* gsf)
{
    if (bad(h, e)) return MCE_ERR_ARG;
    const EstHost& s = h->eng->est[e];
    if (fz) {
        fz[0] = s.raw_fz[0];
        fz[1] = s.raw_fz[1];
    }
    if (mean) memcpy(mean, s.raw_mean.data(), sizeof(double) * s.raw_mean.size());
    if (cov) memcpy(cov, s.raw_cov.data(), sizeof(double) * s.raw_cov.size());
    if (gsf) *gsf = s.gscale;
    return MCE_OK;
}

int mce_get_errors(mce_handle* h, int e) { return bad(h, e) ? MCE_ERR_ARG : h->eng->est[e].errors; }
long long mce_num_terms(mce_handle* h, int e) { return bad(h, e) ? MCE_ERR_ARG : h->eng->est[e].nt; }
int mce_terms_per_shape(mce_handle* h, int e, int* out, int n)
{
    if (bad(h, e) || !out) return MCE_ERR_ARG;
    const auto& t = h->eng->est[e].tps;
    for (int i = 0; i < n; i++) out[i] = i < (int)t.size() ? t[i] : 0;
    return MCE_OK;
}
int mce_cpdf_1d_grid(mce_handle* h, int e, int marg_idx, const double* bar_nu, double grid_low, double grid_high,
                     double grid_res, int max_points, double* x, double* y)
{
    if (bad(h, e)) return MCE_ERR_ARG;
    return h->eng->cpdf_1d_grid(e, marg_idx, bar_nu, grid_low, grid_high, grid_res, max_points, x, y);
}
// shift_cf_by_bias (cauchy_estimator.hpp:1312-1327): no shift after the final MU
int mce_shift_cf_by_bias(mce_handle* h, int e, const double* bias)
{
    if (bad(h, e) || !bias) return MCE_ERR_ARG;
    EngineBase* g = h->eng;
    if (g->master_step >= g->est[e].num_updates) return MCE_OK;
    return g->shift_terms_b(e, bias, 0);
}
// deterministic_time_prop (cauchy_estimator.hpp:1329-1352): B u only when both are given
int mce_deterministic_time_prop(mce_handle* h, int e, const double* Phi, const double* B, const double* u)
{
    if (bad(h, e) || !Phi) return MCE_ERR_ARG;
    if ((B == nullptr) != (u == nullptr)) {
        set_error("deterministic_time_prop: give both B and u or neither");
        return MCE_ERR_ARG;
    }
    EngineBase* g = h->eng;
    const int d = g->d, cm = g->cmcc;
    std::vector<double> Bu;
    if (B && cm > 0) {
        // matvecmul(B, u) in the reference's order (cauchy_term.hpp:449-453)
        Bu.assign(d, 0.0);
        for (int i = 0; i < d; i++) {
            double s = 0.0;
            for (int j = 0; j < cm; j++) s += B[i * cm + j] * u[j];
            Bu[i] = s;
        }
    }
    return g->time_prop_terms(e, Phi, Bu.empty() ? nullptr : Bu.data());
}
// finalize_extended_moments (cauchy_estimator.hpp:1354-1388): b -= Re(mean) for
// every term (not after the final MU), then mean += x_bar, x_bar = Re(mean)
int mce_finalize_extended_moments(mce_handle* h, int e, double* x_bar)
{
    if (bad(h, e) || !x_bar) return MCE_ERR_ARG;
    EngineBase* g = h->eng;
    const int d = g->d;
    EstHost& eh = g->est[e];
    if (g->master_step < g->est[e].num_updates) {
        std::vector<double> dx(d);
        for (int i = 0; i < d; i++) dx[i] = eh.mean[2 * i];
        const int s = g->shift_terms_b(e, dx.data(), 1);
        if (s != MCE_OK) return s;
    }
    for (int i = 0; i < d; i++) eh.mean[2 * i] += x_bar[i];
    for (int i = 0; i < d; i++) x_bar[i] = eh.mean[2 * i];
    return MCE_OK;
}
int mce_cpdf_nd(mce_handle* h, int e, const double* x, int npts, double* out)
{
    if (bad(h, e)) return MCE_ERR_ARG;
    return h->eng->cpdf_nd(e, x, npts, out);
}
int mce_cpdf_marginal(mce_handle* h, int e, const int* marg_idx, int n_marg, const double* nu_bar, const double* x,
                      int npts, double* out)
{
    if (bad(h, e)) return MCE_ERR_ARG;
    return h->eng->cpdf_marginal(e, marg_idx, n_marg, nu_bar, x, npts, out);
}
int mce_cpdf_2d_grid(mce_handle* h, int e, int marg_idx1, int marg_idx2, const double* bar_nu, double gridx_low,
                     double gridx_high, double gridx_res, double gridy_low, double gridy_high, double gridy_res,
                     int reset_cache, int max_points, double* x, double* y, double* z)
{
    if (bad(h, e)) return MCE_ERR_ARG;
    return h->eng->cpdf_2d_grid(e, marg_idx1, marg_idx2, bar_nu, gridx_low, gridx_high, gridx_res, gridy_low,
                                gridy_high, gridy_res, reset_cache, max_points, x, y, z);
}
int mce_draw_bar_nu(long long seed, int d, double* bar_nu)
{
    if (d < 1 || !bar_nu) return MCE_ERR_ARG;
    if (seed >= 0) srand((unsigned)seed);
    // random_uniform_open (random_variables.hpp:36-40), doubled
    for (int i = 0; i < d; i++) bar_nu[i] = 2 * (((double)rand() + 1.0) / ((double)RAND_MAX + 2.0));
    return MCE_OK;
}
mce_rel2d* mce_rel2d_create(mce_handle* primary, int est_p, mce_handle* secondary, int est_s, const double* Trel,
                            const double* bar_nu_full, int full_solve, int with_term_approx, double term_approx_eps,
                            double* moments, long long* counts, int* status)
{
    int s = MCE_ERR_ARG;
    mce_rel2d* r = nullptr;
    if (!bad(primary, est_p) && !bad(secondary, est_s) && Trel && bar_nu_full) {
        r = new mce_rel2d();
        s = rel2d_build(r, *primary->eng, est_p, *secondary->eng, est_s, Trel, bar_nu_full, full_solve,
                        with_term_approx, term_approx_eps, moments, counts);
        if (s != MCE_OK) {
            delete r;
            r = nullptr;
        }
    }
    if (status) *status = s;
    return r;
}
int mce_rel2d_grid(mce_rel2d* r, double xlow, double xhigh, double dx, double ylow, double yhigh, double dy,
                   double norm_factor_prim, double norm_factor_sec, int max_points, double* x, double* y, double* z)
{
    if (!r) return MCE_ERR_ARG;
    return rel2d_grid(r, xlow, xhigh, dx, ylow, yhigh, dy, norm_factor_prim, norm_factor_sec, max_points, x, y, z);
}
long long mce_rel2d_num_pairs(mce_rel2d* r) { return r ? r->npairs : MCE_ERR_ARG; }
long long mce_rel2d_num_terms(mce_rel2d* r) { return r ? r->nkept : MCE_ERR_ARG; }
double mce_rel2d_device_ms(mce_rel2d* r, int which) { return r && which >= 0 && which < 3 ? r->ms[which] : -1.0; }
long long mce_rel2d_launch_count(mce_rel2d* r) { return r ? r->launches : MCE_ERR_ARG; }
void mce_rel2d_destroy(mce_rel2d* r) { delete r; }
long long mce_post_mu_terms(mce_handle* h) { return h ? h->eng->post_mu_terms : MCE_ERR_ARG; }
double mce_host_time_ms(mce_handle* h, int which) { return h && which >= 0 && which < 3 ? h->eng->host_ms[which] : -1.0; }
int mce_master_step(mce_handle* h) { return h ? h->eng->master_step : MCE_ERR_ARG; }
int mce_device_errors(mce_handle* h) { return h ? h->eng->device_errors : MCE_ERR_ARG; }
long long mce_total_cells(mce_handle* h, int e) { return bad(h, e) ? MCE_ERR_ARG : h->eng->total_cells(e); }
int mce_dump_terms(mce_handle* h, int e, int max_shape, int* shape, double* A, double* p, double* b, int* cells,
                   int* keys, double* g)
{
    if (bad(h, e)) return MCE_ERR_ARG;
    return h->eng->dump_terms(e, max_shape, shape, A, p, b, cells, keys, g);
}
int mce_reset(mce_handle* h) { return h ? h->eng->reset() : MCE_ERR_ARG; }
long long mce_trim_memory(mce_handle* h, long long min_bytes)
{
    if (!h || min_bytes < 0) return MCE_ERR_ARG;
    const long long r = h->eng->trim(min_bytes);
    if (r < 0) set_error("mce_trim_memory: only between mce_reset (or creation) and the next step");
    return r;
}
int mce_reinitialize_start_statistics(mce_handle* h, int e, const double* A0, const double* p0, const double* b0)
{
    if (bad(h, e) || !A0 || !p0 || !b0) return MCE_ERR_ARG;
    EstHost& s = h->eng->est[e];
    const int d = h->eng->d;
    s.A0.assign(A0, A0 + d * d);
    s.p0.assign(p0, p0 + d);
    s.b0.assign(b0, b0 + d);
    // the reference re-creates the first term at once (setup_first_term,
    // cauchy_estimator.hpp:1302-1309): the next first update starts from these
    return h->eng->upload_start(e);
}
int mce_set_master_step(mce_handle* h, int ms)
{
    if (!h || ms < 0) return MCE_ERR_ARG;
    h->eng->master_step = ms;
    return MCE_OK;
}
int mce_set_print_basic_info(mce_handle* h, int e, int on)
{
    if (!h) return MCE_ERR_ARG;
    if (e < 0) {
        for (auto& s : h->eng->est) s.print_basic_info = on != 0;
        return MCE_OK;
    }
    if (bad(h, e)) return MCE_ERR_ARG;
    h->eng->est[e].print_basic_info = on != 0;
    return MCE_OK;
}
int mce_set_window_number(mce_handle* h, int w)
{
    if (!h) return MCE_ERR_ARG;
    for (auto& e : h->eng->est) e.win_num = w;
    return MCE_OK;
}
double mce_last_step_ms(mce_handle* h) { return h ? h->eng->last_ms : -1.0; }
double mce_device_time_ms(mce_handle* h) { return h ? h->eng->device_ms_total : -1.0; }
long long mce_launch_count(mce_handle* h) { return h ? h->eng->launches : MCE_ERR_ARG; }
int mce_set_profiling(mce_handle* h, int mode)
{
    if (!h || mode < 0 || mode > 2) return MCE_ERR_ARG;
    h->eng->prof_mode = mode;
    return MCE_OK;
}
int mce_clear_profile(mce_handle* h)
{
    if (!h) return MCE_ERR_ARG;
    h->eng->clear_prof();
    return MCE_OK;
}
int mce_num_kernel_groups(void) { return KID_COUNT; }
const char* mce_kernel_group_name(int k) { return (k >= 0 && k < KID_COUNT) ? kKernelGroupNames[k] : ""; }
int mce_kernel_group_stats(mce_handle* h, int k, double* ms, long long* launches, double* alg_bytes,
                           double* alg_flops)
{
    if (!h || k < 0 || k >= KID_COUNT) return MCE_ERR_ARG;
    EngineBase* g = h->eng;
    if (ms) *ms = g->kms[k];
    if (launches) *launches = g->klaunch[k];
    if (alg_bytes) *alg_bytes = g->kbytes[k];
    if (alg_flops) *alg_flops = g->kflops[k];
    return MCE_OK;
}
int mce_autotune_configure(int enabled)
{
    if (enabled != 0 && enabled != 1) return MCE_ERR_ARG;
    tune_configure(enabled);
    return MCE_OK;
}
int mce_autotune_table(int* rows, float* best_ms, int max_rows)
{
    if (max_rows < 0 || (max_rows > 0 && !rows)) return MCE_ERR_ARG;
    return tune_table(rows, best_ms, max_rows);
}
const char* mce_autotune_kernel_name(int k)
{
    static const char* names[TK_COUNT] = {"tp", "build_B_vertices", "mu_rows", "gtable_eval",
                                          "gtable_combine", "gtable_prom_eval", "compact", "ftr_resolve"};
    return (k >= 0 && k < TK_COUNT) ? names[k] : "";
}
void mce_destroy(mce_handle* h)
{
    if (!h) return;
    delete h->eng;
    delete h;
}

}  // extern "C"

namespace mce {

void report_error(const std::string& s) { set_error(s); }

// mce_batch_step with the g-table kernel's per-warp scratch placed in
// [scratch, scratch + bytes) and every device allocation refused; the
// entry point mce_batch_step_noalloc (mce_no_alloc.cu) owns the region.
int batch_step_in_fixed_scratch(mce_handle* h, void* scratch, size_t bytes, const double* msmt, const double* Phi,
                                const double* Gamma, const double* beta, const double* H, const double* gamma,
                                const double* B, const double* u, int shared_model, int* err_out)
{
    if (!h || !scratch) return MCE_ERR_ARG;
    EngineBase* g = h->eng;
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != g->device) {
        cudaGetLastError();
        set_error("mce_batch_step_noalloc: the current device (" + std::to_string(cur) +
                  ") is not the handle's device (" + std::to_string(g->device) +
                  "); make the handle's device current first");
        return MCE_ERR_DEVICE;
    }
    // the launcher puts up to 4 warps in a block: one block's slots must fit
    const size_t need = 4 * g->gtable_scratch_bytes_per_warp();
    if (need > bytes) {
        set_error("mce_batch_step_noalloc: a term of up to " + std::to_string(g->MC) + " hyperplanes in " +
                  std::to_string(g->d) + " dimensions needs " + std::to_string(need) +
                  " bytes of g-table scratch, more than the " + std::to_string(bytes) + " bytes of the static array");
        return MCE_ERR_SHAPE;
    }
    struct Restore {
        EngineBase* g;
        ~Restore()
        {
            g_device_alloc_forbidden = false;
            g->fixed_gtable_scratch = nullptr;
            g->fixed_gtable_scratch_bytes = 0;
        }
    } restore{g};
    g->fixed_gtable_scratch = scratch;
    g->fixed_gtable_scratch_bytes = bytes;
    g_device_alloc_forbidden = true;
    const int rc = mce_batch_step(h, msmt, Phi, Gamma, beta, H, gamma, B, u, shared_model, err_out);
    // a step refused part-way may have kernels queued: let them finish so
    // the reset that must follow does not race them
    if (rc != MCE_OK) g->drain();
    return rc;
}

}  // namespace mce

#endif  // MCE_ONLY_DIM <= 0
