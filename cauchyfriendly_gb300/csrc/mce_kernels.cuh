// Kernel launch interface of the MCE step path.  The kernels themselves live
// in mce_kernels.cu (templated on the state dimension D, instantiated for
// D = 1..8); the engine (mce_engine.cu) calls these launchers.
#pragma once
#include "mce_device.cuh"

namespace mce {

// Kernels launched by the calling host thread (every launch site counts
// itself; per thread, so handles stepped from several threads count their own).
extern thread_local long long g_launches;

struct LaunchCfg {
    cudaStream_t stream;
    int num_sms;
    // Cell bitmaps (2^m bits per term) live in shared memory up to
    // kSmemBitmapRows hyperplanes; above that each warp of the bitmap kernels
    // takes a region of this global buffer (gbits_warps regions of the largest
    // per-warp size), and the kernels launch at most that many warps.
    unsigned* gbits = nullptr;
    long long gbits_warps = 0;
    // Cells one reduction group may hold in the g-table kernels' per-warp
    // lists and scratch; 0: half_cells_cap(MC, d), the count of a central
    // arrangement in general position.  A step whose groups hold more (nearly
    // degenerate arrangements) raises it and re-runs the table preparation.
    int cells_cap = 0;
};
// Block-size autotuner of the thread-per-item kernels (grid-stride loops with
// no shared memory, no block-wide step and no reductions, so every block size
// gives bit-identical results).  A launch site asks for its block size by
// (kernel, state dimension, hyperplane capacity, log2 of the item count); the
// first launches of a key try 64, 128, 256 and 512 threads, each twice, timed
// with CUDA events on the launch's stream, and later launches take the
// fastest.  Launches of fewer than 2^15 items keep the default size.
// MCE_AUTOTUNE=0 in the environment keeps the fixed sizes.
enum TuneKernel {
    TK_TP = 0,
    TK_BUILD_B_VERTICES,
    TK_MU_ROWS,
    TK_GTABLE_EVAL,
    TK_GTABLE_COMBINE,
    TK_GTABLE_PROM_EVAL,
    TK_COMPACT,
    TK_FTR_RESOLVE,
    TK_COUNT
};
struct TuneLaunch {
    int block = 128;
    void* entry = nullptr;  // set when this launch is a timed measurement
};
TuneLaunch tune_begin(int kernel, int D, int MC, long long items, int def_block, int max_block, cudaStream_t st);
void tune_end(const TuneLaunch& t, cudaStream_t st);
// The settled keys as rows (kernel, D, MC, log2 items, block) and the best
// sample's ms; returns how many there are (fills at most n).
int tune_table(int* out, float* best_ms, int n);
// Drops every tuned key and turns the tuner on or off.
void tune_configure(int enabled);
constexpr int kSmemBitmapRows = 16;
constexpr int kMaxBitmapRows = 24;
inline int cells_cap_of(const LaunchCfg& c, int MC, int D)
{
    return c.cells_cap > 0 ? c.cells_cap : half_cells_cap(MC, D);
}
// words of one warp's bitmap region in the g-table kernels (the largest user)
inline long long gtable_bitmap_words(int MC, int D, int cells_cap = 0)
{
    const long long words = (1LL << MC) > 32 ? (1LL << MC) / 32 : 1;
    return 3 * words + 32 + (cells_cap > 0 ? cells_cap : half_cells_cap(MC, D));
}

// N-D conditional pdf (csrc/mce_ndpdf.cu): one estimator's terms (a
// contiguous range of a parent list) and tables.
struct NdInput {
    int D = 0, MC = 0;
    int MB = 0;  // the most rows any of the terms has (MC: the storage's row capacity)
    long long n = 0;
    const int* m = nullptr;
    const double* A = nullptr;  // [n][MC][D]
    const double* p = nullptr;  // [n][MC]
    const double* b = nullptr;  // [n][D]
    const long long* toff = nullptr;
    const int* tcnt = nullptr;
    const int* keys = nullptr;
    const cd* vals = nullptr;
    double fz = 0;  // Re fz, the normaliser
    // The marginal pdf of nkeep states (0: the pdf of the full state): the
    // state order with the states integrated out first and the kept ones last
    // (reorient[j] = the state in position j), and the point nu_bar[D - nkeep]
    // at which the terms left after nkeep lowerings are looked up (host).
    int nkeep = 0;
    int reorient[kMaxDim] = {0};
    const double* nu_bar = nullptr;
};
struct NdWork;
NdWork* nd_work_create();
void nd_work_destroy(NdWork* w);
// The pdf at npts points x_host[npts][D] (the marginal: [npts][nkeep], the
// kept states in ascending order) into out_host[2 * npts] (re, im); kernels
// launched are added to *launches.
int nd_pdf_eval(const NdInput& in, const double* x_host, int npts, double* out_host, NdWork* w, const LaunchCfg& lc,
                long long* launches);

// Scratch for the device-wide scans.
struct ScanScratch {
    long long* block_sums;  // capacity >= ceil(n / 2048) + 1 at every level
    long long cap;
};

// out[i] = sum_{k<i} in[k] for i in [0, n]; out[n] holds the total.
void scan_int_to_ll(const int* in, long long* out, long long n, ScanScratch& s, const LaunchCfg& c);

// Relative-then-transformed 2-D system of two estimators
// (cauchy_prediction.hpp:306-971).  Pairs are numbered in the reference's
// single-thread order: primary shape, secondary shape, primary term,
// secondary term; a block is one (primary shape, secondary shape) pair.
struct Rel2DBlock {
    long long off;  // first pair of the block
    int po, pc;     // primary terms of the shape: first slot in idxP, count
    int so, sc;     // secondary terms of the shape: first slot in idxS, count
};
struct Rel2DArgs {
    ParentList P, S;  // the two estimators' term lists
    Tables TP, TS;
    int MCp, MCs;
    const long long* idxP;  // term indices of the primary, by shape then position
    const long long* idxS;
    const Rel2DBlock* blk;
    int nblk;
    long long npairs;
    const double* Trel;     // 2 x D, row-major
    const double* nu_full;  // D
    int full;               // FULL_SOLVE: all 2m cells instead of m
    int approx;             // with_term_approx
    int moments;            // get_relative_moments
    double eps, approx_nf;  // term_approx_eps; (1/2pi)^2 / fz_prim / fz_sec
    int CC;                 // cells per cache row
    double* tt;             // npairs x rel2d_stride(CC)
    int* keep;              // npairs: 0 where the term was approximated out
    double* mrows;          // npairs x 14: g, g y_j, -(g y_j y_k) as (re, im)
};
// doubles per cache row: m, b[2], sin[CC+1], cos[CC+1], gamma1 re[CC], gamma2 re[CC], g[CC] (re, im)
__host__ __device__ inline int rel2d_stride(int CC) { return 6 * CC + 5; }

// bucket positions kept per record between term-reduction rounds
constexpr int kFtrResume = 8;

template <int D>
struct Kernels {
    // First measurement update (cauchy_estimator.hpp:1179-1208).
    static void first_count(const double* A0, const EstStep<D>* st, int E, int* cnt, const LaunchCfg& c);
    static void first_build(const double* A0, const double* p0, const double* b0, const EstStep<D>* st,
                            const double* roots, int E, const long long* pstart, ParentList P, int MC,
                            cd* est_raw, const LaunchCfg& c);
    static void first_tables(ParentList P, long long nP, const double* cval, const double* dval,
                             const unsigned* hof, const double* gscale, Tables T, int MC, const LaunchCfg& c);

    // Time propagation, TP coalignment and child counting (cauchy_term.hpp:84-145, 435-531).
    static void tp(ParentList P, long long nP, const EstStep<D>* st, int with_tp, int MC, int* Bcap,
                   int* nvert, int* err, const LaunchCfg& c);
    // B tables: TP enumeration (cell_enumeration.hpp:676-855) or a copy of the parent keys.
    static void build_B(ParentList P, long long nP, const EstStep<D>* st, int with_tp, Tables Told,
                        int* Bkeys, long long Bcap_total, const double* bpert, int MC, const int* combo_off,
                        const unsigned char* combos, const long long* voff, long long nv, int* vsv, int* err,
                        const LaunchCfg& c);
    // Measurement update, g/yei evaluation, moment partials, MU coalignment.
    static void mu(ParentList P, long long nP, const EstStep<D>* st, const long long* pstart,
                   const double* roots, Tables Told, int* Bkeys, TermRecs R, long long nR,
                   const long long* kall_scan, long long nterms, double* frow, int* fint, cd* contrib, int MC,
                   int* err, const LaunchCfg& c);
    // Per-estimator moment sums in the reference's order and finalisation
    // (cauchy_estimator.hpp:307-357); the chains start in the estimator order
    // given by order (null: 0..E-1), longest first when the caller sorts.
    static void moments(const cd* contrib, const long long* pstart, const long long* kall_scan, int E,
                        const int* order, const EstStep<D>* st, double* tot, cd* est_raw, double* gscale,
                        const LaunchCfg& c);
    // Fast term reduction (term_reduction.hpp:159-276) over the post-MU records:
    // grid cells of b, counting-sorted buckets, near predecessors.
    static void ftr_cells(TermRecs R, long long nR, long long hmask, int* slot_of, int* bcount, const LaunchCfg& c);
    static void ftr_scatter(TermRecs R, long long nR, const int* slot_of, const long long* boff, int* bfill,
                            void* ent, const LaunchCfg& c);
    static size_t cell_entry_bytes();
    static void ftr_sort(const void* in, long long n, const int* slot_of, const long long* boff, void* out,
                         const LaunchCfg& c);
    // One resolution round: over every record (wl_in null) or over the
    // worklist of records still waiting, whose length the kernel reads from
    // n_in (device memory, written by the previous round; n_bound, known on
    // the host, bounds it and sizes the grid); the ones that must wait again
    // are appended to wl_out (count n_out); resume holds kFtrResume bucket
    // positions per record.  Rounds thus queue back to back without the host.
    static void ftr_resolve(TermRecs R, long long nR, const void* ent, const long long* boff, long long hmask, int MC,
                            int* status, int* owner, const int* wl_in, const int* n_in, long long n_bound,
                            int* wl_out, int* n_out, int* resume, const LaunchCfg& c);
    // the resolution rounds from first_round on in one persistent cooperative
    // launch (round r: worklist wl[r & 1], count cnt[r % 3]; the counts
    // zeroed, barrier state bar[2] zeroed); MCE_ERR_CUDA when the cooperative
    // launch is not available
    static int ftr_resolve_all(TermRecs R, long long nR, const void* ent, const long long* boff, long long hmask,
                               int MC, int* status, int* owner, int* wl0, int* wl1, int* cnt, int* resume,
                               unsigned* bar, int first_round, int max_rounds, int* err, const LaunchCfg& c);
    // The rounds from round 1 on as a device-side WHILE loop of a CUDA graph
    // (built once per engine by ftr_graph_create; its kernels read their
    // pointers from a device argument block that ftr_graph_launch rewrites);
    // ftr_graph_collect, after the stream has been synchronised, counts the
    // rounds' launches.
    static int ftr_graph_create(void** graph, const LaunchCfg& c);
    static int ftr_graph_launch(void* graph, TermRecs R, long long nR, const void* ent, const long long* boff,
                                long long hmask, int MC, int* status, int* owner, int* wl0, int* wl1, int* cnt,
                                int* resume, int max_rounds, int* err, const LaunchCfg& c);
    static void ftr_graph_collect(void* graph);
    static void ftr_graph_destroy(void* graph);
    // g-tables of every reduction group (flattening.hpp:318-568).
    static void gtable(TermRecs R, const int* roots_list, long long nroots, const int* gcnt,
                       const long long* goff, const int* members, ParentList P, Tables Told, const int* Bkeys,
                       const double* gscale, const long long* toff, Tables Tnew, int* tcnt, int* alive,
                       int* src, cd* scratch, long long scratch_per_warp, const GFlat& f, int MC, int* err,
                       const LaunchCfg& c, long long max_warps = 0);
    // the members left after promotions (GFlat::pr_*), a flat pass
    static void gtable_promoted(TermRecs R, const int* roots_list, long long nroots, long long nmem,
                                long long nitems, long long ncells, const int* members, ParentList P, Tables Told,
                                const int* Bkeys, const double* gscale, const long long* toff, Tables Tnew,
                                const GFlat& f, int MC, const LaunchCfg& c);
    // Root cells into the output keys and each group's flat-pass layout.  A
    // root with more cells than its table slot (toff) or than the cells
    // capacity writes its count to need[r] and sets over[0] = 1, over[1] =
    // max count: the caller re-sizes and runs the preparation again.
    static void gtable_prep(TermRecs R, const int* roots_list, long long nroots, const int* gcnt,
                            const long long* goff, const int* members, ParentList P, Tables Told, const int* Bkeys,
                            const long long* toff, Tables Tnew, const GFlat& f, int* gitems, int* gcells, int MC,
                            int* need, int* over, const LaunchCfg& c);
    static void shift_b(ParentList P, long long a, long long n, const double* v, int sub, const LaunchCfg& c);
    static void det_tp(ParentList P, long long a, long long n, const double* Phi, const double* Bu, int MC,
                       const LaunchCfg& c);
    static void cpdf2d_terms(ParentList P, long long a, long long n, int i1, int i2, const double* bar_nu, Tables T,
                             int MC, double* tt, const LaunchCfg& c);
    static void cpdf1d_terms(ParentList P, long long a, long long n, int marg, const double* bar_nu, Tables T,
                             int MC, double* tt, const LaunchCfg& c);
    static void gtable_combine(TermRecs R, const int* roots_list, long long nroots, const long long* coff,
                               long long ncells, const int* gcnt, const long long* goff, const int* members,
                               ParentList P, Tables Told, const int* Bkeys, const long long* toff, Tables Tnew,
                               int* tcnt, int* alive, int* src, const GFlat& f, int MC, const LaunchCfg& c);
    static void gtable_eval(TermRecs R, const int* roots_list, long long nroots, long long nitems,
                            const long long* goff, const int* members, ParentList P, Tables Told, const int* Bkeys,
                            const double* gscale, const long long* toff, Tables Tnew, const GFlat& f, int MC,
                            const LaunchCfg& c);
    // Moment rows of the current (reduced) terms, compute_moments(false).
    static void post_ftr_terms(ParentList P, long long nP, const double* roots, Tables T, int MC, cd* contrib,
                               const LaunchCfg& c);
    // One relative 2-D term per (primary term, secondary term) pair: its
    // cache row, kept flag and moment contributions.
    static void rel2d_pairs(const Rel2DArgs& a, const LaunchCfg& c);
    // Next parent list (shape-bucketed, stable) from the surviving roots.
    static void compact(TermRecs R, const int* alive, const int* src, long long nR, const int* new_slot,
                        const long long* toff, const int* tcnt, ParentList Pn, int MC, const LaunchCfg& c);
};

// Shape-agnostic kernels.
void group_count(const int* status, const int* owner, long long nR, int* gcnt, const LaunchCfg& c);
// doubles per term record of the marginal 2-D pdf
__host__ __device__ inline int cpdf2d_stride(int MC) { return 6 * MC + 6; }
// marginal 2-D pdf at npts points (xs, ys) from the per-term records of k_cpdf2d_terms
void cpdf2d_points(const double* tt, long long n, int MC, const double* xs, const double* ys, int npts, double fz,
                   double* zs, int* bad, const LaunchCfg& c);
// marginal 1-D pdf at npts points from the per-term records of k_cpdf1d_terms
void cpdf1d_points(const double* tt, long long n, const double* xs, int npts, int exact, double fz, double* ys,
                   const LaunchCfg& c);
// relative 2-D pdf at npts points from the cache rows of the nk kept pairs
// kidx (in order), split into nch chunks: part[nch x npts], then the chunk
// sums in order scaled by (2 - full) (1/2pi)^2 / (nf_prim nf_sec)
void rel2d_points(const double* tt, const long long* kidx, long long nk, int CC, int full, long long chunk,
                  int nch, const double* xs, const double* ys, int npts, double* part, int* bad, const LaunchCfg& c);
// kept pair indices in order from the keep flags and their exclusive scan
void rel2d_compact(const int* keep, const long long* kpos, long long n, long long* kidx, const LaunchCfg& c);
void rel2d_finish(const double* part, int nch, int npts, int full, double nf_prim, double nf_sec, double* zs,
                  const LaunchCfg& c);
// relative moments: the 14 columns of mrows summed over the pairs in order
// (chunks of `chunk` pairs, then the chunk sums), finalised into out[14]
void rel2d_moments(const double* mrows, long long n, long long chunk, double* part, double* out, const LaunchCfg& c);
void group_fill(const int* status, const int* owner, long long nR, const long long* goff, int* gfill,
                int* members, const LaunchCfg& c);
void group_sort(const int* gcnt, const long long* goff, long long nR, const int* members_in, int* members_out,
                const LaunchCfg& c);
void roots_flags(const int* status, const int* m, long long nR, int D, int* is_root, int* cap,
                 const LaunchCfg& c);
void roots_list(const int* is_root, const long long* rscan, long long nR, int* list, const LaunchCfg& c);
// Stable partition of the surviving records of each estimator by shape:
// tiles of records within each estimator (at most partition_tiles_cap(nR, E)
// of them), per-tile shape counts turned into per-tile prefixes (C, in
// place) and the (estimator, shape) histogram; then the slots.
long long partition_tiles_cap(long long nR, int E);
void partition_tiles(const int* alive, const int* m, const long long* rbase, int E, int MCp, long long nR,
                     int* ntile, long long* tstart, int* C, int* hist, ScanScratch& ss, const LaunchCfg& c);
void partition_rank(const int* alive, const int* m, const long long* rbase, int E, int MCp, long long nR,
                    const long long* tstart, const int* P, const long long* bucket_off, int* new_slot,
                    const LaunchCfg& c);
void rbase_kernel(const long long* pstart, const long long* kscan, int E, long long* rbase,
                  const LaunchCfg& c);

}  // namespace mce
