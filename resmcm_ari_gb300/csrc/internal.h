// Internal types shared by the host C++ and the CUDA translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <map>
#include <set>
#include <string>
#include <tuple>
#include <vector>

#include "resmcm_gpu.h"

struct rmcm_handle;
struct rmcm_graph;
struct rmcm_mat;
struct rmcm_batch;

namespace rmcm {

// Device CSR descriptor: rowptr[rows+1] (int64), col[nnz] (int32, rows
// ascending), val[nnz] (uint32 or uint64).  Passed to kernels by value.
struct DevCsr {
    int64_t rows = 0;
    int64_t cols = 0;
    int64_t nnz = 0;
    int64_t *rowptr = nullptr;
    int32_t *col = nullptr;
    void *val = nullptr;
    const uint64_t *rowsum = nullptr;   // per-row sum of values (saturating); null when every value is 1
    // with rowsum: per row {length, row sum saturated to 0xffffffff}, one
    // 8-byte gather where the analysis of a uint32 product needs both
    const uint2 *info = nullptr;
};

// Device-side status words, one int each (set with atomicOr, never cleared by kernels).
enum StatusWord { kOverflow = 0, kInvariant = 1, kArena = 2, kTimeout = 3, kNumStatus = 8 };

// Row bins of the SpGEMM (see spgemm.cu for the kernels that serve them).
enum Bin {
    kBinTiny = 0,      // flops <= 32: one warp per row, register bitonic sort
    kBinHash512 = 1,   // shared-memory hash tables of 512 / 2048 / 8192 slots
    kBinHash2k = 2,
    kBinHash8k = 3,
    kBinDense = 4,     // windowed dense accumulator (presence + counters) in shared memory
    kBinRank = 5,      // whole-row bitmap in shared memory, counts by rank with global atomics
    kBinMicro = 6,     // flops <= G (1, 2, 4, 8 or 16): G lanes per row, one product per lane
    kBinWarp = 7,      // output width <= 2048, few products: a warp per row with its own window
    kNumBins = 8
};

// Tunables of the SpGEMM row binning (the autotuner searches these).
struct Tuning {
    // threads per short row (flops <= 32): 32 = a warp per row (k_tiny);
    // 1..16 = that many lanes per row for rows of at most that many products
    // (k_micro), the rest of the short rows a warp each; 128 = no short-row
    // bins, short rows go to the 128-thread CTAs of the 512-slot hash bin
    int32_t threads_per_row = 4;
    int32_t hash_max_flops = 4096;  // rows above go to the dense / rank bins
    int32_t dense_ratio = 16;       // dense when flops * dense_ratio >= cols (and one window covers cols)
    int32_t warp_max_flops = 2048;  // output width <= 2048 and at most this many flops: warp bin (0: none)
    // dense-bin products: inner indices whose A-column x B-row density reaches
    // 1 / gemm_inv_density go to a tensor-core GEMM (0: never)
    int32_t gemm_inv_density = 512;
    int32_t gemm_min_mflops = 512;   // products with fewer multiply-adds (millions) stay sparse
    double hash_load = 0.5;         // hash table load factor bound: slots >= min(f, cols) / load, load <= 0.75
    bool dense_single_pass = true;  // dense rows in one window: one pass into a padded temporary
    bool short_single_pass = true;  // tiny, micro, hash, warp and unsplit rank rows: one pass into a bounded temporary
    int64_t dense_temp_max_bytes = 8LL << 30;
};

// One profiled product: stats plus the six events that bracket its passes
// (analyze, symbolic + scan, numeric).
struct ProdRecord {
    rmcm_product_stats st{};
    cudaEvent_t ev[8] = {};   // analysis, symbolic, numeric passes; [6..7] the tensor-core GEMMs
};

// Sizes one SpGEMM read back from the device, kept so that the same product
// can be replayed (under CUDA stream capture) without any host round trip.
struct ProductPlan {
    int mode = 0;                    // 0 normal, 1 record, 2 replay
    int32_t counts[kNumBins] = {};
    int32_t dense_max_alen = 0;
    int64_t flops = 0;
    int64_t nnz = 0;
    bool dense_temp = false;
    int64_t max_dense_flops = 0;
    int64_t c_max_row = -1;
    bool split = false;
    int32_t n_front = 0;
    int64_t max_rank_flops = 0;
    int32_t risky_rows = 0;
    bool rank_split = false;
    int32_t rank_n_front = 0;
    int64_t scratch_bytes = 0;
    int32_t pack_cbits = 0;          // column bits of the packed copy of B (0: not packed)
    bool short_temp = false;         // short-row bins ran in one pass into a temporary
    int64_t short_total = 0;         // its slots
    uint32_t short_mask = 0;         // the bins that ran in that pass
};

}  // namespace rmcm

struct rmcm_mat {
    rmcm::DevCsr d;
    int32_t valtype = RMCM_VAL_U32;
    bool graph_owned = false;
    bool ones = false;                  // every value is 1 (leaves): row sums are row lengths
    bool positive = false;              // every value is >= 1 (a counter > 0 then marks presence)
    bool distinct = false;              // no column repeats within a row
    uint64_t *rowsum = nullptr;         // lazily computed row sums (device, rows + 1: the largest value last), owned
                                        // followed by `rows` uint2 {length, sum saturated to 32 bits}
    int64_t max_row = -1;               // longest row (entries); -1 when unknown
    // rows longer than kEstLongRow entries, ascending (device), when known:
    // the estimator gives each a whole CTA
    int32_t *est_long = nullptr;
    int32_t n_est_long = -1;            // -1: not known (the estimator walks every row per warp)
    cudaEvent_t xfer_done = nullptr;    // end of a pending asynchronous download (transfer stream)
    int64_t bytes = 0;
};

struct rmcm_handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int32_t valtype = RMCM_VAL_AUTO;
    int64_t budget = 0;
    int64_t in_use = 0;
    int64_t peak = 0;               // high-water mark of in_use since the last reset
    int64_t launches = 0;
    int sm_count = 0;
    std::string last_error;
    int *d_status = nullptr;        // kNumStatus ints
    int *h_status = nullptr;        // pinned mirror
    int64_t *h_pinned = nullptr;    // small pinned transfer area (64 int64)
    // scratch (grown on demand, stream-ordered)
    void *scratch = nullptr;
    int64_t scratch_bytes = 0;
    cudaEvent_t ev[8] = {};
    // second stream for work that overlaps the main stream's kernels inside
    // one operation (forked and joined with the two events)
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // transfer stream of asynchronous downloads; matrices freed while their
    // download is in flight are released once it has landed
    cudaStream_t xfer = nullptr;
    std::vector<rmcm_mat *> deferred;
    rmcm::Tuning tune;
    int32_t prof_level = 0;
    std::vector<rmcm::ProdRecord> prof;
    std::set<rmcm_graph *> graphs;   // graphs whose leaves live on this handle
    std::set<rmcm_batch *> batches;  // batches recorded on this handle
    bool abort_on_certain_overflow = false;   // spgemm returns EOVERFLOW before computing when sure
    int32_t order_mode = RMCM_ORDER_RES;
};

struct rmcm_graph {
    rmcm_handle *h = nullptr;
    int32_t batches = 0;             // live batches that replay this graph's leaves
    int64_t n = 0, m = 0;
    int32_t max_vt = 0;
    std::vector<int32_t> vtype;
    std::vector<int64_t> adj_ptr;
    std::vector<int32_t> adj_nbr;
    std::vector<int32_t> adj_et;
    std::vector<int64_t> dims;       // per type
    std::vector<int64_t> bin_ptr;    // per type, CSR over bin_ids
    std::vector<int32_t> bin_ids;    // ascending global ids per type
    std::vector<int32_t> local;      // global id -> local id
    std::map<std::tuple<int32_t, int32_t, int32_t, int32_t>, rmcm_mat *> leaves;
};

namespace rmcm {

// Rows with more entries than this get a whole CTA in the estimator.
constexpr int64_t kEstLongRow = 4096;

// ---- error plumbing ------------------------------------------------------
int32_t set_error(rmcm_handle *h, int32_t status, const std::string &msg);
int32_t cuda_error(rmcm_handle *h, cudaError_t e, const char *what);

#define RMCM_CUDA(h, call)                                       \
    do {                                                         \
        cudaError_t _e = (call);                                 \
        if (_e != cudaSuccess) return rmcm::cuda_error((h), _e, #call); \
    } while (0)

#define RMCM_TRY(call)                      \
    do {                                    \
        int32_t _s = (call);                \
        if (_s != RMCM_OK) return _s;       \
    } while (0)

// ---- device memory (stream ordered, budgeted) ----------------------------
int32_t dev_alloc(rmcm_handle *h, void **p, int64_t bytes);
void dev_free(rmcm_handle *h, void *p, int64_t bytes);
// Grow the handle's scratch area to at least `bytes`.
int32_t scratch_reserve(rmcm_handle *h, int64_t bytes);
int32_t mat_alloc(rmcm_handle *h, int64_t rows, int64_t cols, int64_t nnz, int32_t valtype, rmcm_mat **out);
void mat_release(rmcm_handle *h, rmcm_mat *m);
// Copies up to three device ranges into pinned host buffers with a small
// kernel on stream s (chain_dp.cu); false if a buffer is not device-mapped.
bool copy_out_launch(const void *const *src, void *const *dst_host, const int64_t *bytes, cudaStream_t s);
// Read and clear the device status words; maps them to a status code.
int32_t check_status(rmcm_handle *h);

inline int64_t val_bytes(int32_t valtype) { return valtype == RMCM_VAL_U64 ? 8 : 4; }

// ---- kernels (host launchers) --------------------------------------------
// spgemm.cu
int32_t spgemm(rmcm_handle *h, const rmcm_mat *A, const rmcm_mat *B, rmcm_mat **C, int64_t *flops_out,
               ProductPlan *plan = nullptr);
int32_t fill_ones(rmcm_handle *h, void *val, int64_t nnz, int32_t valtype);
// One device pass over an uploaded CSR (val may be null): f[0] bad row
// pointer or column, [1] unsorted row, [2] repeated column, [3] zero value,
// [4] longest row, [5] rows longer than kEstLongRow, listed (unordered, at
// most cap) in long_rows.  Queued on h->stream.
int32_t csr_check(rmcm_handle *h, const DevCsr &M, const void *val, int32_t valtype, unsigned long long *f,
                  int32_t *long_rows, int64_t cap);
int32_t convert_values(rmcm_handle *h, const rmcm_mat *src, int32_t valtype, rmcm_mat **out);
// dense_gemm.cu: tensor-core part of a dense-bin product.  S holds the
// dense part's exact counts in the product's value type (A.rows x ld): the
// sum over the limb GEMMs of G << (bits (i + j)), formed by the GEMM's
// epilogue (tc_gemm.cu).  skip[u] flags the inner indices it covers; the
// entries of A on the others are listed per row (lcol, lval, lcnt).
struct DensePart {
    const void *S = nullptr;
    int64_t ld = 0;
    int32_t limbs = 0, bits = 0;      // B's limbs
    int32_t alimbs = 1, abits = 0;    // A's limbs (limb form; 1 and 0 for the one-limb uint32 form)
    int32_t chunks = 1;               // chunks of the heavy indices (uint64 products)
    int64_t heavy = 0;
    const uint8_t *skip = nullptr;
    // A's light entries: row r's are lcol/lval[rowptr[r] .. + lcnt[r])
    const int32_t *lcol = nullptr;
    const uint32_t *lval = nullptr;
    const int32_t *lcnt = nullptr;
    // with light_flops: row r's light products (B row lengths over its light
    // entries), their largest row sum and their total
    const int64_t *lflops = nullptr;
    int64_t lmax = 0, ltotal = 0;
    void *mem = nullptr, *sel = nullptr, *amem = nullptr;
    int64_t bytes = 0, sel_bytes = 0, abytes = 0;
};
// ev_begin / ev_end (may be null) are recorded around the GEMMs; light_flops
// also counts each row's light products (dp.lflops, dp.lmax, dp.ltotal).
int32_t dense_part_build(rmcm_handle *h, const DevCsr &A, const DevCsr &B, uint64_t bmax, DensePart &dp,
                         cudaEvent_t ev_begin = nullptr, cudaEvent_t ev_end = nullptr, bool light_flops = false);
// uint64 products: A split into limbs too and the heavy indices into chunks.
int32_t dense_part_build64(rmcm_handle *h, const DevCsr &A, const DevCsr &B, DensePart &dp,
                           cudaEvent_t ev_begin = nullptr, cudaEvent_t ev_end = nullptr);
void dense_part_release(rmcm_handle *h, DensePart &dp);
// tc_gemm.cu: S (M x ldn of uint32 or uint64, vbytes) = sum over limbs and
// chunks of Ad_i[:, chunk q] BdT_j[:, chunk q]^T << (bits (i + j)), on
// tcgen05; RMCM_EINVAL for shapes it does not take.
int32_t tc_seed_gemm(rmcm_handle *h, const void *Ad, const void *BdT, int64_t M, int64_t N, int64_t ldn,
                     int32_t la, int32_t lb, int64_t kc, int64_t nq, int32_t bits, int32_t vbytes, void *S,
                     int *err_dev);
// estimator.cu: c_dev[len*len] on the device
int32_t estimate(rmcm_handle *h, rmcm_mat *const *chain, int32_t len, double *c_dev);
// Persistent pinned host memory mirrored by device memory, for small tables
// that kernels read: filled on the host, copied with cudaMemcpyAsync (under
// stream capture the copy node reads the pinned memory at every replay, so
// the table must stay untouched after it is captured).
struct TableArena {
    char *host = nullptr;
    char *dev = nullptr;
    int64_t cap = 0, used = 0;
    bool push(int64_t bytes, void **hp, void **dp) {
        const int64_t b = (bytes + 255) & ~255LL;
        if (used + b > cap) return false;
        *hp = host + used;
        *dp = dev + used;
        used += b;
        return true;
    }
};
// estimator.cu: the estimates of many chains, one launch per level step over
// all of them, each chain bit-identical to estimate()
struct EstChain {
    rmcm_mat *const *mats = nullptr;
    int32_t len = 0;
    double *c_dev = nullptr;     // len x len
};
int32_t estimate_multi(rmcm_handle *h, const EstChain *chains, int32_t n, TableArena &arena);
// chain_dp.cu: split/cost/pairs on the device
int32_t chain_order_dev(rmcm_handle *h, const double *c_dev, int32_t len, int32_t *split_dev, double *cost_dev,
                        int32_t *pairs_dev);
// Launch-only form (no host round trip; usable under stream capture):
// c16/split16/cost16 are 16x16 arrays, pairs32 holds 32 ints.
// ---- executor entry points shared with the server -----------------------
// Leaf CSR of (src, sink, et) in valtype, built on first use (owned by g).
int32_t leaf_of(rmcm_handle *h, rmcm_graph *g, int32_t src, int32_t sink, int32_t et, int32_t valtype,
                rmcm_mat **out);
// Meta-path string -> vertex types (len+1) and edge types (len).
int32_t path_parse(const char *s, std::vector<int32_t> &vts, std::vector<int32_t> &ets);
// Runs a chain in the given post-order pair list (no estimator, no DP);
// widen = uint32 with escalation to uint64 (leaf64 supplies uint64 leaves).
int32_t chain_run_ordered(rmcm_handle *h, rmcm_mat *const *mats, int32_t len, const int32_t *pairs, rmcm_mat **out,
                          rmcm_timings *t, bool widen, const std::function<int32_t(int, rmcm_mat **)> &leaf64);
// Estimates + DP of a chain: c (len*len), split (len*len) and the pair list
// (2*(len-1)) on the host.
int32_t chain_plan(rmcm_handle *h, rmcm_mat *const *mats, int32_t len, double *c, int32_t *split, int32_t *pairs,
                   double *es_s, double *dp_s);

// Launches a digest of m into out_dev[0..1] (nnz, order-free entry hash);
// capture-safe.
int32_t mat_digest_launch(rmcm_handle *h, const rmcm_mat *m, uint64_t *out_dev, int64_t row0 = 0);
// api.cpp: where the blocked final product of a chain delivers its blocks
struct BlockSink {
    int64_t rows_per_block = 0;     // 0: from the estimate and the free budget
    rmcm_block_fn fn = nullptr;
    void *user = nullptr;
};
int32_t chain_order_launch(rmcm_handle *h, const double *c_dev, int32_t len, double *c16, int32_t *split16,
                           double *cost16, int32_t *pairs32);
// chain_dp.cu: the DP of n chains in one launch (c_all, split_all, cost_all:
// 16 x 16 per chain holding its len x len compactly; pairs_all: 32 per chain)
int32_t chain_order_multi(rmcm_handle *h, const double *c_all, const int32_t *lens_dev, int32_t n, int32_t *split_all,
                          double *cost_all, int32_t *pairs_all);
// A row view (rows row pointers from rowptr[0], entries at their positions)
// whose digest goes to out[2 out .. 2 out + 1].
struct DigestJob {
    const int64_t *rowptr = nullptr;
    const int32_t *col = nullptr;
    const void *val = nullptr;
    int64_t rows = 0;
    int32_t vbytes = 4;
    int32_t out = 0;
};
int32_t digest_multi_launch(rmcm_handle *h, const DigestJob *jobs_dev, int32_t njobs, uint64_t *out_dev);
// batch_fused.cu: many chains as block-diagonal waves (see that file)
struct FusedBatch;
int32_t fused_create(rmcm_handle *h, rmcm_graph *g, const char *const *paths, int32_t count, FusedBatch **out);
int32_t fused_run(rmcm_handle *h, FusedBatch *b, int64_t *nnz_out, uint64_t *digest_out, double *seconds);
void fused_info(const FusedBatch *b, int32_t *count, int64_t *launches_per_run, int64_t *nodes);
void fused_free(rmcm_handle *h, FusedBatch *b);

}  // namespace rmcm
