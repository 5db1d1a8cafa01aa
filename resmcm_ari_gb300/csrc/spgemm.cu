// Row-binned Gustavson SpGEMM with exact integer path counts (sm_103a).
//
// Replaces SpGEMM / row_wise_SpGEMM_based_on_bitmap of efficient/resmcm.cpp
// (:586-647).  The reference's product is Boolean: for every row u of A it
// walks B[a] for a in A[u], marks new columns in a per-thread n-byte bitmap
// and appends them in discovery order.  Here every output row is computed
// with its path counts (C[u][v] = sum_a A[u][a] * B[a][v]) and written with
// ascending columns; its column SET is the reference's row.
//
// Pipeline of one product C = A * B (m = A.rows, n = B.cols):
//   1. k_analyze    warp per row: flops(u) = sum |B[a]|, bin of the row.
//   2. k_scatter    row ids into per-bin lists (device-computed offsets).
//   3. symbolic     exact |C[u]| per bin kernel (same kernels, NUMERIC=false).
//   4. scan         device exclusive scan of |C[u]| into C.rowptr (int64).
//   5. numeric      columns + counts per bin kernel (NUMERIC=true).
// Bins (see classify; the thresholds are the handle's tunables):
//   micro   flops <= G      G lanes per row (G = 1..16), one product per lane,
//                           G-wide bitonic sort (only when G is tuned below 32).
//   tiny    flops <= 32     one warp per row; products in registers, bitonic
//                           sort across the warp, segmented sum, ballot compaction.
//   hash*   flops <= 4096   one CTA per row; linear-probing hash table in shared
//                           memory of at least min(flops, n) / load slots
//                           (512/2048/8192; load 0.5 by default, at most 0.75),
//                           then in-place compaction and a bitonic sort.
//   dense   otherwise       one CTA per row; bitmap + counters over a window of
//                           W columns in shared memory; rows wider than W are
//                           processed window by window with per-entry cursors
//                           (B rows are sorted).  Output is emitted word by word
//                           with ballot compaction, so stores are coalesced.
// Overflow: products and sums are checked against the value type; an
// overflow raises the kOverflow status word (the structure stays exact).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>

#include "internal.h"

namespace rmcm {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kEmptyBin = 0x7f;   // bin code of rows with no products
constexpr int kRiskyBit = 0x80;   // bin_of flag: the row's total count may exceed the value type

// Shared-memory windows of the dense bin (columns per window).
constexpr int32_t kDenseWinU32 = 40960;       // 160 KB counters + 40 KB presence bytes
constexpr int32_t kDenseWinU64 = 22528;       // 176 KB counters + 22 KB presence bytes
constexpr int32_t kDenseWinSym = 196608;      // presence bytes only: 192 KB
constexpr int kDenseThreads = 512;
// B is packed for the dense bin when the product has at least this many
// multiply-adds per entry of B.
constexpr int64_t kPackReuse = 64;

__device__ __forceinline__ void raise_status(int *st, int word) { atomicOr(st + word, 1); }

// Overflow of a product or a sum is recorded in a per-thread flag and flushed
// to the kOverflow status word once per warp or CTA (a global atomic per
// overflowing add would serialise the whole GPU on one address).
__device__ __forceinline__ uint32_t mul_chk(uint32_t a, uint32_t b, bool &ovf) {
    const unsigned long long p = (unsigned long long)a * b;
    ovf |= p > 0xffffffffull;
    return (uint32_t)p;
}
__device__ __forceinline__ uint64_t mul_chk(uint64_t a, uint64_t b, bool &ovf) {
    ovf |= __umul64hi(a, b) != 0;
    return a * b;
}
__device__ __forceinline__ void add_shared_chk(uint32_t *p, uint32_t v, bool &ovf) {
    const uint32_t old = atomicAdd(p, v);
    ovf |= old > 0xffffffffu - v;
}
__device__ __forceinline__ void add_shared_chk(uint64_t *p, uint64_t v, bool &ovf) {
    const unsigned long long old = atomicAdd((unsigned long long *)p, (unsigned long long)v);
    ovf |= old > ~0ull - v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(kFull, v, d);
    return v;
}

__device__ __forceinline__ int32_t warp_min(int32_t v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = min(v, __shfl_xor_sync(kFull, v, d));
    return v;
}

// ------------------------------------------------------------------------
// 1. analysis and binning
// ------------------------------------------------------------------------

// Warp bin: output rows of at most kWarpCols columns, kWarpWarps rows per CTA.
constexpr int kWarpCols = 2048;
constexpr int kWarpWarps = 4;

struct BinParams {
    int64_t dense_win;      // columns one numeric dense window covers
    int32_t hash_max;       // flops above -> dense or rank
    int32_t dense_ratio;    // dense when flops * ratio >= cols and one window covers cols
    int32_t micro_max;      // flops <= micro_max -> micro bin (0: none)
    int32_t tiny_max;       // flops <= tiny_max -> tiny bin (32, or 0: none)
    int32_t inv_load_q8;    // 256 / hash load factor, rounded up
    int32_t warp_max;       // flops <= warp_max and cols <= kWarpCols -> warp bin (0: none)
};

// Widest output row the rank bin holds in shared memory (bitmap + prefixes).
constexpr int64_t kRankCols = 1 << 20;

__device__ __forceinline__ int classify(int64_t f, int64_t ncols, const BinParams &bp) {
    if (f == 0) return kEmptyBin;
    if (f <= bp.micro_max) return kBinMicro;
    if (f <= bp.tiny_max) return kBinTiny;
    if (ncols <= kWarpCols && f <= bp.warp_max) return kBinWarp;
    const bool one_window = ncols <= bp.dense_win;
    if (f > bp.hash_max) return (!one_window && ncols <= kRankCols) ? kBinRank : kBinDense;
    if (one_window && f * (int64_t)bp.dense_ratio >= ncols) return kBinDense;
    const int64_t need = (min(f, ncols) * bp.inv_load_q8 + 255) >> 8;
    if (need > 8192) return (!one_window && ncols <= kRankCols) ? kBinRank : kBinDense;
    if (need <= 512) return kBinHash512;
    if (need <= 2048) return kBinHash2k;
    // rows wider than a window that would need the 8192-slot table: the rank
    // bin's bitmap beats sorting up to 8192 entries with block barriers
    if (!one_window && ncols <= kRankCols) return kBinRank;
    return kBinHash8k;
}

__device__ __forceinline__ unsigned long long sat_add(unsigned long long a, unsigned long long b) {
    return a > ~0ull - b ? ~0ull : a + b;
}

// Warp per row of A: flops and bin; per-bin row counts and the longest
// A row of the dense bin (it sizes the cursor scratch).  It also bounds the
// row's total count S = sum_k A[r][k] * rowsum(B[k]) (saturating): no entry
// of the row can exceed S, so a row with S within the value type is marked
// safe (its kernels skip the overflow checks), and a row with S greater than
// (its possible distinct columns) x (largest value) is certain to overflow,
// which raises *certain.
// Per-product totals of the analysis, accumulated per CTA in shared memory
// and added to the global words once per CTA.
struct AnalyzeOut {
    int64_t *flops;                        // per row
    uint8_t *bin_of;                       // per row
    int32_t *bin_count;                    // [kNumBins]
    int32_t *dense_max_alen;
    unsigned long long *flops_total;
    int32_t *certain;
    unsigned long long *dense_max_flops;
    unsigned long long *rank_max_flops;
    int32_t *risky_rows;
    unsigned long long *max_total;        // largest row total bound S
    unsigned long long *short_cap;        // sum of min(flops, cols) over the short-row bins' rows
    unsigned long long *rank_cap;         // the same over the rank bin's rows
};

struct AnalyzeShared {
    int32_t cnt[kNumBins];
    int32_t max_alen;
    int32_t certain;
    int32_t risky;
    unsigned long long flops;
    unsigned long long max_flops;
    unsigned long long max_rank_flops;
    unsigned long long max_total;
    unsigned long long short_cap, rank_cap;
};

__device__ __forceinline__ void analyze_shared_init(AnalyzeShared &sh) {
    if (threadIdx.x < kNumBins) sh.cnt[threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        sh.max_alen = 0;
        sh.certain = 0;
        sh.risky = 0;
        sh.flops = 0;
        sh.max_flops = 0;
        sh.max_rank_flops = 0;
        sh.max_total = 0;
        sh.short_cap = 0;
        sh.rank_cap = 0;
    }
}

__device__ __forceinline__ void analyze_shared_flush(AnalyzeShared &sh, const AnalyzeOut &o) {
    if (threadIdx.x < kNumBins && sh.cnt[threadIdx.x]) atomicAdd(o.bin_count + threadIdx.x, sh.cnt[threadIdx.x]);
    if (threadIdx.x == 0) {
        if (sh.flops) atomicAdd(o.flops_total, sh.flops);
        if (sh.max_alen) atomicMax(o.dense_max_alen, sh.max_alen);
        if (sh.max_flops) atomicMax(o.dense_max_flops, sh.max_flops);
        if (sh.max_rank_flops) atomicMax(o.rank_max_flops, sh.max_rank_flops);
        if (sh.certain) atomicOr(o.certain, 1);
        if (sh.risky) atomicAdd(o.risky_rows, sh.risky);
        if (sh.max_total) atomicMax(o.max_total, sh.max_total);
        if (sh.short_cap) atomicAdd(o.short_cap, sh.short_cap);
        if (sh.rank_cap) atomicAdd(o.rank_cap, sh.rank_cap);
    }
}

// Bin, overflow flags and totals of row r from its products f and its
// saturating count bound srow.
template <typename V>
__device__ __forceinline__ void analyze_row(int64_t r, int64_t f, unsigned long long srow, int64_t alen,
                                            int64_t ncols, const BinParams &bp, const AnalyzeOut &o,
                                            AnalyzeShared &sh) {
    const int b = classify(f, ncols, bp);
    const unsigned long long vmax = sizeof(V) == 4 ? 0xffffffffull : ~0ull;
    const bool risky = sizeof(V) == 4 ? srow > vmax : srow == ~0ull;
    o.flops[r] = f;
    o.bin_of[r] = (uint8_t)(b | (risky ? kRiskyBit : 0));
    if (f) atomicAdd(&sh.flops, (unsigned long long)f);
    if (risky && b != kEmptyBin) atomicAdd(&sh.risky, 1);
    if (sizeof(V) == 4 && risky) atomicMax(&sh.max_total, srow);
    if (sizeof(V) == 4 && risky) {
        const unsigned long long distinct = (unsigned long long)min(f, ncols);
        if (srow == ~0ull || srow / vmax > distinct) sh.certain = 1;
    }
    if (b != kEmptyBin) {
        atomicAdd(&sh.cnt[b], 1);
        // slots of the single-pass temporary, should the row take it
        const unsigned long long cap = (unsigned long long)(f < ncols ? f : ncols);
        if (b == kBinRank) atomicAdd(&sh.rank_cap, cap);
        else if (b != kBinDense) atomicAdd(&sh.short_cap, cap);
        if (b == kBinDense) {
            atomicMax(&sh.max_alen, (int32_t)(alen < (int64_t)INT_MAX ? alen : (int64_t)INT_MAX));
            atomicMax(&sh.max_flops, (unsigned long long)f);
        }
        if (b == kBinRank) atomicMax(&sh.max_rank_flops, (unsigned long long)f);
    }
}

// Products and count bound of A entries [k0, k1) (strided by `step` from k0).
template <typename V>
__device__ __forceinline__ void analyze_entries(const DevCsr &A, const DevCsr &B, int64_t k0, int64_t k1, int step,
                                                int64_t &f, unsigned long long &srow) {
    const V *Aval = (const V *)A.val;
    int64_t k = k0;
    if (sizeof(V) == 4 && B.info) {
        // uint32: one 8-byte gather per entry (length, row sum saturated to
        // 32 bits, read as 2^32 when saturated: the bound stays an upper
        // bound and the exact total stays a lower one)
        auto bsum_of = [](uint32_t s) -> unsigned long long { return s == 0xffffffffu ? (1ull << 32) : s; };
        for (; k + 3 * (int64_t)step < k1; k += 4 * (int64_t)step) {
            int32_t a[4];
            unsigned long long av[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                a[u] = A.col[k + u * step];
                av[u] = Aval[k + u * step];
            }
            uint2 in[4];
#pragma unroll
            for (int u = 0; u < 4; u++) in[u] = B.info[a[u]];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                f += in[u].x;
                const unsigned long long bs = bsum_of(in[u].y);
                const unsigned long long prod = __umul64hi(av[u], bs) ? ~0ull : av[u] * bs;
                srow = sat_add(srow, prod);
            }
        }
        for (; k < k1; k += step) {
            const uint2 in = B.info[A.col[k]];
            f += in.x;
            const unsigned long long av = Aval[k], bs = bsum_of(in.y);
            const unsigned long long prod = __umul64hi(av, bs) ? ~0ull : av * bs;
            srow = sat_add(srow, prod);
        }
        return;
    }
    // four entries per step: their gathers are independent and overlap
    for (; k + 3 * (int64_t)step < k1; k += 4 * (int64_t)step) {
        int32_t a[4];
        unsigned long long av[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            a[u] = A.col[k + u * step];
            av[u] = Aval[k + u * step];
        }
        int64_t lo[4], hi[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            lo[u] = B.rowptr[a[u]];
            hi[u] = B.rowptr[a[u] + 1];
        }
        unsigned long long bsum[4];
#pragma unroll
        for (int u = 0; u < 4; u++) bsum[u] = B.rowsum ? B.rowsum[a[u]] : (unsigned long long)(hi[u] - lo[u]);
#pragma unroll
        for (int u = 0; u < 4; u++) {
            f += hi[u] - lo[u];
            const unsigned long long prod = __umul64hi(av[u], bsum[u]) ? ~0ull : av[u] * bsum[u];
            srow = sat_add(srow, prod);
        }
    }
    for (; k < k1; k += step) {
        const int32_t a = A.col[k];
        const int64_t len = B.rowptr[a + 1] - B.rowptr[a];
        f += len;
        const unsigned long long bsum = B.rowsum ? B.rowsum[a] : (unsigned long long)len;
        const unsigned long long av = Aval[k];
        const unsigned long long prod = __umul64hi(av, bsum) ? ~0ull : av * bsum;
        srow = sat_add(srow, prod);
    }
}

// Warp per row of A: flops and bin; per-bin row counts and the longest
// A row of the dense bin (it sizes the cursor scratch).  It also bounds the
// row's total count S = sum_k A[r][k] * rowsum(B[k]) (saturating): no entry
// of the row can exceed S, so a row with S within the value type is marked
// safe (its kernels skip the overflow checks), and a row with S greater than
// (its possible distinct columns) x (largest value) is certain to overflow,
// which raises *certain.  Rows with more than long_min entries are left to
// k_analyze_long (appended to long_list) so no warp walks a huge row alone.
template <typename V>
__global__ void __launch_bounds__(256) k_analyze(DevCsr A, DevCsr B, BinParams bp, AnalyzeOut o, int64_t long_min,
                                                 int32_t *long_list, int32_t *nlong) {
    __shared__ AnalyzeShared sh;
    analyze_shared_init(sh);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < A.rows; r += nwarps) {
        const int64_t a0 = A.rowptr[r], a1 = A.rowptr[r + 1];
        if (a1 - a0 > long_min) {
            if (lane == 0) long_list[atomicAdd(nlong, 1)] = (int32_t)r;
            continue;
        }
        int64_t f = 0;
        unsigned long long srow = 0;
        analyze_entries<V>(A, B, a0 + lane, a1, 32, f, srow);
        f = warp_sum(f);
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) srow = sat_add(srow, __shfl_xor_sync(kFull, srow, d));
        if (lane == 0) analyze_row<V>(r, f, srow, a1 - a0, B.cols, bp, o, sh);
    }
    __syncthreads();
    analyze_shared_flush(sh, o);
}

// Long rows: the whole grid walks each long row, CTA b taking the b-th slice
// of its entries; partial products (int64) and count bounds (uint64, with a
// saturation flag) meet in per-row accumulators.
template <typename V>
__global__ void __launch_bounds__(256) k_analyze_long(DevCsr A, DevCsr B, const int32_t *long_list,
                                                      const int32_t *nlong, unsigned long long *acc_f,
                                                      unsigned long long *acc_s, int32_t *sat) {
    const int nl = *nlong;
    const int lane = threadIdx.x & 31;
    for (int j = 0; j < nl; j++) {
        const int32_t r = long_list[j];
        const int64_t a0 = A.rowptr[r], alen = A.rowptr[r + 1] - a0;
        const int64_t k0 = a0 + alen * blockIdx.x / gridDim.x, k1 = a0 + alen * (blockIdx.x + 1) / gridDim.x;
        int64_t f = 0;
        unsigned long long srow = 0;
        analyze_entries<V>(A, B, k0 + threadIdx.x, k1, blockDim.x, f, srow);
        f = warp_sum(f);
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) srow = sat_add(srow, __shfl_xor_sync(kFull, srow, d));
        if (lane == 0) {
            if (f) atomicAdd(acc_f + j, (unsigned long long)f);
            if (srow) {
                const unsigned long long old = atomicAdd(acc_s + j, srow);
                if (srow == ~0ull || old > ~0ull - srow) atomicOr(sat + j, 1);
            }
        }
    }
}

template <typename V>
__global__ void __launch_bounds__(256) k_analyze_long_finish(DevCsr A, DevCsr B, BinParams bp, AnalyzeOut o,
                                                             const int32_t *long_list, const int32_t *nlong,
                                                             const unsigned long long *acc_f,
                                                             const unsigned long long *acc_s, const int32_t *sat) {
    __shared__ AnalyzeShared sh;
    analyze_shared_init(sh);
    __syncthreads();
    const int nl = *nlong;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nl; j += gridDim.x * blockDim.x) {
        const int32_t r = long_list[j];
        const unsigned long long srow = sat[j] ? ~0ull : acc_s[j];
        analyze_row<V>(r, (int64_t)acc_f[j], srow, A.rowptr[r + 1] - A.rowptr[r], B.cols, bp, o, sh);
    }
    __syncthreads();
    analyze_shared_flush(sh, o);
}

// Saturating row sums of a matrix's values (warp per row); out[M.rows]
// (zeroed by the caller) receives the largest value, info[r] the row's
// {length, sum saturated to 0xffffffff}.
template <typename V>
__global__ void k_rowsum(DevCsr M, uint64_t *out, uint2 *info) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const V *v = (const V *)M.val;
    unsigned long long vmax = 0;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < M.rows; r += nwarps) {
        unsigned long long sum = 0;
        for (int64_t q = M.rowptr[r] + lane; q < M.rowptr[r + 1]; q += 32) {
            const unsigned long long x = (unsigned long long)v[q];
            sum = sat_add(sum, x);
            vmax = x > vmax ? x : vmax;
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) sum = sat_add(sum, __shfl_xor_sync(kFull, sum, d));
        if (lane == 0) {
            out[r] = sum;
            info[r] = make_uint2((uint32_t)min(M.rowptr[r + 1] - M.rowptr[r], (int64_t)0xffffffff),
                                 sum > 0xffffffffull ? 0xffffffffu : (uint32_t)sum);
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        const unsigned long long o = __shfl_xor_sync(kFull, vmax, d);
        vmax = o > vmax ? o : vmax;
    }
    if (lane == 0 && vmax) atomicMax((unsigned long long *)out + M.rows, vmax);
}

// Packed copy of B for the dense bin's plain path: entry q becomes
// (value << cbits) | column at a position of its own row such that the r-th
// entry of every shared-memory bank (column mod 32) lands in group r, groups
// in order and banks ascending within a group.  Any 32 consecutive positions
// then touch each bank at most twice (once per group they straddle), where
// the sorted order puts several columns of a sparse row on one bank.  Ranks
// within a bank follow the sorted order, so the layout is deterministic.
// An entry's position is start[rank] + (banks below its own in group rank),
// from per-rank tables (group masks and starts) when no bank holds more than
// kPackRanks entries of the row, else from the bank totals directly.
constexpr int kPackWarps = 4;
constexpr int kPackRanks = 1024;

__global__ void __launch_bounds__(kPackWarps * 32) k_pack_banked(DevCsr B, int32_t cbits, uint32_t *pk, int *st) {
    __shared__ int32_t s_cnt[kPackWarps][32];
    __shared__ uint32_t s_mask[kPackWarps][kPackRanks];   // banks with more than r entries
    __shared__ int32_t s_start[kPackWarps][kPackRanks];   // first position of group r
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t *cnt = s_cnt[warp];
    uint32_t *gmask = s_mask[warp];
    int32_t *gstart = s_start[warp];
    const uint32_t *bv = (const uint32_t *)B.val;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < B.rows; r += nwarps) {
        const int64_t q0 = B.rowptr[r], q1 = B.rowptr[r + 1];
        if (q0 == q1) continue;
        cnt[lane] = 0;
        __syncwarp();
        for (int64_t q = q0 + lane; q < q1; q += 32) atomicAdd(&cnt[B.col[q] & 31], 1);
        __syncwarp();
        const int32_t total = cnt[lane];   // entries of bank `lane`
        __syncwarp();
        cnt[lane] = 0;                     // running rank per bank
        const int32_t max_total = __reduce_max_sync(kFull, total);
        const bool tab = max_total <= kPackRanks;
        if (tab) {
            int32_t run = 0;
            for (int32_t g = 0; g < max_total; g++) {
                const uint32_t m = __ballot_sync(kFull, total > g);
                if (lane == 0) {
                    gmask[g] = m;
                    gstart[g] = run;
                }
                run += __popc(m);
            }
        }
        __syncwarp();
        for (int64_t base = q0; base < q1; base += 32) {
            const int64_t q = base + lane;
            const bool ok = q < q1;
            const int32_t c = ok ? B.col[q] : 0;
            const int32_t bank = ok ? (c & 31) : 32 + lane;
            const unsigned peers = __match_any_sync(kFull, bank);
            const int32_t rank = ok ? cnt[bank] + __popc(peers & lt_mask) : 0;
            __syncwarp();
            if (ok && lane == 31 - __clz(peers)) cnt[bank] += __popc(peers);
            __syncwarp();
            int32_t pos = 0;
            if (tab) {
                if (ok) pos = gstart[rank] + __popc(gmask[rank] & ((1u << bank) - 1u));
            } else {
                // entries before (rank, bank): min(total_b, rank) of every
                // bank, plus one of each lower bank that reaches this rank
#pragma unroll 8
                for (int b = 0; b < 32; b++) {
                    const int32_t t = __shfl_sync(kFull, total, b);
                    pos += min(t, rank) + ((b < bank && t > rank) ? 1 : 0);
                }
            }
            if (ok) {
                const uint32_t x = bv[q];
                // the host checked the largest value; a replay on other values would not fit
                if (x >> (32 - cbits)) raise_status(st, kInvariant);
                pk[q0 + pos] = (x << cbits) | (uint32_t)c;
            }
        }
        __syncwarp();
    }
}

// Row ids into per-bin lists laid out back to back (offsets from bin_count).
__global__ void __launch_bounds__(256) k_scatter(int64_t m, const uint8_t *bin_of, const int32_t *bin_count,
                                                 int32_t *bin_cursor, int32_t *lists, int64_t *cnt) {
    // slots are handed out per tile of 256 rows: lanes of a warp with the
    // same bin take consecutive ranks (one shared add per warp and bin), the
    // tile one global add per bin, so a million rows do not queue on a few
    // global counters
    __shared__ int32_t off[kNumBins], s_cnt[kNumBins], s_base[kNumBins];
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid == 0) {
        int32_t s = 0;
        for (int b = 0; b < kNumBins; b++) { off[b] = s; s += bin_count[b]; }
    }
    for (int64_t r0 = (int64_t)blockIdx.x * 256; r0 < m; r0 += (int64_t)gridDim.x * 256) {
        if (tid < kNumBins) s_cnt[tid] = 0;
        __syncthreads();
        const int64_t r = r0 + tid;
        int b = kEmptyBin;
        if (r < m) {
            b = bin_of[r] & ~kRiskyBit;
            if (b == kEmptyBin) cnt[r] = 0;   // rows without products have no entries
        }
        const unsigned peers = __match_any_sync(kFull, b);
        const int leader = __ffs(peers) - 1;
        int32_t wbase = 0;
        if (lane == leader && b != kEmptyBin) wbase = atomicAdd(&s_cnt[b], __popc(peers));
        wbase = __shfl_sync(kFull, wbase, leader);
        const int32_t rank = wbase + __popc(peers & ((1u << lane) - 1u));
        __syncthreads();
        if (tid < kNumBins && s_cnt[tid]) s_base[tid] = atomicAdd(bin_cursor + tid, s_cnt[tid]);
        __syncthreads();
        if (b != kEmptyBin) lists[off[b] + s_base[b] + rank] = (int32_t)r;
        __syncthreads();
    }
}



// ------------------------------------------------------------------------
// tiny bin: one warp per row, <= 32 products held one per lane
// ------------------------------------------------------------------------

template <typename V, bool NUMERIC>
__global__ void __launch_bounds__(256) k_tiny(DevCsr A, DevCsr B, DevCsr C, const int32_t *rows, int32_t nrows,
                                              int64_t *cnt, int *st) {
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const V *Aval = (const V *)A.val;
    const V *Bval = (const V *)B.val;
    bool ovf = false;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nrows; w += nwarps) {
        const int32_t r = rows[w];
        const int64_t a0 = A.rowptr[r], a1 = A.rowptr[r + 1];
        int32_t key = INT_MAX;
        unsigned long long val = 0;
        int filled = 0;                                   // products placed so far (uniform)
        for (int64_t k0 = a0; k0 < a1; k0 += 32) {
            const int64_t k = k0 + lane;
            int32_t len = 0;
            int64_t bs = 0;
            unsigned long long va = 0;
            if (k < a1) {
                const int32_t a = A.col[k];
                bs = B.rowptr[a];
                len = (int32_t)(B.rowptr[a + 1] - bs);
                if (NUMERIC) va = Aval[k];
            }
            int32_t incl = len;                           // inclusive scan of lengths
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int32_t o = __shfl_up_sync(kFull, incl, d);
                if (lane >= d) incl += o;
            }
            const int32_t excl = incl - len;
            const int32_t tot = __shfl_sync(kFull, incl, 31);
            // lanes [filled, filled + tot) take one product each from this chunk
            const unsigned nz = __ballot_sync(kFull, len > 0);
            unsigned starts = (len > 0 && filled + excl < 32) ? (1u << (filled + excl)) : 0u;
            starts = __reduce_or_sync(kFull, starts);
            const int p = lane - filled;
            const bool mine = p >= 0 && p < tot;
            int src = 0;
            if (mine) {
                const unsigned upto = (lane == 31) ? kFull : ((2u << lane) - 1u);
                const int rank = __popc(starts & upto) - 1;   // source = rank-th lane with len > 0
                unsigned rest = nz;
                for (int t = 0; t < rank; t++) rest &= rest - 1u;
                src = __ffs(rest) - 1;
            }
            const int64_t sbs = __shfl_sync(kFull, bs, src);
            const int32_t sex = __shfl_sync(kFull, excl, src);
            const unsigned long long sva = __shfl_sync(kFull, va, src);
            if (mine) {
                const int64_t q = sbs + (p - sex);
                key = B.col[q];
                if (NUMERIC) {
                    const unsigned long long vb = Bval[q];
                    if (sizeof(V) != 4) ovf |= __umul64hi(sva, vb) != 0;
                    val = sva * vb;
                }
            }
            filled += tot;
        }
        // bitonic sort of (key, val) across the warp, ascending keys
#pragma unroll
        for (int kk = 2; kk <= 32; kk <<= 1) {
#pragma unroll
            for (int j = kk >> 1; j > 0; j >>= 1) {
                const int32_t ok = __shfl_xor_sync(kFull, key, j);
                const unsigned long long ov = NUMERIC ? __shfl_xor_sync(kFull, val, j) : 0ull;
                const bool up = (lane & kk) == 0;
                const bool lower = (lane & j) == 0;
                const bool take = (lower == up) ? (ok < key) : (ok > key);
                if (take) { key = ok; if (NUMERIC) val = ov; }
            }
        }
        const int32_t prev = __shfl_up_sync(kFull, key, 1);
        const bool head = key != INT_MAX && (lane == 0 || prev != key);
        const unsigned heads = __ballot_sync(kFull, head);
        if (!NUMERIC) {
            if (lane == 0) cnt[r] = __popc(heads);
        } else {
            // segmented suffix sums: a head ends up with the sum of its run
            unsigned long long s = val;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned long long o = __shfl_down_sync(kFull, s, d);
                const int32_t okey = __shfl_down_sync(kFull, key, d);
                if (lane + d < 32 && okey == key) {
                    ovf |= s > ~0ull - o;
                    s += o;
                }
            }
            if (sizeof(V) == 4 && head) ovf |= s > 0xffffffffull;
            const int64_t base = C.rowptr[r];
            const int64_t rlen = C.rowptr[r + 1] - base;
            if (lane == 0) {
                // single pass (cnt given): the row's slots bound its entries
                const int64_t nh = __popc(heads);
                if (cnt) cnt[r] = nh;
                if (cnt ? nh > rlen : rlen != nh) raise_status(st, kInvariant);
            }
            if (head) {
                const int pos = __popc(heads & lt_mask);
                if (pos < rlen) {
                    C.col[base + pos] = key;
                    ((V *)C.val)[base + pos] = (V)s;
                }
            }
        }
    }
    if (__any_sync(kFull, ovf) && lane == 0) raise_status(st, kOverflow);
}

// Warp bin: rows whose output has at most kWarpCols columns and whose
// products are few (bounded by a tunable): a warp per row with a window of
// its own in shared memory (presence bytes; counters in the numeric pass), so
// a CTA carries several rows at once with no block barrier.  Per chunk of 32
// A entries the warp scans their B row lengths and lane l takes the
// flattened products l, l + 32, ... (four loads in flight); every product
// marks its column's 32-column group in a per-lane mask, and the output pass
// visits only the groups the row touched, 32 columns per ballot, writing the
// columns in order (coalesced) and clearing the window behind it.
template <typename V, bool NUMERIC, bool CHECKED, typename Visit>
__device__ __forceinline__ void warp_row_products(const DevCsr A, const DevCsr B, int64_t a0, int64_t a1,
                                                  int32_t *wpre, int64_t *wbs, V *wva, bool &ovf, Visit visit) {
    const int lane = threadIdx.x & 31;
    const V *Aval = (const V *)A.val;
    const V *Bval = (const V *)B.val;
    for (int64_t k0 = a0; k0 < a1; k0 += 32) {
        const int64_t k = k0 + lane;
        int32_t len = 0;
        int64_t bs = 0;
        V va = 0;
        if (k < a1) {
            const int32_t a = A.col[k];
            bs = B.rowptr[a];
            len = (int32_t)(B.rowptr[a + 1] - bs);
            if (NUMERIC) va = Aval[k];
        }
        int32_t incl = len;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int32_t o = __shfl_up_sync(kFull, incl, d);
            if (lane >= d) incl += o;
        }
        const int32_t tot = __shfl_sync(kFull, incl, 31);
        __syncwarp();   // the previous chunk is done with the staging arrays
        wpre[lane] = incl - len;
        wbs[lane] = bs;
        if (NUMERIC) wva[lane] = va;
        if (lane == 31) wpre[32] = tot;
        __syncwarp();
        int e = 0;
        for (int32_t p0 = 0; p0 < tot; p0 += 128) {
            int32_t c[4];
            V v[4], av[4];
            bool ok[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int32_t p = p0 + 32 * u + lane;
                ok[u] = p < tot;
                c[u] = 0;
                v[u] = 0;
                av[u] = 0;
                if (ok[u]) {
                    while (wpre[e + 1] <= p) e++;
                    const int64_t q = wbs[e] + (p - wpre[e]);
                    c[u] = __ldg(B.col + q);
                    if (NUMERIC) {
                        v[u] = __ldg(Bval + q);
                        av[u] = wva[e];
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                if (!ok[u]) continue;
                V prod = 0;
                if (NUMERIC) prod = CHECKED ? mul_chk(av[u], v[u], ovf) : (V)(av[u] * v[u]);
                visit(c[u], prod);
            }
        }
    }
}

template <typename V, bool NUMERIC>
__global__ void __launch_bounds__(kWarpWarps * 32) k_warp(DevCsr A, DevCsr B, DevCsr C, const int32_t *rows,
                                                          int32_t nrows, int64_t *cnt, int *st,
                                                          const uint8_t *bin_of) {
    using AtomV = typename std::conditional<sizeof(V) == 4, unsigned int, unsigned long long>::type;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int32_t s_pre[kWarpWarps][33];
    __shared__ int64_t s_bs[kWarpWarps][32];
    __shared__ V s_va[kWarpWarps][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    constexpr int W = kWarpCols;
    constexpr int64_t per_warp = W + (NUMERIC ? (int64_t)W * sizeof(V) : 0);
    uint8_t *pres = smem + warp * per_warp;
    V *acc = (V *)(pres + W);
    for (int i = lane; i < (int)(per_warp / 16); i += 32) ((uint4 *)pres)[i] = make_uint4(0, 0, 0, 0);
    __syncwarp();
    bool ovf = false;
    for (int64_t wi = (int64_t)blockIdx.x * kWarpWarps + warp; wi < nrows; wi += (int64_t)gridDim.x * kWarpWarps) {
        const int32_t r = rows[wi];
        const int64_t a0 = A.rowptr[r], a1 = A.rowptr[r + 1];
        const bool checked = NUMERIC && (bin_of[r] & kRiskyBit) != 0;
        uint32_t glo = 0, ghi = 0;   // 32-column groups this lane touched
        auto mark = [&](int32_t c) {
            pres[c] = 1;
            const int g = c >> 5;
            if (g < 32) glo |= 1u << g;
            else ghi |= 1u << (g - 32);
        };
        if (!NUMERIC) {
            warp_row_products<V, false, false>(A, B, a0, a1, s_pre[warp], s_bs[warp], s_va[warp], ovf,
                                               [&](int32_t c, V) { mark(c); });
        } else if (checked) {
            warp_row_products<V, true, true>(A, B, a0, a1, s_pre[warp], s_bs[warp], s_va[warp], ovf,
                                             [&](int32_t c, V p) {
                                                 mark(c);
                                                 add_shared_chk(acc + c, p, ovf);
                                             });
        } else {
            warp_row_products<V, true, false>(A, B, a0, a1, s_pre[warp], s_bs[warp], s_va[warp], ovf,
                                              [&](int32_t c, V p) {
                                                  mark(c);
                                                  atomicAdd((AtomV *)(acc + c), (AtomV)p);
                                              });
        }
        glo = __reduce_or_sync(kFull, glo);
        ghi = __reduce_or_sync(kFull, ghi);
        __syncwarp();   // every product has landed in the window
        const int64_t base = NUMERIC ? C.rowptr[r] : 0;
        const int64_t rlen = NUMERIC ? C.rowptr[r + 1] - base : 0;
        int64_t pos = 0;
        for (int half = 0; half < 2; half++) {
            uint32_t gm = half ? ghi : glo;
            while (gm) {
                const int g = __ffs(gm) - 1 + 32 * half;
                gm &= gm - 1;
                const int lc = g * 32 + lane;
                const bool here = pres[lc] != 0;
                const unsigned bits = __ballot_sync(kFull, here);
                if (here) {
                    if (NUMERIC) {
                        const int64_t o = pos + __popc(bits & lt_mask);
                        if (o < rlen) {
                            C.col[base + o] = lc;
                            ((V *)C.val)[base + o] = acc[lc];
                        }
                        acc[lc] = 0;
                    }
                    pres[lc] = 0;
                }
                pos += __popc(bits);
            }
        }
        if (lane == 0) {
            if (!NUMERIC) {
                cnt[r] = pos;
            } else {
                // single pass (cnt given): the row's slots bound its entries
                if (cnt) cnt[r] = pos;
                if (cnt ? pos > rlen : pos != rlen) raise_status(st, kInvariant);
            }
        }
        __syncwarp();
    }
    if (__any_sync(kFull, ovf) && lane == 0) raise_status(st, kOverflow);
}

// Micro bin: G lanes per row (G = 1, 2, 4, 8 or 16) for rows of at most G
// products, 32/G rows per warp.  Lane g of a group takes the row's g-th
// product (walking the A row until the B lengths pass g), the group sorts
// its keys with a G-wide bitonic network (xor partners stay inside the
// aligned group) and merges equal columns with segmented suffix sums, as
// the warp-per-row bin does for up to 32 products.
template <typename V, bool NUMERIC, int G>
__global__ void __launch_bounds__(256) k_micro(DevCsr A, DevCsr B, DevCsr C, const int32_t *rows, int32_t nrows,
                                               int64_t *cnt, int *st) {
    static_assert(G >= 1 && G <= 16 && (G & (G - 1)) == 0, "G must be a power of two up to 16");
    constexpr int RPW = 32 / G;                       // rows per warp
    const int lane = threadIdx.x & 31;
    const int g = lane & (G - 1);
    const int gbase = lane & ~(G - 1);
    const unsigned gmask = G == 32 ? kFull : (((1u << G) - 1u) << gbase);
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const V *Aval = (const V *)A.val;
    const V *Bval = (const V *)B.val;
    bool ovf = false;
    for (int64_t w0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * RPW; w0 < nrows; w0 += nwarps * RPW) {
        const int64_t w = w0 + lane / G;
        const bool active = w < nrows;
        int32_t r = 0;
        int32_t key = INT_MAX;
        unsigned long long val = 0;
        if (active) {
            r = rows[w];
            const int64_t a1 = A.rowptr[r + 1];
            int64_t acc = 0;
            for (int64_t k = A.rowptr[r]; k < a1 && acc <= g; k++) {
                const int32_t a = A.col[k];
                const int64_t bs = B.rowptr[a];
                const int64_t len = B.rowptr[a + 1] - bs;
                if (g < acc + len) {
                    const int64_t q = bs + (g - acc);
                    key = B.col[q];
                    if (NUMERIC) {
                        const unsigned long long va = Aval[k], vb = Bval[q];
                        if (sizeof(V) != 4) ovf |= __umul64hi(va, vb) != 0;
                        val = va * vb;
                    }
                }
                acc += len;
            }
        }
#pragma unroll
        for (int kk = 2; kk <= G; kk <<= 1) {
#pragma unroll
            for (int j = kk >> 1; j > 0; j >>= 1) {
                const int32_t ok = __shfl_xor_sync(kFull, key, j);
                const unsigned long long ov = NUMERIC ? __shfl_xor_sync(kFull, val, j) : 0ull;
                const bool up = (g & kk) == 0;
                const bool lower = (g & j) == 0;
                const bool take = (lower == up) ? (ok < key) : (ok > key);
                if (take) { key = ok; if (NUMERIC) val = ov; }
            }
        }
        const int32_t prev = __shfl_up_sync(kFull, key, 1, G);
        const bool head = active && key != INT_MAX && (g == 0 || prev != key);
        const unsigned heads = (__ballot_sync(kFull, head) & gmask) >> gbase;
        if (!NUMERIC) {
            if (active && g == 0) cnt[r] = __popc(heads);
        } else {
            unsigned long long sum = val;
#pragma unroll
            for (int d = 1; d < G; d <<= 1) {
                const unsigned long long o = __shfl_down_sync(kFull, sum, d, G);
                const int32_t okey = __shfl_down_sync(kFull, key, d, G);
                if (g + d < G && okey == key) {
                    ovf |= sum > ~0ull - o;
                    sum += o;
                }
            }
            if (sizeof(V) == 4 && head) ovf |= sum > 0xffffffffull;
            if (active) {
                const int64_t base = C.rowptr[r];
                const int64_t rlen = C.rowptr[r + 1] - base;
                if (g == 0) {
                    // single pass (cnt given): the row's slots bound its entries
                    const int64_t nh = __popc(heads);
                    if (cnt) cnt[r] = nh;
                    if (cnt ? nh > rlen : rlen != nh) raise_status(st, kInvariant);
                }
                if (head) {
                    const int pos = __popc(heads & ((1u << g) - 1u));
                    if (pos < rlen) {
                        C.col[base + pos] = key;
                        ((V *)C.val)[base + pos] = (V)sum;
                    }
                }
            }
        }
    }
    if (__any_sync(kFull, ovf) && lane == 0) raise_status(st, kOverflow);
}

// ------------------------------------------------------------------------
// product stream shared by the hash and dense bins
// ------------------------------------------------------------------------
//
// A CTA walks one A row in chunks of kChunk entries.  For a chunk it stages
// in shared memory, per entry t: pre[t] (first flattened product index),
// bs[t] (first B position) and va[t] (the A value); then the flattened
// products pre[0] .. pre[cnt] are split into one contiguous range per warp
// and lane l of a warp visits products base + l, base + 32 + l, ...  Every
// lane is busy whatever the B row lengths, consecutive lanes read
// consecutive B positions (coalesced), and four products are loaded before
// any is consumed so four loads per lane are in flight.

constexpr int kChunk = 512;

template <typename V>
struct ChunkStage {
    int64_t pre[kChunk + 1];   // first flattened product of each entry (short entries only when split)
    int64_t bs[kChunk];        // first B position of each entry
    V va[kChunk];              // A value of each entry
    int32_t len[kChunk];       // B positions of each entry
    int64_t warp_tot[32];
    int32_t ctr;               // next entry for the long-row warps
    int32_t nlong, nfull;      // dense kernel: entries in llist / flist
    int32_t llist[kChunk];     // dense kernel: entries with long B segments
    int32_t flist[kChunk];     // dense kernel: entries whose B segment fills the window
    int32_t wl[32], wf[32];    // per-warp counts while the lists are built
};

// B rows with at least this many products go to the warp-per-row path.
constexpr int kLongRow = 32;

// Block-wide exclusive scan of kChunk int64 lengths held kChunk/NT per thread.
template <int NT>
__device__ __forceinline__ void stage_scan(int64_t (&len)[kChunk / NT], int64_t *pre, int64_t *warp_tot) {
    constexpr int IPT = kChunk / NT;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t mine = 0;
#pragma unroll
    for (int i = 0; i < IPT; i++) mine += len[i];
    int64_t incl = mine;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int64_t o = __shfl_up_sync(kFull, incl, d);
        if (lane >= d) incl += o;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    int64_t base = 0, total = 0;
#pragma unroll
    for (int w = 0; w < NT / 32; w++) {
        const int64_t t = warp_tot[w];
        if (w < warp) base += t;
        total += t;
    }
    int64_t run = base + incl - mine;
#pragma unroll
    for (int i = 0; i < IPT; i++) {
        pre[threadIdx.x * IPT + i] = run;
        run += len[i];
    }
    if (threadIdx.x == 0) pre[kChunk] = total;
    __syncthreads();
}

// Visits every staged product of the chunk: visit(col, product value).
template <int NT, typename V, bool NUMERIC, typename Visit>
__device__ __forceinline__ void stream_chunk(const ChunkStage<V> &sg, int cnt, const DevCsr B, bool checked, bool &ovf,
                                             Visit visit) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int NW = NT / 32;
    const int64_t total = sg.pre[cnt];
    if (total == 0) return;
    const int64_t per = (((total + NW - 1) / NW) + 31) & ~(int64_t)31;
    const int64_t pbeg = (int64_t)warp * per;
    const int64_t pend = min(pbeg + per, total);
    if (pbeg >= pend) return;
    // k = last staged entry with pre[k] <= p (entries with no products are skipped)
    int64_t p0 = min(pbeg + lane, pend - 1);
    int lo = 0, hi = cnt - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sg.pre[mid] <= p0) lo = mid;
        else hi = mid - 1;
    }
    int k = lo;
    const V *Bval = (const V *)B.val;
    for (int64_t base = pbeg; base < pend; base += 128) {
        int32_t c[4];
        V pv[4];
        bool ok[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int64_t p = base + u * 32 + lane;
            ok[u] = p < pend;
            c[u] = 0;
            pv[u] = 0;
            if (ok[u]) {
                while (sg.pre[k + 1] <= p) k++;
                const int64_t q = sg.bs[k] + (p - sg.pre[k]);
                c[u] = B.col[q];
                if (NUMERIC) pv[u] = checked ? mul_chk(sg.va[k], Bval[q], ovf) : (V)(sg.va[k] * Bval[q]);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (ok[u]) visit(c[u], pv[u]);
    }
}

// Visits the products of the staged entries whose B segment has at least
// kLongRow positions: warps take such entries one at a time from a shared
// counter (sg.ctr, zeroed by the caller before staging) and sweep the segment
// 128 positions per step, four loads per lane in flight, no per-product search.
template <typename V, bool NUMERIC, typename Visit>
__device__ __forceinline__ void stream_long(ChunkStage<V> &sg, int cnt, const DevCsr B, bool checked, bool &ovf,
                                            Visit visit) {
    const int lane = threadIdx.x & 31;
    while (true) {
        int i = 0;
        if (lane == 0) i = atomicAdd(&sg.ctr, 1);
        i = __shfl_sync(kFull, i, 0);
        if (i >= cnt) break;
        const int t = sg.llist[i];
        const int32_t L = sg.len[t];
        const int32_t *bc = B.col + sg.bs[t];
        const V *bv = (const V *)B.val + sg.bs[t];
        const V a = NUMERIC ? sg.va[t] : (V)0;
        for (int32_t base = 0; base < L; base += 128) {
            int32_t c[4];
            V v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int32_t o = base + u * 32 + lane;
                c[u] = o < L ? bc[o] : -1;
                if (NUMERIC) v[u] = o < L ? bv[o] : (V)0;
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (c[u] >= 0) visit(c[u], NUMERIC ? (checked ? mul_chk(a, v[u], ovf) : (V)(a * v[u])) : (V)0);
        }
    }
}

// Shared-memory add at a 32-bit shared address (no value returned).
__device__ __forceinline__ void red_shared_add(uint32_t addr, uint32_t v) {
    asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(addr), "r"(v));
}
__device__ __forceinline__ void red_shared_add(uint32_t addr, uint64_t v) {
    asm volatile("red.shared.add.u64 [%0], %1;" ::"r"(addr), "l"(v));
}

// stream_long for rows that need neither overflow checks nor presence bytes:
// add(col, product) only.  Each lane keeps one pointer pair into the B
// segment; whole blocks of 128 positions run unpredicated (eight loads per
// lane in flight, immediate offsets), the remainder once with predicates.
template <typename V, typename Add>
__device__ __forceinline__ void stream_long_plain(ChunkStage<V> &sg, int cnt, const DevCsr B, Add add) {
    const int lane = threadIdx.x & 31;
    while (true) {
        int i = 0;
        if (lane == 0) i = atomicAdd(&sg.ctr, 1);
        i = __shfl_sync(kFull, i, 0);
        if (i >= cnt) break;
        const int t = sg.llist[i];
        const int32_t L = sg.len[t];
        const int64_t q0 = sg.bs[t] + lane;
        const int32_t *pc = B.col + q0;
        const V *pv = (const V *)B.val + q0;
        const V a = sg.va[t];
        for (int32_t nb = L >> 7; nb > 0; nb--, pc += 128, pv += 128) {
            int32_t c[4];
            V v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                c[u] = __ldg(pc + 32 * u);
                v[u] = __ldg(pv + 32 * u);
            }
#pragma unroll
            for (int u = 0; u < 4; u++) add(c[u], (V)(a * v[u]));
        }
        const int32_t rest = (L & 127) - lane;   // this lane's positions: lane, lane + 32, ...
        int32_t c[4];
        V v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            c[u] = 0;
            v[u] = 0;
            if (32 * u < rest) {
                c[u] = __ldg(pc + 32 * u);
                v[u] = __ldg(pv + 32 * u);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (32 * u < rest) add(c[u], (V)(a * v[u]));
    }
}

// stream_long_plain over the packed copy of B (k_pack_banked): one load per
// position, column and value split from the word.
template <typename Add>
__device__ __forceinline__ void stream_long_packed(ChunkStage<uint32_t> &sg, int cnt, const uint32_t *pk,
                                                   int32_t cbits, Add add) {
    const int lane = threadIdx.x & 31;
    const uint32_t cmask = (1u << cbits) - 1u;
    while (true) {
        int i = 0;
        if (lane == 0) i = atomicAdd(&sg.ctr, 1);
        i = __shfl_sync(kFull, i, 0);
        if (i >= cnt) break;
        const int t = sg.llist[i];
        const int32_t L = sg.len[t];
        const uint32_t *pw = pk + sg.bs[t] + lane;
        const uint32_t a = sg.va[t];
        for (int32_t nb = L >> 7; nb > 0; nb--, pw += 128) {
            uint32_t w[4];
#pragma unroll
            for (int u = 0; u < 4; u++) w[u] = __ldg(pw + 32 * u);
#pragma unroll
            for (int u = 0; u < 4; u++) add((int32_t)(w[u] & cmask), a * (w[u] >> cbits));
        }
        const int32_t rest = (L & 127) - lane;
        uint32_t w[4];
#pragma unroll
        for (int u = 0; u < 4; u++) w[u] = 32 * u < rest ? __ldg(pw + 32 * u) : 0u;
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (32 * u < rest) add((int32_t)(w[u] & cmask), a * (w[u] >> cbits));
    }
}

// ------------------------------------------------------------------------
// hash bins: one CTA per row, shared-memory linear probing
// ------------------------------------------------------------------------

template <int S>
__device__ __forceinline__ uint32_t hash_slot(int32_t c) {
    constexpr int LOG = 31 - __builtin_clz(S);
    return ((uint32_t)c * 2654435761u) >> (32 - LOG);
}

template <typename V, bool NUMERIC, int S>
__device__ __forceinline__ void hash_add(V *slot, V p, bool checked, bool &ovf) {
    if (checked) add_shared_chk(slot, p, ovf);
    else atomicAdd((typename std::conditional<sizeof(V) == 4, unsigned int, unsigned long long>::type *)slot, p);
}

template <typename V, bool NUMERIC, int S>
__device__ __forceinline__ int hash_insert(int32_t *keys, V *vals, int32_t c, V p, int *st, bool checked, bool &ovf) {
    uint32_t h = hash_slot<S>(c);
    for (int probe = 0; probe < S; probe++) {
        const int32_t k = ((volatile int32_t *)keys)[h];
        if (k == c) {
            if (NUMERIC) hash_add<V, NUMERIC, S>(vals + h, p, checked, ovf);
            return 0;
        }
        if (k == -1) {
            const int32_t old = atomicCAS(keys + h, -1, c);
            if (old == -1 || old == c) {
                if (NUMERIC) hash_add<V, NUMERIC, S>(vals + h, p, checked, ovf);
                return old == -1;
            }
        }
        h = (h + 1) & (S - 1);
    }
    raise_status(st, kInvariant);   // table full: cannot happen, the bin keeps nnz <= 0.75 * slots
    return 0;
}

// Inclusive prefix sum of v over the lanes of a full warp.
__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int o = __shfl_up_sync(kFull, v, d);
        if (lane >= d) v += o;
    }
    return v;
}

// Block-wide exclusive scan of one int per thread; returns the total.
template <int NT>
__device__ __forceinline__ int block_excl_scan(int v, int *excl, int *s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int o = __shfl_up_sync(kFull, incl, d);
        if (lane >= d) incl += o;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    int base = 0, total = 0;
#pragma unroll
    for (int w = 0; w < NT / 32; w++) {
        const int t = s_warp[w];
        if (w < warp) base += t;
        total += t;
    }
    *excl = base + incl - v;
    __syncthreads();
    return total;
}

// Stages entries [k0, k0 + cnt) of an A row with their whole B rows.
template <int NT, typename V, bool NUMERIC>
__device__ __forceinline__ void stage_full_rows(ChunkStage<V> &sg, const DevCsr A, const DevCsr B, int64_t k0,
                                                int cnt) {
    constexpr int IPT = kChunk / NT;
    int64_t len[IPT];
    const V *Aval = (const V *)A.val;
#pragma unroll
    for (int i = 0; i < IPT; i++) {
        const int t = threadIdx.x * IPT + i;
        len[i] = 0;
        if (t < cnt) {
            const int32_t a = A.col[k0 + t];
            const int64_t b0 = B.rowptr[a];
            len[i] = B.rowptr[a + 1] - b0;
            sg.bs[t] = b0;
            sg.len[t] = (int32_t)len[i];
            if (NUMERIC) sg.va[t] = Aval[k0 + t];
        }
    }
    stage_scan<NT>(len, sg.pre, sg.warp_tot);
}

// stage_full_rows that also lists the entries whose B rows have at least
// kLongRow positions (sg.llist / sg.nlong, sg.ctr zeroed): their length in
// the flattened stream is 0, stream_long_fast takes them a warp at a time.
// One entry per thread (NT == kChunk).
template <int NT, typename V, bool NUMERIC>
__device__ __forceinline__ void stage_rows_split(ChunkStage<V> &sg, const DevCsr A, const DevCsr B, int64_t k0,
                                                 int cnt) {
    static_assert(kChunk == NT, "one A entry per thread");
    constexpr int NW = NT / 32;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    int64_t len[1] = {0};
    bool lng = false;
    if (t < cnt) {
        const int32_t a = A.col[k0 + t];
        const int64_t b0 = B.rowptr[a];
        const int64_t L = B.rowptr[a + 1] - b0;
        sg.bs[t] = b0;
        sg.len[t] = (int32_t)L;
        if (NUMERIC) sg.va[t] = ((const V *)A.val)[k0 + t];
        lng = L >= kLongRow;
        len[0] = lng ? 0 : L;
    }
    const unsigned lb = __ballot_sync(kFull, lng);
    if (lane == 0) sg.wl[warp] = __popc(lb);
    if (t == 0) sg.ctr = 0;
    stage_scan<NT>(len, sg.pre, sg.warp_tot);
    int pl = 0, tl = 0;
#pragma unroll
    for (int w = 0; w < NW; w++) {
        const int x = sg.wl[w];
        if (w < warp) pl += x;
        tl += x;
    }
    if (lng) sg.llist[pl + __popc(lb & ((1u << lane) - 1u))] = t;
    if (t == 0) sg.nlong = tl;
    __syncthreads();
}

// Products of the listed long entries: a warp per entry (taken from sg.ctr),
// whole blocks of 128 positions unpredicated, the rest once with predicates;
// visit(col, product).  CHECKED records overflowing products in ovf.
template <typename V, bool NUMERIC, bool CHECKED, typename Visit>
__device__ __forceinline__ void stream_long_fast(ChunkStage<V> &sg, int cnt, const DevCsr B, bool &ovf,
                                                 Visit visit) {
    const int lane = threadIdx.x & 31;
    while (true) {
        int i = 0;
        if (lane == 0) i = atomicAdd(&sg.ctr, 1);
        i = __shfl_sync(kFull, i, 0);
        if (i >= cnt) break;
        const int t = sg.llist[i];
        const int32_t L = sg.len[t];
        const int64_t q0 = sg.bs[t] + lane;
        const int32_t *pc = B.col + q0;
        const V *pv = (const V *)B.val + q0;
        const V a = NUMERIC ? sg.va[t] : (V)0;
        auto prod = [&](V b) -> V {
            if (!NUMERIC) return (V)0;
            if (CHECKED) return mul_chk(a, b, ovf);
            return (V)(a * b);
        };
        for (int32_t nb = L >> 7; nb > 0; nb--, pc += 128, pv += 128) {
            int32_t c[4];
            V v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                c[u] = __ldg(pc + 32 * u);
                v[u] = NUMERIC ? __ldg(pv + 32 * u) : (V)0;
            }
#pragma unroll
            for (int u = 0; u < 4; u++) visit(c[u], prod(v[u]));
        }
        const int32_t rest = (L & 127) - lane;
        int32_t c[4];
        V v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            c[u] = 0;
            v[u] = 0;
            if (32 * u < rest) {
                c[u] = __ldg(pc + 32 * u);
                if (NUMERIC) v[u] = __ldg(pv + 32 * u);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (32 * u < rest) visit(c[u], prod(v[u]));
    }
}

template <typename V, bool NUMERIC, int S, int NT>
__global__ void __launch_bounds__(NT) k_hash(DevCsr A, DevCsr B, DevCsr C, const int32_t *rows, int32_t nrows,
                                             int64_t *cnt, int *st, const uint8_t *bin_of) {
    extern __shared__ __align__(16) unsigned char smem[];
    int32_t *keys = (int32_t *)smem;
    V *vals = (V *)(keys + S);
    __shared__ ChunkStage<V> sg;
    __shared__ int s_warp[NT / 32];
    const int tid = threadIdx.x;
    bool ovf = false;
    for (int32_t ri = blockIdx.x; ri < nrows; ri += gridDim.x) {
        const int32_t r = rows[ri];
        const int64_t a0 = A.rowptr[r], a1 = A.rowptr[r + 1];
        const bool checked = (bin_of[r] & kRiskyBit) != 0;
        for (int i = tid; i < S; i += NT) {
            keys[i] = -1;
            if (NUMERIC) vals[i] = 0;
        }
        __syncthreads();
        int fresh = 0;
        for (int64_t k0 = a0; k0 < a1; k0 += kChunk) {
            const int n = (int)(a1 - k0 < (int64_t)kChunk ? a1 - k0 : (int64_t)kChunk);
            stage_full_rows<NT, V, NUMERIC>(sg, A, B, k0, n);
            stream_chunk<NT, V, NUMERIC>(sg, n, B, checked, ovf, [&](int32_t c, V p) {
                fresh += hash_insert<V, NUMERIC, S>(keys, vals, c, p, st, checked, ovf);
            });
            __syncthreads();
        }
        if (!NUMERIC) {
            int excl;
            const int total = block_excl_scan<NT>(fresh, &excl, s_warp);
            if (tid == 0) cnt[r] = total;
        } else {
            // compact the occupied slots to the front of the table itself
            // (each thread holds its slots in registers across the scan's
            // barriers), then sort them there
            constexpr int PER = S / NT;
            int32_t kr[PER];
            V vr[PER];
            int mine = 0;
#pragma unroll
            for (int i = 0; i < PER; i++) {
                kr[i] = keys[tid * PER + i];
                vr[i] = vals[tid * PER + i];
                mine += kr[i] != -1;
            }
            int off;
            const int n = block_excl_scan<NT>(mine, &off, s_warp);
#pragma unroll
            for (int i = 0; i < PER; i++) {
                if (kr[i] != -1) {
                    keys[off] = kr[i];
                    vals[off] = vr[i];
                    off++;
                }
            }
            int P = 1;
            while (P < n) P <<= 1;
            for (int i = n + tid; i < P; i += NT) keys[i] = INT_MAX;
            int32_t *sk = keys;
            V *sv = vals;
            __syncthreads();
            for (int kk = 2; kk <= P; kk <<= 1) {
                for (int j = kk >> 1; j > 0; j >>= 1) {
                    for (int i = tid; i < P; i += NT) {
                        const int ixj = i ^ j;
                        if (ixj > i) {
                            const bool up = (i & kk) == 0;
                            const int32_t x = sk[i], y = sk[ixj];
                            if ((x > y) == up) {
                                sk[i] = y;
                                sk[ixj] = x;
                                const V t = sv[i];
                                sv[i] = sv[ixj];
                                sv[ixj] = t;
                            }
                        }
                    }
                    __syncthreads();
                }
            }
            const int64_t base = C.rowptr[r];
            const int64_t rlen = C.rowptr[r + 1] - base;
            if (tid == 0) {
                // single pass (cnt given): the row's slots bound its entries
                if (cnt) cnt[r] = n;
                if (cnt ? (int64_t)n > rlen : rlen != n) raise_status(st, kInvariant);
            }
            const int lim = (int)((int64_t)n < rlen ? (int64_t)n : rlen);
            for (int i = tid; i < lim; i += NT) {
                C.col[base + i] = sk[i];
                ((V *)C.val)[base + i] = sv[i];
            }
        }
        __syncthreads();
    }
    if (__syncthreads_or(ovf) && tid == 0) raise_status(st, kOverflow);
}

// ------------------------------------------------------------------------
// dense bin: one CTA per row, windowed presence bytes + counters in shared memory
// ------------------------------------------------------------------------
//
// Presence is a byte per column written with plain stores (no read-modify-
// write, so lanes hitting neighbouring columns never contend); counters are
// shared-memory atomics.  Output columns of a window are emitted 32 at a time
// with a ballot over the presence bytes, so global stores are coalesced.  A
// row wider than one window is processed window by window: per A entry the
// staging step finds the part of its (sorted) B row inside the window by a
// binary search from a per-entry cursor and records where the next window
// starts; the next window is the one holding the smallest remaining column.

//
// TEMP mode (numeric, single window only): row ri of the bin list is written
// to slot ri of a row-padded temporary (C.col / C.val point at it, slot
// stride `tstride` entries) and its length goes to cnt[r]; the symbolic pass
// is skipped for these rows and k_copy_rows compacts the slots into C.
// Per-product extras of the dense bin (single-window rows only): the packed
// copy of B (k_pack_banked) and the tensor-core part of the product (S: the
// dense part's counts in the product's value type, one row of gld per row of
// A; skip[u] flags the inner indices it covers, whose A entries the kernel
// leaves out).
struct DenseExtra {
    const uint32_t *pk = nullptr;
    int32_t cbits = 0;
    const void *S = nullptr;
    int64_t gld = 0;
    const uint8_t *skip = nullptr;
    const int32_t *lcnt = nullptr;   // with S: row r has lcnt[r] entries (A's light ones) from rowptr[r]
};

template <typename V, bool NUMERIC, bool TEMP, bool PRES = true>
__global__ void __launch_bounds__(kDenseThreads) k_dense(DevCsr A, DevCsr B, DevCsr C, const int32_t *rows,
                                                         int32_t nrows, int64_t *cnt, int32_t *cursors,
                                                         int64_t cur_stride, int32_t W, int *st, int64_t tstride,
                                                         const uint8_t *bin_of, bool positive, bool b_distinct,
                                                         bool abort_mode, DenseExtra ex) {
    constexpr int NT = kDenseThreads;
    constexpr int kPull = 4;   // register accumulators per thread: windows of up to 4 * NT columns
    static_assert(kChunk == NT, "the dense kernel stages one A entry per thread");
    constexpr int IPT = kChunk / NT;
    constexpr int NW = NT / 32;
    using AtomV = typename std::conditional<sizeof(V) == 4, unsigned int, unsigned long long>::type;
    extern __shared__ __align__(16) unsigned char smem[];
    // PRES = false: no presence bytes (every row's counters mark presence;
    // launched only when every value is >= 1 and no row can overflow)
    uint8_t *present = smem;
    V *acc = (V *)(PRES ? smem + (((size_t)W + 15) & ~(size_t)15) : smem);
    __shared__ ChunkStage<V> sg;
    __shared__ int64_t s_warp[NW];
    __shared__ int32_t s_next;
    __shared__ int32_t s_abort;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    const V *Aval = (const V *)A.val;
    const V *Bval = (const V *)B.val;
    if (PRES)
        for (int i = tid; i < W / 16; i += NT) ((uint4 *)present)[i] = make_uint4(0, 0, 0, 0);
    if (NUMERIC)
        for (int i = tid; i < W; i += NT) acc[i] = 0;
    const bool multi = B.cols > W;
    int32_t *cur = multi ? cursors + (int64_t)blockIdx.x * cur_stride : nullptr;
    bool ovf = false;
    __syncthreads();
    for (int32_t ri = blockIdx.x; ri < nrows; ri += gridDim.x) {
        if (abort_mode) {
            // another CTA saw an overflow: the caller recomputes in uint64
            if (tid == 0) s_abort = *(volatile int *)(st + kOverflow);
            __syncthreads();
            if (s_abort) break;
        }
        const int32_t r = rows[ri];
        const int64_t a0 = A.rowptr[r], a1 = ex.lcnt ? a0 + ex.lcnt[r] : A.rowptr[r + 1];
        // A row that cannot overflow needs no checks, and when every input
        // value is >= 1 its counters alone mark presence (no count is 0).
        const bool checked = NUMERIC && (bin_of[r] & kRiskyBit) != 0;
        const bool track = PRES && (!NUMERIC || checked || !positive);
        const int64_t row_base = TEMP ? (int64_t)ri * tstride : (NUMERIC ? C.rowptr[r] : 0);
        const int64_t row_end = TEMP ? row_base + tstride : (NUMERIC ? C.rowptr[r + 1] : 0);
        int64_t out = row_base;
        int64_t total = 0;
        int64_t w0 = 0;
        bool first = true;
        auto visit = [&](int32_t c, V p) {
            const int32_t lc = (int32_t)(c - w0);
            if (track) present[lc] = 1;
            if (NUMERIC) {
                if (checked) add_shared_chk(acc + lc, p, ovf);
                else atomicAdd((AtomV *)(acc + lc), (AtomV)p);
            }
        };
        if constexpr (NUMERIC) {
            if (ex.S) {
                // the row's tensor-core part seeds the counters (one window)
                const V *g = (const V *)ex.S + (int64_t)r * ex.gld;
                for (int c = tid; c < (int)B.cols; c += NT) acc[c] = g[c];
                __syncthreads();
            }
        }
        while (true) {
            const int64_t w1 = min(w0 + (int64_t)W, B.cols);
            if (tid == 0) s_next = INT_MAX;
            int32_t my_next = INT_MAX;
            // B segments covering every column of a narrow window ("full") are
            // accumulated in registers by column owner: no atomics, no presence
            const int32_t wc = (int32_t)(w1 - w0);
            const bool pull_ok = NUMERIC && b_distinct && wc <= kPull * NT;
            V preg[kPull];
#pragma unroll
            for (int j = 0; j < kPull; j++) preg[j] = 0;
            bool pulled = false;
            for (int64_t k0 = a0; k0 < a1; k0 += kChunk) {
                const int n = (int)(a1 - k0 < (int64_t)kChunk ? a1 - k0 : (int64_t)kChunk);
                int64_t len[IPT];
                bool full = false, lng = false;
                int64_t own_lo = 0, own_hi = 0;   // this thread's entry (plain path)
                V own_a = 0;
#pragma unroll
                for (int i = 0; i < IPT; i++) {
                    const int t = tid * IPT + i;
                    len[i] = 0;
                    if (t < n) {
                        const int64_t k = k0 + t;
                        const int32_t a = A.col[k];
                        const int64_t bs = B.rowptr[a];
                        // inner indices of the tensor-core part contribute through G
                        const int64_t be = (ex.skip && ex.skip[a]) ? bs : B.rowptr[a + 1];
                        int64_t lo = bs, hi = be;
                        if (multi) {
                            if (!first) lo = bs + cur[k - a0];
                            // first position with column >= w1
                            int64_t L = lo, R = be;
                            while (L < R) {
                                const int64_t mid = (L + R) >> 1;
                                if (B.col[mid] < w1) L = mid + 1;
                                else R = mid;
                            }
                            hi = L;
                            cur[k - a0] = (int32_t)(hi - bs);
                            if (hi < be) my_next = min(my_next, B.col[hi]);
                        }
                        sg.bs[t] = lo;
                        full = pull_ok && hi - lo == wc;
                        lng = !full && hi - lo >= kLongRow;
                        sg.len[t] = (int32_t)(hi - lo);
                        if (NUMERIC) sg.va[t] = Aval[k];
                        len[i] = (full || lng) ? 0 : hi - lo;   // short segments: flattened stream
                        if (!full && !lng) {
                            own_lo = lo;
                            own_hi = hi;
                            if (NUMERIC) own_a = Aval[k];
                        }
                    }
                }
                // lists of long and full entries (one entry per thread: kChunk == NT)
                const unsigned lb = __ballot_sync(kFull, lng), fb = __ballot_sync(kFull, full);
                if (lane == 0) {
                    sg.wl[warp] = __popc(lb);
                    sg.wf[warp] = __popc(fb);
                }
                if (tid == 0) sg.ctr = 0;
                stage_scan<NT>(len, sg.pre, sg.warp_tot);
                {
                    int pl = 0, pf = 0, tl = 0, tf = 0;
#pragma unroll
                    for (int w = 0; w < NW; w++) {
                        if (w < warp) {
                            pl += sg.wl[w];
                            pf += sg.wf[w];
                        }
                        tl += sg.wl[w];
                        tf += sg.wf[w];
                    }
                    if (lng) sg.llist[pl + __popc(lb & lt_mask)] = tid;
                    if (full) sg.flist[pf + __popc(fb & lt_mask)] = tid;
                    if (tid == 0) {
                        sg.nlong = tl;
                        sg.nfull = tf;
                    }
                }
                __syncthreads();
                bool plain = false;
                if constexpr (NUMERIC && sizeof(V) == 4) {
                    // uint32 counters only: 32-bit shared addresses, no flag tests per
                    // product (the uint64 kernel keeps the general path: the plain one
                    // costs it registers and spills)
                    plain = !checked && !track;
                    if (plain) {
                        const uint32_t acc_s =
                            (uint32_t)__cvta_generic_to_shared(acc) - (uint32_t)w0 * (uint32_t)sizeof(V);
                        auto add = [&](int32_t c, V p) {
                            red_shared_add(acc_s + (uint32_t)c * (uint32_t)sizeof(V), p);
                        };
                        if (sg.nlong) {
                            // pk: packed copy of B (single window only)
                            if (ex.pk) stream_long_packed(sg, sg.nlong, ex.pk, ex.cbits, add);
                            else stream_long_plain<V>(sg, sg.nlong, B, add);
                        }
                        // short segments: each thread adds its own entry's
                        // products (four loads in flight), no flattening
                        const int32_t *bc = B.col;
                        int64_t q = own_lo;
                        for (; q + 3 < own_hi; q += 4) {
                            int32_t c[4];
                            V v[4];
#pragma unroll
                            for (int u = 0; u < 4; u++) {
                                c[u] = __ldg(bc + q + u);
                                v[u] = __ldg(Bval + q + u);
                            }
#pragma unroll
                            for (int u = 0; u < 4; u++) add(c[u], (V)(own_a * v[u]));
                        }
                        for (; q < own_hi; q++) add(__ldg(bc + q), (V)(own_a * __ldg(Bval + q)));
                    }
                }
                if (!plain) {
                    if (sg.nlong) stream_long<V, NUMERIC>(sg, sg.nlong, B, checked, ovf, visit);
                    stream_chunk<NT, V, NUMERIC>(sg, n, B, checked, ovf, visit);
                }
                const int nfull = sg.nfull;
                for (int i0 = 0; i0 < nfull; i0 += 4) {
                    // four full entries per step: sixteen independent loads per thread
                    pulled = true;
                    V bvals[4][kPull];
                    V av[4];
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        const bool ok = i0 + e < nfull;
                        const int t = sg.flist[ok ? i0 + e : i0];
                        av[e] = ok ? sg.va[t] : (V)0;
                        const V *bv = Bval + sg.bs[t];
#pragma unroll
                        for (int j = 0; j < kPull; j++) {
                            const int c = tid + j * NT;
                            bvals[e][j] = (ok && c < wc) ? bv[c] : (V)0;
                        }
                    }
#pragma unroll
                    for (int e = 0; e < 4; e++)
#pragma unroll
                        for (int j = 0; j < kPull; j++) {
                            const V p = checked ? mul_chk(av[e], bvals[e][j], ovf) : (V)(av[e] * bvals[e][j]);
                            if (checked) ovf |= preg[j] > (V)~(V)0 - p;
                            preg[j] += p;
                        }
                }
                __syncthreads();
            }
            if (pulled) {
                // fold the register sums in: each column has one owner, the
                // atomics of this window finished at the barrier above
#pragma unroll
                for (int j = 0; j < kPull; j++) {
                    const int c = tid + j * NT;
                    if (c < wc) {
                        if (checked) ovf |= acc[c] > (V)~(V)0 - preg[j];
                        acc[c] += preg[j];
                        if (track) present[c] = 1;
                    }
                }
                __syncthreads();
            }
            if (multi) {
                my_next = warp_min(my_next);
                if (lane == 0 && my_next != INT_MAX) atomicMin(&s_next, my_next);
            }
            // count the window: warps own contiguous ranges of 32-column groups
            const int groups = (int)((w1 - w0 + 31) >> 5);
            const int gchunk = (groups + NW - 1) / NW;
            const int gb = min(warp * gchunk, groups), ge = min(gb + gchunk, groups);
            int64_t c_w = 0;
            for (int g = gb; g < ge; g++) {
                const int lc = g * 32 + lane;
                const bool here = track ? present[lc] != 0 : acc[lc] != 0;
                c_w += __popc(__ballot_sync(kFull, here));
                if (!NUMERIC && here) present[lc] = 0;
            }
            if (lane == 0) s_warp[warp] = c_w;
            __syncthreads();
            int64_t base = 0, wtot = 0;
#pragma unroll
            for (int w = 0; w < NW; w++) {
                const int64_t t = s_warp[w];
                if (w < warp) base += t;
                wtot += t;
            }
            if (NUMERIC) {
                int64_t pos = out + base;
                for (int g = gb; g < ge; g++) {
                    const int lc = g * 32 + lane;
                    const bool here = track ? present[lc] != 0 : acc[lc] != 0;
                    const unsigned bits = __ballot_sync(kFull, here);
                    if (here) {
                        const int64_t o = pos + __popc(bits & lt_mask);
                        if (o < row_end) {
                            C.col[o] = (int32_t)(w0 + lc);
                            ((V *)C.val)[o] = acc[lc];
                        }
                        acc[lc] = 0;
                        if (track) present[lc] = 0;
                    }
                    pos += __popc(bits);
                }
            }
            out += wtot;
            total += wtot;
            const int32_t nx = multi ? s_next : INT_MAX;
            __syncthreads();
            if (nx == INT_MAX) break;
            w0 = ((int64_t)nx / W) * W;
            first = false;
        }
        if (tid == 0) {
            if (!NUMERIC || TEMP) cnt[r] = total;
            else if (total != row_end - row_base) raise_status(st, kInvariant);
        }
        if (abort_mode && __syncthreads_or(ovf) && tid == 0) raise_status(st, kOverflow);
    }
    if (__syncthreads_or(ovf) && tid == 0) raise_status(st, kOverflow);
}

// ------------------------------------------------------------------------
// split dense rows (single-window rows whose products exceed a fair share)
// ------------------------------------------------------------------------
//
// One CTA per dense row leaves the device idle behind the heaviest row when
// rows are skewed (a few Zipf-popular rows holding most of the products).
// Such a row is split by ranges of its A entries into parts; a CTA per part
// accumulates its range in a shared-memory window (presence bytes + counters,
// as the dense bin does) and adds the window's nonzero counters into a global
// per-row accumulator (uint64 counters + presence bits).  One CTA per split
// row then writes the row in column order.  Counts are non-negative, so a
// part overflows only if the whole row does.

constexpr int kSplitThreads = 512;

// Per dense-list row: split rows (products above fpart, at most max_slots of
// them) go to the back of the permuted list `perm` with a slot and a number
// of parts, the other rows to the front; k_dense then runs over the front.
__global__ void k_split_select(const int32_t *rows, int32_t n, const int64_t *flops, int64_t fpart, int32_t pmax,
                               int32_t *perm, int32_t *front, int32_t *nslots, int32_t *row_of_slot, int32_t *parts,
                               int32_t max_slots) {
    for (int64_t ri = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ri < n; ri += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = rows[ri];
        const int64_t f = flops[r];
        bool split = false;
        if (f > fpart) {
            const int32_t s_ = atomicAdd(nslots, 1);
            if (s_ < max_slots) {
                const int32_t pos = n - 1 - s_;
                perm[pos] = r;
                row_of_slot[s_] = pos;
                parts[s_] = (int32_t)min((int64_t)pmax, (f + fpart - 1) / fpart);
                split = true;
            }
        }
        if (!split) perm[atomicAdd(front, 1)] = r;
    }
}

// Exclusive scan of the parts of the used slots (one block, max_slots <= 1024).
__global__ void __launch_bounds__(1024) k_split_tasks(const int32_t *parts, const int32_t *nslots, int32_t max_slots,
                                                      int32_t *task_start) {
    __shared__ int s_warp[32];
    const int ns = min(*nslots, max_slots);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int v = tid < ns ? parts[tid] : 0;
    int incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int o = __shfl_up_sync(kFull, incl, d);
        if (lane >= d) incl += o;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    int base = 0;
    for (int w = 0; w < warp; w++) base += s_warp[w];
    if (tid < ns) task_start[tid] = base + incl - v;
    if (tid == ns - 1) task_start[ns] = base + incl;
    if (ns == 0 && tid == 0) task_start[0] = 0;
}

// One CTA per task (slot, part): the part's A-entry range into the shared
// window, then its nonzero counters into the slot's global accumulator.
template <typename V, bool PRES = true>
__global__ void __launch_bounds__(kSplitThreads) k_dense_split(DevCsr A, DevCsr B, const int32_t *rows,
                                                               const int32_t *row_of_slot, const int32_t *parts,
                                                               const int32_t *task_start, const int32_t *nslots,
                                                               int32_t max_slots, int32_t W,
                                                               unsigned long long *G, uint32_t *Gbits,
                                                               const uint8_t *bin_of, int *st, int32_t wc,
                                                               bool pull_ok, const uint32_t *pk, int32_t cbits,
                                                               const int32_t *lcnt) {
    constexpr int NT = kSplitThreads;
    constexpr int kPull = 4;   // register accumulators per thread: rows of up to 4 * NT columns
    static_assert(kChunk == NT, "one staged A entry per thread");
    using AtomV = typename std::conditional<sizeof(V) == 4, unsigned int, unsigned long long>::type;
    const V *Aval = (const V *)A.val;
    const V *Bval = (const V *)B.val;
    extern __shared__ __align__(16) unsigned char smem[];
    // PRES = false (every value >= 1, no row can overflow): counters alone
    // mark presence and the window holds only them
    uint8_t *present = smem;
    V *acc = (V *)(PRES ? smem + (((size_t)W + 15) & ~(size_t)15) : smem);
    __shared__ ChunkStage<V> sg;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int ns = min(*nslots, max_slots);
    const int ntasks = task_start[ns];
    if (PRES)
        for (int i = tid; i < W / 16; i += NT) ((uint4 *)present)[i] = make_uint4(0, 0, 0, 0);
    for (int i = tid; i < W; i += NT) acc[i] = 0;
    bool ovf = false;
    __syncthreads();
    for (int task = blockIdx.x; task < ntasks; task += gridDim.x) {
        int lo = 0, hi = ns - 1;   // last slot with task_start <= task
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (task_start[mid] <= task) lo = mid;
            else hi = mid - 1;
        }
        const int slot = lo;
        const int part = task - task_start[slot];
        const int np = parts[slot];
        const int32_t r = rows[row_of_slot[slot]];
        // (lcnt: A holds the row's light entries only, lcnt[r] of them)
        const int64_t a0 = A.rowptr[r], alen = lcnt ? (int64_t)lcnt[r] : A.rowptr[r + 1] - a0;
        const int64_t ka = a0 + alen * part / np, kb = a0 + alen * (part + 1) / np;
        const bool checked = (bin_of[r] & kRiskyBit) != 0;
        // B rows covering all wc columns ("full", as in the dense bin) are
        // accumulated in registers by column owner; the rest stream through
        // the shared-memory counters
        V preg[kPull];
#pragma unroll
        for (int j = 0; j < kPull; j++) preg[j] = 0;
        bool pulled = false;
        for (int64_t k0 = ka; k0 < kb; k0 += kChunk) {
            const int n = (int)(kb - k0 < (int64_t)kChunk ? kb - k0 : (int64_t)kChunk);
            int64_t len1[1] = {0};
            bool full = false, lng = false;
            if (tid < n) {
                const int32_t a = A.col[k0 + tid];
                const int64_t b0 = B.rowptr[a];
                const int64_t len = B.rowptr[a + 1] - b0;
                full = pull_ok && len == wc;
                lng = sizeof(V) == 4 && !full && len >= kLongRow;   // uint64: flattened stream only
                sg.bs[tid] = b0;
                sg.len[tid] = (int32_t)len;
                sg.va[tid] = Aval[k0 + tid];
                len1[0] = (full || lng) ? 0 : len;
            }
            // lists of full entries (register path) and long ones (a warp each)
            const unsigned fb = __ballot_sync(kFull, full), lb = __ballot_sync(kFull, lng);
            if (lane == 0) {
                sg.wf[warp] = __popc(fb);
                sg.wl[warp] = __popc(lb);
            }
            if (tid == 0) sg.ctr = 0;
            stage_scan<NT>(len1, sg.pre, sg.warp_tot);
            int pf = 0, tf = 0, pl = 0, tl = 0;
            for (int w = 0; w < NT / 32; w++) {
                if (w < warp) {
                    pf += sg.wf[w];
                    pl += sg.wl[w];
                }
                tf += sg.wf[w];
                tl += sg.wl[w];
            }
            if (full) sg.flist[pf + __popc(fb & lt_mask)] = tid;
            if (lng) sg.llist[pl + __popc(lb & lt_mask)] = tid;
            __syncthreads();
            // the row's overflow test is chosen here, not per product (uint64
            // keeps the single flattened stream: the split costs it spills)
            if constexpr (sizeof(V) == 8) {
                stream_chunk<NT, V, true>(sg, n, B, checked, ovf, [&](int32_t c, V p) {
                    if (PRES) present[c] = 1;
                    if (checked) add_shared_chk(acc + c, p, ovf);
                    else atomicAdd((AtomV *)(acc + c), (AtomV)p);
                });
            } else if (checked) {
                auto vis = [&](int32_t c, V p) {
                    if (PRES) present[c] = 1;
                    add_shared_chk(acc + c, p, ovf);
                };
                if (tl) stream_long_fast<V, true, true>(sg, tl, B, ovf, vis);
                stream_chunk<NT, V, true>(sg, n, B, true, ovf, vis);
            } else {
                bool done = false;
                if constexpr (sizeof(V) == 4 && !PRES) {
                    // uint32 counters alone: 32-bit shared addresses, packed B when given
                    const uint32_t acc_s = (uint32_t)__cvta_generic_to_shared(acc);
                    auto add = [&](int32_t c, V p) { red_shared_add(acc_s + (uint32_t)c * 4u, p); };
                    if (tl) {
                        if (pk) stream_long_packed(sg, tl, pk, cbits, add);
                        else stream_long_fast<V, true, false>(sg, tl, B, ovf, add);
                    }
                    stream_chunk<NT, V, true>(sg, n, B, false, ovf, add);
                    done = true;
                }
                if (!done) {
                    auto vis = [&](int32_t c, V p) {
                        if (PRES) present[c] = 1;
                        atomicAdd((AtomV *)(acc + c), (AtomV)p);
                    };
                    if (tl) stream_long_fast<V, true, false>(sg, tl, B, ovf, vis);
                    stream_chunk<NT, V, true>(sg, n, B, false, ovf, vis);
                }
            }
            for (int i0 = 0; i0 < tf; i0 += 4) {
                pulled = true;
                V bvals[4][kPull];
                V av[4];
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const bool ok = i0 + e < tf;
                    const int t = sg.flist[ok ? i0 + e : i0];
                    av[e] = ok ? sg.va[t] : (V)0;
                    const V *bv = Bval + sg.bs[t];
#pragma unroll
                    for (int j = 0; j < kPull; j++) {
                        const int c = tid + j * NT;
                        bvals[e][j] = (ok && c < wc) ? bv[c] : (V)0;
                    }
                }
#pragma unroll
                for (int e = 0; e < 4; e++)
#pragma unroll
                    for (int j = 0; j < kPull; j++) {
                        const V p = checked ? mul_chk(av[e], bvals[e][j], ovf) : (V)(av[e] * bvals[e][j]);
                        if (checked) ovf |= preg[j] > (V)~(V)0 - p;
                        preg[j] += p;
                    }
            }
            __syncthreads();
        }
        if (pulled) {
            // each column has one owner; the window's atomics ended at the barrier above
#pragma unroll
            for (int j = 0; j < kPull; j++) {
                const int c = tid + j * NT;
                if (c < wc) {
                    if (checked) ovf |= acc[c] > (V)~(V)0 - preg[j];
                    acc[c] += preg[j];
                    if (PRES) present[c] = 1;
                }
            }
            __syncthreads();
        }
        // merge: one global atomic per present column, then clear the window
        unsigned long long *g = G + (int64_t)slot * W;
        uint32_t *gb = Gbits + (int64_t)slot * (W / 32);
        for (int c = tid; c < W; c += NT) {
            const bool here = PRES ? present[c] != 0 : acc[c] != 0;
            const unsigned bits = __ballot_sync(kFull, here);
            if (here) {
                const unsigned long long v = (unsigned long long)acc[c];
                if (v) {
                    const unsigned long long old = atomicAdd(g + c, v);
                    ovf |= old > ~0ull - v;
                }
                if (PRES) present[c] = 0;
                acc[c] = 0;
            }
            if (lane == 0 && bits) atomicOr(gb + (c >> 5), bits);
        }
        __syncthreads();
    }
    if (__syncthreads_or(ovf) && tid == 0) raise_status(st, kOverflow);
}

// One CTA per split row: the accumulated row, in column order, into its
// padded slot of the temporary (row ri at ri * tstride); its length to cnt.
// With S (the tensor-core part's counts, row r at r * gld; every value
// positive) a column is present when either part has it and its count is
// the sum of both.
template <typename V>
__global__ void __launch_bounds__(kSplitThreads) k_split_finish(DevCsr T, const int32_t *rows,
                                                                const int32_t *row_of_slot, const int32_t *nslots,
                                                                int32_t max_slots, int64_t ncols, int32_t W,
                                                                const unsigned long long *G, const uint32_t *Gbits,
                                                                int64_t tstride, int64_t *cnt, int *st,
                                                                const V *S, int64_t gld) {
    constexpr int NT = kSplitThreads, NW = NT / 32;
    __shared__ int64_t s_warp[NW];
    const int ns = min(*nslots, max_slots);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    bool ovf = false;
    for (int slot = blockIdx.x; slot < ns; slot += gridDim.x) {
        const int32_t ri = row_of_slot[slot];
        const int32_t r = rows[ri];
        const unsigned long long *g = G + (int64_t)slot * W;
        const uint32_t *gb = Gbits + (int64_t)slot * (W / 32);
        const V *srow = S ? S + (int64_t)r * gld : nullptr;
        const int groups = (int)((ncols + 31) >> 5);
        const int gchunk = (groups + NW - 1) / NW;
        const int g0 = min(warp * gchunk, groups), g1 = min(g0 + gchunk, groups);
        // presence bits of group q (warp-uniform)
        auto word = [&](int q) -> unsigned {
            unsigned bits = gb[q];
            if (srow) {
                const int64_t c = (int64_t)q * 32 + lane;
                bits |= __ballot_sync(kFull, c < ncols && srow[c] != 0);
            }
            return bits;
        };
        int64_t mine = 0;
        for (int q = g0; q < g1; q++) mine += __popc(word(q));
        if (lane == 0) s_warp[warp] = mine;
        __syncthreads();
        int64_t base = 0, total = 0;
        for (int w = 0; w < NW; w++) {
            if (w < warp) base += s_warp[w];
            total += s_warp[w];
        }
        int64_t pos = (int64_t)ri * tstride + base;
        for (int q = g0; q < g1; q++) {
            const unsigned bits = word(q);
            if (bits & (1u << lane)) {
                const int64_t o = pos + __popc(bits & lt_mask);
                const int32_t c = q * 32 + lane;
                unsigned long long v = g[c];
                if (srow) {
                    const unsigned long long sv = (unsigned long long)srow[c];
                    ovf |= v > ~0ull - sv;
                    v += sv;
                }
                if (sizeof(V) == 4) ovf |= v > 0xffffffffull;
                T.col[o] = c;
                ((V *)T.val)[o] = (V)v;
            }
            pos += __popc(bits);
        }
        if (tid == 0) cnt[r] = total;
        __syncthreads();
    }
    if (__syncthreads_or(ovf) && tid == 0) raise_status(st, kOverflow);
}

// ------------------------------------------------------------------------
// rank bin: wide rows (more columns than a dense window, at most kRankCols)
// ------------------------------------------------------------------------
//
// A CTA per row holds a bitmap of the whole output row in shared memory.
// Symbolic: set the bit of every product's column, count the bits.  Numeric:
// rebuild the bitmap, turn it into ranks (per 128-word group a prefix of set
// bits, per word a prefix inside its group), write the sorted columns
// straight from the bitmap, zero the row's values, then stream the products
// again and add each one at C.val[row start + rank(column)] with a global
// atomic.  The cost per row is two or three passes over its products plus two
// scans of the bitmap, whatever the row's width or product count; the scans
// take a group per warp and four words per lane (one 16-byte load), since
// most words of a wide row are empty.

constexpr int kRankThreads = 512;

template <typename V, bool NUMERIC>
__global__ void __launch_bounds__(kRankThreads) k_rank(DevCsr A, DevCsr B, DevCsr C, const int32_t *rows,
                                                       int32_t nrows, int64_t *cnt, int *st, const uint8_t *bin_of) {
    constexpr int NT = kRankThreads;
    using AtomV = typename std::conditional<sizeof(V) == 4, unsigned int, unsigned long long>::type;
    extern __shared__ __align__(16) unsigned char smem[];
    const int ngroups = (int)((B.cols + 4095) >> 12);       // 128-word (4096-column) groups
    const int nwords = ngroups * 128;
    uint32_t *bits = (uint32_t *)smem;
    uint16_t *wpre = (uint16_t *)(bits + nwords);             // NUMERIC only
    uint32_t *gpre = (uint32_t *)(wpre + nwords);             // NUMERIC only
    __shared__ ChunkStage<V> sg;
    __shared__ int s_warp[NT / 32];
    __shared__ int64_t s_cnt;
    const int tid = threadIdx.x;
    bool ovf = false;
    for (int32_t ri = blockIdx.x; ri < nrows; ri += gridDim.x) {
        const int32_t r = rows[ri];
        const int64_t a0 = A.rowptr[r], a1 = A.rowptr[r + 1];
        const bool checked = NUMERIC && (bin_of[r] & kRiskyBit) != 0;
        for (int i = tid; i < nwords / 4; i += NT) ((uint4 *)bits)[i] = make_uint4(0, 0, 0, 0);
        __syncthreads();
        auto set_bit = [&](int32_t c, V) { atomicOr(bits + (c >> 5), 1u << (c & 31)); };
        for (int64_t k0 = a0; k0 < a1; k0 += kChunk) {
            const int n = (int)(a1 - k0 < (int64_t)kChunk ? a1 - k0 : (int64_t)kChunk);
            stage_rows_split<NT, V, false>(sg, A, B, k0, n);
            if (sg.nlong) stream_long_fast<V, false, false>(sg, sg.nlong, B, ovf, set_bit);
            stream_chunk<NT, V, false>(sg, n, B, false, ovf, set_bit);
            __syncthreads();
        }
        if (!NUMERIC) {
            int mine = 0;
            for (int i = tid; i < nwords / 4; i += NT) {
                const uint4 q = ((const uint4 *)bits)[i];
                mine += __popc(q.x) + __popc(q.y) + __popc(q.z) + __popc(q.w);
            }
            int excl;
            const int total = block_excl_scan<NT>(mine, &excl, s_warp);
            if (tid == 0) cnt[r] = total;
            continue;
        }
        const int lane = tid & 31;
        // ranks: a warp per group, four words per lane: per word the set bits
        // before it inside its group (the lane's own words, then a shuffle
        // scan over the lanes; four uint16 in one 8-byte store), per group the
        // set bits before it (a block scan over the group totals)
        {
            for (int g = tid >> 5; g < ngroups; g += NT / 32) {
                const int w0 = g * 128 + lane * 4;
                const uint4 q = *(const uint4 *)(bits + w0);
                const int p0 = __popc(q.x), p1 = __popc(q.y), p2 = __popc(q.z);
                const int t = p0 + p1 + p2 + __popc(q.w);
                const int x = warp_incl_scan(t);
                const uint32_t e = (uint32_t)(x - t);
                *(uint2 *)(wpre + w0) = make_uint2(e | ((e + p0) << 16), (e + p0 + p1) | ((e + p0 + p1 + p2) << 16));
                if (lane == 31) gpre[g] = (uint32_t)x;
            }
            __syncthreads();
            const int per = (ngroups + NT - 1) / NT;
            const int g0 = min(tid * per, ngroups), g1 = min(g0 + per, ngroups);
            int mine = 0;
            for (int g = g0; g < g1; g++) mine += (int)gpre[g];
            int excl;
            const int total = block_excl_scan<NT>(mine, &excl, s_warp);
            for (int g = g0; g < g1; g++) {
                const uint32_t t = gpre[g];
                gpre[g] = (uint32_t)excl;
                excl += (int)t;
            }
            if (tid == 0) s_cnt = total;
            __syncthreads();
        }
        // (with cnt: C is the single-pass temporary, rlen the row's capacity,
        // and the row's length is reported)
        const int64_t base = C.rowptr[r];
        const int64_t rlen = C.rowptr[r + 1] - base;
        if (tid == 0) {
            if (cnt) cnt[r] = s_cnt;
            if (cnt ? s_cnt > rlen : s_cnt != rlen) raise_status(st, kInvariant);
        }
        // sorted columns straight from the bitmap (four words per lane, from
        // the first one's rank); zero the row's values
        for (int g = tid >> 5; g < ngroups; g += NT / 32) {
            const int w0 = g * 128 + lane * 4;
            const uint4 q = *(const uint4 *)(bits + w0);
            int64_t pos = (int64_t)gpre[g] + wpre[w0];
            const uint32_t ws[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
            for (int j = 0; j < 4; j++) {
                uint32_t word = ws[j];
                while (word) {
                    const int b = __ffs(word) - 1;
                    word &= word - 1;
                    if (pos < rlen) {
                        C.col[base + pos] = (w0 + j) * 32 + b;
                        ((V *)C.val)[base + pos] = 0;
                    }
                    pos++;
                }
            }
        }
        __syncthreads();
        // values: every product lands on its column's rank
        V *vals = (V *)C.val + base;
        auto rank_of = [&](int32_t c) -> int64_t {
            const int w = c >> 5;
            return (int64_t)gpre[w >> 7] + wpre[w] + __popc(bits[w] & ((1u << (c & 31)) - 1u));
        };
        auto add_plain = [&](int32_t c, V p) {
            const int64_t pos = rank_of(c);
            if (pos < rlen) atomicAdd((AtomV *)(vals + pos), (AtomV)p);
        };
        auto add_chk = [&](int32_t c, V p) {
            const int64_t pos = rank_of(c);
            if (pos < rlen) {
                const AtomV old = atomicAdd((AtomV *)(vals + pos), (AtomV)p);
                ovf |= old > (AtomV)~(AtomV)0 - (AtomV)p;
            }
        };
        // the overflow test is chosen once per row, not per product
        for (int64_t k0 = a0; k0 < a1; k0 += kChunk) {
            const int n = (int)(a1 - k0 < (int64_t)kChunk ? a1 - k0 : (int64_t)kChunk);
            stage_rows_split<NT, V, true>(sg, A, B, k0, n);
            if (checked) {
                if (sg.nlong) stream_long_fast<V, true, true>(sg, sg.nlong, B, ovf, add_chk);
                stream_chunk<NT, V, true>(sg, n, B, true, ovf, add_chk);
            } else {
                if (sg.nlong) stream_long_fast<V, true, false>(sg, sg.nlong, B, ovf, add_plain);
                stream_chunk<NT, V, true>(sg, n, B, false, ovf, add_plain);
            }
            __syncthreads();
        }

    }
    if (__syncthreads_or(ovf) && tid == 0) raise_status(st, kOverflow);
}

// ------------------------------------------------------------------------
// split rank rows (wide rows whose products exceed a fair share)
// ------------------------------------------------------------------------
//
// As for dense rows: a heavy rank row is cut into parts of its A entries.
// Symbolic: a CTA per part sets the bits of its products in a shared-memory
// bitmap and ORs the nonzero words into the row's global bitmap; one CTA per
// row counts the bits.  Numeric: one CTA per row turns the global bitmap into
// per-word ranks, writes the sorted columns and zeroes the values; then a CTA
// per part adds its products at their ranks with global atomics.

// Task -> slot (last slot whose first task is <= task).
__device__ __forceinline__ int split_slot_of(const int32_t *task_start, int ns, int task) {
    int lo = 0, hi = ns - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (task_start[mid] <= task) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <typename V>
__global__ void __launch_bounds__(kRankThreads) k_rank_split_sym(DevCsr A, DevCsr B, const int32_t *rows,
                                                                 const int32_t *row_of_slot, const int32_t *parts,
                                                                 const int32_t *task_start, const int32_t *nslots,
                                                                 int32_t max_slots, int32_t nwords, uint32_t *gbits) {
    constexpr int NT = kRankThreads;
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t *bits = (uint32_t *)smem;
    __shared__ ChunkStage<V> sg;
    const int tid = threadIdx.x;
    const int ns = min(*nslots, max_slots);
    const int ntasks = task_start[ns];
    bool ovf = false;
    for (int task = blockIdx.x; task < ntasks; task += gridDim.x) {
        const int slot = split_slot_of(task_start, ns, task);
        const int part = task - task_start[slot], np = parts[slot];
        const int32_t r = rows[row_of_slot[slot]];
        const int64_t a0 = A.rowptr[r], alen = A.rowptr[r + 1] - a0;
        const int64_t ka = a0 + alen * part / np, kb = a0 + alen * (part + 1) / np;
        for (int i = tid; i < nwords / 4; i += NT) ((uint4 *)bits)[i] = make_uint4(0, 0, 0, 0);
        __syncthreads();
        auto set_bit = [&](int32_t c, V) { atomicOr(bits + (c >> 5), 1u << (c & 31)); };
        for (int64_t k0 = ka; k0 < kb; k0 += kChunk) {
            const int n = (int)(kb - k0 < (int64_t)kChunk ? kb - k0 : (int64_t)kChunk);
            stage_rows_split<NT, V, false>(sg, A, B, k0, n);
            if (sg.nlong) stream_long_fast<V, false, false>(sg, sg.nlong, B, ovf, set_bit);
            stream_chunk<NT, V, false>(sg, n, B, false, ovf, set_bit);
            __syncthreads();
        }
        uint32_t *g = gbits + (int64_t)slot * nwords;
        for (int w = tid; w < nwords; w += NT) {
            const uint32_t b = bits[w];
            if (b) atomicOr(g + w, b);
        }
        __syncthreads();
    }
}

// One CTA per split row: its length from the global bitmap.
__global__ void __launch_bounds__(512) k_rank_split_count(const int32_t *rows, const int32_t *row_of_slot,
                                                          const int32_t *nslots, int32_t max_slots, int32_t nwords,
                                                          const uint32_t *gbits, int64_t *cnt) {
    __shared__ int s_warp[16];
    const int ns = min(*nslots, max_slots);
    for (int slot = blockIdx.x; slot < ns; slot += gridDim.x) {
        const uint32_t *g = gbits + (int64_t)slot * nwords;
        int mine = 0;
        for (int w = threadIdx.x; w < nwords; w += 512) mine += __popc(g[w]);
        int excl;
        const int total = block_excl_scan<512>(mine, &excl, s_warp);
        if (threadIdx.x == 0) cnt[rows[row_of_slot[slot]]] = total;
    }
}

// One CTA per split row: per-word ranks (set bits before the word) into
// gpre, the sorted columns into C, the row's values zeroed.
template <typename V>
__global__ void __launch_bounds__(kRankThreads) k_rank_split_prep(DevCsr C, const int32_t *rows,
                                                                  const int32_t *row_of_slot, const int32_t *nslots,
                                                                  int32_t max_slots, int32_t nwords,
                                                                  const uint32_t *gbits, uint32_t *gpre, int *st) {
    constexpr int NT = kRankThreads, NW = NT / 32;
    __shared__ int s_warp[NW];
    __shared__ uint32_t s_bpre[kRankCols / 1024];
    const int ns = min(*nslots, max_slots);
    const int tid = threadIdx.x, lane = tid & 31;
    const int nblocks = nwords >> 5;                          // nwords is a multiple of 32
    const int per = (nblocks + NT - 1) / NT;
    const int b0 = min(tid * per, nblocks), b1 = min(b0 + per, nblocks);
    for (int slot = blockIdx.x; slot < ns; slot += gridDim.x) {
        const int32_t r = rows[row_of_slot[slot]];
        const uint32_t *g = gbits + (int64_t)slot * nwords;
        uint32_t *pre = gpre + (int64_t)slot * nwords;
        // set bits per 32-word block (a warp per block, coalesced)
        for (int b = tid >> 5; b < nblocks; b += NW) {
            const int x = warp_incl_scan(__popc(g[b * 32 + lane]));
            if (lane == 31) s_bpre[b] = (uint32_t)x;
        }
        __syncthreads();
        int mine = 0;
        for (int b = b0; b < b1; b++) mine += (int)s_bpre[b];
        int excl;
        const int total = block_excl_scan<NT>(mine, &excl, s_warp);
        for (int b = b0; b < b1; b++) {
            const uint32_t t = s_bpre[b];
            s_bpre[b] = (uint32_t)excl;
            excl += (int)t;
        }
        __syncthreads();
        const int64_t base = C.rowptr[r];
        const int64_t rlen = C.rowptr[r + 1] - base;
        if (tid == 0 && total != rlen) raise_status(st, kInvariant);
        // per-word ranks and the sorted columns, a warp per block again
        for (int b = tid >> 5; b < nblocks; b += NW) {
            const int w = b * 32 + lane;
            uint32_t word = g[w];
            const int p = __popc(word);
            int64_t pos = (int64_t)s_bpre[b] + warp_incl_scan(p) - p;
            pre[w] = (uint32_t)pos;
            while (word) {
                const int bit = __ffs(word) - 1;
                word &= word - 1;
                if (pos < rlen) {
                    C.col[base + pos] = w * 32 + bit;
                    ((V *)C.val)[base + pos] = 0;
                }
                pos++;
            }
        }
        __syncthreads();
    }
}

// One CTA per task: the part's products added at their ranks.
template <typename V>
__global__ void __launch_bounds__(kRankThreads) k_rank_split_val(DevCsr A, DevCsr B, DevCsr C, const int32_t *rows,
                                                                 const int32_t *row_of_slot, const int32_t *parts,
                                                                 const int32_t *task_start, const int32_t *nslots,
                                                                 int32_t max_slots, int32_t nwords,
                                                                 const uint32_t *gbits, const uint32_t *gpre,
                                                                 const uint8_t *bin_of, int *st) {
    constexpr int NT = kRankThreads;
    using AtomV = typename std::conditional<sizeof(V) == 4, unsigned int, unsigned long long>::type;
    __shared__ ChunkStage<V> sg;
    const int ns = min(*nslots, max_slots);
    const int ntasks = task_start[ns];
    bool ovf = false;
    for (int task = blockIdx.x; task < ntasks; task += gridDim.x) {
        const int slot = split_slot_of(task_start, ns, task);
        const int part = task - task_start[slot], np = parts[slot];
        const int32_t r = rows[row_of_slot[slot]];
        const int64_t a0 = A.rowptr[r], alen = A.rowptr[r + 1] - a0;
        const int64_t ka = a0 + alen * part / np, kb = a0 + alen * (part + 1) / np;
        const bool checked = (bin_of[r] & kRiskyBit) != 0;
        const uint32_t *g = gbits + (int64_t)slot * nwords;
        const uint32_t *pre = gpre + (int64_t)slot * nwords;
        const int64_t base = C.rowptr[r];
        const int64_t rlen = C.rowptr[r + 1] - base;
        V *vals = (V *)C.val + base;
        auto rank_of = [&](int32_t c) -> int64_t {
            const int w = c >> 5;
            return (int64_t)pre[w] + __popc(g[w] & ((1u << (c & 31)) - 1u));
        };
        auto add_plain = [&](int32_t c, V p) {
            const int64_t pos = rank_of(c);
            if (pos < rlen) atomicAdd((AtomV *)(vals + pos), (AtomV)p);
        };
        auto add_chk = [&](int32_t c, V p) {
            const int64_t pos = rank_of(c);
            if (pos < rlen) {
                const AtomV old = atomicAdd((AtomV *)(vals + pos), (AtomV)p);
                ovf |= old > (AtomV)~(AtomV)0 - (AtomV)p;
            }
        };
        for (int64_t k0 = ka; k0 < kb; k0 += kChunk) {
            const int n = (int)(kb - k0 < (int64_t)kChunk ? kb - k0 : (int64_t)kChunk);
            stage_rows_split<NT, V, true>(sg, A, B, k0, n);
            if (checked) {
                if (sg.nlong) stream_long_fast<V, true, true>(sg, sg.nlong, B, ovf, add_chk);
                stream_chunk<NT, V, true>(sg, n, B, true, ovf, add_chk);
            } else {
                if (sg.nlong) stream_long_fast<V, true, false>(sg, sg.nlong, B, ovf, add_plain);
                stream_chunk<NT, V, true>(sg, n, B, false, ovf, add_plain);
            }
            __syncthreads();
        }
    }
    if (__syncthreads_or(ovf) && threadIdx.x == 0) raise_status(st, kOverflow);
}

// Slots of the short-row temporary: min(products, columns) for a row of
// the short-row bins, none for the others.
__global__ void k_short_cap(int64_t m, const uint8_t *bin_of, const int64_t *flops, int64_t cols, uint32_t mask,
                            int64_t *cap) {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
        const int b = bin_of[r] & ~kRiskyBit;
        cap[r] = (b != kEmptyBin && ((mask >> b) & 1u)) ? (flops[r] < cols ? flops[r] : cols) : 0;
    }
}

// The single-pass bins' rows from their slots in the temporary into C (a
// warp per row, four entries per lane in flight; the row's length is C's,
// from the scan of the reported lengths).
template <typename V>
__global__ void __launch_bounds__(256) k_copy_short(int64_t m, const uint8_t *bin_of, uint32_t mask,
                                                    const int64_t *trow, const int32_t *tcol, const V *tval,
                                                    DevCsr C) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < m; r += nw) {
        const int b = bin_of[r] & ~kRiskyBit;
        if (b == kEmptyBin || !((mask >> b) & 1u)) continue;
        const int64_t d0 = C.rowptr[r], len = C.rowptr[r + 1] - d0, s0 = trow[r];
        for (int64_t i0 = lane; i0 < len; i0 += 128) {
            int32_t c[4];
            V v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int64_t i = i0 + 32 * u;
                if (i < len) {
                    c[u] = tcol[s0 + i];
                    v[u] = tval[s0 + i];
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int64_t i = i0 + 32 * u;
                if (i < len) {
                    C.col[d0 + i] = c[u];
                    ((V *)C.val)[d0 + i] = v[u];
                }
            }
        }
    }
}

__global__ void k_iota(int32_t *v, int32_t n) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

// Compacts TEMP-mode slots into C: row rows[ri] has cnt = rowptr[r+1]-rowptr[r]
// entries at slot ri of the temporary.
template <typename V>
__global__ void __launch_bounds__(256) k_copy_rows(const int32_t *rows, int32_t nrows, DevCsr C, const int32_t *tcol,
                                                   const V *tval, int64_t tstride) {
    for (int32_t ri = blockIdx.x; ri < nrows; ri += gridDim.x) {
        const int32_t r = rows[ri];
        const int64_t b = C.rowptr[r], n = C.rowptr[r + 1] - b;
        const int32_t *sc = tcol + (int64_t)ri * tstride;
        const V *sv = tval + (int64_t)ri * tstride;
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
            C.col[b + i] = sc[i];
            ((V *)C.val)[b + i] = sv[i];
        }
    }
}

// ------------------------------------------------------------------------
// scan of row counts into the row pointer (int64), three phases
// ------------------------------------------------------------------------

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int64_t block_scan_i64(int64_t v, int64_t *s_warp, int64_t *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int64_t o = __shfl_up_sync(kFull, incl, d);
        if (lane >= d) incl += o;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    int64_t base = 0, tot = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
        const int64_t t = s_warp[w];
        if (w < warp) base += t;
        tot += t;
    }
    __syncthreads();
    *total = tot;
    return base + incl - v;
}

// rowptr[i+1] = inclusive partial sums within a tile; tile sums to tile_sum.
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int64_t *cnt, int64_t m, int64_t *rowptr,
                                                             int64_t *tile_sum, unsigned long long *row_max,
                                                             int64_t expect, int *st) {
    __shared__ int64_t s_warp[32];
    const int64_t t0 = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t s = 0, mx = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        v[i] = (t0 + i < m) ? cnt[t0 + i] : 0;
        s += v[i];
        mx = max(mx, v[i]);
    }
    if (row_max) {
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) mx = max(mx, (int64_t)__shfl_xor_sync(kFull, mx, d));
        if ((threadIdx.x & 31) == 0 && mx > 0) atomicMax(row_max, (unsigned long long)mx);
    }
    int64_t tot;
    int64_t run = block_scan_i64(s, s_warp, &tot);
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        run += v[i];
        if (t0 + i < m) rowptr[t0 + i + 1] = run;
        // one tile: the scan is complete here (a replay checks its size)
        if (gridDim.x == 1 && t0 + i == m - 1 && expect >= 0 && run != expect) raise_status(st, kInvariant);
    }
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = tot;
    if (gridDim.x == 1 && threadIdx.x == 0) rowptr[0] = 0;
}

// One block: exclusive scan of the tile sums in place.
__global__ void __launch_bounds__(1024) k_scan_sums(int64_t *tile_sum, int64_t ntiles, int64_t *rowptr) {
    __shared__ int64_t s_warp[32];
    __shared__ int64_t s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int64_t b = 0; b < ntiles; b += blockDim.x) {
        const int64_t i = b + threadIdx.x;
        const int64_t v = i < ntiles ? tile_sum[i] : 0;
        int64_t tot;
        const int64_t ex = block_scan_i64(v, s_warp, &tot);
        const int64_t carry = s_carry;
        if (i < ntiles) tile_sum[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) s_carry = carry + tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) rowptr[0] = 0;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_add(int64_t m, int64_t *rowptr, const int64_t *tile_sum,
                                                           int64_t expect, int *st) {
    const int64_t t0 = (int64_t)blockIdx.x * kScanTile;
    const int64_t add = tile_sum[blockIdx.x];
    if (add == 0 && (expect < 0 || t0 + kScanTile < m)) return;
    for (int i = threadIdx.x; i < kScanTile; i += kScanThreads) {
        const int64_t r = t0 + i;
        if (r < m) {
            const int64_t v = rowptr[r + 1] + add;
            if (add) rowptr[r + 1] = v;
            // the last row's end is the product's size (a replay checks it)
            if (r == m - 1 && expect >= 0 && v != expect) raise_status(st, kInvariant);
        }
    }
}

// ------------------------------------------------------------------------
// small helpers
// ------------------------------------------------------------------------

// Profiling only: B rows touched by A (distinct columns of A) and their entries.
__global__ void k_mark_touched(DevCsr A, uint8_t *mark) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < A.nnz; q += (int64_t)gridDim.x * blockDim.x)
        mark[A.col[q]] = 1;
}

__global__ void k_sum_touched(DevCsr B, const uint8_t *mark, unsigned long long *out) {
    unsigned long long rows = 0, ent = 0;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < B.rows; c += (int64_t)gridDim.x * blockDim.x)
        if (mark[c]) {
            rows++;
            ent += (unsigned long long)(B.rowptr[c + 1] - B.rowptr[c]);
        }
    rows = warp_sum(rows);
    ent = warp_sum(ent);
    if ((threadIdx.x & 31) == 0 && (rows || ent)) {
        atomicAdd(out, rows);
        atomicAdd(out + 1, ent);
    }
}

__global__ void k_widen(const uint32_t *src, uint64_t *dst, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

template <typename V>
__global__ void k_fill_ones(V *v, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] = 1;
}

int grid_for(rmcm_handle *h, int64_t work, int threads, int per_sm) {
    int64_t g = (work + threads - 1) / threads;
    const int64_t cap = (int64_t)h->sm_count * per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

// Opt a kernel in to `bytes` of dynamic shared memory (static shared memory
// counts against the same 48 KB default, so the attribute is set whenever the
// request is non-zero and above what this kernel was last given).
template <typename F>
int32_t set_smem(rmcm_handle *h, F *kernel, int64_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, int64_t> given;
    std::lock_guard<std::mutex> lock(mu);
    auto key = std::make_pair(h->device, (const void *)kernel);
    auto it = given.find(key);
    if (it != given.end() && it->second >= bytes) return RMCM_OK;
    RMCM_CUDA(h, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    given[key] = bytes;
    return RMCM_OK;
}

// Resident CTAs per SM of `kernel` at `threads` threads and `bytes` of dynamic
// shared memory (cached per device, kernel and size; the kernel's shared
// memory limit must already be set).
template <typename F>
int occupancy(rmcm_handle *h, F *kernel, int threads, int64_t bytes) {
    static std::mutex mu;
    static std::map<std::tuple<int, const void *, int64_t>, int> known;
    std::lock_guard<std::mutex> lock(mu);
    auto key = std::make_tuple(h->device, (const void *)kernel, bytes);
    auto it = known.find(key);
    if (it != known.end()) return it->second;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, (size_t)bytes) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    known[key] = n;
    return n;
}

// Row-padded temporary of the single-pass dense rows, and the buffers of the
// rows split over several CTAs.
struct DenseTemp {
    bool active = false;
    int32_t *col = nullptr;
    void *val = nullptr;
    int64_t stride = 0;
    int64_t bytes = 0, vbytes = 0;   // the two allocations (columns, counts)
    bool no_risky = false;            // no row can overflow: with positive inputs, no presence bytes
    // packed copy of B (k_pack_banked) for the plain path of single-window rows
    const uint32_t *pk = nullptr;
    int32_t cbits = 0;
    void *pk_mem = nullptr;
    int64_t pk_bytes = 0;
    DensePart dpart;                  // tensor-core part of the product (single-pass rows)
    // split rows
    bool split = false;
    const int64_t *flops = nullptr;   // per-row products (scratch)
    int64_t fpart = 0;                // products per part
    int32_t pmax = 0;                 // parts per row at most
    int32_t max_slots = 0;            // split rows at most
    int32_t *nslots = nullptr;        // device counter
    int32_t *front = nullptr;         // device counter: rows of the dense list not split
    int32_t n_front = 0;              // its value on the host
    int32_t *perm = nullptr;          // dense list, unsplit rows first
    int32_t *row_of_slot = nullptr, *parts = nullptr, *task_start = nullptr;
    unsigned long long *G = nullptr;
    uint32_t *Gbits = nullptr;
    void *split_mem = nullptr;
    int64_t split_bytes = 0;
};

// Buffers of the split rank rows (alive from the symbolic to the numeric pass).
struct RankSplit {
    bool active = false;
    int32_t *perm = nullptr;          // rank list, unsplit rows first
    int32_t *front = nullptr, *nslots = nullptr;
    int32_t n_front = 0;
    int32_t *row_of_slot = nullptr, *parts = nullptr, *task_start = nullptr;
    int32_t max_slots = 0, pmax = 0;
    int64_t fpart = 0;
    int32_t nwords = 0;
    uint32_t *gbits = nullptr, *gpre = nullptr;
    void *mem = nullptr;
    int64_t bytes = 0;
};

// Rows with fewer products than this are never split.
constexpr int64_t kSplitMinFlops = 1 << 20;
constexpr int64_t kSplitMinLight = 1 << 18;   // light products of rows beside a tensor-core part

// A rows with more entries than this are analysed by the whole grid.
constexpr int64_t kLongAnalyze = 16384;

// Extras of a dense-bin launch: the packed copy of B, and (single-pass rows
// only) the tensor-core part.
DenseExtra dense_extra(const DenseTemp *t, bool single_pass) {
    DenseExtra e;
    if (!t) return e;
    e.pk = t->pk;
    e.cbits = t->cbits;
    if (single_pass && t->dpart.S) {
        e.S = t->dpart.S;
        e.gld = t->dpart.ld;
        e.lcnt = t->dpart.lcnt;
    }
    return e;
}

template <typename V, bool NUMERIC>
int32_t launch_bins(rmcm_handle *h, const DevCsr &A, const DevCsr &B, const DevCsr &C, const int32_t *lists,
                    const int32_t *counts, int32_t dense_max_alen, int64_t *cnt, int32_t *cursor_base,
                    int64_t cursor_cap, const DenseTemp *temp, const uint8_t *bin_of, bool positive,
                    bool b_distinct, const RankSplit *rs, uint32_t bin_mask = ~0u) {
    cudaStream_t s = h->stream;
    int *st = h->d_status;
    int32_t off = 0;
    const int64_t ncols = B.cols;
    const int micro_g = h->tune.threads_per_row;
    for (int b = 0; b < kNumBins; b++) {
        const int32_t n = counts[b];
        const int32_t *list = lists + off;
        off += n;
        if (n == 0 || !((bin_mask >> b) & 1u)) continue;
        switch (b) {
            case kBinWarp: {
                const int64_t sm = (int64_t)kWarpWarps * (kWarpCols + (NUMERIC ? (int64_t)kWarpCols * sizeof(V) : 0));
                auto kern = k_warp<V, NUMERIC>;
                RMCM_TRY(set_smem(h, kern, sm));
                const int per_sm = std::max(1, occupancy(h, kern, kWarpWarps * 32, sm));
                const int grid = grid_for(h, (int64_t)n * 32, kWarpWarps * 32, per_sm);
                kern<<<grid, kWarpWarps * 32, sm, s>>>(A, B, C, list, n, cnt, st, bin_of);
                break;
            }
            case kBinTiny: {
                const int grid = grid_for(h, (int64_t)n * 32, 256, 8);
                k_tiny<V, NUMERIC><<<grid, 256, 0, s>>>(A, B, C, list, n, cnt, st);
                break;
            }
            case kBinMicro: {
                const int grid = grid_for(h, ((int64_t)n * micro_g + 31) / 32 * 32, 256, 8);
                switch (micro_g) {
                    case 1: k_micro<V, NUMERIC, 1><<<grid, 256, 0, s>>>(A, B, C, list, n, cnt, st); break;
                    case 2: k_micro<V, NUMERIC, 2><<<grid, 256, 0, s>>>(A, B, C, list, n, cnt, st); break;
                    case 4: k_micro<V, NUMERIC, 4><<<grid, 256, 0, s>>>(A, B, C, list, n, cnt, st); break;
                    case 8: k_micro<V, NUMERIC, 8><<<grid, 256, 0, s>>>(A, B, C, list, n, cnt, st); break;
                    default: k_micro<V, NUMERIC, 16><<<grid, 256, 0, s>>>(A, B, C, list, n, cnt, st); break;
                }
                break;
            }
            case kBinHash512: {
                constexpr int S = 512, NT = 128;
                const int64_t sm = S * 4 + (NUMERIC ? S * sizeof(V) : 0);
                auto kern = k_hash<V, NUMERIC, S, NT>;
                RMCM_TRY(set_smem(h, kern, sm));
                kern<<<grid_for(h, (int64_t)n * NT, NT, 16), NT, sm, s>>>(A, B, C, list, n, cnt, st, bin_of);
                break;
            }
            case kBinHash2k: {
                constexpr int S = 2048, NT = 256;
                const int64_t sm = S * 4 + (NUMERIC ? S * sizeof(V) : 0);
                auto kern = k_hash<V, NUMERIC, S, NT>;
                RMCM_TRY(set_smem(h, kern, sm));
                kern<<<grid_for(h, (int64_t)n * NT, NT, 8), NT, sm, s>>>(A, B, C, list, n, cnt, st, bin_of);
                break;
            }
            case kBinHash8k: {
                constexpr int S = 8192, NT = 512;
                const int64_t sm = S * 4 + (NUMERIC ? S * sizeof(V) : 0);
                auto kern = k_hash<V, NUMERIC, S, NT>;
                RMCM_TRY(set_smem(h, kern, sm));
                kern<<<grid_for(h, (int64_t)n * NT, NT, 2), NT, sm, s>>>(A, B, C, list, n, cnt, st, bin_of);
                break;
            }
            case kBinRank: {
                // k_rank: 128-word groups (bitmap, per-word and per-group prefixes)
                const int64_t nwords = (ncols + 4095) / 4096 * 128;
                const int64_t sm = NUMERIC ? nwords * 4 + nwords * 2 + (nwords / 128) * 4 : nwords * 4;
                auto kern = k_rank<V, NUMERIC>;
                RMCM_TRY(set_smem(h, kern, sm));
                const int per_sm = (int)std::max<int64_t>(1, std::min<int64_t>(4, (200 * 1024) / std::max<int64_t>(sm, 1)));
                const int grid = (int)std::min<int64_t>((int64_t)n, (int64_t)h->sm_count * per_sm);
                const bool split = rs && rs->active;
                if (split) {
                    // split rows on the second stream, beside the unsplit ones
                    RMCM_CUDA(h, cudaEventRecord(h->ev_fork, s));
                    RMCM_CUDA(h, cudaStreamWaitEvent(h->aux, h->ev_fork, 0));
                    const int sgrid = h->sm_count * 2;
                    // (the split kernels' bitmaps: 32-word blocks, rs->nwords per slot)
                    const int64_t snw = rs->nwords;
                    if (!NUMERIC) {
                        auto ks = k_rank_split_sym<V>;
                        RMCM_TRY(set_smem(h, ks, snw * 4));
                        k_rank_split_sym<V><<<sgrid, kRankThreads, snw * 4, h->aux>>>(
                            A, B, rs->perm, rs->row_of_slot, rs->parts, rs->task_start, rs->nslots, rs->max_slots,
                            (int32_t)snw, rs->gbits);
                        k_rank_split_count<<<rs->max_slots, 512, 0, h->aux>>>(
                            rs->perm, rs->row_of_slot, rs->nslots, rs->max_slots, (int32_t)snw, rs->gbits, cnt);
                    } else {
                        k_rank_split_prep<V><<<rs->max_slots, kRankThreads, 0, h->aux>>>(
                            C, rs->perm, rs->row_of_slot, rs->nslots, rs->max_slots, (int32_t)snw, rs->gbits,
                            rs->gpre, st);
                        k_rank_split_val<V><<<sgrid, kRankThreads, 0, h->aux>>>(
                            A, B, C, rs->perm, rs->row_of_slot, rs->parts, rs->task_start, rs->nslots,
                            rs->max_slots, (int32_t)snw, rs->gbits, rs->gpre, bin_of, st);
                    }
                    h->launches += 2;
                }
                const int32_t *rl = split ? rs->perm : list;
                const int32_t rn = split ? rs->n_front : n;
                if (rn > 0)
                    kern<<<std::max(1, std::min(grid, rn)), kRankThreads, sm, s>>>(A, B, C, rl, rn, cnt, st, bin_of);
                if (split) {
                    RMCM_CUDA(h, cudaEventRecord(h->ev_join, h->aux));
                    RMCM_CUDA(h, cudaStreamWaitEvent(s, h->ev_join, 0));
                }
                break;
            }
            case kBinDense: {
                if (temp && temp->active) {
                    if (!NUMERIC) {
                        // one pass: columns + counts into the padded slots, lengths to cnt
                        const int64_t W = (ncols + 31) / 32 * 32;
                        // every value >= 1 and no row able to overflow: the
                        // counters alone mark presence, so the window holds only
                        // them (a smaller CTA, more of them per SM)
                        const int64_t sm_full = ((W + 15) & ~15LL) + W * (int64_t)sizeof(V);
                        const int64_t sm_lite = W * (int64_t)sizeof(V);
                        bool lite = false;
                        if (positive && temp->no_risky) {
                            RMCM_TRY(set_smem(h, k_dense<V, true, true>, sm_full));
                            RMCM_TRY(set_smem(h, k_dense<V, true, true, false>, sm_lite));
                            // only where dropping the bytes fits more CTAs per SM
                            lite = occupancy(h, k_dense<V, true, true, false>, kDenseThreads, sm_lite) >
                                   occupancy(h, k_dense<V, true, true>, kDenseThreads, sm_full);
                        }
                        const int64_t sm = lite ? sm_lite : sm_full;
                        auto kern = lite ? k_dense<V, true, true, false> : k_dense<V, true, true>;
                        RMCM_TRY(set_smem(h, kern, sm));
                        const int per_sm = (int)std::max<int64_t>(1, std::min<int64_t>(4, (200 * 1024) / std::max<int64_t>(sm, 1)));
                        const int grid = (int)std::min<int64_t>((int64_t)n, (int64_t)h->sm_count * per_sm);
                        DevCsr T = C;
                        T.col = temp->col;
                        T.val = temp->val;
                        // with a tensor-core part, A's light entries only
                        DevCsr Al = A;
                        if (temp->dpart.S) {
                            Al.col = const_cast<int32_t *>(temp->dpart.lcol);
                            Al.val = const_cast<uint32_t *>(temp->dpart.lval);
                        }
                        if (temp->split) {
                            // the split rows run on the second stream, beside the dense bin
                            const bool slite = positive && temp->no_risky;
                            const int64_t ssm = slite ? sm_lite : sm_full;
                            auto ks = slite ? k_dense_split<V, false> : k_dense_split<V, true>;
                            RMCM_TRY(set_smem(h, ks, ssm));
                            RMCM_CUDA(h, cudaEventRecord(h->ev_fork, s));
                            RMCM_CUDA(h, cudaStreamWaitEvent(h->aux, h->ev_fork, 0));
                            const int sper = (int)std::max<int64_t>(1, std::min<int64_t>(4, (200 * 1024) / std::max<int64_t>(ssm, 1)));
                            ks<<<(int)((int64_t)h->sm_count * sper), kSplitThreads, ssm, h->aux>>>(
                                Al, B, temp->perm, temp->row_of_slot, temp->parts, temp->task_start, temp->nslots,
                                temp->max_slots, (int32_t)W, temp->G, temp->Gbits, bin_of, st, (int32_t)ncols,
                                b_distinct && ncols <= 4 * kSplitThreads, temp->pk, temp->cbits,
                                temp->dpart.S ? temp->dpart.lcnt : nullptr);
                            k_split_finish<V><<<temp->max_slots, kSplitThreads, 0, h->aux>>>(
                                T, temp->perm, temp->row_of_slot, temp->nslots, temp->max_slots, ncols, (int32_t)W,
                                temp->G, temp->Gbits, temp->stride, cnt, st, (const V *)temp->dpart.S,
                                temp->dpart.ld);
                            h->launches += 2;
                        }
                        // split rows sit at the back of the permuted list: the dense
                        // kernel takes its front
                        const int32_t *dl = temp->split ? temp->perm : list;
                        const int32_t dn = temp->split ? temp->n_front : n;
                        if (dn > 0)
                            kern<<<std::max(1, std::min(grid, dn)), kDenseThreads, sm, s>>>(
                                Al, B, T, dl, dn, cnt, nullptr, 0, (int32_t)W, st, temp->stride, bin_of, positive,
                                b_distinct, h->abort_on_certain_overflow, dense_extra(temp, true));
                        if (temp->split) {
                            RMCM_CUDA(h, cudaEventRecord(h->ev_join, h->aux));
                            RMCM_CUDA(h, cudaStreamWaitEvent(s, h->ev_join, 0));
                        }
                    } else {
                        const int grid = (int)std::min<int64_t>((int64_t)n, (int64_t)h->sm_count * 8);
                        k_copy_rows<V><<<grid, 256, 0, s>>>(temp->split ? temp->perm : list, n, C, temp->col,
                                                             (const V *)temp->val, temp->stride);
                    }
                    break;
                }
                const int64_t wmax = NUMERIC ? (sizeof(V) == 4 ? kDenseWinU32 : kDenseWinU64) : kDenseWinSym;
                const int64_t W = std::min<int64_t>(wmax, (ncols + 31) / 32 * 32);
                const int64_t pres_bytes = (W + 15) & ~15LL;
                const int64_t sm = pres_bytes + (NUMERIC ? W * (int64_t)sizeof(V) : 0);
                auto kern = k_dense<V, NUMERIC, false>;
                RMCM_TRY(set_smem(h, kern, sm));
                int per_sm = (int)std::max<int64_t>(1, std::min<int64_t>(4, (200 * 1024) / std::max<int64_t>(sm, 1)));
                int grid = (int)std::min<int64_t>((int64_t)n, (int64_t)h->sm_count * per_sm);
                const bool multi = ncols > W;
                int64_t stride = multi ? std::max<int32_t>(dense_max_alen, 1) : 0;
                if (multi && (int64_t)grid * stride > cursor_cap) {
                    grid = (int)std::max<int64_t>(1, cursor_cap / stride);
                }
                kern<<<grid, kDenseThreads, sm, s>>>(A, B, C, list, n, cnt, cursor_base, stride, (int32_t)W, st, 0, bin_of,
                                                     positive, b_distinct, h->abort_on_certain_overflow,
                                                     NUMERIC && !multi ? dense_extra(temp, false) : DenseExtra{});
                break;
            }
        }
        h->launches++;
        RMCM_CUDA(h, cudaGetLastError());
    }
    return RMCM_OK;
}

// Exclusive scan of the row lengths into rowptr (rowptr[0] = 0); one tile
// needs one launch.  expect >= 0 checks the total (replays).
int32_t scan_rowptr(rmcm_handle *h, const int64_t *cnt, int64_t m, int64_t *rowptr, int64_t *tile_sum,
                    unsigned long long *row_max, int64_t expect) {
    cudaStream_t s = h->stream;
    const int64_t ntiles = std::max<int64_t>(1, (m + kScanTile - 1) / kScanTile);
    if (m == 0) {
        RMCM_CUDA(h, cudaMemsetAsync(rowptr, 0, sizeof(int64_t), s));
        return RMCM_OK;
    }
    k_scan_tiles<<<(unsigned)ntiles, kScanThreads, 0, s>>>(cnt, m, rowptr, tile_sum, row_max, expect, h->d_status);
    h->launches++;
    if (ntiles > 1) {
        k_scan_sums<<<1, 1024, 0, s>>>(tile_sum, ntiles, rowptr);
        k_scan_add<<<(unsigned)ntiles, kScanThreads, 0, s>>>(m, rowptr, tile_sum, expect, h->d_status);
        h->launches += 2;
    }
    RMCM_CUDA(h, cudaGetLastError());
    return RMCM_OK;
}


template <typename V>
int32_t spgemm_t(rmcm_handle *h, const rmcm_mat *Am, const rmcm_mat *Bm, rmcm_mat **Cout, int64_t *flops_out,
                 ProductPlan *plan) {
    cudaStream_t s = h->stream;
    const bool replay = plan && plan->mode == 2;
    const bool record = plan && plan->mode == 1;
    // row sums of B bound the counts of every output row (computed once per matrix)
    if (!Bm->ones && !Bm->rowsum && Bm->d.rows > 0) {
        rmcm_mat *Bw = const_cast<rmcm_mat *>(Bm);
        RMCM_TRY(dev_alloc(h, (void **)&Bw->rowsum, 8 * (Bm->d.rows + 1) + 8 * Bm->d.rows));
        RMCM_CUDA(h, cudaMemsetAsync(Bw->rowsum + Bm->d.rows, 0, 8, s));
        k_rowsum<V><<<grid_for(h, Bm->d.rows * 32, 256, 8), 256, 0, s>>>(Bm->d, Bw->rowsum,
                                                                          (uint2 *)(Bw->rowsum + Bm->d.rows + 1));
        h->launches++;
        RMCM_CUDA(h, cudaGetLastError());
    }
    const DevCsr A = Am->d;
    DevCsr B = Bm->d;
    B.rowsum = Bm->ones ? nullptr : Bm->rowsum;
    B.info = B.rowsum ? (const uint2 *)(Bm->rowsum + Bm->d.rows + 1) : nullptr;
    const bool positive = Am->positive && Bm->positive;
    const int64_t m = A.rows;
    // scratch layout: flops[m] i64 | cnt[m] i64 | tile sums | bin_of[m] u8 | lists[m] i32 | small counters | cursors
    const int64_t ntiles = std::max<int64_t>(1, (m + kScanTile - 1) / kScanTile);
    auto al = [](int64_t x) { return (x + 255) & ~255LL; };
    const int64_t o_flops = 0;
    const int64_t o_cnt = o_flops + al(8 * m);
    const int64_t o_tiles = o_cnt + al(8 * m);
    const int64_t o_bin = o_tiles + al(8 * ntiles);
    const int64_t o_lists = o_bin + al(m);
    const int64_t o_small = o_lists + al(4 * m);
    const int64_t o_cur = o_small + 256;
    int64_t need = o_cur;
    if (record) plan->scratch_bytes = need;
    if (replay && need > h->scratch_bytes)
        return set_error(h, RMCM_EINTERNAL, "replay: scratch not reserved before capture");
    RMCM_TRY(scratch_reserve(h, need));
    char *sc = (char *)h->scratch;
    int64_t *flops = (int64_t *)(sc + o_flops);
    int64_t *cnt = (int64_t *)(sc + o_cnt);
    int64_t *tiles = (int64_t *)(sc + o_tiles);
    uint8_t *bin_of = (uint8_t *)(sc + o_bin);
    int32_t *lists = (int32_t *)(sc + o_lists);
    // small: [0..6] bin counts, [8..14] bin cursors, [16] longest dense A row,
    // [32..33] total flops (u64), [36..37] largest dense-row flops (u64),
    // [40] overflow certain, [42] dense split slots, [43] long A rows,
    // [44..45] longest C row (u64), [46] unsplit dense rows, [48..51]
    // profiling sums, [52] rank split slots, [53] unsplit rank rows,
    // [54..55] largest rank-row flops (u64), [56] rows that may overflow,
    // [58..59] largest value of B (u64, when B may be packed), [60..61]
    // largest total bound S of a row that may overflow (uint32), [18..19]
    // and [20..21] slots of the single-pass temporary for the short-row bins'
    // and the rank bin's rows (u64)
    int32_t *small = (int32_t *)(sc + o_small);
    RMCM_CUDA(h, cudaMemsetAsync(small, 0, 256, s));
    // B may be packed for the dense bin (uint32, positive, one window)
    const bool pack_cand = sizeof(V) == 4 && positive && B.cols >= 2 && B.cols <= kDenseWinU32 && B.nnz > 0;
    if (pack_cand && !Bm->ones && !replay)
        RMCM_CUDA(h, cudaMemcpyAsync(small + 58, Bm->rowsum + Bm->d.rows, 8, cudaMemcpyDeviceToDevice, s));

    ProdRecord *rec = nullptr;
    size_t rec_idx = 0;
    if (h->prof_level > 0 && !replay) {
        h->prof.emplace_back();
        rec_idx = h->prof.size() - 1;
        rec = &h->prof[rec_idx];
        for (auto &e : rec->ev) RMCM_CUDA(h, cudaEventCreate(&e));
        RMCM_CUDA(h, cudaEventRecord(rec->ev[0], s));
    }
    void *long_mem = nullptr;
    int64_t long_bytes = 0;
    BinParams bp;
    bp.dense_win = sizeof(V) == 4 ? kDenseWinU32 : kDenseWinU64;
    bp.hash_max = h->tune.hash_max_flops;
    bp.dense_ratio = h->tune.dense_ratio;
    {
        const int tpr = h->tune.threads_per_row;
        bp.micro_max = tpr < 32 ? tpr : 0;
        bp.tiny_max = tpr <= 32 ? 32 : 0;
        bp.inv_load_q8 = (int32_t)std::ceil(256.0 / h->tune.hash_load);
        bp.warp_max = h->tune.warp_max_flops;
    }
    if (m > 0) {
        AnalyzeOut ao{flops,
                      bin_of,
                      small,
                      small + 16,
                      (unsigned long long *)(small + 32),
                      small + 40,
                      (unsigned long long *)(small + 36),
                      (unsigned long long *)(small + 54),
                      small + 56,
                      (unsigned long long *)(small + 60),
                      (unsigned long long *)(small + 18),
                      (unsigned long long *)(small + 20)};
        // rows longer than kLongAnalyze entries: walked by the whole grid
        const bool long_rows = Am->max_row > kLongAnalyze;
        const int64_t max_long = A.nnz / kLongAnalyze + 1;
        if (long_rows) {
            long_bytes = 24 * max_long + 256;
            RMCM_TRY(dev_alloc(h, (void **)&long_mem, long_bytes));
            RMCM_CUDA(h, cudaMemsetAsync(long_mem, 0, long_bytes, s));
        }
        int32_t *nlong = small + 43;
        unsigned long long *acc_f = long_rows ? (unsigned long long *)long_mem : nullptr;
        unsigned long long *acc_s = long_rows ? acc_f + max_long : nullptr;
        int32_t *lsat = long_rows ? (int32_t *)(acc_s + max_long) : nullptr;
        int32_t *llist = long_rows ? lsat + max_long : nullptr;
        k_analyze<V><<<grid_for(h, m * 32, 256, 8), 256, 0, s>>>(A, B, bp, ao, long_rows ? kLongAnalyze : INT64_MAX,
                                                                  llist, nlong);
        h->launches++;
        if (long_rows) {
            k_analyze_long<V><<<h->sm_count * 4, 256, 0, s>>>(A, B, llist, nlong, acc_f, acc_s, lsat);
            k_analyze_long_finish<V><<<4, 256, 0, s>>>(A, B, bp, ao, llist, nlong, acc_f, acc_s, lsat);
            h->launches += 2;
        }
        k_scatter<<<grid_for(h, m, 256, 8), 256, 0, s>>>(m, bin_of, small, small + 8, lists, cnt);
        h->launches += 1;
        if (long_mem) {
            dev_free(h, long_mem, long_bytes);
            long_mem = nullptr;
        }
        RMCM_CUDA(h, cudaGetLastError());
    }
    if (rec) {
        // the symbolic time starts here: it includes the product's setup
        // (temporaries, packing, the tensor-core part, split preparation)
        RMCM_CUDA(h, cudaEventRecord(h->prof[rec_idx].ev[1], s));
        RMCM_CUDA(h, cudaEventRecord(h->prof[rec_idx].ev[2], s));
    }
    // bin counts, the longest dense A row and the flops to the host (a replay
    // takes them from the recorded plan)
    int32_t counts[kNumBins];
    int32_t dense_max_alen = 0;
    int64_t flops_total = 0;
    int64_t cap_short = 0, cap_rank = 0;
    bool certain = false;
    if (replay) {
        memcpy(counts, plan->counts, sizeof(counts));
        dense_max_alen = plan->dense_max_alen;
        flops_total = plan->flops;
    } else {
        RMCM_CUDA(h, cudaMemcpyAsync(h->h_pinned, small, 64 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        RMCM_CUDA(h, cudaStreamSynchronize(s));
        memcpy(counts, h->h_pinned, sizeof(counts));
        dense_max_alen = ((int32_t *)h->h_pinned)[16];
        memcpy(&flops_total, (int32_t *)h->h_pinned + 32, sizeof(int64_t));
        memcpy(&cap_short, (int32_t *)h->h_pinned + 18, sizeof(int64_t));
        memcpy(&cap_rank, (int32_t *)h->h_pinned + 20, sizeof(int64_t));
        certain = ((int32_t *)h->h_pinned)[40] != 0;
        if (sizeof(V) == 4 && h->abort_on_certain_overflow && !certain) {
            // a row whose total exceeds 16 x 2^32 averages more than 2^32/128
            // per column: with skewed counts an entry overflows all but
            // surely, so widen before computing (a wrong guess only costs
            // uint64 arithmetic)
            uint64_t mt = 0;
            memcpy(&mt, (int32_t *)h->h_pinned + 60, sizeof(uint64_t));
            if (mt / 16 > 0xffffffffull) certain = true;
        }
    }
    if (record) {
        memcpy(plan->counts, counts, sizeof(counts));
        plan->dense_max_alen = dense_max_alen;
        plan->flops = flops_total;
    }
    if (flops_out) *flops_out = flops_total;
    if (certain && h->abort_on_certain_overflow) {
        // some row's total count exceeds (its distinct columns) x (largest
        // value): an overflow is certain, so the caller widens first
        if (rec) {
            for (auto &e : h->prof[rec_idx].ev) cudaEventDestroy(e);
            h->prof.pop_back();
        }
        return set_error(h, RMCM_EOVERFLOW, "path counts certainly exceed the value type");
    }

    // Cursor buffer for multi-window dense rows.  It is a separate allocation:
    // growing the scratch area here would move the row lists built above.
    const int64_t wnum = sizeof(V) == 4 ? kDenseWinU32 : kDenseWinU64;
    int64_t cursor_cap = 0;
    int32_t *cursors = nullptr;
    if (counts[kBinDense] > 0 && B.cols > wnum) {
        const int64_t stride = std::max<int32_t>(dense_max_alen, 1);
        cursor_cap = stride * std::min<int64_t>((int64_t)h->sm_count * 4, 1024);
        RMCM_TRY(dev_alloc(h, (void **)&cursors, 4 * cursor_cap));
    }
    auto drop_cursors = [&]() {
        if (cursors) dev_free(h, cursors, 4 * cursor_cap);
        cursors = nullptr;
    };
    // Single-pass dense rows: when every dense row fits one numeric window,
    // compute them once into a row-padded temporary (bounded in size).
    DenseTemp dtemp;
    if (counts[kBinDense] > 0 && B.cols <= wnum && h->tune.dense_single_pass && (!replay || plan->dense_temp)) {
        const int64_t stride = (B.cols + 3) & ~3LL;
        const int64_t bytes = (int64_t)counts[kBinDense] * stride * (4 + (int64_t)sizeof(V));
        const int64_t room = h->budget - h->in_use;
        if (replay || (bytes <= h->tune.dense_temp_max_bytes && bytes < room / 2)) {
            // columns and counts in two allocations: a product whose rows all
            // come out full can take them over as its own arrays
            const int64_t cb = (int64_t)counts[kBinDense] * stride * 4, vb = bytes - cb;
            void *pc = nullptr, *pv = nullptr;
            if (dev_alloc(h, &pc, cb) == RMCM_OK && dev_alloc(h, &pv, vb) == RMCM_OK) {
                dtemp.active = true;
                dtemp.col = (int32_t *)pc;
                dtemp.val = pv;
                dtemp.stride = stride;
                dtemp.bytes = cb;
                dtemp.vbytes = vb;
            } else {
                if (pc) dev_free(h, pc, cb);
                h->last_error.clear();
            }
        }
    }
    if (replay && plan->dense_temp && !dtemp.active)
        return set_error(h, RMCM_ENOMEM, "replay: dense temporary could not be allocated");
    if (record) plan->dense_temp = dtemp.active;
    {
        int32_t risky_rows = 0;
        if (replay) risky_rows = plan->risky_rows;
        else risky_rows = ((int32_t *)h->h_pinned)[56];
        if (record) plan->risky_rows = risky_rows;
        dtemp.no_risky = risky_rows == 0;
    }
    {
        // Tensor-core part (dense_gemm.cu): every row with products in the
        // single-pass dense bin, uint32, positive, no row able to overflow, a
        // large product whose rows need no split over CTAs (skewed rows keep
        // the split kernels); not inside a batch recording (plain runs only).
        int64_t mdf = 0;
        if (!replay) memcpy(&mdf, (int32_t *)h->h_pinned + 36, sizeof(int64_t));
        const int64_t fpart0 = std::max<int64_t>(kSplitMinFlops, flops_total / ((int64_t)h->sm_count * 4));
        // (uint64 products, whose dense parts are whole-row GEMMs in the
        // retail and stress chains, take it even with skewed rows; uint32
        // products with skewed rows count each row's light products, and the
        // rows heavy in those are split over CTAs like skewed dense rows)
        // (the panel gathers store one value per (row, index): no repeated
        // column within a row of A or B)
        const bool skewed = mdf > fpart0;
        bool want = !plan && dtemp.active && positive && dtemp.no_risky && Am->distinct && Bm->distinct &&
                    flops_total >= (int64_t)h->tune.gemm_min_mflops * 1000000 && h->tune.gemm_inv_density > 0;
        for (int b = 0; b < kNumBins && want; b++)
            if (b != kBinDense && counts[b] > 0) want = false;
        if (want) {
            cudaEvent_t e0 = rec ? h->prof[rec_idx].ev[6] : nullptr, e1 = rec ? h->prof[rec_idx].ev[7] : nullptr;
            int32_t drc = RMCM_OK;
            if (sizeof(V) == 4) {
                uint64_t bmax = 1;
                if (!Bm->ones) memcpy(&bmax, (int32_t *)h->h_pinned + 58, sizeof(uint64_t));
                drc = dense_part_build(h, A, B, bmax, dtemp.dpart, e0, e1, skewed);
            } else {
                drc = dense_part_build64(h, A, B, dtemp.dpart, e0, e1);
            }
            if (drc != RMCM_OK) {
                dense_part_release(h, dtemp.dpart);
                if (dtemp.pk_mem) dev_free(h, dtemp.pk_mem, dtemp.pk_bytes);
                if (dtemp.active) {
                    dev_free(h, dtemp.col, dtemp.bytes);
                    dev_free(h, dtemp.val, dtemp.vbytes);
                }
                return drc;
            }
        }
    }
    {
        // Pack B when the dense bin reuses its entries many times and every
        // value fits beside the column bits.
        int32_t cbits = 0;
        if (replay) {
            cbits = plan->pack_cbits;
        } else if (pack_cand && counts[kBinDense] > 0 && flops_total >= kPackReuse * B.nnz && !dtemp.dpart.S) {
            // (with a tensor-core part the light rows left are short: no packing)
            uint64_t bmax = 1;
            if (!Bm->ones) memcpy(&bmax, (int32_t *)h->h_pinned + 58, sizeof(uint64_t));
            const int32_t cb = 32 - __builtin_clz((uint32_t)(B.cols - 1));
            if (cb < 32 && bmax < (1ull << (32 - cb))) cbits = cb;
        }
        if (cbits > 0) {
            void *p = nullptr;
            if (dev_alloc(h, &p, 4 * B.nnz) == RMCM_OK) {
                dtemp.pk = (const uint32_t *)p;
                dtemp.cbits = cbits;
                dtemp.pk_mem = p;
                dtemp.pk_bytes = 4 * B.nnz;
                k_pack_banked<<<grid_for(h, B.rows * 32, kPackWarps * 32, 6), kPackWarps * 32, 0, s>>>(
                    B, cbits, (uint32_t *)p, h->d_status);
                h->launches++;
                RMCM_CUDA(h, cudaGetLastError());
            } else if (replay) {
                return set_error(h, RMCM_ENOMEM, "replay: packed copy of B could not be allocated");
            } else {
                h->last_error.clear();
                cbits = 0;
            }
        }
        if (record) plan->pack_cbits = cbits;
    }
    // Dense rows with far more products than a fair share of the device are
    // split over several CTAs (k_dense_split).
    int64_t max_dense_f = 0;
    if (replay) max_dense_f = plan->max_dense_flops;
    else memcpy(&max_dense_f, (int32_t *)h->h_pinned + 36, sizeof(int64_t));
    if (record) plan->max_dense_flops = max_dense_f;
    if (dtemp.active && (!dtemp.dpart.S || dtemp.dpart.lflops)) {
        // (with a tensor-core part the rows' light products decide, in
        // smaller parts: the GEMM has taken the bulk of the work; without
        // their counts there is no split)
        const bool light = dtemp.dpart.S != nullptr;
        const int64_t ftot = light ? dtemp.dpart.ltotal : flops_total;
        const int64_t fmax = light ? dtemp.dpart.lmax : max_dense_f;
        const int64_t fpart =
            std::max<int64_t>(light ? kSplitMinLight : kSplitMinFlops, ftot / ((int64_t)h->sm_count * 4));
        if (fmax > fpart) {
            const int32_t nd = counts[kBinDense];
            const int32_t max_slots = (int32_t)std::min<int64_t>(std::min<int64_t>(1024, nd), ftot / fpart + 1);
            const int64_t Wt = (B.cols + 31) / 32 * 32;
            auto al = [](int64_t x) { return (x + 255) & ~255LL; };
            const int64_t o_perm = 0;
            const int64_t o_row = o_perm + al(4LL * nd);
            const int64_t o_parts = o_row + al(4LL * max_slots);
            const int64_t o_ts = o_parts + al(4LL * max_slots);
            const int64_t o_g = o_ts + al(4LL * (max_slots + 1));
            const int64_t o_gb = o_g + al(8LL * max_slots * Wt);
            const int64_t total = o_gb + al(4LL * max_slots * (Wt / 32));
            void *mem = nullptr;
            if (dev_alloc(h, &mem, total) == RMCM_OK) {
                char *b = (char *)mem;
                dtemp.split = true;
                dtemp.flops = light ? dtemp.dpart.lflops : flops;
                dtemp.fpart = fpart;
                dtemp.pmax = h->sm_count * 2;
                dtemp.max_slots = max_slots;
                dtemp.nslots = small + 42;
                dtemp.front = small + 46;
                dtemp.perm = (int32_t *)(b + o_perm);
                dtemp.row_of_slot = (int32_t *)(b + o_row);
                dtemp.parts = (int32_t *)(b + o_parts);
                dtemp.task_start = (int32_t *)(b + o_ts);
                dtemp.G = (unsigned long long *)(b + o_g);
                dtemp.Gbits = (uint32_t *)(b + o_gb);
                dtemp.split_mem = mem;
                dtemp.split_bytes = total;
                RMCM_CUDA(h, cudaMemsetAsync(b + o_g, 0, total - o_g, s));
            } else {
                h->last_error.clear();
            }
        }
    }
    if (replay && plan->split && !dtemp.split)
        return set_error(h, RMCM_ENOMEM, "replay: split-row buffers could not be allocated");
    if (record) plan->split = dtemp.split;
    if (dtemp.split) {
        // choose the split rows now: the dense kernel needs the count of the others
        int32_t dense_off = 0;
        for (int b = 0; b < kBinDense; b++) dense_off += counts[b];
        const int32_t nd = counts[kBinDense];
        k_split_select<<<grid_for(h, nd, 256, 8), 256, 0, s>>>(lists + dense_off, nd, dtemp.flops, dtemp.fpart, dtemp.pmax,
                                                               dtemp.perm, dtemp.front, dtemp.nslots,
                                                               dtemp.row_of_slot, dtemp.parts, dtemp.max_slots);
        k_split_tasks<<<1, 1024, 0, s>>>(dtemp.parts, dtemp.nslots, dtemp.max_slots, dtemp.task_start);
        h->launches += 2;
        RMCM_CUDA(h, cudaGetLastError());
        if (replay) {
            dtemp.n_front = plan->n_front;
        } else {
            RMCM_CUDA(h, cudaMemcpyAsync(h->h_pinned + 2, dtemp.front, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
            RMCM_CUDA(h, cudaStreamSynchronize(s));
            dtemp.n_front = ((int32_t *)(h->h_pinned + 2))[0];
        }
        if (record) plan->n_front = dtemp.n_front;
    }
    // Rank-bin rows likewise (k_rank_split_*)
    RankSplit rsplit;
    int64_t max_rank_f = 0;
    if (replay) max_rank_f = plan->max_rank_flops;
    else memcpy(&max_rank_f, (int32_t *)h->h_pinned + 54, sizeof(int64_t));
    if (record) plan->max_rank_flops = max_rank_f;
    if (counts[kBinRank] > 0) {
        const int64_t fpart = std::max<int64_t>(kSplitMinFlops, flops_total / ((int64_t)h->sm_count * 4));
        if (max_rank_f > fpart) {
            const int32_t nr = counts[kBinRank];
            const int32_t max_slots = (int32_t)std::min<int64_t>(std::min<int64_t>(1024, nr), flops_total / fpart + 1);
            const int64_t nwords = (B.cols + 1023) / 1024 * 32;
            auto al = [](int64_t x) { return (x + 255) & ~255LL; };
            const int64_t o_perm = 0;
            const int64_t o_row = o_perm + al(4LL * nr);
            const int64_t o_parts = o_row + al(4LL * max_slots);
            const int64_t o_ts = o_parts + al(4LL * max_slots);
            const int64_t o_bits = o_ts + al(4LL * (max_slots + 1));
            const int64_t o_pre = o_bits + al(4LL * max_slots * nwords);
            const int64_t total = o_pre + al(4LL * max_slots * nwords);
            void *mem = nullptr;
            if (dev_alloc(h, &mem, total) == RMCM_OK) {
                char *b = (char *)mem;
                rsplit.active = true;
                rsplit.perm = (int32_t *)(b + o_perm);
                rsplit.row_of_slot = (int32_t *)(b + o_row);
                rsplit.parts = (int32_t *)(b + o_parts);
                rsplit.task_start = (int32_t *)(b + o_ts);
                rsplit.gbits = (uint32_t *)(b + o_bits);
                rsplit.gpre = (uint32_t *)(b + o_pre);
                rsplit.nslots = small + 52;
                rsplit.front = small + 53;
                rsplit.max_slots = max_slots;
                rsplit.pmax = h->sm_count * 2;
                rsplit.fpart = fpart;
                rsplit.nwords = (int32_t)nwords;
                rsplit.mem = mem;
                rsplit.bytes = total;
                RMCM_CUDA(h, cudaMemsetAsync(b + o_bits, 0, 4LL * max_slots * nwords, s));
                int32_t roff = 0;
                for (int b2 = 0; b2 < kBinRank; b2++) roff += counts[b2];
                k_split_select<<<grid_for(h, nr, 256, 8), 256, 0, s>>>(lists + roff, nr, flops, fpart, rsplit.pmax,
                                                                       rsplit.perm, rsplit.front, rsplit.nslots,
                                                                       rsplit.row_of_slot, rsplit.parts, max_slots);
                k_split_tasks<<<1, 1024, 0, s>>>(rsplit.parts, rsplit.nslots, max_slots, rsplit.task_start);
                h->launches += 2;
                RMCM_CUDA(h, cudaGetLastError());
                if (replay) {
                    rsplit.n_front = plan->rank_n_front;
                } else {
                    RMCM_CUDA(h, cudaMemcpyAsync(h->h_pinned + 3, rsplit.front, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
                    RMCM_CUDA(h, cudaStreamSynchronize(s));
                    rsplit.n_front = ((int32_t *)(h->h_pinned + 3))[0];
                }
                if (record) plan->rank_n_front = rsplit.n_front;
            } else {
                h->last_error.clear();
            }
        }
    }
    if (replay && plan->rank_split && !rsplit.active)
        return set_error(h, RMCM_ENOMEM, "replay: split rank-row buffers could not be allocated");
    if (record) plan->rank_split = rsplit.active;
    auto drop_rank = [&]() {
        if (rsplit.active) dev_free(h, rsplit.mem, rsplit.bytes);
        rsplit.active = false;
    };
    auto drop_temp = [&]() {
        dense_part_release(h, dtemp.dpart);
        if (dtemp.pk_mem) dev_free(h, dtemp.pk_mem, dtemp.pk_bytes);
        dtemp.pk_mem = nullptr;
        dtemp.pk = nullptr;
        if (dtemp.active) {
            dev_free(h, dtemp.col, dtemp.bytes);
            dev_free(h, dtemp.val, dtemp.vbytes);
        }
        if (dtemp.split) dev_free(h, dtemp.split_mem, dtemp.split_bytes);
        dtemp.active = false;
        dtemp.split = false;
    };

    // Single pass for the short-row bins (tiny, micro, hash, warp) and, when
    // none of its rows is split over CTAs, the rank bin: each such row gets
    // min(products, columns) slots in a temporary, their numeric kernels
    // write there and report each row's length (the symbolic pass is skipped
    // for them), and after the scan the rows are copied into C.
    constexpr uint32_t kShortBins = (1u << kBinTiny) | (1u << kBinHash512) | (1u << kBinHash2k) |
                                    (1u << kBinHash8k) | (1u << kBinMicro) | (1u << kBinWarp);
    uint32_t short_mask = kShortBins | (rsplit.active ? 0u : (1u << kBinRank));
    if (replay && plan->short_temp) short_mask = plan->short_mask;
    struct {
        bool active = false;
        int64_t *rowptr = nullptr;
        int32_t *col = nullptr;
        void *val = nullptr;
        int64_t total = 0, rp_bytes = 0, c_bytes = 0, v_bytes = 0;
    } stemp;
    auto drop_short = [&]() {
        if (stemp.rowptr) dev_free(h, stemp.rowptr, stemp.rp_bytes);
        if (stemp.col) dev_free(h, stemp.col, stemp.c_bytes);
        if (stemp.val) dev_free(h, stemp.val, stemp.v_bytes);
        stemp.rowptr = nullptr;
        stemp.col = nullptr;
        stemp.val = nullptr;
        stemp.active = false;
    };
    {
        int64_t n_short = 0;
        for (int b = 0; b < kNumBins; b++)
            if ((short_mask >> b) & 1u) n_short += counts[b];
        bool want = replay ? plan->short_temp : (n_short > 0 && h->tune.short_single_pass);
        if (want) {
            // slots: a capacity per row (m of them, then scanned in place of
            // a copy) and the row pointers of the temporary
            stemp.rp_bytes = 16 * (m + 1);
            if (dev_alloc(h, (void **)&stemp.rowptr, stemp.rp_bytes) == RMCM_OK) {
                int64_t *capr = stemp.rowptr + (m + 1);
                k_short_cap<<<grid_for(h, m, 256, 8), 256, 0, s>>>(m, bin_of, flops, B.cols, short_mask, capr);
                h->launches++;
                int32_t src = cudaGetLastError() == cudaSuccess ? RMCM_OK : set_error(h, RMCM_ECUDA, "short capacity");
                // the total came with the analysis (no read-back here); the
                // scan checks it on the device
                stemp.total = replay ? plan->short_total
                                     : cap_short + (((short_mask >> kBinRank) & 1u) ? cap_rank : 0);
                if (src == RMCM_OK)
                    src = scan_rowptr(h, capr, m, stemp.rowptr, tiles, (unsigned long long *)(small + 44), stemp.total);
                const int64_t room = h->budget - h->in_use;
                stemp.c_bytes = 4 * std::max<int64_t>(stemp.total, 1);
                stemp.v_bytes = (int64_t)sizeof(V) * std::max<int64_t>(stemp.total, 1);
                if (src == RMCM_OK &&
                    (replay || stemp.c_bytes + stemp.v_bytes <= std::min<int64_t>(h->tune.dense_temp_max_bytes, room / 2)) &&
                    dev_alloc(h, (void **)&stemp.col, stemp.c_bytes) == RMCM_OK &&
                    dev_alloc(h, &stemp.val, stemp.v_bytes) == RMCM_OK) {
                    stemp.active = true;
                } else {
                    if (src != RMCM_OK) {
                        drop_short();
                        drop_cursors();
                        drop_temp();
                        drop_rank();
                        return src;
                    }
                    drop_short();
                    h->last_error.clear();
                }
            } else {
                h->last_error.clear();
            }
        }
        if (replay && plan->short_temp && !stemp.active)
            return set_error(h, RMCM_ENOMEM, "replay: short-row temporary could not be allocated");
        if (record) {
            plan->short_temp = stemp.active;
            plan->short_total = stemp.total;
            plan->short_mask = short_mask;
        }
    }
    const uint32_t other_bins = stemp.active ? ~short_mask : ~0u;

    // symbolic
    rmcm_mat *C = nullptr;
    int32_t rc = mat_alloc(h, m, B.cols, -1, Am->valtype, &C);
    if (rc != RMCM_OK) {
        drop_short();
        drop_cursors();
        drop_temp();
        drop_rank();
        return rc;
    }
    // every row single-pass dense (no split): slot i of the temporary is row i,
    // so a product whose rows all come out full can keep it as C
    const bool all_dense = dtemp.active && !dtemp.split && counts[kBinDense] == m;
    if (all_dense) {
        k_iota<<<grid_for(h, m, 256, 8), 256, 0, s>>>(lists, (int32_t)m);
        h->launches++;
        if (cudaGetLastError() != cudaSuccess) rc = set_error(h, RMCM_ECUDA, "row list launch");
    }
    if (rc == RMCM_OK && stemp.active) {
        // the short-row bins, once, into the temporary (lengths to cnt)
        DevCsr T = C->d;
        T.rowptr = stemp.rowptr;
        T.col = stemp.col;
        T.val = stemp.val;
        T.nnz = stemp.total;
        rc = launch_bins<V, true>(h, A, B, T, lists, counts, dense_max_alen, cnt, cursors, cursor_cap, &dtemp, bin_of,
                                  positive, Bm->distinct, &rsplit, short_mask);
    }
    if (rc == RMCM_OK)
        rc = launch_bins<V, false>(h, A, B, C->d, lists, counts, dense_max_alen, cnt, cursors, cursor_cap, &dtemp,
                                   bin_of, positive, Bm->distinct, &rsplit, other_bins);
    if (rc == RMCM_OK)
        rc = scan_rowptr(h, cnt, m, C->d.rowptr, tiles, (unsigned long long *)(small + 44), replay ? plan->nnz : -1);
    if (rec) cudaEventRecord(h->prof[rec_idx].ev[3], s);
    // nnz to the host, then the output arrays
    int64_t *hp = h->h_pinned;
    if (rc == RMCM_OK && !replay) {
        cudaError_t e = cudaMemcpyAsync(hp, C->d.rowptr + m, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hp + 1, small + 44, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_error(h, e, "spgemm nnz download");
    }
    const int64_t nnz = replay ? plan->nnz : hp[0];
    const int64_t c_max_row = replay ? plan->c_max_row : hp[1];
    if (record) {
        plan->nnz = nnz;
        plan->c_max_row = c_max_row;
    }
    if (rc == RMCM_OK && h->abort_on_certain_overflow && !replay) {
        // single-pass dense rows already computed their counts: stop early if
        // any of them overflowed, so the caller can recompute in uint64
        cudaError_t e = cudaMemcpyAsync(h->h_status, h->d_status, sizeof(int) * kNumStatus, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_error(h, e, "spgemm status download");
        else if (h->h_status[kOverflow]) {
            cudaMemsetAsync(h->d_status + kOverflow, 0, sizeof(int), s);
            drop_short();
            drop_cursors();
            drop_temp();
            drop_rank();
            mat_release(h, C);
            if (rec) {
                for (auto &e : h->prof[rec_idx].ev) cudaEventDestroy(e);
                h->prof.pop_back();
            }
            return set_error(h, RMCM_EOVERFLOW, "path counts exceed the value type");
        }
    }
    // every row full: the temporary's layout (row i at i * stride) is C's
    const bool adopt = rc == RMCM_OK && all_dense && nnz == m * dtemp.stride;
    if (adopt) {
        C->d.col = dtemp.col;
        C->d.val = dtemp.val;
        C->d.nnz = nnz;
        C->bytes += (4 + (int64_t)sizeof(V)) * nnz;
        dtemp.active = false;   // owned by C now
    } else if (rc == RMCM_OK) {
        rc = mat_alloc(h, m, B.cols, nnz, Am->valtype, &C);
    }
    if (rec) cudaEventRecord(h->prof[rec_idx].ev[4], s);
    if (rc == RMCM_OK && !adopt && stemp.active) {
        k_copy_short<V><<<grid_for(h, m * 32, 256, 16), 256, 0, s>>>(m, bin_of, short_mask, stemp.rowptr, stemp.col,
                                                                       (const V *)stemp.val, C->d);
        h->launches++;
        if (cudaGetLastError() != cudaSuccess) rc = set_error(h, RMCM_ECUDA, "short-row copy launch");
    }
    if (rc == RMCM_OK && !adopt)
        rc = launch_bins<V, true>(h, A, B, C->d, lists, counts, dense_max_alen, nullptr, cursors, cursor_cap, &dtemp,
                                  bin_of, positive, Bm->distinct, &rsplit, other_bins);
    drop_short();
    const int32_t gemm_limbs = dtemp.dpart.S ? dtemp.dpart.limbs * dtemp.dpart.alimbs : 0;
    const int64_t gemm_inner = dtemp.dpart.S ? dtemp.dpart.heavy : 0;
    drop_cursors();
    drop_temp();
    drop_rank();
    if (rc != RMCM_OK) {
        mat_release(h, C);
        return rc;
    }
    if (rec) {
        ProdRecord &R = h->prof[rec_idx];
        RMCM_CUDA(h, cudaEventRecord(R.ev[5], s));
        rmcm_product_stats &st = R.st;
        st.rows = m;
        st.inner = A.cols;
        st.cols = B.cols;
        st.nnz_a = A.nnz;
        st.nnz_b = B.nnz;
        st.nnz_c = nnz;
        st.flops = flops_total;
        st.valtype = Am->valtype;
        for (int b = 0; b < kNumBins; b++) st.bin_rows[b] = counts[b];
        st.gemm_limbs = gemm_limbs;
        st.gemm_inner = gemm_inner;
        if (h->prof_level >= 2 && A.cols > 0) {
            // after the numeric pass: the row lists are no longer needed, reuse them
            uint8_t *mark = (uint8_t *)lists;
            unsigned long long *acc = (unsigned long long *)(small + 48);
            if (A.cols + 64 <= 4 * m) {
                RMCM_CUDA(h, cudaMemsetAsync(mark, 0, A.cols, s));
                RMCM_CUDA(h, cudaMemsetAsync(acc, 0, 16, s));
                k_mark_touched<<<grid_for(h, std::max<int64_t>(A.nnz, 1), 256, 8), 256, 0, s>>>(A, mark);
                k_sum_touched<<<grid_for(h, std::max<int64_t>(B.rows, 1), 256, 8), 256, 0, s>>>(B, mark, acc);
                RMCM_CUDA(h, cudaMemcpyAsync(hp, acc, 16, cudaMemcpyDeviceToHost, s));
                RMCM_CUDA(h, cudaStreamSynchronize(s));
                st.touched_rows = hp[0];
                st.touched_nnz = hp[1];
            } else {
                std::vector<uint8_t> hm(A.cols, 0);
                std::vector<int32_t> hc(A.nnz);
                std::vector<int64_t> hr(B.rows + 1);
                RMCM_CUDA(h, cudaMemcpyAsync(hc.data(), A.col, 4 * A.nnz, cudaMemcpyDeviceToHost, s));
                RMCM_CUDA(h, cudaMemcpyAsync(hr.data(), B.rowptr, 8 * (B.rows + 1), cudaMemcpyDeviceToHost, s));
                RMCM_CUDA(h, cudaStreamSynchronize(s));
                for (int32_t c : hc) hm[c] = 1;
                for (int64_t c = 0; c < B.rows; c++)
                    if (hm[c]) {
                        st.touched_rows++;
                        st.touched_nnz += hr[c + 1] - hr[c];
                    }
            }
            const int64_t iv = sizeof(V);
            st.bytes_a = (m + 1) * 8 + A.nnz * (4 + iv);
            st.bytes_b_touched = st.touched_rows * 16 + st.touched_nnz * (4 + iv);
            st.bytes_c = (m + 1) * 8 + nnz * (4 + iv);
        }
    }
    C->positive = positive;
    C->distinct = true;
    C->max_row = c_max_row;
    *Cout = C;
    return RMCM_OK;
}

}  // namespace

int32_t spgemm(rmcm_handle *h, const rmcm_mat *A, const rmcm_mat *B, rmcm_mat **C, int64_t *flops_out,
               ProductPlan *plan) {
    if (!A || !B || !C) return set_error(h, RMCM_EINVAL, "spgemm: null matrix");
    if (A->d.cols != B->d.rows)
        return set_error(h, RMCM_EINVAL, "spgemm: shape mismatch (A.cols != B.rows)");
    if (A->valtype != B->valtype) return set_error(h, RMCM_EINVAL, "spgemm: value types differ");
    if (A->valtype == RMCM_VAL_U64) return spgemm_t<uint64_t>(h, A, B, C, flops_out, plan);
    return spgemm_t<uint32_t>(h, A, B, C, flops_out, plan);
}

int32_t convert_values(rmcm_handle *h, const rmcm_mat *src, int32_t valtype, rmcm_mat **out) {
    if (src->valtype != RMCM_VAL_U32 || valtype != RMCM_VAL_U64)
        return set_error(h, RMCM_EINVAL, "convert: only uint32 -> uint64 widening is supported");
    rmcm_mat *m = nullptr;
    RMCM_TRY(mat_alloc(h, src->d.rows, src->d.cols, src->d.nnz, valtype, &m));
    cudaStream_t s = h->stream;
    cudaError_t e = cudaMemcpyAsync(m->d.rowptr, src->d.rowptr, 8 * (src->d.rows + 1), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && src->d.nnz)
        e = cudaMemcpyAsync(m->d.col, src->d.col, 4 * src->d.nnz, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && src->d.nnz) {
        k_widen<<<grid_for(h, src->d.nnz, 256, 8), 256, 0, s>>>((const uint32_t *)src->d.val, (uint64_t *)m->d.val,
                                                                 src->d.nnz);
        h->launches++;
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        mat_release(h, m);
        return cuda_error(h, e, "convert");
    }
    m->ones = src->ones;
    m->positive = src->positive;
    m->distinct = src->distinct;
    m->max_row = src->max_row;
    *out = m;
    return RMCM_OK;
}

// Checks of an uploaded CSR in one pass, a warp per row: row pointers
// non-decreasing and within [0, nnz], columns in [0, cols), each row's
// columns ascending and distinct, and (with val) whether a value is 0; the
// longest row and the rows longer than kEstLongRow (in any order, at most
// cap of them).  f[0] bad, [1] unsorted, [2] duplicate, [3] zero value,
// [4] longest row, [5] long rows.
template <typename V>
__global__ void __launch_bounds__(256) k_check_csr(DevCsr M, int64_t nnz, const V *val, unsigned long long *f,
                                                   int32_t *long_rows, int64_t cap) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    bool bad = false, unsorted = false, dup = false, zero = false;
    unsigned long long longest = 0;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < M.rows; r += nwarps) {
        const int64_t a = M.rowptr[r], b = M.rowptr[r + 1];
        if (a < 0 || b < a || b > nnz) {
            bad = true;
            continue;
        }
        for (int64_t q = a + lane; q < b; q += 32) {
            const int32_t c = M.col[q];
            if (c < 0 || c >= M.cols) bad = true;
            if (q > a) {
                const int32_t p = M.col[q - 1];
                unsorted |= c < p;
                dup |= c == p;
            }
            if (val) zero |= val[q] == 0;
        }
        const unsigned long long len = (unsigned long long)(b - a);
        longest = len > longest ? len : longest;
        if (lane == 0 && len > (unsigned long long)kEstLongRow) {
            const unsigned long long slot = atomicAdd(f + 5, 1ull);
            if ((int64_t)slot < cap) long_rows[slot] = (int32_t)r;
        }
    }
    bad = __any_sync(kFull, bad);
    unsorted = __any_sync(kFull, unsorted);
    dup = __any_sync(kFull, dup);
    zero = __any_sync(kFull, zero);
    if (lane == 0) {
        if (bad) atomicOr(f, 1ull);
        if (unsorted) atomicOr(f + 1, 1ull);
        if (dup) atomicOr(f + 2, 1ull);
        if (zero) atomicOr(f + 3, 1ull);
        if (longest) atomicMax(f + 4, longest);
    }
}

int32_t csr_check(rmcm_handle *h, const DevCsr &M, const void *val, int32_t valtype, unsigned long long *f,
                  int32_t *long_rows, int64_t cap) {
    RMCM_CUDA(h, cudaMemsetAsync(f, 0, 6 * sizeof(unsigned long long), h->stream));
    if (M.rows > 0) {
        const int grid = grid_for(h, M.rows * 32, 256, 8);
        if (valtype == RMCM_VAL_U64)
            k_check_csr<uint64_t><<<grid, 256, 0, h->stream>>>(M, M.nnz, (const uint64_t *)val, f, long_rows, cap);
        else
            k_check_csr<uint32_t><<<grid, 256, 0, h->stream>>>(M, M.nnz, (const uint32_t *)val, f, long_rows, cap);
        h->launches++;
        RMCM_CUDA(h, cudaGetLastError());
    }
    return RMCM_OK;
}

int32_t fill_ones(rmcm_handle *h, void *val, int64_t nnz, int32_t valtype) {
    if (nnz <= 0) return RMCM_OK;
    const int grid = grid_for(h, nnz, 256, 8);
    if (valtype == RMCM_VAL_U64) k_fill_ones<uint64_t><<<grid, 256, 0, h->stream>>>((uint64_t *)val, nnz);
    else k_fill_ones<uint32_t><<<grid, 256, 0, h->stream>>>((uint32_t *)val, nnz);
    h->launches++;
    RMCM_CUDA(h, cudaGetLastError());
    return RMCM_OK;
}

}  // namespace rmcm
