// RES row-wise sparsity estimator (sm_103a, FP64).
//
// Replaces the estimator loop of DynamicOptimizer::rows_sparse_optimal_matrix_chain_order
// (efficient/resmcm.cpp:506-517), getSparsities (:442-452) and
// compute_sparsities (:468-485):
//   r_ii[u] = min(1, |M_i[u]| / dim(vts[i+1]))
//   r_ij[u] = 1 - prod_{v in M_i[u]} (1 - r_{i+1,j}[v])          (j > i)
//   c_ij    = sum_u r_ij[u] * dim(vts[j+1])
// for i = len-1 .. 0.  dim(vts[j+1]) is the column count of M_j.
//
// One launch per level i computes every j > i at once, so each M_i is read
// once: a level stores q = 1 - r (r rounded first, then 1 - r rounded, the
// value the reference's next level forms) row-major as q[v * len + j], so
// the next level multiplies the gathered q directly and a row's gathers for
// all j are one contiguous run of doubles.
// Mapping: a warp per row; the warp is split into G groups of JP lanes
// (JP = next power of two >= number of j), lane (g, j) multiplies the factors
// of entries g, g+G, ... for target j, and the G partial products are
// combined with shuffles in a fixed order.  Sums of c_ij are per-warp, then
// per-block (fixed warp order), then a one-block pass over the block partials
// (fixed order): the estimate is bit-for-bit reproducible run to run.
// Every multiply and add is an explicit round-to-nearest intrinsic, so no
// fused multiply-add changes the rounding against the reference's
// `tmp_rho *= (1 - r)` and `nnz += s * dim`.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <mutex>
#include <vector>

#include "internal.h"

namespace rmcm {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kEstThreads = 256;
constexpr int kMaxLen = 16;

struct LevelArgs {
    int32_t len;            // chain length (matrices)
    int32_t i;              // level
    int32_t nj;             // number of j > i (len - 1 - i)
    int32_t jp;             // lanes per group (power of two >= nj, >= 1)
    int32_t tile;           // rows a warp takes per step (1 .. 32)
    double dim_leaf;        // dim(vts[i+1]) = cols of M_i
    double dims[kMaxLen];   // dims[j] = cols of M_j
};

// prod over entries k = k0, k0 + G, ... < k1 of q_next[col_k][j] (= 1 - r).
// A lane with at least four entries keeps four independent partial products
// (entries taken in turn) so four gathers and multiply chains are in flight,
// combined in a fixed order ((p0 p1)(p2 p3)); a shorter run multiplies
// serially (no combining multiplies).  Reproducible run to run.
__device__ __forceinline__ double factor_product(const DevCsr &M, const double *q_next, int32_t len, int j,
                                                 int64_t k0, int64_t k1, int G) {
    int64_t k = k0;
    if (k + 3 * (int64_t)G < k1) {
        double p[4] = {1.0, 1.0, 1.0, 1.0};
        for (; k + 3 * (int64_t)G < k1; k += 4 * (int64_t)G) {
            int32_t v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = M.col[k + u * G];
            double q[4];
#pragma unroll
            for (int u = 0; u < 4; u++) q[u] = q_next[(int64_t)v[u] * len + j];
#pragma unroll
            for (int u = 0; u < 4; u++) p[u] = __dmul_rn(p[u], q[u]);
        }
        // the last 0..3 entries, into p[0], p[1], p[2] in turn
#pragma unroll
        for (int u = 0; u < 3; u++) {
            if (k < k1) {
                p[u] = __dmul_rn(p[u], q_next[(int64_t)M.col[k] * len + j]);
                k += G;
            }
        }
        return __dmul_rn(__dmul_rn(p[0], p[1]), __dmul_rn(p[2], p[3]));
    }
    double p = 1.0;
    for (; k < k1; k += G) p = __dmul_rn(p, q_next[(int64_t)M.col[k] * len + j]);
    return p;
}

// Rows per warp step: 32 when every warp of a full grid (blocks_cap CTAs)
// still gets several steps, fewer for short matrices so that warps stay busy.
inline int32_t level_tile(int64_t rows, int64_t blocks_cap) {
    const int64_t warps = blocks_cap * (kEstThreads / 32);
    int32_t t = 32;
    while (t > 1 && rows < warps * t * 4) t >>= 1;
    return t;
}

// One level of one chain, as CTA `bid` of `nblk` (the same work split and
// summation order whether the CTA belongs to a one-chain launch or to a
// launch over many chains).
__device__ __forceinline__ void res_level_body(const DevCsr &M, const double *q_next, double *q_cur,
                                               const LevelArgs &la, double *partial, bool skip_long, int64_t bid,
                                               int64_t nblk) {
    __shared__ double s_tp[kEstThreads / 32][32 * kMaxLen];   // tile products: [t * jp + jo]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int G = 32 / la.jp;
    const int g = lane / la.jp;
    const int jo = lane % la.jp;                 // offset of j above i+1
    const bool active_j = jo < la.nj;
    const int j = la.i + 1 + jo;
    const double dimj = active_j ? la.dims[j] : 0.0;
    double term_sum = 0.0;                       // this lane's rows of target j
    const int T = la.tile;                       // rows per warp step (1 .. 32)
    double *tp = s_tp[warp];
    const int64_t nwarps = (nblk * blockDim.x) >> 5;
    for (int64_t t0 = ((bid * blockDim.x + threadIdx.x) >> 5) * T; t0 < M.rows; t0 += nwarps * T) {
        // r_ii of the tile's rows, a lane each (one division for T rows)
        int64_t my_a0 = 0, my_len = 0;
        if (lane < T && t0 + lane < M.rows) {
            const int64_t ul = t0 + lane;
            my_a0 = M.rowptr[ul];
            my_len = M.rowptr[ul + 1] - my_a0;
            double r = __ddiv_rn((double)my_len, la.dim_leaf);
            r = r > 1.0 ? 1.0 : r;
            q_cur[ul * la.len + la.i] = __dsub_rn(1.0, r);
        }
        if (la.nj == 0) continue;
        const int nrow = M.rows - t0 < (int64_t)T ? (int)(M.rows - t0) : T;
        uint32_t skipped = 0;
        for (int t = 0; t < nrow; t++) {
            const int64_t a0 = __shfl_sync(kFull, my_a0, t), rl = __shfl_sync(kFull, my_len, t);
            if (skip_long && rl > kEstLongRow) {   // a CTA of k_res_long takes it
                skipped |= 1u << t;
                continue;
            }
            double prod = 1.0;
            if (active_j) prod = factor_product(M, q_next, la.len, j, a0 + g, a0 + rl, G);
            // combine the group products (fixed butterfly order); groups past
            // the row's entries hold exactly 1.0, so those steps are skipped
            const int ng = rl < (int64_t)G ? (int)rl : G;
            for (int d = la.jp; d < 32 && d < la.jp * ng; d <<= 1) {
                const double o = __shfl_xor_sync(kFull, prod, d);
                prod = __dmul_rn(prod, o);
            }
            if (g == 0 && active_j) tp[t * la.jp + jo] = prod;
        }
        __syncwarp();
        // per (row, target): r = 1 - prod, its term r * dim_j, and q = 1 - r
        // for the next level; lane (g, jo) takes rows g, g + G, ...
        if (active_j) {
            for (int t = g; t < nrow; t += G) {
                if ((skipped >> t) & 1u) continue;
                const double r = __dsub_rn(1.0, tp[t * la.jp + jo]);
                q_cur[(t0 + t) * la.len + j] = __dsub_rn(1.0, r);
                term_sum = __dadd_rn(term_sum, __dmul_rn(r, dimj));
            }
        }
        __syncwarp();
    }
    // this warp's sums per target, over the groups in a fixed order
    for (int d = la.jp; d < 32; d <<= 1) term_sum = __dadd_rn(term_sum, __shfl_xor_sync(kFull, term_sum, d));
    // block partials: partial[block * len + j]
    __shared__ double s_part[kEstThreads / 32][kMaxLen];
    if (g == 0 && active_j) s_part[warp][jo] = term_sum;
    __syncthreads();
    if (threadIdx.x < la.nj) {
        double acc = 0.0;
        for (int w = 0; w < kEstThreads / 32; w++) acc = __dadd_rn(acc, s_part[w][threadIdx.x]);
        partial[bid * kMaxLen + threadIdx.x] = acc;
    }
}

__global__ void __launch_bounds__(kEstThreads) k_res_level(DevCsr M, const double *q_next, double *q_cur,
                                                           LevelArgs la, double *partial, bool skip_long) {
    res_level_body(M, q_next, q_cur, la, partial, skip_long, blockIdx.x, gridDim.x);
}

// A CTA per long row (rows listed ascending): warp w multiplies the factors
// of the w-th of 32 equal slices of the row, grouped as in k_res_level, and
// the 32 warp products are combined in warp order.  The row's terms
// s * dim_j go to partial[block], after the partials of k_res_level, so the
// reduction still adds them in a fixed order.
constexpr int kEstLongThreads = 1024;

__device__ __forceinline__ void res_long_body(const DevCsr &M, const double *q_next, double *q_cur,
                                              const LevelArgs &la, const int32_t *long_rows, double *partial,
                                              int64_t bid) {
    __shared__ double s_prod[kEstLongThreads / 32][kMaxLen];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int G = 32 / la.jp;
    const int g = lane / la.jp;
    const int jo = lane % la.jp;
    const bool active_j = jo < la.nj && g < G;
    const int j = la.i + 1 + jo;
    const int64_t u = long_rows[bid];
    const int64_t a0 = M.rowptr[u], len = M.rowptr[u + 1] - a0;
    const int64_t k0 = a0 + len * warp / (kEstLongThreads / 32), k1 = a0 + len * (warp + 1) / (kEstLongThreads / 32);
    double prod = 1.0;
    if (active_j) prod = factor_product(M, q_next, la.len, j, k0 + g, k1, G);
    for (int d = la.jp; d < 32; d <<= 1) {
        const double o = __shfl_xor_sync(kFull, prod, d);
        prod = __dmul_rn(prod, o);
    }
    if (g == 0 && active_j) s_prod[warp][jo] = prod;
    __syncthreads();
    if ((int)threadIdx.x < la.nj) {
        double p = 1.0;
        for (int w = 0; w < kEstLongThreads / 32; w++) p = __dmul_rn(p, s_prod[w][threadIdx.x]);
        const int jj = la.i + 1 + threadIdx.x;
        const double sv = __dsub_rn(1.0, p);
        q_cur[u * la.len + jj] = __dsub_rn(1.0, sv);   // q = 1 - r for the next level
        partial[bid * kMaxLen + threadIdx.x] = __dmul_rn(sv, la.dims[jj]);
    }
}

__global__ void __launch_bounds__(kEstLongThreads) k_res_long(DevCsr M, const double *q_next, double *q_cur,
                                                              LevelArgs la, const int32_t *long_rows,
                                                              double *partial) {
    res_long_body(M, q_next, q_cur, la, long_rows, partial, blockIdx.x);
}

// One block: c[i*len + j] = sum over blocks (fixed pairwise order).
__device__ __forceinline__ void res_reduce_body(const double *partial, int32_t nblocks, const LevelArgs &la, double *c) {
    __shared__ double s[256];
    for (int jo = 0; jo < la.nj; jo++) {
        double acc = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) acc = __dadd_rn(acc, partial[(int64_t)b * kMaxLen + jo]);
        s[threadIdx.x] = acc;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) s[threadIdx.x] = __dadd_rn(s[threadIdx.x], s[threadIdx.x + w]);
            __syncthreads();
        }
        if (threadIdx.x == 0) c[la.i * la.len + la.i + 1 + jo] = s[0];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_res_reduce(const double *partial, int32_t nblocks, LevelArgs la, double *c) {
    res_reduce_body(partial, nblocks, la, c);
}

// Many chains at once: job j is one level of one chain, exactly the launch
// the one-chain estimator makes for it (its CTAs are blocks first .. first +
// blocks - 1 of this grid), so every chain's estimates are bit-identical to
// rmcm_estimate's.
struct LevelJob {
    DevCsr M;
    const double *q_next;
    double *q_cur;
    double *partial;
    double *c;                  // the chain's len x len estimates
    const int32_t *long_rows;   // rows with a CTA of their own (nlong of them)
    LevelArgs la;
    int64_t first, blocks;      // CTAs of the level launch
    int64_t lfirst;             // CTAs of the long-row launch: lfirst .. lfirst + nlong - 1
    int32_t nlong;
};

__device__ __forceinline__ int find_job(const LevelJob *jobs, int njobs, int64_t b, bool longs) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((longs ? jobs[mid].lfirst : jobs[mid].first) <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(kEstThreads) k_res_level_multi(const LevelJob *jobs, int32_t njobs) {
    const LevelJob &jb = jobs[find_job(jobs, njobs, blockIdx.x, false)];
    res_level_body(jb.M, jb.q_next, jb.q_cur, jb.la, jb.partial, jb.nlong > 0, (int64_t)blockIdx.x - jb.first,
                   jb.blocks);
}

__global__ void __launch_bounds__(kEstLongThreads) k_res_long_multi(const LevelJob *jobs, int32_t njobs) {
    const LevelJob &jb = jobs[find_job(jobs, njobs, blockIdx.x, true)];
    res_long_body(jb.M, jb.q_next, jb.q_cur, jb.la, jb.long_rows, jb.partial + jb.blocks * kMaxLen,
                  (int64_t)blockIdx.x - jb.lfirst);
}

__global__ void __launch_bounds__(256) k_res_reduce_multi(const LevelJob *jobs) {
    const LevelJob &jb = jobs[blockIdx.x];
    if (jb.la.nj > 0) res_reduce_body(jb.partial, (int32_t)(jb.blocks + jb.nlong), jb.la, jb.c);
}

}  // namespace

int32_t estimate(rmcm_handle *h, rmcm_mat *const *chain, int32_t len, double *c_dev) {
    if (len < 1 || len > kMaxLen) return set_error(h, RMCM_EINVAL, "estimate: chain length must be 1..16");
    cudaStream_t s = h->stream;
    int64_t max_rows = 1;
    for (int i = 0; i < len; i++) {
        if (!chain[i]) return set_error(h, RMCM_EINVAL, "estimate: null matrix");
        if (i + 1 < len && chain[i]->d.cols != chain[i + 1]->d.rows)
            return set_error(h, RMCM_EINVAL, "estimate: consecutive matrices do not chain");
        max_rows = std::max(max_rows, chain[i]->d.rows);
    }
    // grid is fixed by the row count only, so the reduction order is stable
    const int64_t blocks_cap = (int64_t)h->sm_count * 8;
    int64_t long_cap = 0;
    for (int i = 0; i < len; i++) long_cap = std::max<int64_t>(long_cap, chain[i]->n_est_long);
    auto al = [](int64_t x) { return (x + 255) & ~255LL; };
    const int64_t rbytes = al(8 * max_rows * len);
    const int64_t pbytes = al(8 * (blocks_cap + long_cap) * kMaxLen);
    double *r_a = nullptr, *r_b = nullptr, *part = nullptr;
    RMCM_TRY(dev_alloc(h, (void **)&r_a, 2 * rbytes + pbytes));
    r_b = (double *)((char *)r_a + rbytes);
    part = (double *)((char *)r_a + 2 * rbytes);
    cudaError_t e = cudaMemsetAsync(c_dev, 0, sizeof(double) * len * len, s);
    double *r_cur = r_a, *r_next = r_b;
    for (int i = len - 1; i >= 0 && e == cudaSuccess; i--) {
        const DevCsr &M = chain[i]->d;
        LevelArgs la{};
        la.len = len;
        la.i = i;
        la.nj = len - 1 - i;
        int jp = 1;
        while (jp < la.nj) jp <<= 1;
        la.jp = jp;
        la.dim_leaf = (double)M.cols;
        for (int j = 0; j < len; j++) la.dims[j] = (double)chain[j]->d.cols;
        la.tile = level_tile(M.rows, blocks_cap);
        int64_t blocks = (M.rows + (int64_t)la.tile * (kEstThreads / 32) - 1) / ((int64_t)la.tile * (kEstThreads / 32));
        blocks = std::max<int64_t>(1, std::min(blocks, blocks_cap));
        // rows of more than kEstLongRow entries (known for uploaded matrices)
        // get a whole CTA each
        const int32_t nlong = la.nj > 0 && chain[i]->n_est_long > 0 ? chain[i]->n_est_long : 0;
        k_res_level<<<(unsigned)blocks, kEstThreads, 0, s>>>(M, r_next, r_cur, la, part, nlong > 0);
        h->launches++;
        if (nlong > 0) {
            k_res_long<<<(unsigned)nlong, kEstLongThreads, 0, s>>>(M, r_next, r_cur, la, chain[i]->est_long,
                                                                   part + blocks * kMaxLen);
            h->launches++;
        }
        if (la.nj > 0) {
            k_res_reduce<<<1, 256, 0, s>>>(part, (int32_t)(blocks + nlong), la, c_dev);
            h->launches++;
        }
        e = cudaGetLastError();
        std::swap(r_cur, r_next);
    }
    dev_free(h, r_a, 2 * rbytes + pbytes);
    if (e != cudaSuccess) return cuda_error(h, e, "estimator launch");
    return RMCM_OK;
}


// Estimates of many chains, a launch per level step over all of them: step s
// runs level len_c - 1 - s of every chain c longer than s.  Job tables go to
// the device through the arena (persistent pinned host memory and device
// memory, so that a stream capture records copies that stay valid).
int32_t estimate_multi(rmcm_handle *h, const EstChain *chains, int32_t n, TableArena &arena) {
    cudaStream_t s = h->stream;
    const int64_t blocks_cap = (int64_t)h->sm_count * 8;
    auto al = [](int64_t x) { return (x + 255) & ~255LL; };
    int32_t max_len = 0;
    std::vector<int64_t> off(n + 1, 0);
    for (int32_t c = 0; c < n; c++) {
        const int32_t len = chains[c].len;
        if (len < 1 || len > kMaxLen) return set_error(h, RMCM_EINVAL, "estimate: chain length must be 1..16");
        max_len = std::max(max_len, len);
        int64_t max_rows = 1, long_cap = 0;
        for (int i = 0; i < len; i++) {
            max_rows = std::max(max_rows, chains[c].mats[i]->d.rows);
            long_cap = std::max<int64_t>(long_cap, chains[c].mats[i]->n_est_long);
        }
        off[c + 1] = off[c] + 2 * al(8 * max_rows * len) + al(8 * (blocks_cap + long_cap) * kMaxLen);
    }
    char *buf = nullptr;
    RMCM_TRY(dev_alloc(h, (void **)&buf, std::max<int64_t>(off[n], 256)));
    cudaError_t e = cudaSuccess;
    for (int32_t c = 0; c < n && e == cudaSuccess; c++)
        e = cudaMemsetAsync(chains[c].c_dev, 0, sizeof(double) * chains[c].len * chains[c].len, s);
    std::vector<LevelJob> jobs;
    for (int32_t st = 0; st < max_len && e == cudaSuccess; st++) {
        jobs.clear();
        int64_t nb = 0, nl = 0;
        for (int32_t c = 0; c < n; c++) {
            const int32_t len = chains[c].len;
            if (st >= len) continue;
            const int i = len - 1 - st;
            int64_t max_rows = 1;
            for (int q = 0; q < len; q++) max_rows = std::max(max_rows, chains[c].mats[q]->d.rows);
            const int64_t rbytes = al(8 * max_rows * len);
            // the one-chain estimator swaps its two level buffers every level
            double *ra = (double *)(buf + off[c]), *rb = (double *)(buf + off[c] + rbytes);
            double *r_cur = (st % 2 == 0) ? ra : rb, *r_next = (st % 2 == 0) ? rb : ra;
            const rmcm_mat *Mi = chains[c].mats[i];
            LevelJob jb{};
            jb.M = Mi->d;
            jb.q_next = r_next;
            jb.q_cur = r_cur;
            jb.partial = (double *)(buf + off[c] + 2 * rbytes);
            jb.c = chains[c].c_dev;
            jb.la.len = len;
            jb.la.i = i;
            jb.la.nj = len - 1 - i;
            int jp = 1;
            while (jp < jb.la.nj) jp <<= 1;
            jb.la.jp = jp;
            jb.la.dim_leaf = (double)Mi->d.cols;
            for (int q = 0; q < len; q++) jb.la.dims[q] = (double)chains[c].mats[q]->d.cols;
            jb.la.tile = level_tile(Mi->d.rows, blocks_cap);
            int64_t blocks = (Mi->d.rows + (int64_t)jb.la.tile * (kEstThreads / 32) - 1) /
                             ((int64_t)jb.la.tile * (kEstThreads / 32));
            jb.blocks = std::max<int64_t>(1, std::min(blocks, blocks_cap));
            jb.nlong = jb.la.nj > 0 && Mi->n_est_long > 0 ? Mi->n_est_long : 0;
            jb.long_rows = Mi->est_long;
            jb.first = nb;
            jb.lfirst = nl;
            nb += jb.blocks;
            nl += jb.nlong;
            jobs.push_back(jb);
        }
        void *hp = nullptr, *dp = nullptr;
        const int64_t tbytes = (int64_t)sizeof(LevelJob) * (int64_t)jobs.size();
        if (!arena.push(tbytes, &hp, &dp)) {
            dev_free(h, buf, std::max<int64_t>(off[n], 256));
            return set_error(h, RMCM_EINTERNAL, "estimate: job table arena full");
        }
        memcpy(hp, jobs.data(), tbytes);
        e = cudaMemcpyAsync(dp, hp, tbytes, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) break;
        k_res_level_multi<<<(unsigned)nb, kEstThreads, 0, s>>>((const LevelJob *)dp, (int32_t)jobs.size());
        h->launches++;
        if (nl > 0) {
            k_res_long_multi<<<(unsigned)nl, kEstLongThreads, 0, s>>>((const LevelJob *)dp, (int32_t)jobs.size());
            h->launches++;
        }
        k_res_reduce_multi<<<(unsigned)jobs.size(), 256, 0, s>>>((const LevelJob *)dp);
        h->launches++;
        e = cudaGetLastError();
    }
    dev_free(h, buf, std::max<int64_t>(off[n], 256));
    if (e != cudaSuccess) return cuda_error(h, e, "multi-chain estimator launch");
    return RMCM_OK;
}

// ---------------------------------------------------------------------------
// RES estimator for callers that cannot allocate device memory
// ---------------------------------------------------------------------------
//
// Some callers of this library may not call cudaMalloc (or any allocating
// routine) at the point where they need an estimate: a host framework that
// owns every byte of device memory through its own pool and forbids plugins
// from allocating behind its back, or a latency-critical serving loop that
// allows no allocation after start-up (an allocation can synchronise the
// device or fail under memory pressure at the worst moment).
// rmcm_estimate_noalloc serves them.  The caller passes
// its chain as plain device CSR arrays it already owns and a host array for
// the estimates; every temporary the estimator needs (two levels of row
// sparsities, per-block partial sums and the estimate matrix) lives in the
// file-scope array below, a fixed 32 MiB that every GPU which loads this
// library holds until the process exits.  The array's address is looked up
// once per device, on the first call made with that device current.

namespace {

constexpr int64_t kNoAllocScratchBytes = 32LL << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct NoAllocDevice {
    bool ready = false;
    unsigned char *scratch = nullptr;   // device address of g_noalloc_scratch
    int sm_count = 0;
};
std::mutex g_noalloc_mu;
NoAllocDevice g_noalloc_dev[128];

}  // namespace
}  // namespace rmcm

extern "C" RMCM_API int32_t rmcm_estimate_noalloc(int32_t len, const int64_t *rows, const int64_t *cols,
                                                  const int64_t *const *rowptr, const int32_t *const *col,
                                                  double *c_out, void *stream) {
    using namespace rmcm;
    if (len < 1 || len > kMaxLen || !rows || !cols || !rowptr || !col || !c_out) return RMCM_EINVAL;
    int64_t max_rows = 1;
    for (int i = 0; i < len; i++) {
        if (rows[i] < 0 || cols[i] < 0 || cols[i] > INT32_MAX || (rows[i] > 0 && !rowptr[i])) return RMCM_EINVAL;
        // two FP64 levels of len values per row must fit the array: refuse
        // before any size product can wrap around
        if (rows[i] > kNoAllocScratchBytes / (16 * (int64_t)len)) return RMCM_EINVAL;
        if (i + 1 < len && cols[i] != rows[i + 1]) return RMCM_EINVAL;
        max_rows = std::max(max_rows, rows[i]);
    }
    // set-up, once per device, with that device current
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) return RMCM_ECUDA;
    NoAllocDevice nd;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        NoAllocDevice &d = g_noalloc_dev[dev];
        if (!d.ready) {
            void *ptr = nullptr;
            if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) {
                cudaGetLastError();
                return RMCM_ECUDA;
            }
            int sm = 0;
            if (cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sm <= 0) {
                cudaGetLastError();
                return RMCM_ECUDA;
            }
            d.scratch = (unsigned char *)ptr;
            d.sm_count = sm;
            d.ready = true;
        }
        nd = d;
    }
    // scratch layout: estimates | level r | level r' | block partials
    const int64_t blocks_cap = (int64_t)nd.sm_count * 8;
    auto al = [](int64_t x) { return (x + 255) & ~255LL; };
    const int64_t cbytes = al(8 * kMaxLen * kMaxLen);
    const int64_t rbytes = al(8 * max_rows * len);
    const int64_t pbytes = al(8 * blocks_cap * kMaxLen);
    if (cbytes + 2 * rbytes + pbytes > kNoAllocScratchBytes) return RMCM_EINVAL;   // chain too large
    cudaStream_t s = (cudaStream_t)stream;
    double *c_dev = (double *)nd.scratch;
    double *r_cur = (double *)(nd.scratch + cbytes);
    double *r_next = (double *)(nd.scratch + cbytes + rbytes);
    double *part = (double *)(nd.scratch + cbytes + 2 * rbytes);
    cudaError_t e = cudaMemsetAsync(c_dev, 0, sizeof(double) * len * len, s);
    for (int i = len - 1; i >= 0 && e == cudaSuccess; i--) {
        DevCsr M;
        M.rows = rows[i];
        M.cols = cols[i];
        M.rowptr = const_cast<int64_t *>(rowptr[i]);
        M.col = const_cast<int32_t *>(col[i]);
        LevelArgs la{};
        la.len = len;
        la.i = i;
        la.nj = len - 1 - i;
        int jp = 1;
        while (jp < la.nj) jp <<= 1;
        la.jp = jp;
        la.dim_leaf = (double)M.cols;
        for (int j = 0; j < len; j++) la.dims[j] = (double)cols[j];
        la.tile = level_tile(M.rows, blocks_cap);
        int64_t blocks = (M.rows + (int64_t)la.tile * (kEstThreads / 32) - 1) / ((int64_t)la.tile * (kEstThreads / 32));
        blocks = std::max<int64_t>(1, std::min(blocks, blocks_cap));
        k_res_level<<<(unsigned)blocks, kEstThreads, 0, s>>>(M, r_next, r_cur, la, part, false);
        if (la.nj > 0) k_res_reduce<<<1, 256, 0, s>>>(part, (int32_t)blocks, la, c_dev);
        e = cudaGetLastError();
        std::swap(r_cur, r_next);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(c_out, c_dev, sizeof(double) * len * len, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return RMCM_ECUDA;
    }
    return RMCM_OK;
}
