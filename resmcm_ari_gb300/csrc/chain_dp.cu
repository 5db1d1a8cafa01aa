// Chain-order dynamic program as a single warp (sm_103a).
//
// Replaces the DP of DynamicOptimizer::rows_sparse_optimal_matrix_chain_order
// (efficient/resmcm.cpp:519-536) and get_optimal_chain_order (:563-573):
//   m[i][j] = min_k  m[i][k] + m[k+1][j] + (c[i][k] + c[k+1][j] + c[i][j])
// with c[i][i] = 0 and m[i][i] = 0, the smallest k winning ties (the
// reference's strict '<' while k ascends).  Both sums are evaluated in the
// reference's left-to-right order with explicit round-to-nearest adds, so the
// same c gives the same split table bit for bit.
// Lane i owns the interval [i, i+l] of each length l; the lengths advance in
// lock step (__syncwarp between them).  Lane 0 then walks the split table in
// post-order with an explicit stack and emits the (k, l) pair list, -1
// standing for "the top of the temporary stack".
// One warp per chain: `nchains` chains are ordered by one launch.
// The file also holds the result digest used to compare chain results
// computed by different routes without copying them to the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>

#include "internal.h"

namespace rmcm {
namespace {

constexpr int kMaxLen = 16;

__global__ void __launch_bounds__(32) k_chain_dp(const double *c_all, const int32_t *lens, int32_t nchains,
                                                 int32_t *split_all, double *cost_all, int32_t *pairs_all,
                                                 int32_t one_len) {
    const int chain = blockIdx.x;
    if (chain >= nchains) return;
    const int lane = threadIdx.x;
    const int len = lens ? lens[chain] : one_len;
    const double *c = c_all + (int64_t)chain * kMaxLen * kMaxLen;
    __shared__ double sc[kMaxLen * kMaxLen];
    __shared__ double sm[kMaxLen * kMaxLen];
    __shared__ int32_t ss[kMaxLen * kMaxLen];
    for (int q = lane; q < kMaxLen * kMaxLen; q += 32) {
        const int i = q / kMaxLen, j = q % kMaxLen;
        sc[q] = (i < len && j < len && i != j) ? c[i * len + j] : 0.0;
        sm[q] = 0.0;
        ss[q] = 0;
    }
    __syncwarp();
    for (int l = 1; l < len; l++) {
        const int i = lane;
        if (i < len - l) {
            const int j = i + l;
            double best = DBL_MAX;
            int bk = 0;
            for (int k = i; k < j; k++) {
                const double tmp = __dadd_rn(__dadd_rn(sc[i * kMaxLen + k], sc[(k + 1) * kMaxLen + j]), sc[i * kMaxLen + j]);
                const double cost = __dadd_rn(__dadd_rn(sm[i * kMaxLen + k], sm[(k + 1) * kMaxLen + j]), tmp);
                if (cost < best) {
                    best = cost;
                    bk = k;
                }
            }
            sm[i * kMaxLen + j] = best;
            ss[i * kMaxLen + j] = bk;
        }
        __syncwarp();
    }
    int32_t *split = split_all + (int64_t)chain * kMaxLen * kMaxLen;
    double *cost = cost_all + (int64_t)chain * kMaxLen * kMaxLen;
    for (int q = lane; q < len * len; q += 32) {
        const int i = q / len, j = q % len;
        split[q] = ss[i * kMaxLen + j];
        cost[q] = sm[i * kMaxLen + j];
    }
    if (lane == 0 && len > 1) {
        // iterative post-order over the split tree
        int32_t *pairs = pairs_all + (int64_t)chain * 2 * kMaxLen;
        int st_i[2 * kMaxLen], st_j[2 * kMaxLen], st_state[2 * kMaxLen], st_left[2 * kMaxLen];
        int sp = 0, np = 0, ret = 0;
        st_i[0] = 0; st_j[0] = len - 1; st_state[0] = 0; sp = 1;
        while (sp > 0) {
            const int t = sp - 1;
            const int i = st_i[t], j = st_j[t];
            if (i == j) { ret = i; sp--; continue; }
            const int k = ss[i * kMaxLen + j];
            if (st_state[t] == 0) {
                st_state[t] = 1;
                st_i[sp] = i; st_j[sp] = k; st_state[sp] = 0; sp++;
            } else if (st_state[t] == 1) {
                st_left[t] = ret;
                st_state[t] = 2;
                st_i[sp] = k + 1; st_j[sp] = j; st_state[sp] = 0; sp++;
            } else {
                pairs[2 * np] = st_left[t];
                pairs[2 * np + 1] = ret;
                np++;
                ret = -1;
                sp--;
            }
        }
    }
}

}  // namespace

namespace {

// splitmix64 output function (Steele, Lea and Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014)
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}

// out[0] = nnz (rowptr[rows]); out[1] += sum over entries (r, c, v) of
// mix64(mix64(r * 2^32 + c) + v), mod 2^64, with r counted from row0 (a block
// of rows of a larger matrix adds its share of that matrix's digest).  The sum
// does not depend on the entry order, so equal matrices give equal digests
// whatever the launch shape.
template <typename V>
__global__ void __launch_bounds__(256) k_digest(DevCsr C, unsigned long long *out, int64_t row0) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    uint64_t acc = 0;
    const V *val = (const V *)C.val;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < C.rows; r += warps) {
        const int64_t e1 = C.rowptr[r + 1];
        for (int64_t e = C.rowptr[r] + lane; e < e1; e += 32) {
            const uint64_t key = ((uint64_t)(r + row0) << 32) | (uint32_t)C.col[e];
            const uint64_t v = val ? (uint64_t)val[e] : 1ULL;
            acc += mix64(mix64(key) + v);
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0 && acc) atomicAdd(out + 1, (unsigned long long)acc);
    if (blockIdx.x == 0 && threadIdx.x == 0) out[0] = (unsigned long long)C.rowptr[C.rows];
}

// Digests of many row views in one launch: blockIdx.y picks the view.
// out[2 o] = the view's nnz, out[2 o + 1] += its entries' hash sum (rows
// counted from the view's first row); out must start zeroed.
__global__ void __launch_bounds__(256) k_digest_multi(const DigestJob *jobs, unsigned long long *out) {
    const DigestJob jb = jobs[blockIdx.y];
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    uint64_t acc = 0;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < jb.rows; r += warps) {
        const int64_t e1 = jb.rowptr[r + 1];
        for (int64_t e = jb.rowptr[r] + lane; e < e1; e += 32) {
            const uint64_t key = ((uint64_t)r << 32) | (uint32_t)jb.col[e];
            uint64_t v = 1ULL;
            if (jb.val) v = jb.vbytes == 8 ? ((const uint64_t *)jb.val)[e] : (uint64_t)((const uint32_t *)jb.val)[e];
            acc += mix64(mix64(key) + v);
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0 && acc) atomicAdd(out + 2 * jb.out + 1, (unsigned long long)acc);
    if (blockIdx.x == 0 && threadIdx.x == 0) out[2 * jb.out] = (unsigned long long)(jb.rowptr[jb.rows] - jb.rowptr[0]);
}

}  // namespace

namespace {

// Copy of up to three device ranges into host memory (device addresses of
// pinned host buffers) by SM stores: the copy engines stay free for the small
// read-backs of the executor.  Ranges whose source and destination share
// their 16-byte alignment move in 16-byte words between byte-wise ends.
struct OutRange {
    const char *src;
    char *dst;
    int64_t bytes;
};

__global__ void __launch_bounds__(512) k_copy_out(OutRange r0, OutRange r1, OutRange r2) {
    const OutRange rs[3] = {r0, r1, r2};
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
    for (int i = 0; i < 3; i++) {
        const OutRange r = rs[i];
        if (r.bytes <= 0) continue;
        const int64_t head = ((16 - ((uintptr_t)r.src & 15)) & 15) < r.bytes ? ((16 - ((uintptr_t)r.src & 15)) & 15)
                                                                             : r.bytes;
        const bool same = (((uintptr_t)r.src ^ (uintptr_t)r.dst) & 15) == 0;
        const int64_t body = same ? (r.bytes - head) / 16 : 0;
        const int64_t tail0 = same ? head + body * 16 : 0;
        if (same) {
            for (int64_t b = tid; b < head; b += nt) r.dst[b] = r.src[b];
            const uint4 *s4 = (const uint4 *)(r.src + head);
            uint4 *d4 = (uint4 *)(r.dst + head);
            for (int64_t w = tid; w < body; w += nt) d4[w] = s4[w];
        }
        for (int64_t b = tail0 + tid; b < r.bytes; b += nt) r.dst[b] = r.src[b];
    }
}

}  // namespace

// Page-locked host memory (allocated or registered with CUDA).  Only such
// buffers go through the copy kernels: a pageable buffer may be device-
// addressable too (the GPU reaches all host memory here), but its owner may
// free it as soon as the call returns, before an asynchronous kernel has read
// it -- pageable copies stay on the copy engine, which stages them before
// returning.
static bool pinned_host(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Download of a result's arrays by k_copy_out on stream s; false when some
// destination is not page-locked: the caller copies.
bool copy_out_launch(const void *const *src, void *const *dst_host, const int64_t *bytes, cudaStream_t s) {
    OutRange r[3] = {};
    for (int i = 0; i < 3; i++) {
        if (!dst_host[i] || bytes[i] <= 0) continue;
        if (!pinned_host(dst_host[i])) return false;
        void *alias = nullptr;
        if (cudaHostGetDevicePointer(&alias, dst_host[i], 0) != cudaSuccess || !alias) {
            cudaGetLastError();
            return false;
        }
        r[i] = OutRange{(const char *)src[i], (char *)alias, bytes[i]};
    }
    k_copy_out<<<16, 512, 0, s>>>(r[0], r[1], r[2]);
    return cudaGetLastError() == cudaSuccess;
}

int32_t digest_multi_launch(rmcm_handle *h, const DigestJob *jobs_dev, int32_t njobs, uint64_t *out_dev) {
    if (njobs <= 0) return RMCM_OK;
    if (njobs > 65535) return set_error(h, RMCM_EINVAL, "digest: too many views");
    k_digest_multi<<<dim3(16, (unsigned)njobs), 256, 0, h->stream>>>(jobs_dev, (unsigned long long *)out_dev);
    h->launches++;
    RMCM_CUDA(h, cudaGetLastError());
    return RMCM_OK;
}

int32_t chain_order_multi(rmcm_handle *h, const double *c_all, const int32_t *lens_dev, int32_t n, int32_t *split_all,
                          double *cost_all, int32_t *pairs_all) {
    if (n <= 0) return RMCM_OK;
    k_chain_dp<<<(unsigned)n, 32, 0, h->stream>>>(c_all, lens_dev, n, split_all, cost_all, pairs_all, 0);
    h->launches++;
    RMCM_CUDA(h, cudaGetLastError());
    return RMCM_OK;
}

int32_t mat_digest_launch(rmcm_handle *h, const rmcm_mat *m, uint64_t *out_dev, int64_t row0) {
    cudaStream_t s = h->stream;
    RMCM_CUDA(h, cudaMemsetAsync(out_dev, 0, 2 * sizeof(uint64_t), s));
    const int64_t want = (m->d.rows * 32 + 255) / 256;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)h->sm_count * 8));
    if (m->valtype == RMCM_VAL_U64)
        k_digest<uint64_t><<<grid, 256, 0, s>>>(m->d, (unsigned long long *)out_dev, row0);
    else
        k_digest<uint32_t><<<grid, 256, 0, s>>>(m->d, (unsigned long long *)out_dev, row0);
    h->launches++;
    RMCM_CUDA(h, cudaGetLastError());
    return RMCM_OK;
}

int32_t chain_order_dev(rmcm_handle *h, const double *c_dev, int32_t len, int32_t *split_dev, double *cost_dev,
                        int32_t *pairs_dev) {
    // single-chain form: c_dev is len*len; stage it into the 16x16 batched layout
    if (len < 1 || len > kMaxLen) return set_error(h, RMCM_EINVAL, "order: chain length must be 1..16");
    cudaStream_t s = h->stream;
    const int64_t cbytes = sizeof(double) * kMaxLen * kMaxLen;
    char *buf = nullptr;
    const int64_t total = cbytes + 256 + 4 * kMaxLen * kMaxLen + cbytes + 4 * 2 * kMaxLen;
    RMCM_TRY(dev_alloc(h, (void **)&buf, total + 1024));
    double *c16 = (double *)buf;
    int32_t *lens = (int32_t *)(buf + cbytes);
    int32_t *sp16 = (int32_t *)(buf + cbytes + 256);
    double *cost16 = (double *)(buf + cbytes + 256 + 4 * kMaxLen * kMaxLen);
    int32_t *pairs16 = (int32_t *)((char *)cost16 + cbytes);
    cudaError_t e = cudaMemcpyAsync(c16, c_dev, sizeof(double) * len * len, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) {
        int32_t L = len;
        e = cudaMemcpyAsync(lens, &L, sizeof(int32_t), cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess) {
        k_chain_dp<<<1, 32, 0, s>>>(c16, lens, 1, sp16, cost16, pairs16, 0);
        h->launches++;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && split_dev)
        e = cudaMemcpyAsync(split_dev, sp16, sizeof(int32_t) * len * len, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && cost_dev)
        e = cudaMemcpyAsync(cost_dev, cost16, sizeof(double) * len * len, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && pairs_dev && len > 1)
        e = cudaMemcpyAsync(pairs_dev, pairs16, sizeof(int32_t) * 2 * (len - 1), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);   // host value of L must outlive the copy
    dev_free(h, buf, total + 1024);
    if (e != cudaSuccess) return cuda_error(h, e, "chain order");
    return RMCM_OK;
}

int32_t chain_order_launch(rmcm_handle *h, const double *c_dev, int32_t len, double *c16, int32_t *split16,
                           double *cost16, int32_t *pairs32) {
    if (len < 1 || len > kMaxLen) return set_error(h, RMCM_EINVAL, "order: chain length must be 1..16");
    cudaStream_t s = h->stream;
    RMCM_CUDA(h, cudaMemcpyAsync(c16, c_dev, sizeof(double) * len * len, cudaMemcpyDeviceToDevice, s));
    k_chain_dp<<<1, 32, 0, s>>>(c16, nullptr, 1, split16, cost16, pairs32, len);
    h->launches++;
    RMCM_CUDA(h, cudaGetLastError());
    return RMCM_OK;
}

}  // namespace rmcm
