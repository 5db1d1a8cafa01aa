// Tensor-core part of dense-bin products (sm_103a; FP16 limb GEMMs on
// tcgen05 with FP32 accumulation in TMEM, exact integer results).
//
// A product C = A B whose output rows all sit in the dense bin often has a
// few inner indices u (columns of A, rows of B) that carry most of its
// multiply-adds: A's column u is nearly full and so is B's row u (in the
// retail workload, the heaviest users of T x U . U x C).  For those, the
// sub-product A[:, H] B[H, :] is dense work: it runs as a GEMM on the tensor
// cores (k_tc_seed, tc_gemm.cu), and the dense-bin kernel streams only the
// remaining entries of A into counters seeded with the GEMM's rows.
//
// Exactness.  A's heavy values (<= 2048) and B's heavy values split into L
// limbs of `bits` bits (each <= 2047) are integers that FP16 holds exactly;
// their products and every partial sum of a GEMM output are non-negative
// integers no larger than S_A * (2^bits - 1) <= 2^24, S_A being the largest
// sum of a row's heavy A values, so FP32 holds each of them exactly in any
// summation order.  The row's counter then takes sum_l G_l << (bits * l)
// modulo 2^32, the uint32 value of the exact product (rows that could
// overflow uint32 never come here); the GEMM's epilogue forms that sum and
// writes one uint32 seed per output.
//
// The heavy set: an inner index is heavy when (A column count / rows) x
// (B row length / cols) reaches 1 / inv_density, the point where a dense
// multiply-add on the tensor cores costs less than the sparse ones it
// replaces; column counts are sampled (every 8th entry of A).  Which indices
// are heavy only moves work between the two parts, never changes a result.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "internal.h"

namespace rmcm {
namespace {

constexpr int kSample = 8;            // A entries per counted one (column counts)
constexpr int64_t kMaxHeavy = 65536;  // heavy indices at most (A panel row in shared memory)
constexpr int kGatherThreads = 256;
constexpr int kGatherPer = 8;          // A entries per thread per step of k_gather_a

// Sampled column counts of A: cnt[u] += 1 for every kSample-th entry.
__global__ void k_col_sample(DevCsr A, uint32_t *cnt) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x * kSample;
    for (int64_t k = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kSample; k < A.nnz; k += stride)
        atomicAdd(cnt + A.col[k], 1u);
}

// heavy[u] = score threshold met; slot[u] = its index in the heavy list
// (order of discovery: the list order never changes a result), list[slot] = u.
__global__ void k_heavy_select(int64_t nin, const uint32_t *cnt, const int64_t *browptr, double thr,
                               uint8_t *heavy, int32_t *slot, int32_t *list, int32_t *nheavy, int32_t cap) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t u0 = (int64_t)blockIdx.x * blockDim.x; u0 < nin; u0 += stride) {
        const int64_t u = u0 + threadIdx.x;
        bool hv = false;
        if (u < nin) {
            const double score = (double)cnt[u] * kSample * (double)(browptr[u + 1] - browptr[u]);
            hv = score >= thr;
        }
        const unsigned b = __ballot_sync(0xffffffffu, hv);
        int base = 0;
        if (lane == 0 && b) base = atomicAdd(nheavy, __popc(b));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (u < nin) {
            int32_t s = -1;
            if (hv) {
                s = base + __popc(b & ((1u << lane) - 1u));
                if (s < cap) list[s] = (int32_t)u;
                else s = -1;
            }
            heavy[u] = s >= 0;
            slot[u] = s;
        }
    }
}

// Row panel of A over the heavy indices: Ad[r][slot[u]] = A[r][u] as FP16
// (ld columns, zero elsewhere), built in shared memory and written whole.
// The row's other (light) entries go, in any order, to the front of its
// segment of (lcol, lval); lcnt[r] = their number.  stats[0] = largest row
// sum of heavy values, stats[1] = largest heavy value.  With lflops (B's row
// pointers in browptr) also the row's light products: lflops[r] = the sum of
// B's row lengths over its light entries, stats[5] = their largest row sum,
// stats[6] = their total.  stats[7] = the most heavy entries in a row.
__global__ void __launch_bounds__(kGatherThreads) k_gather_a(DevCsr A, const int32_t *slot, int32_t ld, __half *Ad,
                                                             int32_t *lcol, uint32_t *lval, int32_t *lcnt,
                                                             unsigned long long *stats, const int64_t *browptr,
                                                             int64_t *lflops) {
    extern __shared__ __align__(16) unsigned char smem[];
    __half *row = (__half *)smem;
    __shared__ unsigned long long s_sum, s_max, s_lf;
    __shared__ int32_t s_light, s_heavy;
    const int lane = threadIdx.x & 31;
    const uint32_t *av = (const uint32_t *)A.val;
    for (int64_t r = blockIdx.x; r < A.rows; r += gridDim.x) {
        for (int i = threadIdx.x; i < ld / 8; i += kGatherThreads) ((uint4 *)row)[i] = make_uint4(0, 0, 0, 0);
        if (threadIdx.x == 0) {
            s_sum = 0;
            s_max = 0;
            s_lf = 0;
            s_light = 0;
            s_heavy = 0;
        }
        __syncthreads();
        const int64_t a0 = A.rowptr[r], a1 = A.rowptr[r + 1];
        unsigned long long sum = 0, mx = 0, lf = 0;
        int32_t nheavy = 0;
        // kGatherPer entries per thread per step: their gathers overlap; the
        // light ones are placed with one shared reservation per warp and step
        for (int64_t k0 = a0; k0 < a1; k0 += kGatherPer * kGatherThreads) {
            int32_t c[kGatherPer], sl[kGatherPer];
            uint32_t v[kGatherPer];
#pragma unroll
            for (int u = 0; u < kGatherPer; u++) {
                const int64_t k = k0 + u * kGatherThreads + threadIdx.x;
                c[u] = k < a1 ? A.col[k] : -1;
                v[u] = k < a1 ? av[k] : 0u;
            }
#pragma unroll
            for (int u = 0; u < kGatherPer; u++) sl[u] = c[u] >= 0 ? slot[c[u]] : -1;
            uint32_t lm = 0;
#pragma unroll
            for (int u = 0; u < kGatherPer; u++) {
                if (sl[u] >= 0) {
                    row[sl[u]] = __uint2half_rn(v[u]);
                    sum += v[u];
                    mx = v[u] > mx ? v[u] : mx;
                    nheavy++;
                } else if (c[u] >= 0) {
                    lm |= 1u << u;
                }
            }
            const int nl = __popc(lm);
            int incl = nl;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += t;
            }
            const int wtot = __shfl_sync(0xffffffffu, incl, 31);
            int base = 0;
            if (lane == 0 && wtot) base = atomicAdd(&s_light, wtot);
            base = __shfl_sync(0xffffffffu, base, 0);
            int64_t o = a0 + base + incl - nl;
#pragma unroll
            for (int u = 0; u < kGatherPer; u++) {
                if ((lm >> u) & 1u) {
                    lcol[o] = c[u];
                    lval[o] = v[u];
                    o++;
                }
            }
            if (lflops) {
#pragma unroll
                for (int u = 0; u < kGatherPer; u++)
                    if ((lm >> u) & 1u) lf += (unsigned long long)(browptr[c[u] + 1] - browptr[c[u]]);
            }
        }
        if (sum) atomicAdd(&s_sum, sum);
        if (mx) atomicMax(&s_max, mx);
        if (lf) atomicAdd(&s_lf, lf);
        if (nheavy) atomicAdd(&s_heavy, nheavy);
        __syncthreads();
        uint4 *dst = (uint4 *)(Ad + r * (int64_t)ld);
        for (int i = threadIdx.x; i < ld / 8; i += kGatherThreads) dst[i] = ((const uint4 *)row)[i];
        if (threadIdx.x == 0) {
            lcnt[r] = s_light;
            if (s_sum) atomicMax(stats, s_sum);
            if (s_max) atomicMax(stats + 1, s_max);
            if (s_heavy) atomicMax(stats + 7, (unsigned long long)s_heavy);
            if (lflops) {
                lflops[r] = (int64_t)s_lf;
                if (s_lf) {
                    atomicMax(stats + 5, s_lf);
                    atomicAdd(stats + 6, s_lf);
                }
            }
        }
        __syncthreads();
    }
}

// Limb l of B's heavy rows, transposed for the tensor cores (K contiguous):
// BdT[l][c][h] = (B[list[h]][c] >> (bits l)) & (2^bits - 1) as FP16, for
// c < ldn and h < ldk (zero where B has no entry, for h >= nh and c >= cols).
// A CTA stages the 64 heavy rows h0.. over kBtCols columns in shared memory,
// one tile per limb filled in a single pass over the entries (33-word pitch:
// the scatter of a warp's columns hits distinct banks), and writes each
// output row's 128 bytes coalesced.  stats[2] = largest value.
constexpr int kBtCols = 256;
constexpr int kBtPitch = 66;   // halves per staged row: 64 heavy rows + 2
constexpr int64_t kBtTileBytes = (int64_t)kBtCols * kBtPitch * 2;

template <typename V>
__global__ void __launch_bounds__(kGatherThreads) k_gather_bt(DevCsr B, const int32_t *list, int32_t nh, int32_t ldk,
                                                              int32_t ldn, int32_t limbs, int32_t bits, __half *BdT,
                                                              int64_t limb_stride, unsigned long long *stats) {
    extern __shared__ __align__(16) unsigned char smem[];
    __half *tiles = (__half *)smem;   // limbs x kBtCols x kBtPitch
    __shared__ int64_t s_beg[64], s_end[64];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int32_t h0 = (int32_t)blockIdx.x * 64;
    const int32_t c0 = (int32_t)blockIdx.y * kBtCols;
    const int32_t nc = min(kBtCols, ldn - c0);
    if (threadIdx.x < 64) {
        // the row's entries with columns in [c0, c0 + kBtCols): two lower bounds
        const int32_t hr = h0 + (int32_t)threadIdx.x;
        int64_t b = 0, e = 0;
        if (hr < nh) {
            const int32_t u = list[hr];
            const int64_t end = B.rowptr[u + 1];
            int64_t lo = B.rowptr[u], hi = end;
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (B.col[mid] < c0) lo = mid + 1;
                else hi = mid;
            }
            b = lo;
            hi = end;
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (B.col[mid] < c0 + kBtCols) lo = mid + 1;
                else hi = mid;
            }
            e = lo;
        }
        s_beg[threadIdx.x] = b;
        s_end[threadIdx.x] = e;
    }
    const V *bv = (const V *)B.val;
    const V mask = ((V)1 << bits) - (V)1;
    unsigned long long mx = 0;
    uint32_t *tw = (uint32_t *)tiles;
    for (int i = threadIdx.x; i < limbs * (kBtCols * kBtPitch / 2); i += kGatherThreads) tw[i] = 0u;
    __syncthreads();
    for (int hr = warp; hr < 64; hr += kGatherThreads / 32) {
        const int64_t e = s_end[hr];
        for (int64_t k = s_beg[hr] + lane; k < e; k += 32) {
            const int32_t c = B.col[k];
            const V v = bv[k];
            mx = (unsigned long long)v > mx ? (unsigned long long)v : mx;
            for (int l = 0; l < limbs; l++)
                tiles[(int64_t)l * (kBtCols * kBtPitch) + (c - c0) * kBtPitch + hr] =
                    __uint2half_rn((uint32_t)((v >> (bits * l)) & mask));
        }
    }
    __syncthreads();
    for (int l = 0; l < limbs; l++) {
        const uint32_t *tl = tw + (int64_t)l * (kBtCols * kBtPitch / 2);
        for (int cr = warp; cr < nc; cr += kGatherThreads / 32) {
            uint32_t *dst = (uint32_t *)(BdT + l * limb_stride + (int64_t)(c0 + cr) * ldk + h0);
            dst[lane] = tl[cr * (kBtPitch / 2) + lane];
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, mx, d);
        mx = o > mx ? o : mx;
    }
    if (lane == 0 && mx) atomicMax(stats + 2, mx);
}

// Per row of A the number of heavy entries and the largest heavy value
// (stats[3], stats[4]: maxima over rows); TA is A's value type.  A CTA per
// row, kGatherPer entries per thread per step (the column -> slot gathers
// overlap, so a long row does not serialise a warp).
template <typename TA>
__global__ void __launch_bounds__(kGatherThreads) k_heavy_stats(DevCsr A, const int32_t *slot,
                                                                unsigned long long *stats) {
    __shared__ unsigned long long s_cnt;
    const int lane = threadIdx.x & 31;
    const TA *av = (const TA *)A.val;
    unsigned long long cmax = 0, vmax = 0;
    for (int64_t r = blockIdx.x; r < A.rows; r += gridDim.x) {
        if (threadIdx.x == 0) s_cnt = 0;
        __syncthreads();
        const int64_t a0 = A.rowptr[r], a1 = A.rowptr[r + 1];
        unsigned long long c = 0;
        for (int64_t k0 = a0; k0 < a1; k0 += kGatherPer * kGatherThreads) {
            int32_t col[kGatherPer];
#pragma unroll
            for (int u = 0; u < kGatherPer; u++) {
                const int64_t k = k0 + u * kGatherThreads + threadIdx.x;
                col[u] = k < a1 ? A.col[k] : -1;
            }
#pragma unroll
            for (int u = 0; u < kGatherPer; u++) {
                if (col[u] >= 0 && slot[col[u]] >= 0) {
                    c++;
                    const unsigned long long v = (unsigned long long)av[k0 + u * kGatherThreads + threadIdx.x];
                    vmax = v > vmax ? v : vmax;
                }
            }
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) c += __shfl_xor_sync(0xffffffffu, c, d);
        if (lane == 0 && c) atomicAdd(&s_cnt, c);
        __syncthreads();
        if (threadIdx.x == 0) cmax = s_cnt > cmax ? s_cnt : cmax;
        __syncthreads();
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, vmax, d);
        vmax = o > vmax ? o : vmax;
    }
    if (lane == 0 && vmax) atomicMax(stats + 4, vmax);
    if (threadIdx.x == 0 && cmax) atomicMax(stats + 3, cmax);
}

// Row panels of A in limbs (TA: A's value type): limb l of each heavy
// value, (A[r][u] >> (bits l)) & (2^bits - 1) as FP16 at Ad[l][r][slot[u]].
// A CTA per row holds `group` limb rows in shared memory and fills them in
// one pass over the row's entries, kGatherPer entries per thread per step
// (the column -> slot gathers overlap); a row with more limbs than fit takes
// one pass per group.  With lcol (first pass only) the light entries are
// compacted per row and, with lflops, their products counted, as in
// k_gather_a.
template <typename TA>
__global__ void __launch_bounds__(kGatherThreads) k_gather_al(DevCsr A, const int32_t *slot, int32_t ld,
                                                              int32_t limbs, int32_t group, int32_t bits,
                                                              __half *Ad, int64_t limb_stride, int32_t *lcol,
                                                              TA *lval, int32_t *lcnt, unsigned long long *stats,
                                                              const int64_t *browptr, int64_t *lflops) {
    extern __shared__ __align__(16) unsigned char smem[];
    __half *rows = (__half *)smem;
    __shared__ int32_t s_light;
    __shared__ unsigned long long s_lf;
    const int lane = threadIdx.x & 31;
    const TA *av = (const TA *)A.val;
    const uint64_t mask = (1ull << bits) - 1ull;
    for (int64_t r = blockIdx.x; r < A.rows; r += gridDim.x) {
        const int64_t a0 = A.rowptr[r], a1 = A.rowptr[r + 1];
        if (threadIdx.x == 0) {
            s_light = 0;
            s_lf = 0;
        }
        unsigned long long lf = 0;
        for (int l0 = 0; l0 < limbs; l0 += group) {
            const int ng = min(group, limbs - l0);
            const bool compact = lcol && l0 == 0;
            for (int i = threadIdx.x; i < ng * ld / 8; i += kGatherThreads) ((uint4 *)rows)[i] = make_uint4(0, 0, 0, 0);
            __syncthreads();
            for (int64_t k0 = a0; k0 < a1; k0 += kGatherPer * kGatherThreads) {
                int32_t c[kGatherPer], sl[kGatherPer];
                uint64_t v[kGatherPer];
#pragma unroll
                for (int u = 0; u < kGatherPer; u++) {
                    const int64_t k = k0 + u * kGatherThreads + threadIdx.x;
                    c[u] = k < a1 ? A.col[k] : -1;
                    v[u] = k < a1 ? (uint64_t)av[k] : 0ull;
                }
#pragma unroll
                for (int u = 0; u < kGatherPer; u++) sl[u] = c[u] >= 0 ? slot[c[u]] : -1;
                uint32_t lm = 0;
#pragma unroll
                for (int u = 0; u < kGatherPer; u++) {
                    if (sl[u] >= 0) {
                        for (int l = 0; l < ng; l++)
                            rows[l * ld + sl[u]] = __uint2half_rn((uint32_t)((v[u] >> (bits * (l0 + l))) & mask));
                    } else if (c[u] >= 0) {
                        lm |= 1u << u;
                    }
                }
                if (compact) {
                    // one shared reservation per warp and step for its light entries
                    const int nl = __popc(lm);
                    int incl = nl;
#pragma unroll
                    for (int d = 1; d < 32; d <<= 1) {
                        const int t = __shfl_up_sync(0xffffffffu, incl, d);
                        if (lane >= d) incl += t;
                    }
                    const int wtot = __shfl_sync(0xffffffffu, incl, 31);
                    int base = 0;
                    if (lane == 0 && wtot) base = atomicAdd(&s_light, wtot);
                    base = __shfl_sync(0xffffffffu, base, 0);
                    int64_t o = a0 + base + incl - nl;
#pragma unroll
                    for (int u = 0; u < kGatherPer; u++) {
                        if ((lm >> u) & 1u) {
                            lcol[o] = c[u];
                            lval[o] = (TA)v[u];
                            o++;
                            if (lflops) lf += (unsigned long long)(browptr[c[u] + 1] - browptr[c[u]]);
                        }
                    }
                }
            }
            __syncthreads();
            for (int l = 0; l < ng; l++) {
                uint4 *dst = (uint4 *)(Ad + (l0 + l) * limb_stride + r * (int64_t)ld);
                const uint4 *src = (const uint4 *)(rows + (int64_t)l * ld);
                for (int i = threadIdx.x; i < ld / 8; i += kGatherThreads) dst[i] = src[i];
            }
            __syncthreads();
        }
        if (lcol) {
            if (lf) atomicAdd(&s_lf, lf);
            __syncthreads();
            if (threadIdx.x == 0) {
                lcnt[r] = s_light;
                if (lflops) {
                    lflops[r] = (int64_t)s_lf;
                    if (s_lf) {
                        atomicMax(stats + 5, s_lf);
                        atomicAdd(stats + 6, s_lf);
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Opts k_gather_bt<V> in to the shared memory of `limbs` tiles; false when
// the device refuses (the caller keeps the product sparse).
template <typename V>
bool gather_bt_smem(int32_t limbs) {
    const int64_t bytes = limbs * kBtTileBytes;
    if (bytes <= 48 * 1024) return true;
    if (cudaFuncSetAttribute(k_gather_bt<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess)
        return true;
    cudaGetLastError();
    return false;
}

}  // namespace

// Heavy inner indices of C = A B: sampled column counts of A and the density
// rule give each heavy index a slot (k_heavy_select).  With stats64 also the
// largest number of heavy entries in a row of A and the largest heavy value
// (k_heavy_stats64).  On success hs.sel holds the buffers (the caller frees
// it); nh < 64 means the caller gives up.
struct HeavySet {
    char *sel = nullptr;
    int64_t sel_bytes = 0;
    uint8_t *flag = nullptr;
    int32_t *slot = nullptr, *list = nullptr;
    unsigned long long *stats = nullptr;   // device: [2] largest B value seen, [3..4] as above
    int64_t nh = 0;
    uint64_t hrow = 0, amax = 0;
};

int32_t select_heavy(rmcm_handle *h, const DevCsr &A, const DevCsr &B, bool stats64, HeavySet &hs) {
    hs = HeavySet{};
    cudaStream_t s = h->stream;
    const int64_t M = A.rows, N = B.cols, K = A.cols;
    const double thr = (double)M * (double)N / (double)h->tune.gemm_inv_density;
    auto al = [](int64_t x) { return (x + 255) & ~255LL; };
    const int64_t o_cnt = 0, o_flag = o_cnt + al(4 * K), o_slot = o_flag + al(K), o_list = o_slot + al(4 * K);
    const int64_t o_small = o_list + al(4 * kMaxHeavy);
    hs.sel_bytes = o_small + 256;
    RMCM_TRY(dev_alloc(h, (void **)&hs.sel, hs.sel_bytes));
    uint32_t *cnt = (uint32_t *)(hs.sel + o_cnt);
    hs.flag = (uint8_t *)(hs.sel + o_flag);
    hs.slot = (int32_t *)(hs.sel + o_slot);
    hs.list = (int32_t *)(hs.sel + o_list);
    int32_t *nheavy = (int32_t *)(hs.sel + o_small);
    hs.stats = (unsigned long long *)(hs.sel + o_small + 64);
    RMCM_CUDA(h, cudaMemsetAsync(cnt, 0, 4 * K, s));
    RMCM_CUDA(h, cudaMemsetAsync(hs.sel + o_small, 0, 256, s));
    k_col_sample<<<h->sm_count * 8, 256, 0, s>>>(A, cnt);
    k_heavy_select<<<h->sm_count * 8, 256, 0, s>>>(K, cnt, B.rowptr, thr, hs.flag, hs.slot, hs.list, nheavy,
                                                  (int32_t)kMaxHeavy);
    h->launches += 2;
    if (stats64) {
        k_heavy_stats<uint64_t><<<(int)std::min<int64_t>(std::max<int64_t>(A.rows, 1), (int64_t)h->sm_count * 8),
                                  kGatherThreads, 0, s>>>(A, hs.slot, hs.stats);
        h->launches++;
    }
    RMCM_CUDA(h, cudaGetLastError());
    // the count (and the stats) in one read-back: h_pinned[8..] = small area
    RMCM_CUDA(h, cudaMemcpyAsync(h->h_pinned + 8, hs.sel + o_small, 64 + 40, cudaMemcpyDeviceToHost, s));
    RMCM_CUDA(h, cudaStreamSynchronize(s));
    hs.nh = std::min<int64_t>(((int32_t *)(h->h_pinned + 8))[0], kMaxHeavy);
    hs.hrow = (uint64_t)h->h_pinned[8 + 8 + 3];
    hs.amax = (uint64_t)h->h_pinned[8 + 8 + 4];
    return RMCM_OK;
}

// A's light entries, compacted per row (with their products per row when
// lflops is set), as a limb-form build can take them over.
struct LightPart {
    char *amem = nullptr;
    int64_t bytes = 0;
    int32_t *lcol = nullptr;
    void *lval = nullptr;
    int32_t *lcnt = nullptr;
    int64_t *lflops = nullptr;
    int64_t lmax = 0, ltotal = 0;
};

template <typename V>
int32_t build_limbs(rmcm_handle *h, const DevCsr &A, const DevCsr &B, uint64_t bmax, HeavySet &hs, DensePart &dp,
                    cudaEvent_t ev_begin, cudaEvent_t ev_end, bool light_flops, const LightPart *pre);

// Builds the tensor-core part of C = A B (uint32, single-window dense rows):
// on success dp.S holds the uint32 seeds (rows x ld) and dp.skip
// flags the heavy inner indices; otherwise dp stays empty (and the product
// runs sparse).  bmax: an upper bound on B's values.
int32_t dense_part_build(rmcm_handle *h, const DevCsr &A, const DevCsr &B, uint64_t bmax, DensePart &dp,
                         cudaEvent_t ev_begin, cudaEvent_t ev_end, bool light_flops) {
    dp = DensePart{};
    const int32_t inv_density = h->tune.gemm_inv_density;
    if (inv_density <= 0 || A.rows == 0 || B.cols == 0 || A.cols == 0) return RMCM_OK;
    cudaStream_t s = h->stream;
    const int64_t M = A.rows, N = B.cols;
    const int64_t ldn = (N + 7) / 8 * 8;
    auto al = [](int64_t x) { return (x + 255) & ~255LL; };
    HeavySet hs;
    RMCM_TRY(select_heavy(h, A, B, false, hs));
    char *sel = hs.sel;
    const int64_t sel_bytes = hs.sel_bytes;
    uint8_t *flag = hs.flag;
    int32_t *slot = hs.slot, *list = hs.list;
    unsigned long long *stats = hs.stats;
    auto fail = [&](int32_t rc) {
        dev_free(h, sel, sel_bytes);
        dp = DensePart{};
        return rc;
    };
    const int64_t nh = hs.nh;
    // worth a GEMM only when the heavy part is a real share of the work
    if (nh < 64) return fail(RMCM_OK);
    const int64_t ldk = (nh + 63) / 64 * 64;
    // dense panels: A (M x ldk) and up to 3 limbs of B held transposed
    // (ldn x ldk), FP16; the seeds S (M x ldn), uint32
    const int64_t a_bytes = al(2 * M * ldk), b_limb = ldk * ldn, g_limb = M * ldn;
    const int64_t max_bytes = (h->budget - h->in_use) / 3;
    const int64_t l_bytes = al(8 * A.nnz) + al(4 * M) + (light_flops ? al(8 * M) : 0);
    if (a_bytes + l_bytes + al(2 * 3 * b_limb) + al(4 * g_limb) > max_bytes) return fail(RMCM_OK);
    if (ldk * 2 > 160 * 1024) return fail(RMCM_OK);
    // A panel (freed once the GEMMs are queued); A's light entries
    // (compacted per row) and their counts (kept for the dense kernel)
    __half *Ad = nullptr;
    char *amem = nullptr;
    RMCM_TRY(dev_alloc(h, (void **)&Ad, a_bytes));
    if (dev_alloc(h, (void **)&amem, l_bytes) != RMCM_OK) {
        dev_free(h, Ad, a_bytes);
        h->last_error.clear();
        return fail(RMCM_OK);
    }
    int32_t *lcol = (int32_t *)amem;
    uint32_t *lval = (uint32_t *)(lcol + A.nnz);
    int32_t *lcnt = (int32_t *)(amem + al(8 * A.nnz));
    int64_t *lflops = light_flops ? (int64_t *)(amem + al(8 * A.nnz) + al(4 * M)) : nullptr;
    auto fail2 = [&](int32_t rc) {
        dev_free(h, Ad, a_bytes);
        dev_free(h, amem, l_bytes);
        return fail(rc);
    };
    {
        const int64_t smem = ldk * 2;
        if (smem > 48 * 1024 &&
            cudaFuncSetAttribute(k_gather_a, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
            cudaGetLastError();
            return fail2(RMCM_OK);
        }
        const int grid = (int)std::min<int64_t>(M, (int64_t)h->sm_count * 8);
        k_gather_a<<<grid, kGatherThreads, smem, s>>>(A, slot, (int32_t)ldk, Ad, lcol, lval, lcnt, stats, B.rowptr,
                                                      lflops);
        h->launches++;
        RMCM_CUDA(h, cudaGetLastError());
    }
    RMCM_CUDA(h, cudaMemcpyAsync(h->h_pinned + 8, stats, 8 * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    RMCM_CUDA(h, cudaStreamSynchronize(s));
    const uint64_t s_a = ((uint64_t *)(h->h_pinned + 8))[0], a_max = ((uint64_t *)(h->h_pinned + 8))[1];
    const int64_t l_max = (int64_t)((uint64_t *)(h->h_pinned + 8))[5];
    const int64_t l_total = (int64_t)((uint64_t *)(h->h_pinned + 8))[6];
    const uint64_t h_row = ((uint64_t *)(h->h_pinned + 8))[7];
    if (s_a == 0) return fail2(RMCM_OK);
    // limb width: S_A * (2^bits - 1) <= 2^24 and 2^bits - 1 <= 2047
    int32_t bits = 0;
    while (bits < 11 && (double)s_a * (double)((1ull << (bits + 1)) - 1) <= 16777216.0) bits++;
    int32_t bbits = 0;
    while (bbits < 64 && (bmax >> bbits) != 0) bbits++;
    const int32_t limbs = bits ? std::max(1, (bbits + bits - 1) / bits) : 0;
    if (a_max > 2048 || bits == 0 || limbs > 3 || bits * (limbs - 1) >= 32) {
        // one limb of A cannot keep the partial sums exact: the limb form
        // (limbs of A too, chunks of the heavy indices) on the same heavy set,
        // taking over the light entries compacted above
        dev_free(h, Ad, a_bytes);
        hs.hrow = h_row;
        hs.amax = a_max;
        LightPart lp;
        lp.amem = amem;
        lp.bytes = l_bytes;
        lp.lcol = lcol;
        lp.lval = lval;
        lp.lcnt = lcnt;
        lp.lflops = lflops;
        lp.lmax = l_max;
        lp.ltotal = l_total;
        return build_limbs<uint32_t>(h, A, B, bmax, hs, dp, ev_begin, ev_end, light_flops, &lp);
    }
    const int64_t bd_bytes = al(2 * limbs * b_limb), g_bytes = al(4 * g_limb);
    char *mem = nullptr;
    if (dev_alloc(h, (void **)&mem, bd_bytes + g_bytes) != RMCM_OK) {
        h->last_error.clear();
        return fail2(RMCM_OK);
    }
    __half *BdT = (__half *)mem;
    uint32_t *S = (uint32_t *)(mem + bd_bytes);
    auto fail3 = [&](int32_t rc) {
        dev_free(h, mem, bd_bytes + g_bytes);
        return fail2(rc);
    };
    {
        dim3 grid((unsigned)(ldk / 64), (unsigned)((ldn + kBtCols - 1) / kBtCols));
        if (!gather_bt_smem<uint32_t>(limbs)) return fail3(RMCM_OK);
        k_gather_bt<uint32_t><<<grid, kGatherThreads, limbs * kBtTileBytes, s>>>(B, list, (int32_t)nh, (int32_t)ldk,
                                                                                  (int32_t)ldn,
                                                             limbs, bits, BdT, b_limb, stats);
        h->launches++;
        RMCM_CUDA(h, cudaGetLastError());
    }
    if (ev_begin) cudaEventRecord(ev_begin, s);
    {
        const int32_t rc = tc_seed_gemm(h, Ad, BdT, M, N, ldn, 1, limbs, ldk, 1, bits, 4, S, h->d_status + kTimeout);
        if (rc == RMCM_EINVAL) return fail3(RMCM_OK);   // a shape the kernel does not take: stay sparse
        if (rc != RMCM_OK) return fail3(rc);
    }
    if (ev_end) cudaEventRecord(ev_end, s);
    // the B gather saw no value wider than the limbs
    RMCM_CUDA(h, cudaMemcpyAsync(h->h_pinned + 8, stats + 2, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    RMCM_CUDA(h, cudaStreamSynchronize(s));
    const uint64_t seen = ((uint64_t *)(h->h_pinned + 8))[0];
    if (bits * limbs < 64 && (seen >> (bits * limbs)) != 0) return fail3(RMCM_OK);
    dev_free(h, Ad, a_bytes);
    dp.amem = amem;
    dp.abytes = l_bytes;
    dp.lcol = lcol;
    dp.lval = lval;
    dp.lcnt = lcnt;
    dp.lflops = lflops;
    dp.lmax = l_max;
    dp.ltotal = l_total;
    dp.mem = mem;
    dp.bytes = bd_bytes + g_bytes;
    dp.S = S;
    dp.ld = ldn;
    dp.limbs = limbs;
    dp.bits = bits;
    dp.heavy = nh;
    dp.sel = sel;
    dp.sel_bytes = sel_bytes;
    dp.skip = flag;
    return RMCM_OK;
}

// Limb form (uint64 products, and uint32 ones whose heavy row sums are too
// large for a single limb of A): A's heavy values are split into limbs as
// well, and the heavy indices into chunks of kc so that every partial sum of
// a GEMM output, at most min(heavy entries of a row, kc) x (A limb max) x
// (B limb max), stays <= 2^24.  G holds la x lb x nq panels, ((i lb + j) nq
// + q) in order; the row's counter takes sum G << (bits (i + j)) modulo
// 2^(8 sizeof(V)) (the epilogue drops the terms shifted out).  hs carries
// the heavy set with hrow and amax, pre (may be null) A's light entries
// already compacted for that set; both are freed on failure.
template <typename V>
int32_t build_limbs(rmcm_handle *h, const DevCsr &A, const DevCsr &B, uint64_t bmax, HeavySet &hs, DensePart &dp,
                    cudaEvent_t ev_begin, cudaEvent_t ev_end, bool light_flops, const LightPart *pre) {
    cudaStream_t s = h->stream;
    const int64_t M = A.rows, N = B.cols;
    const int64_t ldn = (N + 7) / 8 * 8;
    auto al = [](int64_t x) { return (x + 255) & ~255LL; };
    char *sel = hs.sel;
    const int64_t sel_bytes = hs.sel_bytes;
    uint8_t *flag = hs.flag;
    int32_t *slot = hs.slot, *list = hs.list;
    unsigned long long *stats = hs.stats;
    auto fail = [&](int32_t rc) {
        dev_free(h, sel, sel_bytes);
        if (pre) dev_free(h, pre->amem, pre->bytes);
        dp = DensePart{};
        return rc;
    };
    const int64_t nh = hs.nh;
    const uint64_t hrow = hs.hrow, amax = hs.amax;
    if (nh < 64 || amax == 0 || bmax == 0) return fail(RMCM_OK);
    auto bitlen = [](uint64_t v) {
        int b = 0;
        while (b < 64 && (v >> b) != 0) b++;
        return b;
    };
    // limb width: the fewest dense multiply-adds (limb pairs x padded heavy
    // indices), with at most 16 chunks of at least 64 indices each
    int32_t best_bits = 0, best_la = 0, best_lb = 0;
    int64_t best_kc = 0, best_nq = 0;
    for (int32_t bits = 11; bits >= 1; bits--) {
        const int32_t la = (bitlen(amax) + bits - 1) / bits, lb = (bitlen(bmax) + bits - 1) / bits;
        if (la > 4 || lb > 4 || bits * (la - 1 + lb - 1) >= 64) continue;
        const uint64_t mask = (1ull << bits) - 1;
        const double prod = (double)std::min(amax, mask) * (double)std::min(bmax, mask);
        int64_t kc = (int64_t)(16777216.0 / prod) / 64 * 64;
        int64_t nq = 1;
        if ((double)hrow * prod <= 16777216.0) {
            kc = (nh + 63) / 64 * 64;
        } else {
            if (kc < 64) continue;
            nq = (nh + kc - 1) / kc;
            if (nq > 16) continue;
            // the same number of chunks over evenly filled ones
            kc = ((nh + nq - 1) / nq + 63) / 64 * 64;
        }
        const int64_t cost = (int64_t)la * lb * kc * nq, best_cost = (int64_t)best_la * best_lb * best_kc * best_nq;
        if (best_bits == 0 || cost < best_cost || (cost == best_cost && nq < best_nq)) {
            best_bits = bits;
            best_la = la;
            best_lb = lb;
            best_kc = kc;
            best_nq = nq;
        }
    }
    if (best_bits == 0) return fail(RMCM_OK);
    const int32_t bits = best_bits, la = best_la, lb = best_lb;
    const int64_t kc = best_kc, nq = best_nq, ldk = kc * nq;
    const int64_t a_limb = M * ldk, b_limb = ldk * ldn, g_panel = M * ldn;
    const int64_t o_lval = al(4 * A.nnz), o_lcnt = o_lval + al((int64_t)sizeof(V) * A.nnz);
    const int64_t o_lf = o_lcnt + al(4 * M);
    const int64_t a_bytes = al(2 * la * a_limb);
    const int64_t l_bytes = pre ? pre->bytes : o_lf + (light_flops ? al(8 * M) : 0);
    const int64_t bd_bytes = al(2 * lb * b_limb), g_bytes = al((int64_t)sizeof(V) * g_panel);
    if (a_bytes + (pre ? 0 : l_bytes) + bd_bytes + g_bytes > (h->budget - h->in_use) / 3) return fail(RMCM_OK);
    // limb rows of A a gather CTA holds at once (~200 KB of shared memory)
    const int64_t group = std::min<int64_t>(la, (200 * 1024) / (ldk * 2));
    if (group < 1) return fail(RMCM_OK);
    __half *Ad = nullptr;
    char *amem = pre ? pre->amem : nullptr, *mem = nullptr;
    if (dev_alloc(h, (void **)&Ad, a_bytes) != RMCM_OK) {
        h->last_error.clear();
        return fail(RMCM_OK);
    }
    if ((!pre && dev_alloc(h, (void **)&amem, l_bytes) != RMCM_OK) ||
        dev_alloc(h, (void **)&mem, bd_bytes + g_bytes) != RMCM_OK) {
        if (amem && !pre) dev_free(h, amem, l_bytes);
        dev_free(h, Ad, a_bytes);
        h->last_error.clear();
        return fail(RMCM_OK);
    }
    auto fail3 = [&](int32_t rc) {
        dev_free(h, mem, bd_bytes + g_bytes);
        if (!pre) dev_free(h, amem, l_bytes);
        dev_free(h, Ad, a_bytes);
        return fail(rc);
    };
    int32_t *lcol = pre ? pre->lcol : (int32_t *)amem;
    V *lval = pre ? (V *)pre->lval : (V *)(amem + o_lval);
    int32_t *lcnt = pre ? pre->lcnt : (int32_t *)(amem + o_lcnt);
    int64_t *lflops = pre ? pre->lflops : (light_flops ? (int64_t *)(amem + o_lf) : nullptr);
    __half *BdT = (__half *)mem;
    V *S = (V *)(mem + bd_bytes);
    {
        const int64_t smem = group * ldk * 2;
        if (smem > 48 * 1024 &&
            cudaFuncSetAttribute(k_gather_al<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                cudaSuccess) {
            cudaGetLastError();
            return fail3(RMCM_OK);
        }
        const int grid = (int)std::min<int64_t>(M, (int64_t)h->sm_count * 8);
        // (with pre the light entries are already compacted: panels only)
        k_gather_al<V><<<grid, kGatherThreads, smem, s>>>(A, slot, (int32_t)ldk, la, (int32_t)group, bits, Ad,
                                                          a_limb, pre ? nullptr : lcol, lval, lcnt, stats, B.rowptr,
                                                          pre ? nullptr : lflops);
        dim3 bgrid((unsigned)(ldk / 64), (unsigned)((ldn + kBtCols - 1) / kBtCols));
        if (!gather_bt_smem<V>(lb)) return fail3(RMCM_OK);
        k_gather_bt<V><<<bgrid, kGatherThreads, lb * kBtTileBytes, s>>>(B, list, (int32_t)nh, (int32_t)ldk, (int32_t)ldn,
                                                                        lb, bits,
                                                       BdT, b_limb, stats);
        h->launches += 2;
        RMCM_CUDA(h, cudaGetLastError());
    }
    // every limb pair and chunk of the heavy indices in one kernel, summed
    // with its shift into one seed per output
    if (ev_begin) cudaEventRecord(ev_begin, s);
    {
        const int32_t rc = tc_seed_gemm(h, Ad, BdT, M, N, ldn, la, lb, kc, nq, bits, (int32_t)sizeof(V), S,
                                        h->d_status + kTimeout);
        if (rc == RMCM_EINVAL) return fail3(RMCM_OK);
        if (rc != RMCM_OK) return fail3(rc);
    }
    if (ev_end) cudaEventRecord(ev_end, s);
    if (light_flops || sizeof(V) == 4) {
        // light products (stats[5], stats[6]) and, for uint32, the largest
        // B value the gather saw (stats[2]: bmax came from the row scan)
        RMCM_CUDA(h, cudaMemcpyAsync(h->h_pinned + 8, stats, 7 * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        RMCM_CUDA(h, cudaStreamSynchronize(s));
        const uint64_t *st = (const uint64_t *)(h->h_pinned + 8);
        if (bits * lb < 64 && (st[2] >> (bits * lb)) != 0) return fail3(RMCM_OK);
        dp.lmax = pre ? pre->lmax : (int64_t)st[5];
        dp.ltotal = pre ? pre->ltotal : (int64_t)st[6];
    }
    dev_free(h, Ad, a_bytes);
    dp.amem = amem;
    dp.abytes = l_bytes;
    dp.lcol = lcol;
    dp.lval = (const uint32_t *)lval;
    dp.lcnt = lcnt;
    dp.lflops = lflops;
    dp.mem = mem;
    dp.bytes = bd_bytes + g_bytes;
    dp.S = S;
    dp.ld = ldn;
    dp.limbs = lb;
    dp.bits = bits;
    dp.alimbs = la;
    dp.abits = bits;
    dp.chunks = (int32_t)nq;
    dp.heavy = nh;
    dp.sel = sel;
    dp.sel_bytes = sel_bytes;
    dp.skip = flag;
    return RMCM_OK;
}

int32_t dense_part_build64(rmcm_handle *h, const DevCsr &A, const DevCsr &B, DensePart &dp, cudaEvent_t ev_begin,
                           cudaEvent_t ev_end) {
    dp = DensePart{};
    const int32_t inv_density = h->tune.gemm_inv_density;
    if (inv_density <= 0 || A.rows == 0 || B.cols == 0 || A.cols == 0) return RMCM_OK;
    HeavySet hs;
    RMCM_TRY(select_heavy(h, A, B, true, hs));
    // B's largest value (row sums' last slot; 1 for a matrix of ones)
    uint64_t bmax = 1;
    if (B.rowsum) {
        RMCM_CUDA(h, cudaMemcpyAsync(h->h_pinned + 24, B.rowsum + B.rows, 8, cudaMemcpyDeviceToHost, h->stream));
        RMCM_CUDA(h, cudaStreamSynchronize(h->stream));
        bmax = (uint64_t)h->h_pinned[24];
    }
    return build_limbs<uint64_t>(h, A, B, bmax, hs, dp, ev_begin, ev_end, false, nullptr);
}

void dense_part_release(rmcm_handle *h, DensePart &dp) {
    if (dp.amem) dev_free(h, dp.amem, dp.abytes);
    if (dp.mem) dev_free(h, dp.mem, dp.bytes);
    if (dp.sel) dev_free(h, dp.sel, dp.sel_bytes);
    dp = DensePart{};
}

}  // namespace rmcm
