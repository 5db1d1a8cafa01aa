// Tensor-core GEMM of the dense part (sm_103a: tcgen05 + TMA + mbarrier).
//
// The dense part of a product C = A B (dense_gemm.cu) is a sum of FP16
// GEMMs over limbs: A's heavy columns as la limb panels Ad_i (M x ldk, K
// contiguous), B's heavy rows as lb limb panels held transposed, BdT_j
// (ldn x ldk, K contiguous), and the heavy indices in nq chunks of kc.  Every
// partial sum of G_(i,j,q) = Ad_i[:, chunk q] BdT_j[:, chunk q]^T is an
// integer <= 2^24, so FP32 accumulation is exact in any order, and the
// product's dense part is
//
//     S[r][c] = sum_(i,j,q) G_(i,j,q)[r][c] << (bits (i + j))   mod 2^(8 sizeof V)
//
// This kernel computes S directly: per 128 x 128 output tile, for each
// (i, q) group it accumulates the lb limb products of B in TMEM (one
// 128-column accumulator per limb j) and its epilogue converts them to V,
// shifts and adds them into S.  The FP32 panels never reach HBM.
//
// Roles (192 threads): warp 0 lane 0 issues TMA loads into a ring of shared
// memory stages (one A tile and lb B tiles per 64-wide K block, 128-byte
// swizzle); warp 1 owns the TMEM allocation and its lane 0 issues
// tcgen05.mma (M = 128, N = 128, K = 16, FP16 in, FP32 accumulate) and the
// commits that release stages and hand accumulators to the epilogue; warps
// 2-5 read TMEM with tcgen05.ld (warp w reads lanes 32 (w mod 4) .. + 31,
// its TMEM sub-partition) and write S.
//
// Every wait is bounded (kWaitNs of wall time): a wait that runs out sets
// the kernel's error word and the shared abort flag; every role then leaves
// its loop, waits (bounded) for its own copies and MMAs in flight, and the
// TMEM is freed before the CTA exits.  The host reads the error word.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "internal.h"

namespace rmcm {
namespace {

constexpr int kTcThreads = 192;
constexpr int kBM = 128, kBK = 64;                    // MMA rows; kBK FP16 = one 128-byte swizzle row
constexpr uint32_t kTileBytes = kBM * kBK * 2;        // 16 KB per 128-row A tile
constexpr uint64_t kWaitNs = 2000000000ull;           // 2 s per wait
constexpr int kMaxStages = 8;
constexpr int kTmemCols = 512;
constexpr int kSegPitchBytes = 144;                   // staged 128-byte row segment + 16 (bank spread)
constexpr int kEpiBytes = 4 * 32 * kSegPitchBytes;    // 4 epilogue warps x 32 rows

struct TcParams {
    int32_t M, N, ldn;          // output rows, columns, row stride of S (elements)
    int32_t la, lb, nq, kc;     // A limbs, B limbs (<= 4), chunks, K per chunk (multiple of 64)
    int32_t bits;               // limb width
    int32_t stages;             // shared-memory ring depth
    // work units: CTA u < full_tiles computes tile u whole; the others split
    // the remaining tiles' K blocks `splits` ways and add their parts into
    // S (zeroed for those tiles) with atomics: the last, partial wave of
    // tiles then spreads over every SM
    int32_t n_tiles, full_tiles, splits;
    void *S;                    // seeds, M x ldn of V
    int *err;                   // error word (0 = ok)
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase of `bar` with the given parity; false when the wait
// ran out of time or another role aborted (the error word is then set).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort, int *err,
                                          int code) {
    if (mbar_try(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t it = 1;; it++) {
        if (mbar_try(bar, parity)) return true;
        if ((it & 255u) == 0) {
            if (*abort) return false;
            if (global_ns() - t0 > kWaitNs) {
                *abort = 1;
                atomicCAS(err, 0, code);
                return false;
            }
        }
    }
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int32_t x,
                                            int32_t y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor of a K-major tile with 128-byte swizzle:
// start address >> 4 (bits 0-13), leading byte offset 16 >> 4 (unused for
// this layout), stride byte offset 1024 >> 4 (8 rows of 128 bytes apart),
// the fixed 0b001 at bits 46-48, base offset 0 (tiles are 1024-aligned),
// swizzle mode 2 (128-byte) at bits 61-63.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(16 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
           (1ull << 46) | (2ull << 61);
}

// Instruction descriptor of kind::f16: D F32 (bits 4-5 = 1), A and B F16
// (bits 7-9, 10-12 = 0), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
template <int BN>
__host__ __device__ constexpr uint32_t idesc_f16() {
    return (1u << 4) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrives on `bar` once every tcgen05.mma issued so far by this thread has completed.
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 32 consecutive FP32 columns of this warp's 32 TMEM lanes (one row per thread).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// The epilogue's way of writing S: first contribution of a whole tile, a
// later group's contribution (read, add, write: the same thread wrote the
// element before), or a split unit's part (atomic add into a zeroed S).
enum EpiMode { kStore = 0, kAdd = 1, kAtomic = 2 };

template <typename V>
__device__ __forceinline__ void store16(V *dst, uint4 w, int mode) {
    if (mode == kStore) {
        *(uint4 *)dst = w;
    } else if (mode == kAdd) {
        const uint4 o = *(const uint4 *)dst;
        V *wv = (V *)&w;
        const V *ov = (const V *)&o;
#pragma unroll
        for (int e = 0; e < 16 / (int)sizeof(V); e++) wv[e] += ov[e];
        *(uint4 *)dst = w;
    } else {
        const V *wv = (const V *)&w;
#pragma unroll
        for (int e = 0; e < 16 / (int)sizeof(V); e++) {
            if constexpr (sizeof(V) == 8) atomicAdd((unsigned long long *)dst + e, (unsigned long long)wv[e]);
            else atomicAdd((unsigned int *)dst + e, (unsigned int)wv[e]);
        }
    }
}

// One CTA computes (part of) a (MSUB x 128) x BN tile of S: MSUB A tiles of
// 128 rows share each B tile, accumulator (j, msub) at TMEM columns
// (j MSUB + msub) BN (lb MSUB BN <= 512).  Larger tiles need fewer bytes from
// L2 per MMA: a 256 x 256 tile moves 64 KB per 64-wide K block for 8.4 MFLOP.
// The K loop runs over iterations it = group * kblocks + kb, group (i, q) =
// (A limb, chunk of the heavy indices); a unit covers iterations [ib, ie).
template <typename V, int BN, int MSUB>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_tc_seed(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, TcParams p) {
    constexpr uint32_t kBTile = (uint32_t)BN * kBK * 2;
    constexpr uint32_t kIdesc = idesc_f16<BN>();
    constexpr int kChunks = MSUB * (BN / 32);      // 32-column TMEM chunks per accumulator set
    extern __shared__ __align__(1024) unsigned char dyn[];
    __shared__ __align__(8) uint64_t full_bar[kMaxStages], empty_bar[kMaxStages];
    __shared__ __align__(8) uint64_t acc_full, acc_empty, drain_bar;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int abort_flag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // stage ring, 1024-byte aligned (the swizzle atoms need it)
    unsigned char *ring = (unsigned char *)(((uintptr_t)dyn + 1023) & ~(uintptr_t)1023);
    const uint32_t stage_bytes = kTileBytes * MSUB + kBTile * p.lb;
    const int kblocks = p.kc / kBK;
    const int iters = p.la * p.nq * kblocks;
    // this CTA's unit: a whole tile, or one of `splits` parts of a tail tile
    int tile, ib, ie;
    bool split;
    if ((int)blockIdx.x < p.full_tiles) {
        tile = (int)blockIdx.x;
        ib = 0;
        ie = iters;
        split = false;
    } else {
        const int v = (int)blockIdx.x - p.full_tiles, sp = v % p.splits;
        tile = p.full_tiles + v / p.splits;
        ib = (int)((int64_t)iters * sp / p.splits);
        ie = (int)((int64_t)iters * (sp + 1) / p.splits);
        split = true;
    }
    // the n tiles of one row block are consecutive: they run together and
    // share the A tiles through L2
    const int n0 = (tile % p.n_tiles) * BN;
    const int m0 = (tile / p.n_tiles) * (kBM * MSUB);

    if (threadIdx.x == 0) {
        for (int s = 0; s < p.stages; s++) {
            mbar_init(&full_bar[s], 1);
            mbar_init(&empty_bar[s], 1);
        }
        mbar_init(&acc_full, 1);
        mbar_init(&acc_empty, 128);
        mbar_init(&drain_bar, 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"((uint32_t)kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;

    if (warp == 0) {
        if (lane == 0) {
            // producer: MSUB A tiles and lb B tiles per K block
            int it = ib;
            for (; it < ie; it++) {
                const uint32_t l = (uint32_t)(it - ib);
                const int s = (int)(l % (uint32_t)p.stages);
                if (!mbar_wait(&empty_bar[s], ((l / (uint32_t)p.stages) & 1u) ^ 1u, &abort_flag, p.err, 1)) break;
                const int g = it / kblocks, kb = it % kblocks;
                const int i = g / p.nq, q = g % p.nq;
                unsigned char *st = ring + (size_t)s * stage_bytes;
                mbar_expect_tx(&full_bar[s], stage_bytes);
                const int32_t kx = q * p.kc + kb * kBK;
#pragma unroll
                for (int ms = 0; ms < MSUB; ms++)
                    tma_load_2d(st + kTileBytes * ms, &map_a, &full_bar[s], kx, i * p.M + m0 + kBM * ms);
                for (int j = 0; j < p.lb; j++)
                    tma_load_2d(st + kTileBytes * MSUB + kBTile * j, &map_b, &full_bar[s], kx, j * p.ldn + n0);
            }
            // every copy issued has landed before the CTA may exit (after a
            // normal run these phases completed long ago)
            const uint32_t issued = (uint32_t)(it - ib);
            const uint32_t first = issued >= (uint32_t)p.stages ? issued - (uint32_t)p.stages : 0u;
            for (uint32_t l = first; l < issued; l++) {
                volatile int never = 0;
                mbar_wait(&full_bar[l % (uint32_t)p.stages], (l / (uint32_t)p.stages) & 1u, &never, p.err, 1);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer: a group's first iteration in the unit starts its
            // accumulators, its last hands them to the epilogue
            bool issued = false;
            int lg = -1;
            for (int it = ib; it < ie; it++) {
                const uint32_t l = (uint32_t)(it - ib);
                const int kb = it % kblocks;
                const bool first = it == ib || kb == 0;
                if (first) {
                    lg++;
                    if (lg > 0) {
                        if (!mbar_wait(&acc_empty, (uint32_t)(lg - 1) & 1u, &abort_flag, p.err, 2)) break;
                        tc_fence_after();
                    }
                }
                const int s = (int)(l % (uint32_t)p.stages);
                if (!mbar_wait(&full_bar[s], (l / (uint32_t)p.stages) & 1u, &abort_flag, p.err, 3)) break;
                tc_fence_after();
                const uint32_t sa = smem_u32(ring + (size_t)s * stage_bytes);
                for (int j = 0; j < p.lb; j++) {
                    const uint32_t sb = sa + kTileBytes * MSUB + kBTile * j;
#pragma unroll
                    for (int ms = 0; ms < MSUB; ms++)
#pragma unroll
                        for (int k = 0; k < kBK / 16; k++)
                            mma_f16(tmem + (uint32_t)((j * MSUB + ms) * BN), sw128_desc(sa + kTileBytes * ms + 32 * k),
                                    sw128_desc(sb + 32 * k), kIdesc, (!first || k > 0) ? 1u : 0u);
                }
                issued = true;
                mma_commit(&empty_bar[s]);
                if (it == ie - 1 || kb == kblocks - 1) mma_commit(&acc_full);
            }
            if (issued) {
                // every MMA issued has completed before the TMEM is freed
                mma_commit(&drain_bar);
                volatile int never = 0;
                mbar_wait(&drain_bar, 0u, &never, p.err, 2);
            }
        }
    } else {
        // epilogue: thread t of warps 2-5 reads TMEM lane 32 (warp mod 4) + t,
        // row 32 (warp mod 4) + t of each 128-row sub-tile; a warp stages its
        // 32 rows' 128-byte segments in shared memory and writes them as
        // 16-byte pieces, eight lanes per row segment
        const int sub = warp & 3;
        const uint32_t tl = tmem + ((uint32_t)(sub * 32) << 16);
        unsigned char *wb = ring + (size_t)p.stages * stage_bytes + (size_t)(warp - 2) * 32 * kSegPitchBytes;
        const int rq = lane >> 3, q = lane & 7;   // read side: row within a group of 4, 16-byte piece
        const int g_first = ib / kblocks, g_last = (ie - 1) / kblocks;
        for (int g = g_first; g <= g_last && ie > ib; g++) {
            const int lg = g - g_first;
            if (!mbar_wait(&acc_full, (uint32_t)lg & 1u, &abort_flag, p.err, 4)) break;
            tc_fence_after();
            const int i = g / p.nq;
            const int mode = split ? kAtomic : (lg == 0 ? kStore : kAdd);
#pragma unroll 1
            for (int cc = 0; cc < kChunks; cc++) {
                const int ms = cc / (BN / 32), c = cc % (BN / 32);
                V acc[32];
#pragma unroll
                for (int t = 0; t < 32; t++) acc[t] = 0;
                for (int j = 0; j < p.lb; j++) {
                    const int sh = p.bits * (i + j);
                    float f[32];
                    tmem_ld32(tl + (uint32_t)((j * MSUB + ms) * BN + c * 32), f);
                    if (sh < 8 * (int)sizeof(V)) {
#pragma unroll
                        for (int t = 0; t < 32; t++) acc[t] += (V)__float2uint_rn(f[t]) << sh;
                    }
                }
                const int rbase = m0 + kBM * ms + sub * 32;   // the warp's first row
                const int col0 = n0 + c * 32;
#pragma unroll
                for (int hh = 0; hh < (int)sizeof(V) / 4; hh++) {   // 128-byte rounds: uint32 one, uint64 two
                    const V *seg = acc + hh * (128 / (int)sizeof(V));
                    __syncwarp();
#pragma unroll
                    for (int t = 0; t < 8; t++)
                        *(uint4 *)(wb + lane * kSegPitchBytes + 16 * t) = *(const uint4 *)(seg + t * (16 / (int)sizeof(V)));
                    __syncwarp();
                    const int col = col0 + hh * (128 / (int)sizeof(V)) + q * (16 / (int)sizeof(V));
#pragma unroll
                    for (int t = 0; t < 8; t++) {
                        const int rr = 4 * t + rq;
                        const int r = rbase + rr;
                        const uint4 w = *(const uint4 *)(wb + rr * kSegPitchBytes + 16 * q);
                        // ldn and col are multiples of the piece: a piece is in or out whole
                        if (r < p.M && col < p.ldn) store16<V>((V *)p.S + (int64_t)r * p.ldn + col, w, mode);
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(&acc_empty);
        }
    }
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)kTmemCols)
                     : "memory");
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        else
            cudaGetLastError();
    }
    return fn;
}

// 2-D FP16 tensor map over rows x k (k contiguous, row stride ldk elements),
// boxes of 64 x box_rows with the 128-byte swizzle.
bool make_map(CUtensorMap *m, const void *base, int64_t ldk, int64_t rows, int box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn || ((uintptr_t)base & 15) || (ldk * 2) % 16 || ldk % kBK) return false;
    cuuint64_t dims[2] = {(cuuint64_t)ldk, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(ldk * 2)};
    cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void *>(base), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Fewest K blocks a split unit takes (the ring's fill and the epilogue
// would dominate shorter ones).
constexpr int kMinSplitIters = 8;

template <typename V, int BN, int MSUB>
int32_t launch_tc(rmcm_handle *h, const CUtensorMap &ma, const CUtensorMap &mb, TcParams p, int64_t M, int64_t N) {
    const int64_t stage_bytes = (int64_t)kTileBytes * MSUB + (int64_t)BN * kBK * 2 * p.lb;
    // the ring fills ~200 KB: one CTA per SM, so the 512-column TMEM
    // allocation never waits for another CTA's
    p.stages = (int32_t)std::min<int64_t>(kMaxStages, (200 * 1024) / stage_bytes);
    if (p.stages < 2) return RMCM_EINVAL;
    const int smem = (int)(p.stages * stage_bytes + 1024 + kEpiBytes);
    const int64_t bm = (int64_t)kBM * MSUB;
    const int64_t m_tiles = (M + bm - 1) / bm, n_tiles = (N + BN - 1) / BN, tiles = m_tiles * n_tiles;
    const int64_t iters = (int64_t)p.la * p.nq * (p.kc / kBK);
    if (tiles > INT32_MAX / 64 || iters > INT32_MAX) return RMCM_EINVAL;
    // the last, partial wave of tiles is split over the K blocks so that it
    // occupies every SM
    const int64_t sms = std::max(1, h->sm_count);
    const int64_t tail = tiles < sms ? tiles : tiles % sms;
    int64_t splits = tail ? std::min<int64_t>(sms / tail, iters / kMinSplitIters) : 1;
    if (splits < 2) splits = 1;
    const int64_t full = splits > 1 ? tiles - tail : tiles;
    p.n_tiles = (int32_t)n_tiles;
    p.full_tiles = (int32_t)full;
    p.splits = (int32_t)splits;
    cudaStream_t s = h->stream;
    if (splits > 1) {
        // split units add into S: zero the rows of the tiles they cover
        const int64_t r0 = std::min<int64_t>(M, (full / n_tiles) * bm);
        RMCM_CUDA(h, cudaMemsetAsync((char *)p.S + r0 * (int64_t)p.ldn * (int64_t)sizeof(V), 0,
                                     (M - r0) * (int64_t)p.ldn * (int64_t)sizeof(V), s));
    }
    const int64_t grid = full + (tiles - full) * splits;
    if (cudaFuncSetAttribute(k_tc_seed<V, BN, MSUB>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
        cudaSuccess)
        return set_error(h, RMCM_ECUDA, "tc_seed_gemm: shared memory opt-in");
    k_tc_seed<V, BN, MSUB><<<(unsigned)grid, kTcThreads, smem, s>>>(ma, mb, p);
    h->launches++;
    RMCM_CUDA(h, cudaGetLastError());
    return RMCM_OK;
}

}  // namespace

// S (M x ldn of V) = the exact dense part from the FP16 limb panels:
// Ad (la panels of M x ldk) and BdT (lb panels of ldn x ldk), ldk = kc nq.
// Tile shape by B's limbs (the accumulators fill the 512 TMEM columns):
// one limb 256 x 256, two 128 x 256, three or four 128 x 128.
// Returns RMCM_EINVAL when the shape is outside what the kernel takes (the
// caller then keeps the product sparse), RMCM_ECUDA on a launch error.
int32_t tc_seed_gemm(rmcm_handle *h, const void *Ad, const void *BdT, int64_t M, int64_t N, int64_t ldn,
                     int32_t la, int32_t lb, int64_t kc, int64_t nq, int32_t bits, int32_t vbytes, void *S,
                     int *err_dev) {
    if (M <= 0 || N <= 0 || ldn < N || lb < 1 || lb > 4 || la < 1 || nq < 1 || kc < kBK || kc % kBK ||
        (vbytes != 4 && vbytes != 8) || M * la > INT32_MAX || ldn * lb > INT32_MAX || kc * nq > INT32_MAX)
        return RMCM_EINVAL;
    const int64_t ldk = kc * nq;
    const int bn = lb <= 2 ? 256 : 128;
    CUtensorMap ma, mb;
    if (!make_map(&ma, Ad, ldk, M * la, kBM) || !make_map(&mb, BdT, ldk, ldn * lb, bn)) return RMCM_EINVAL;
    TcParams p;
    p.M = (int32_t)M;
    p.N = (int32_t)N;
    p.ldn = (int32_t)ldn;
    p.la = la;
    p.lb = lb;
    p.nq = (int32_t)nq;
    p.kc = (int32_t)kc;
    p.bits = bits;
    p.stages = 0;
    p.n_tiles = p.full_tiles = p.splits = 0;
    p.S = S;
    p.err = err_dev;
    if (vbytes == 4) {
        if (lb == 1) return launch_tc<uint32_t, 256, 2>(h, ma, mb, p, M, N);
        if (lb == 2) return launch_tc<uint32_t, 256, 1>(h, ma, mb, p, M, N);
        return launch_tc<uint32_t, 128, 1>(h, ma, mb, p, M, N);
    }
    if (lb == 1) return launch_tc<uint64_t, 256, 2>(h, ma, mb, p, M, N);
    if (lb == 2) return launch_tc<uint64_t, 256, 1>(h, ma, mb, p, M, N);
    return launch_tc<uint64_t, 128, 1>(h, ma, mb, p, M, N);
}

}  // namespace rmcm
