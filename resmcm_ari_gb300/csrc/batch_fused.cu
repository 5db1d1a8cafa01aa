// Many meta-path chains in fused launches ("waves"), recorded once and
// replayed as one CUDA graph.
//
// The per-path loop of efficient/resmcm.cpp (main :834-889, SSP_dynamic
// :653-772 for every path) becomes three fused stages over the whole batch:
//
// * estimator: one launch per level step over all chains (estimate_multi:
//   step s runs level len - 1 - s of every chain, each chain's CTAs exactly
//   those of its own one-chain launch, so its estimates are bit-identical);
// * DP + order: one launch, a warp per chain (chain_order_multi);
// * products: wave w computes the w-th product (post-order pair) of every
//   chain that has one, as ONE SpGEMM of block-diagonal operands: the left
//   operands' rows are stacked with their columns shifted to the stacked
//   rows of the right operands (A_all = diag(A_c), B_all = diag(B_c), columns
//   of B_all kept local: every row of A_all only reaches its own chain's
//   rows of B_all).  Chain c's result is the row range of C_all its A_c
//   rows produced; the next wave reads it in place through a row view.
//   Operands are gathered into A_all / B_all by one k_concat launch each.
//
// A batch of 512 chains of up to 10 matrices is then some 10 estimator
// steps, one DP and 9 waves of one SpGEMM each, instead of a SpGEMM per
// product per chain.  The record pass runs this with the usual read-backs
// (the orders, every wave's bin counts and sizes, the row ranges' sizes)
// and logs them; the capture pass issues the same work with the recorded
// sizes and no host round trip, into one CUDA graph.  AUTO value types: a
// wave whose counts overflow uint32 widens the whole batch to uint64 (live
// intermediates converted, leaves swapped) and runs again, in the record and
// in the replay alike.  Results are compared by (nnz, order-free digest).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

namespace rmcm {
namespace {

// One operand's rows copied into a stacked operand: rows [0, rows) of the
// view whose row pointers start at rowptr (entries at their absolute
// positions e0 .. e0 + nnz), to rows dst_row0.. and entries dst_e0.., with
// col_add added to every column.
struct CatSeg {
    const int64_t *rowptr;
    const int32_t *col;
    const void *val;     // null: every value 1
    int64_t rows, e0, nnz, dst_row0, dst_e0;
    int32_t col_add;
    int32_t pad;
};

__device__ __forceinline__ int last_seg(const CatSeg *segs, int nseg, int64_t x, bool by_entry) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((by_entry ? segs[mid].dst_e0 : segs[mid].dst_row0) <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <typename V>
__global__ void __launch_bounds__(256) k_concat(const CatSeg *segs, int32_t nseg, int64_t rows, int64_t nnz,
                                                int64_t *rowptr, int32_t *col, V *val) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int64_t r = t0; r < rows; r += stride) {
        const CatSeg &sg = segs[last_seg(segs, nseg, r, false)];
        rowptr[r] = sg.rowptr[r - sg.dst_row0] - sg.e0 + sg.dst_e0;
    }
    if (t0 == 0) rowptr[rows] = nnz;
    for (int64_t x = t0; x < nnz; x += stride) {
        const CatSeg &sg = segs[last_seg(segs, nseg, x, true)];
        const int64_t k = sg.e0 + (x - sg.dst_e0);
        col[x] = sg.col[k] + sg.col_add;
        val[x] = sg.val ? ((const V *)sg.val)[k] : (V)1;
    }
}

// A chain's operand: rows [row0, row0 + rows) of a matrix (a leaf, or the
// stacked result of an earlier wave: `owner` >= 0), entries e0 .. e0 + nnz.
struct Opnd {
    int owner = -1;
    const rmcm_mat *m = nullptr;   // the leaf (owner < 0)
    int64_t row0 = 0, rows = 0, e0 = 0, nnz = 0;
};

struct FusedWave {
    ProductPlan plan;
    bool widen_before = false;      // the batch widened to uint64 before this wave
    std::vector<int64_t> seg_e0;    // per participating chain: first entry of its rows in C_all
    std::vector<int64_t> seg_nnz;   // and their entries
};

}  // namespace

struct FusedBatch {
    rmcm_handle *h = nullptr;
    rmcm_graph *g = nullptr;
    std::vector<std::string> paths;
    std::vector<std::vector<int32_t>> vts, ets;
    std::vector<int32_t> lens;
    std::vector<std::vector<int32_t>> pairs;   // recorded orders
    std::vector<FusedWave> waves;
    std::vector<int64_t> nnz;                  // recorded result sizes
    int32_t start_vt = RMCM_VAL_U32;
    bool widen = false;
    int64_t scratch_need = 256;
    TableArena arena;
    char *persist = nullptr;                   // c_all | lens | split_all | cost_all | pairs_all | digests
    int64_t persist_bytes = 0;
    double *c_all = nullptr;
    int32_t *lens_dev = nullptr, *split_all = nullptr, *pairs_all = nullptr;
    double *cost_all = nullptr;
    uint64_t *d_digest = nullptr, *h_digest = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t launches_per_run = 0, nodes = 0;
};

namespace {

constexpr int kMaxLen = 16;
constexpr int64_t kEstGroupBytes = 4LL << 30;   // level buffers of one estimator launch group

void set_flags_from(rmcm_mat *dst, const std::vector<const rmcm_mat *> &srcs) {
    bool ones = true, positive = true, distinct = true;
    int64_t max_row = 0;
    for (const rmcm_mat *m : srcs) {
        ones = ones && m->ones;
        positive = positive && m->positive;
        distinct = distinct && m->distinct;
        if (max_row >= 0) max_row = m->max_row < 0 ? -1 : std::max(max_row, m->max_row);
    }
    dst->ones = ones;
    dst->positive = positive;
    dst->distinct = distinct;
    dst->max_row = max_row;
}

// Gathers the segments into a stacked operand allocated here.
int32_t concat(rmcm_handle *h, FusedBatch *b, const std::vector<CatSeg> &segs, int64_t rows, int64_t cols,
               int64_t nnz, int32_t vt, rmcm_mat **out) {
    RMCM_TRY(mat_alloc(h, rows, cols, nnz, vt, out));
    void *hp = nullptr, *dp = nullptr;
    const int64_t bytes = (int64_t)sizeof(CatSeg) * (int64_t)segs.size();
    if (!b->arena.push(bytes, &hp, &dp)) {
        mat_release(h, *out);
        *out = nullptr;
        return set_error(h, RMCM_EINTERNAL, "batch: table arena full");
    }
    memcpy(hp, segs.data(), bytes);
    cudaStream_t s = h->stream;
    RMCM_CUDA(h, cudaMemcpyAsync(dp, hp, bytes, cudaMemcpyHostToDevice, s));
    const int64_t work = std::max<int64_t>(std::max(rows, nnz), 1);
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((work + 255) / 256, (int64_t)h->sm_count * 16));
    if (vt == RMCM_VAL_U64)
        k_concat<uint64_t><<<grid, 256, 0, s>>>((const CatSeg *)dp, (int32_t)segs.size(), rows, nnz, (*out)->d.rowptr,
                                               (*out)->d.col, (uint64_t *)(*out)->d.val);
    else
        k_concat<uint32_t><<<grid, 256, 0, s>>>((const CatSeg *)dp, (int32_t)segs.size(), rows, nnz, (*out)->d.rowptr,
                                               (*out)->d.col, (uint32_t *)(*out)->d.val);
    h->launches++;
    RMCM_CUDA(h, cudaGetLastError());
    return RMCM_OK;
}

CatSeg seg_of(const Opnd &o, const std::vector<rmcm_mat *> &owners, int64_t dst_row0, int64_t dst_e0,
              int32_t col_add) {
    const rmcm_mat *m = o.owner >= 0 ? owners[o.owner] : o.m;
    CatSeg sg{};
    sg.rowptr = m->d.rowptr + o.row0;
    sg.col = m->d.col;
    sg.val = m->d.val;
    sg.rows = o.rows;
    sg.e0 = o.e0;
    sg.nnz = o.nnz;
    sg.dst_row0 = dst_row0;
    sg.dst_e0 = dst_e0;
    sg.col_add = col_add;
    return sg;
}

// Record (record = true: read-backs, logs into b) or replay (the logged
// sizes, no host round trip) of the whole batch on h's stream.
int32_t fused_exec(FusedBatch *b, bool record) {
    rmcm_handle *h = b->h;
    cudaStream_t s = h->stream;
    const int32_t n = (int32_t)b->paths.size();
    int32_t cur = b->start_vt;
    b->arena.used = 0;
    // leaves of every chain in the current value type
    std::vector<std::vector<rmcm_mat *>> mats(n);
    auto load_leaves = [&]() -> int32_t {
        for (int32_t c = 0; c < n; c++) {
            mats[c].assign(b->lens[c], nullptr);
            for (int i = 0; i < b->lens[c]; i++)
                RMCM_TRY(leaf_of(h, b->g, b->vts[c][i], b->vts[c][i + 1], b->ets[c][i], cur, &mats[c][i]));
        }
        return RMCM_OK;
    };
    RMCM_TRY(load_leaves());
    // (a) estimates, in launch groups bounded by their level buffers
    {
        std::vector<EstChain> group;
        int64_t gbytes = 0;
        auto flush = [&]() -> int32_t {
            if (group.empty()) return RMCM_OK;
            const int32_t rc = estimate_multi(h, group.data(), (int32_t)group.size(), b->arena);
            group.clear();
            gbytes = 0;
            return rc;
        };
        for (int32_t c = 0; c < n; c++) {
            if (b->lens[c] < 2) continue;
            int64_t rows = 1;
            for (auto *m : mats[c]) rows = std::max(rows, m->d.rows);
            const int64_t need = 16 * rows * b->lens[c];
            if (gbytes + need > kEstGroupBytes && !group.empty()) RMCM_TRY(flush());
            EstChain ec;
            ec.mats = mats[c].data();
            ec.len = b->lens[c];
            ec.c_dev = b->c_all + (int64_t)c * kMaxLen * kMaxLen;
            group.push_back(ec);
            gbytes += need;
        }
        RMCM_TRY(flush());
    }
    // (b) DP + order of every chain, one launch
    {
        void *hp = nullptr, *dp = nullptr;
        if (!b->arena.push(4 * (int64_t)n, &hp, &dp)) return set_error(h, RMCM_EINTERNAL, "batch: table arena full");
        memcpy(hp, b->lens.data(), 4 * (size_t)n);
        RMCM_CUDA(h, cudaMemcpyAsync(dp, hp, 4 * (size_t)n, cudaMemcpyHostToDevice, s));
        RMCM_TRY(chain_order_multi(h, b->c_all, (const int32_t *)dp, n, b->split_all, b->cost_all, b->pairs_all));
    }
    if (record) {
        std::vector<int32_t> hp(32 * (size_t)n);
        RMCM_CUDA(h, cudaMemcpyAsync(hp.data(), b->pairs_all, 4 * hp.size(), cudaMemcpyDeviceToHost, s));
        RMCM_CUDA(h, cudaStreamSynchronize(s));
        b->pairs.assign(n, {});
        for (int32_t c = 0; c < n; c++)
            b->pairs[c].assign(hp.begin() + 32 * (size_t)c, hp.begin() + 32 * (size_t)c + 2 * std::max(0, b->lens[c] - 1));
        b->waves.clear();
    }
    // (c) waves
    std::vector<rmcm_mat *> owners;
    std::vector<int> refs;
    std::vector<std::vector<Opnd>> stack(n);
    std::vector<int32_t> next(n, 0);
    auto unref = [&](const Opnd &o) {
        if (o.owner >= 0 && --refs[o.owner] == 0) {
            mat_release(h, owners[o.owner]);
            owners[o.owner] = nullptr;
        }
    };
    auto widen_all = [&]() -> int32_t {
        cur = RMCM_VAL_U64;
        for (size_t o = 0; o < owners.size(); o++) {
            if (!owners[o]) continue;
            rmcm_mat *w = nullptr;
            RMCM_TRY(convert_values(h, owners[o], RMCM_VAL_U64, &w));
            mat_release(h, owners[o]);
            owners[o] = w;
        }
        return load_leaves();
    };
    int32_t rc = RMCM_OK;
    for (int w = 0; rc == RMCM_OK; w++) {
        std::vector<int32_t> part;
        for (int32_t c = 0; c < n; c++)
            if (next[c] < b->lens[c] - 1) part.push_back(c);
        if (part.empty()) break;
        if (!record) {
            if (w >= (int)b->waves.size()) return set_error(h, RMCM_EINTERNAL, "batch replay: more waves than recorded");
            if (b->waves[w].widen_before) RMCM_TRY(widen_all());
        }
        bool retry = true;
        while (retry && rc == RMCM_OK) {
            retry = false;
            // operands of this wave
            std::vector<Opnd> A(part.size()), B(part.size());
            for (size_t q = 0; q < part.size(); q++) {
                const int32_t c = part[q];
                const int32_t k = b->pairs[c][2 * next[c]], l = b->pairs[c][2 * next[c] + 1];
                auto leaf_op = [&](int i) {
                    Opnd o;
                    o.m = mats[c][i];
                    o.rows = o.m->d.rows;
                    o.nnz = o.m->d.nnz;
                    return o;
                };
                const size_t sz = stack[c].size();
                if (k >= 0 && l >= 0) {
                    A[q] = leaf_op(k);
                    B[q] = leaf_op(l);
                } else if (k < 0 && l >= 0) {
                    A[q] = stack[c][sz - 1];
                    B[q] = leaf_op(l);
                } else if (k >= 0 && l < 0) {
                    A[q] = leaf_op(k);
                    B[q] = stack[c][sz - 1];
                } else {
                    A[q] = stack[c][sz - 2];
                    B[q] = stack[c][sz - 1];
                }
            }
            // stacked operands: B's rows one after another (columns local),
            // A's columns shifted onto its chain's rows of B_all
            std::vector<CatSeg> sa, sb;
            std::vector<const rmcm_mat *> fa, fb;
            int64_t arows = 0, annz = 0, brows = 0, bnnz = 0, bcols = 1;
            std::vector<int64_t> a_row0(part.size());
            for (size_t q = 0; q < part.size(); q++) {
                sb.push_back(seg_of(B[q], owners, brows, bnnz, 0));
                fb.push_back(B[q].owner >= 0 ? owners[B[q].owner] : B[q].m);
                const rmcm_mat *bm = fb.back();
                bcols = std::max(bcols, bm->d.cols);
                a_row0[q] = arows;
                sa.push_back(seg_of(A[q], owners, arows, annz, (int32_t)brows));
                fa.push_back(A[q].owner >= 0 ? owners[A[q].owner] : A[q].m);
                arows += A[q].rows;
                annz += A[q].nnz;
                brows += B[q].rows;
                bnnz += B[q].nnz;
            }
            if (brows > INT32_MAX) return set_error(h, RMCM_EINVAL, "batch: stacked operands exceed 2^31 rows");
            rmcm_mat *Aall = nullptr, *Ball = nullptr, *Call = nullptr;
            RMCM_TRY(concat(h, b, sa, arows, brows, annz, cur, &Aall));
            rc = concat(h, b, sb, brows, bcols, bnnz, cur, &Ball);
            if (rc != RMCM_OK) {
                mat_release(h, Aall);
                return rc;
            }
            set_flags_from(Aall, fa);
            set_flags_from(Ball, fb);
            ProductPlan plan;
            if (record) {
                plan.mode = 1;
            } else {
                plan = b->waves[w].plan;
                plan.mode = 2;
            }
            int64_t fl = 0;
            h->abort_on_certain_overflow = record && b->widen && cur == RMCM_VAL_U32;
            rc = spgemm(h, Aall, Ball, &Call, &fl, &plan);
            h->abort_on_certain_overflow = false;
            mat_release(h, Aall);
            mat_release(h, Ball);
            if (record && rc == RMCM_EOVERFLOW && b->widen && cur == RMCM_VAL_U32 && !Call) {
                rc = widen_all();
                retry = true;
                if (b->waves.size() <= (size_t)w) b->waves.resize(w + 1);
                b->waves[w].widen_before = true;
                continue;
            }
            if (rc != RMCM_OK) {
                if (Call) mat_release(h, Call);
                return rc;
            }
            if (record) {
                const int32_t st = check_status(h);
                if (st == RMCM_EOVERFLOW && b->widen && cur == RMCM_VAL_U32) {
                    mat_release(h, Call);
                    rc = widen_all();
                    retry = true;
                    if (b->waves.size() <= (size_t)w) b->waves.resize(w + 1);
                    b->waves[w].widen_before = true;
                    continue;
                }
                if (st != RMCM_OK) {
                    mat_release(h, Call);
                    return st;
                }
                // sizes of every chain's row range of C_all
                std::vector<int64_t> at(part.size() + 1);
                for (size_t q = 0; q < part.size(); q++) at[q] = a_row0[q];
                at[part.size()] = arows;
                std::vector<int64_t> e(part.size() + 1);
                for (size_t q = 0; q <= part.size(); q++) {
                    RMCM_CUDA(h, cudaMemcpyAsync(h->h_pinned + (q % 16), Call->d.rowptr + at[q], 8, cudaMemcpyDeviceToHost, s));
                    if (q % 16 == 15 || q == part.size()) {
                        RMCM_CUDA(h, cudaStreamSynchronize(s));
                        for (size_t r = q - (q % 16); r <= q; r++) e[r] = h->h_pinned[r % 16];
                    }
                }
                if (b->waves.size() <= (size_t)w) b->waves.resize(w + 1);
                FusedWave &fw = b->waves[w];
                fw.plan = plan;
                fw.seg_e0.assign(part.size(), 0);
                fw.seg_nnz.assign(part.size(), 0);
                for (size_t q = 0; q < part.size(); q++) {
                    fw.seg_e0[q] = e[q];
                    fw.seg_nnz[q] = e[q + 1] - e[q];
                }
                b->scratch_need = std::max(b->scratch_need, plan.scratch_bytes);
            }
            const FusedWave &fw = b->waves[w];
            const int oid = (int)owners.size();
            owners.push_back(Call);
            refs.push_back((int)part.size());
            for (size_t q = 0; q < part.size(); q++) {
                const int32_t c = part[q];
                Opnd r;
                r.owner = oid;
                r.row0 = a_row0[q];
                r.rows = A[q].rows;
                r.e0 = fw.seg_e0[q];
                r.nnz = fw.seg_nnz[q];
                const int32_t k = b->pairs[c][2 * next[c]], l = b->pairs[c][2 * next[c] + 1];
                auto &stk = stack[c];
                if (k >= 0 && l >= 0) {
                    stk.push_back(r);
                } else if (k >= 0 || l >= 0) {
                    unref(stk.back());
                    stk.back() = r;
                } else {
                    unref(stk[stk.size() - 1]);
                    unref(stk[stk.size() - 2]);
                    stk.pop_back();
                    stk.back() = r;
                }
                next[c]++;
            }
        }
    }
    // digests of every result (a leaf for one-matrix chains), one launch
    std::vector<DigestJob> jobs(n);
    for (int32_t c = 0; c < n && rc == RMCM_OK; c++) {
        DigestJob &jb = jobs[c];
        jb.out = c;
        if (b->lens[c] < 2) {
            const rmcm_mat *m = mats[c][0];
            jb.rowptr = m->d.rowptr;
            jb.col = m->d.col;
            jb.val = m->d.val;
            jb.rows = m->d.rows;
            jb.vbytes = (int32_t)val_bytes(m->valtype);
        } else {
            const Opnd &r = stack[c].back();
            const rmcm_mat *m = owners[r.owner];
            jb.rowptr = m->d.rowptr + r.row0;
            jb.col = m->d.col;
            jb.val = m->d.val;
            jb.rows = r.rows;
            jb.vbytes = (int32_t)val_bytes(m->valtype);
        }
        if (record) b->nnz[c] = b->lens[c] < 2 ? mats[c][0]->d.nnz : stack[c].back().nnz;
    }
    if (rc == RMCM_OK) {
        void *hp = nullptr, *dp = nullptr;
        const int64_t bytes = (int64_t)sizeof(DigestJob) * n;
        if (!b->arena.push(bytes, &hp, &dp)) rc = set_error(h, RMCM_EINTERNAL, "batch: table arena full");
        if (rc == RMCM_OK) {
            memcpy(hp, jobs.data(), bytes);
            cudaError_t e = cudaMemsetAsync(b->d_digest, 0, 16 * (size_t)n, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(dp, hp, bytes, cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) rc = cuda_error(h, e, "batch digests");
        }
        if (rc == RMCM_OK) rc = digest_multi_launch(h, (const DigestJob *)dp, n, b->d_digest);
    }
    for (auto *m : owners)
        if (m) mat_release(h, m);
    return rc;
}

}  // namespace

int32_t fused_create(rmcm_handle *h, rmcm_graph *g, const char *const *paths, int32_t count, FusedBatch **out) {
    *out = nullptr;
    FusedBatch *b = new FusedBatch();
    b->h = h;
    b->g = g;
    b->start_vt = h->valtype == RMCM_VAL_U64 ? RMCM_VAL_U64 : RMCM_VAL_U32;
    b->widen = h->valtype == RMCM_VAL_AUTO;
    int32_t rc = RMCM_OK;
    for (int32_t i = 0; i < count && rc == RMCM_OK; i++) {
        std::vector<int32_t> vts, ets;
        if (!paths[i] || path_parse(paths[i], vts, ets) != RMCM_OK) {
            rc = set_error(h, RMCM_EINVAL, std::string("the meta-path is incorrect: ") + (paths[i] ? paths[i] : "(null)"));
            break;
        }
        if (ets.empty() || ets.size() > (size_t)kMaxLen) {
            rc = set_error(h, RMCM_EINVAL, "meta-path must have 1..16 edge types");
            break;
        }
        b->paths.emplace_back(paths[i]);
        b->lens.push_back((int32_t)ets.size());
        b->vts.push_back(vts);
        b->ets.push_back(ets);
    }
    const int32_t n = (int32_t)b->paths.size();
    b->nnz.assign(n, 0);
    // persistent buffers, outside any capture
    if (rc == RMCM_OK) {
        auto al = [](int64_t x) { return (x + 255) & ~255LL; };
        const int64_t c_b = al(8LL * kMaxLen * kMaxLen * n), l_b = al(4LL * n), s_b = al(4LL * kMaxLen * kMaxLen * n),
                      p_b = al(4LL * 32 * n), d_b = al(16LL * n);
        b->persist_bytes = 2 * c_b + l_b + s_b + p_b + d_b;
        rc = dev_alloc(h, (void **)&b->persist, b->persist_bytes);
        if (rc == RMCM_OK) {
            char *p = b->persist;
            b->c_all = (double *)p;
            b->cost_all = (double *)(p + c_b);
            b->lens_dev = (int32_t *)(p + 2 * c_b);
            b->split_all = (int32_t *)(p + 2 * c_b + l_b);
            b->pairs_all = (int32_t *)(p + 2 * c_b + l_b + s_b);
            b->d_digest = (uint64_t *)(p + 2 * c_b + l_b + s_b + p_b);
        }
    }
    if (rc == RMCM_OK) {
        b->arena.cap = 64LL << 20;
        if (cudaMallocHost((void **)&b->arena.host, (size_t)b->arena.cap) != cudaSuccess) {
            b->arena.host = nullptr;
            rc = set_error(h, RMCM_ECUDA, "batch: pinned table arena");
        } else {
            rc = dev_alloc(h, (void **)&b->arena.dev, b->arena.cap);
        }
        if (rc == RMCM_OK && cudaMallocHost((void **)&b->h_digest, 16 * (size_t)std::max(n, 1)) != cudaSuccess) {
            b->h_digest = nullptr;
            rc = set_error(h, RMCM_ECUDA, "batch: pinned digest buffer");
        }
    }
    // record pass
    const int32_t prof = h->prof_level;
    h->prof_level = 0;
    if (rc == RMCM_OK) rc = fused_exec(b, true);
    if (rc == RMCM_OK) {
        cudaError_t e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) rc = cuda_error(h, e, "batch record");
    }
    // capture pass: the same work from the record, no host round trip
    if (rc == RMCM_OK) rc = scratch_reserve(h, b->scratch_need);
    if (rc == RMCM_OK) {
        cudaError_t e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) rc = cuda_error(h, e, "batch scratch");
    }
    if (rc == RMCM_OK) {
        const int64_t l0 = h->launches;
        cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) rc = cuda_error(h, e, "batch capture begin");
        if (rc == RMCM_OK) {
            rc = fused_exec(b, false);
            if (rc == RMCM_OK) {
                e = cudaMemcpyAsync(b->h_digest, b->d_digest, 16 * (size_t)n, cudaMemcpyDeviceToHost, h->stream);
                if (e != cudaSuccess) rc = cuda_error(h, e, "batch digest copy");
            }
            cudaGraph_t graph = nullptr;
            e = cudaStreamEndCapture(h->stream, &graph);
            if (rc == RMCM_OK && e != cudaSuccess) rc = cuda_error(h, e, "cudaStreamEndCapture");
            if (rc != RMCM_OK) {
                if (graph) cudaGraphDestroy(graph);
                cudaGetLastError();
            } else {
                b->graph = graph;
                e = cudaGraphInstantiate(&b->exec, graph, 0);
                if (e != cudaSuccess) {
                    b->exec = nullptr;
                    rc = cuda_error(h, e, "cudaGraphInstantiate");
                } else {
                    size_t nodes = 0;
                    cudaGraphGetNodes(graph, nullptr, &nodes);
                    b->nodes = (int64_t)nodes;
                    b->launches_per_run = h->launches - l0;
                    h->launches = l0;
                }
            }
        }
    }
    h->prof_level = prof;
    if (rc != RMCM_OK) {
        const std::string why = h->last_error;
        fused_free(h, b);
        h->last_error = why;
        return rc;
    }
    *out = b;
    return RMCM_OK;
}

int32_t fused_run(rmcm_handle *h, FusedBatch *b, int64_t *nnz_out, uint64_t *digest_out, double *seconds) {
    if (!b->exec) return set_error(h, RMCM_EINVAL, "batch: not instantiated");
    cudaEvent_t *ev = h->ev;
    RMCM_CUDA(h, cudaEventRecord(ev[6], h->stream));
    RMCM_CUDA(h, cudaGraphLaunch(b->exec, h->stream));
    RMCM_CUDA(h, cudaEventRecord(ev[7], h->stream));
    RMCM_CUDA(h, cudaStreamSynchronize(h->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, ev[6], ev[7]);
    if (seconds) *seconds = ms * 1e-3;
    h->launches += b->launches_per_run;
    RMCM_TRY(check_status(h));
    for (size_t i = 0; i < b->paths.size(); i++) {
        if ((int64_t)b->h_digest[2 * i] != b->nnz[i])
            return set_error(h, RMCM_EINTERNAL, "batch run: result size of " + b->paths[i] + " differs from its record");
        if (nnz_out) nnz_out[i] = (int64_t)b->h_digest[2 * i];
        if (digest_out) digest_out[i] = b->h_digest[2 * i + 1];
    }
    return RMCM_OK;
}

void fused_info(const FusedBatch *b, int32_t *count, int64_t *launches_per_run, int64_t *nodes) {
    if (count) *count = (int32_t)b->paths.size();
    if (launches_per_run) *launches_per_run = b->launches_per_run;
    if (nodes) *nodes = b->nodes;
}

void fused_free(rmcm_handle *h, FusedBatch *b) {
    if (!b) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->persist) dev_free(h, b->persist, b->persist_bytes);
    if (b->arena.dev) dev_free(h, b->arena.dev, b->arena.cap);
    if (b->arena.host) cudaFreeHost(b->arena.host);
    if (b->h_digest) cudaFreeHost(b->h_digest);
    delete b;
}

}  // namespace rmcm
