// C ABI of the GB300 chain engine: handle, device memory, typed graph, leaf
// matrices, the three stages and the chain executor.
//
// The executor restates SSP_dynamic (efficient/resmcm.cpp:653-772): leaf
// matrices first (not timed, :664-667), then inside the timed region the
// estimator, the DP, the order and a stack machine over the (k, l) pairs
// (:709-760) that multiplies leaves and temporaries and frees every operand
// right after its last use.  Leaves stay resident in the graph's cache.
#include <cuda_runtime.h>
#include <omp.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "internal.h"

using namespace rmcm;

namespace rmcm {

int32_t set_error(rmcm_handle *h, int32_t status, const std::string &msg) {
    if (h) h->last_error = msg;
    return status;
}

int32_t cuda_error(rmcm_handle *h, cudaError_t e, const char *what) {
    std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return set_error(h, RMCM_ENOMEM, msg);
    return set_error(h, RMCM_ECUDA, msg);
}

int32_t dev_alloc(rmcm_handle *h, void **p, int64_t bytes) {
    *p = nullptr;
    if (bytes <= 0) bytes = 256;
    if (h->in_use + bytes > h->budget)
        return set_error(h, RMCM_ENOMEM,
                         "device memory budget exhausted: need " + std::to_string(bytes) + " bytes, " +
                             std::to_string(h->budget - h->in_use) + " left");
    cudaError_t e = cudaMallocAsync(p, (size_t)bytes, h->stream);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return cuda_error(h, e, "cudaMallocAsync");
    }
    h->in_use += bytes;
    if (h->in_use > h->peak) h->peak = h->in_use;
    return RMCM_OK;
}

void dev_free(rmcm_handle *h, void *p, int64_t bytes) {
    if (!p) return;
    if (bytes <= 0) bytes = 256;
    cudaFreeAsync(p, h->stream);
    h->in_use -= bytes;
}

int32_t scratch_reserve(rmcm_handle *h, int64_t bytes) {
    if (bytes <= h->scratch_bytes) return RMCM_OK;
    int64_t want = std::max<int64_t>(bytes, h->scratch_bytes + h->scratch_bytes / 2);
    if (h->scratch) {
        dev_free(h, h->scratch, h->scratch_bytes);
        h->scratch = nullptr;
        h->scratch_bytes = 0;
    }
    int32_t rc = dev_alloc(h, &h->scratch, want);
    if (rc != RMCM_OK) {
        rc = dev_alloc(h, &h->scratch, bytes);
        if (rc != RMCM_OK) return rc;
        want = bytes;
    }
    h->scratch_bytes = want;
    return RMCM_OK;
}

// Creates *out with its row pointer when *out is null; allocates col/val for
// nnz entries when nnz >= 0.
int32_t mat_alloc(rmcm_handle *h, int64_t rows, int64_t cols, int64_t nnz, int32_t valtype, rmcm_mat **out) {
    rmcm_mat *m = *out;
    if (!m) {
        m = new rmcm_mat();
        m->valtype = valtype;
        m->d.rows = rows;
        m->d.cols = cols;
        void *rp = nullptr;
        int32_t rc = dev_alloc(h, &rp, 8 * (rows + 1));
        if (rc != RMCM_OK) {
            delete m;
            return rc;
        }
        m->d.rowptr = (int64_t *)rp;
        m->bytes = 8 * (rows + 1);
        *out = m;
    }
    if (nnz >= 0) {
        void *c = nullptr, *v = nullptr;
        RMCM_TRY(dev_alloc(h, &c, 4 * nnz));
        int32_t rc = dev_alloc(h, &v, val_bytes(m->valtype) * nnz);
        if (rc != RMCM_OK) {
            dev_free(h, c, 4 * nnz);
            return rc;
        }
        m->d.col = (int32_t *)c;
        m->d.val = v;
        m->d.nnz = nnz;
        m->bytes += (4 + val_bytes(m->valtype)) * nnz;
    }
    return RMCM_OK;
}

void mat_release(rmcm_handle *h, rmcm_mat *m) {
    if (!m) return;
    if (m->rowsum) dev_free(h, m->rowsum, 8 * (m->d.rows + 1) + 8 * m->d.rows);
    if (m->est_long) dev_free(h, m->est_long, 4 * (int64_t)m->n_est_long);
    if (m->xfer_done) cudaEventDestroy(m->xfer_done);
    dev_free(h, m->d.rowptr, 8 * (m->d.rows + 1));
    if (m->d.col) dev_free(h, m->d.col, 4 * m->d.nnz);
    if (m->d.val) dev_free(h, m->d.val, val_bytes(m->valtype) * m->d.nnz);
    delete m;
}

// Queues the copy of the device status words to the host (read them with
// status_eval once the stream has passed it).
int32_t status_fetch(rmcm_handle *h) {
    RMCM_CUDA(h, cudaMemcpyAsync(h->h_status, h->d_status, sizeof(int) * kNumStatus, cudaMemcpyDeviceToHost, h->stream));
    return RMCM_OK;
}

// The status words fetched last: RMCM_OK, or the error they report (the
// words are cleared on the device).
int32_t status_eval(rmcm_handle *h) {
    int st[kNumStatus];
    memcpy(st, h->h_status, sizeof(st));
    bool any = false;
    for (int i = 0; i < kNumStatus; i++) any |= st[i] != 0;
    if (!any) return RMCM_OK;
    RMCM_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(int) * kNumStatus, h->stream));
    if (st[kInvariant]) return set_error(h, RMCM_EINTERNAL, "device invariant check failed");
    if (st[kTimeout]) return set_error(h, RMCM_ETIMEOUT, "a bounded device wait gave up");
    if (st[kArena]) return set_error(h, RMCM_ENOMEM, "device arena exhausted");
    return set_error(h, RMCM_EOVERFLOW, "a path count overflowed the value type");
}

int32_t check_status(rmcm_handle *h) {
    RMCM_TRY(status_fetch(h));
    RMCM_CUDA(h, cudaStreamSynchronize(h->stream));
    return status_eval(h);
}

}  // namespace rmcm

namespace {

// ---------------------------------------------------------------------------
// text loader (reference file formats of DataReader, efficient/resmcm.cpp:49-177)
// ---------------------------------------------------------------------------

bool read_file(const char *path, std::string &buf) {
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    if (fseek(f, 0, SEEK_END) != 0) {
        fclose(f);
        return false;
    }
    long sz = ftell(f);
    if (sz < 0) {
        fclose(f);
        return false;
    }
    rewind(f);
    buf.resize((size_t)sz);
    size_t got = sz ? fread(&buf[0], 1, (size_t)sz, f) : 0;
    fclose(f);
    buf.resize(got);
    return true;
}

// One line at a time; numbers are non-negative decimal integers separated by
// blanks (a leading '+' is accepted, as istringstream does).
struct LineReader {
    const char *p, *end;
    explicit LineReader(const std::string &s) : p(s.data()), end(s.data() + s.size()) {}
    bool next_line(const char *&b, const char *&e) {
        if (p >= end) return false;
        b = p;
        const char *q = (const char *)memchr(p, '\n', (size_t)(end - p));
        e = q ? q : end;
        p = q ? q + 1 : end;
        return true;
    }
};

inline bool is_blank(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// 1 = number read, 0 = end of line, -1 = malformed
inline int parse_num(const char *&p, const char *e, int64_t &out) {
    while (p < e && is_blank(*p)) p++;
    if (p >= e) return 0;
    if (*p == '+') p++;
    if (p >= e || *p < '0' || *p > '9') return -1;
    int64_t v = 0;
    while (p < e && *p >= '0' && *p <= '9') {
        v = v * 10 + (*p - '0');
        if (v > ((int64_t)1 << 50)) return -1;
        p++;
    }
    if (p < e && !is_blank(*p)) return -1;
    out = v;
    return 1;
}

int32_t graph_finish(rmcm_graph *g) {
    const int32_t nt = g->max_vt + 1;
    g->dims.assign(nt, 0);
    for (int64_t v = 0; v < g->n; v++) g->dims[g->vtype[v]]++;
    g->bin_ptr.assign(nt + 1, 0);
    for (int32_t t = 0; t < nt; t++) g->bin_ptr[t + 1] = g->bin_ptr[t] + g->dims[t];
    g->bin_ids.resize(g->n);
    g->local.resize(g->n);
    std::vector<int64_t> fill(nt, 0);
    for (int64_t v = 0; v < g->n; v++) {
        const int32_t t = g->vtype[v];
        g->local[v] = (int32_t)fill[t];
        g->bin_ids[g->bin_ptr[t] + fill[t]++] = (int32_t)v;
    }
    return RMCM_OK;
}

int32_t load_text(rmcm_handle *h, const char *gfile, const char *vfile, const char *efile, rmcm_graph *g) {
    std::string vb, eb, gb;
    if (!read_file(vfile, vb)) return set_error(h, RMCM_EIO, std::string("cannot open ") + vfile);
    if (!read_file(efile, eb)) return set_error(h, RMCM_EIO, std::string("cannot open ") + efile);
    if (!read_file(gfile, gb)) return set_error(h, RMCM_EIO, std::string("cannot open ") + gfile);
    // n = number of lines of vertex.txt
    int64_t n = 0;
    for (char c : vb) n += c == '\n';
    if (!vb.empty() && vb.back() != '\n') n++;
    g->n = n;
    g->vtype.assign(n, 0);
    g->max_vt = 0;
    {
        LineReader lr(vb);
        const char *b, *e;
        int64_t line = 0;
        while (lr.next_line(b, e)) {
            line++;
            int64_t v, t;
            int a = parse_num(b, e, v);
            if (a == 0) continue;
            if (a < 0 || parse_num(b, e, t) != 1 || v >= n || t > 1000000)
                return set_error(h, RMCM_EPARSE, "vertex file line " + std::to_string(line) + ": expected 'vid vt'");
            g->vtype[v] = (int32_t)t;
            g->max_vt = std::max<int32_t>(g->max_vt, (int32_t)t);
        }
    }
    // graph.txt, pass 1: m and per-vertex counts
    std::vector<int64_t> cnt(n + 1, 0);
    std::vector<unsigned char> seen(n, 0);
    int64_t m = 0;
    {
        LineReader lr(gb);
        const char *b, *e;
        int64_t line = 0;
        while (lr.next_line(b, e)) {
            line++;
            int64_t vid, x;
            int a = parse_num(b, e, vid);
            if (a == 0) continue;
            if (a < 0 || vid >= n) return set_error(h, RMCM_EPARSE, "graph file line " + std::to_string(line) + ": bad vertex id");
            if (seen[vid]) return set_error(h, RMCM_EPARSE, "graph file: vertex " + std::to_string(vid) + " listed twice");
            seen[vid] = 1;
            int64_t toks = 0;
            while ((a = parse_num(b, e, x)) == 1) toks++;
            if (a < 0 || toks % 2) return set_error(h, RMCM_EPARSE, "graph file line " + std::to_string(line) + ": expected 'vid (nbr eid)*'");
            cnt[vid] = toks / 2;
            m += toks / 2;
        }
    }
    g->m = m;
    std::vector<int32_t> etype(m, -1);
    {
        LineReader lr(eb);
        const char *b, *e;
        int64_t line = 0;
        while (lr.next_line(b, e)) {
            line++;
            int64_t id, t;
            int a = parse_num(b, e, id);
            if (a == 0) continue;
            if (a < 0 || parse_num(b, e, t) != 1 || id >= m)
                return set_error(h, RMCM_EPARSE, "edge file line " + std::to_string(line) + ": expected 'eid et' with eid < m");
            etype[id] = (int32_t)t;
        }
    }
    g->adj_ptr.assign(n + 1, 0);
    for (int64_t v = 0; v < n; v++) g->adj_ptr[v + 1] = g->adj_ptr[v] + cnt[v];
    g->adj_nbr.resize(m);
    g->adj_et.resize(m);
    {
        LineReader lr(gb);
        const char *b, *e;
        while (lr.next_line(b, e)) {
            int64_t vid, nb, id;
            if (parse_num(b, e, vid) != 1) continue;
            int64_t pos = g->adj_ptr[vid];
            while (parse_num(b, e, nb) == 1) {
                parse_num(b, e, id);
                if (nb >= n || id >= m || etype[id] < 0)
                    return set_error(h, RMCM_EPARSE, "graph file: neighbour or edge id out of range at vertex " + std::to_string(vid));
                g->adj_nbr[pos] = (int32_t)nb;
                g->adj_et[pos] = etype[id];
                pos++;
            }
        }
    }
    return graph_finish(g);
}

// ---------------------------------------------------------------------------
// leaf matrices (BoolMatrix(HIN, vt, src, sink, et, n), efficient/resmcm.cpp:374-396)
// ---------------------------------------------------------------------------

// What the device check of an upload found.
struct CsrFlags {
    bool bad = false, unsorted = false, dup = false, zero = false;
};

// Copies a host CSR to the device and checks it there (csr_check: one pass
// of a warp per row, no host loop over the arrays); the longest row and the
// estimator's list of long rows (ascending) come from the same pass.  With
// ck the check's flags are returned for the caller to act on; without it
// the arrays are trusted (built here, rows sorted).
int32_t upload_csr(rmcm_handle *h, int64_t rows, int64_t cols, const int64_t *rowptr, const int32_t *col,
                   const void *val, int32_t valtype, rmcm_mat **out, CsrFlags *ck) {
    const int64_t nnz = rows > 0 ? rowptr[rows] : 0;
    rmcm_mat *m = nullptr;
    RMCM_TRY(mat_alloc(h, rows, cols, nnz, valtype, &m));
    cudaStream_t s = h->stream;
    cudaError_t e = cudaMemcpyAsync(m->d.rowptr, rowptr, 8 * (rows + 1), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && nnz > 0) e = cudaMemcpyAsync(m->d.col, col, 4 * nnz, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && nnz > 0 && val)
        e = cudaMemcpyAsync(m->d.val, val, val_bytes(valtype) * nnz, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
        mat_release(h, m);
        return cuda_error(h, e, "upload");
    }
    {
        // flags, then room for every row longer than kEstLongRow
        const int64_t cap = nnz / (kEstLongRow + 1) + 1;
        char *tmp = nullptr;
        int32_t rc = dev_alloc(h, (void **)&tmp, 64 + 4 * cap);
        if (rc != RMCM_OK) {
            mat_release(h, m);
            return rc;
        }
        unsigned long long *f = (unsigned long long *)tmp;
        int32_t *lng = (int32_t *)(tmp + 64);
        rc = csr_check(h, m->d, val ? m->d.val : nullptr, valtype, f, lng, cap);
        if (rc == RMCM_OK) {
            e = cudaMemcpyAsync(h->h_pinned, f, 6 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) rc = cuda_error(h, e, "upload");
        }
        const uint64_t *hf = (const uint64_t *)h->h_pinned;
        const int64_t nlong = rc == RMCM_OK ? std::min<int64_t>((int64_t)hf[5], cap) : 0;
        if (rc == RMCM_OK) {
            if (ck) {
                ck->bad = hf[0] != 0;
                ck->unsorted = hf[1] != 0;
                ck->dup = hf[2] != 0;
                ck->zero = hf[3] != 0;
            }
            m->max_row = (int64_t)hf[4];
        }
        if (rc == RMCM_OK && nlong > 0 && !(ck && (ck->bad || ck->unsorted))) {
            // ascending: the estimator adds the long rows' terms in list order
            std::vector<int32_t> list((size_t)nlong);
            e = cudaMemcpy(list.data(), lng, 4 * nlong, cudaMemcpyDeviceToHost);
            if (e == cudaSuccess) {
                std::sort(list.begin(), list.end());
                rc = dev_alloc(h, (void **)&m->est_long, 4 * nlong);
                if (rc == RMCM_OK) {
                    m->n_est_long = (int32_t)nlong;
                    e = cudaMemcpyAsync(m->est_long, list.data(), 4 * nlong, cudaMemcpyHostToDevice, s);
                    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
                }
            }
            if (rc == RMCM_OK && e != cudaSuccess) rc = cuda_error(h, e, "upload");
        }
        dev_free(h, tmp, 64 + 4 * cap);
        if (rc != RMCM_OK) {
            mat_release(h, m);
            return rc;
        }
    }
    if (!val) {
        int32_t rc = fill_ones(h, m->d.val, nnz, valtype);
        if (rc != RMCM_OK) {
            mat_release(h, m);
            return rc;
        }
        m->ones = true;
        m->positive = true;
    }
    *out = m;
    return RMCM_OK;
}

int32_t build_leaf(rmcm_handle *h, rmcm_graph *g, int32_t src, int32_t sink, int32_t et, int32_t valtype,
                   rmcm_mat **out) {
    const int64_t rows = g->dims[src], cols = g->dims[sink];
    const int64_t b0 = g->bin_ptr[src];
    std::vector<int64_t> rp(rows + 1, 0);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t r = 0; r < rows; r++) {
        const int32_t u = g->bin_ids[b0 + r];
        int64_t c = 0;
        for (int64_t q = g->adj_ptr[u]; q < g->adj_ptr[u + 1]; q++)
            c += (g->adj_et[q] == et && g->vtype[g->adj_nbr[q]] == sink);
        rp[r + 1] = c;
    }
    for (int64_t r = 0; r < rows; r++) rp[r + 1] += rp[r];
    std::vector<int32_t> col(std::max<int64_t>(rp[rows], 1));
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t r = 0; r < rows; r++) {
        const int32_t u = g->bin_ids[b0 + r];
        int64_t o = rp[r];
        for (int64_t q = g->adj_ptr[u]; q < g->adj_ptr[u + 1]; q++)
            if (g->adj_et[q] == et && g->vtype[g->adj_nbr[q]] == sink) col[o++] = g->local[g->adj_nbr[q]];
        std::sort(col.begin() + rp[r], col.begin() + rp[r + 1]);
    }
    int dup = 0;
#pragma omp parallel for schedule(dynamic, 4096) reduction(| : dup)
    for (int64_t r = 0; r < rows; r++)
        for (int64_t q = rp[r] + 1; q < rp[r + 1]; q++) dup |= col[q] == col[q - 1];
    int32_t rc = upload_csr(h, rows, cols, rp.data(), col.data(), nullptr, valtype, out, nullptr);
    if (rc == RMCM_OK) (*out)->distinct = !dup;
    return rc;
}

int32_t get_leaf(rmcm_handle *h, rmcm_graph *g, int32_t src, int32_t sink, int32_t et, int32_t valtype,
                 rmcm_mat **out) {
    if (g->h != h) return set_error(h, RMCM_EINVAL, "graph belongs to another (or a destroyed) handle");
    if (src < 0 || src > g->max_vt || sink < 0 || sink > g->max_vt)
        return set_error(h, RMCM_EINVAL, "meta-path names a vertex type the graph does not have");
    auto key = std::make_tuple(src, sink, et, valtype);
    auto it = g->leaves.find(key);
    if (it != g->leaves.end()) {
        *out = it->second;
        return RMCM_OK;
    }
    rmcm_mat *m = nullptr;
    RMCM_TRY(build_leaf(h, g, src, sink, et, valtype, &m));
    m->graph_owned = true;
    g->leaves[key] = m;
    *out = m;
    return RMCM_OK;
}

int32_t parse_path(const char *s, std::vector<int32_t> &vts, std::vector<int32_t> &ets) {
    // MetaPath(string), efficient/resmcm.cpp:269-299: maximal digit runs; every
    // non-digit closes a number (0 when no digit preceded it); alternate vt, et.
    vts.clear();
    ets.clear();
    if (!s) return RMCM_EINVAL;
    const size_t L = strlen(s);
    if (L == 0) return RMCM_EPARSE;
    int64_t num = 0;
    int i = 0;
    for (size_t q = 0; q < L; q++) {
        const char ch = s[q];
        if (ch >= '0' && ch <= '9') {
            num = num * 10 + (ch - '0');
            if (num > 1000000000) return RMCM_EPARSE;
        } else {
            (i % 2 == 0 ? vts : ets).push_back((int32_t)num);
            num = 0;
            i++;
        }
    }
    if (s[L - 1] >= '0' && s[L - 1] <= '9') {
        (i % 2 == 0 ? vts : ets).push_back((int32_t)num);
        i++;
    }
    if (vts.size() != ets.size() + 1) return RMCM_EPARSE;
    return RMCM_OK;
}

double elapsed_s(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms / 1000.0;
}

int32_t copy_mat(rmcm_handle *h, const rmcm_mat *src, rmcm_mat **out) {
    rmcm_mat *m = nullptr;
    RMCM_TRY(mat_alloc(h, src->d.rows, src->d.cols, src->d.nnz, src->valtype, &m));
    cudaStream_t s = h->stream;
    cudaError_t e = cudaMemcpyAsync(m->d.rowptr, src->d.rowptr, 8 * (src->d.rows + 1), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && src->d.nnz)
        e = cudaMemcpyAsync(m->d.col, src->d.col, 4 * src->d.nnz, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && src->d.nnz)
        e = cudaMemcpyAsync(m->d.val, src->d.val, val_bytes(src->valtype) * src->d.nnz, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) {
        mat_release(h, m);
        return cuda_error(h, e, "copy");
    }
    m->ones = src->ones;
    m->positive = src->positive;
    m->max_row = src->max_row;
    m->distinct = src->distinct;
    *out = m;
    return RMCM_OK;
}

// Device operations of one chain as the executor issued them, with every
// size the executor read back from the device.  Replaying the log issues the
// same work with no host round trip, so it can be captured into a CUDA graph.
struct LogOp {
    enum Kind { kEst, kDp, kBind, kSpgemm, kWiden, kFree } kind;
    int a = -1, b = -1, c = -1;          // matrix slots
    rmcm_mat *ext = nullptr;             // kBind: a graph-owned leaf
    ProductPlan plan;                    // kSpgemm
};
struct ChainLog {
    int32_t len = 0;
    std::vector<rmcm_mat *> leaves;      // slots 0 .. len-1
    std::vector<LogOp> ops;
    int32_t nslots = 0;
    int32_t result = -1;
    int64_t nnz = 0;
    int32_t valtype = RMCM_VAL_U32;
};

// Post-order (k, l) pair list of a split table (get_optimal_chain_order,
// efficient/resmcm.cpp:563-573).
int32_t post_order(const std::vector<int32_t> &split, int32_t len, int32_t i, int32_t j, std::vector<int32_t> &out) {
    if (i == j) return i;
    const int32_t k = split[i * len + j];
    const int32_t a = post_order(split, len, i, k, out);
    const int32_t b = post_order(split, len, k + 1, j, out);
    out.push_back(a);
    out.push_back(b);
    return -1;
}

// DP of efficient/naive.cpp:506-523 (dense dimension costs).
void dense_order(const int64_t *d, int32_t len, std::vector<int32_t> &split, std::vector<double> &m) {
    split.assign(len * len, 0);
    m.assign(len * len, 0.0);
    for (int32_t l = 1; l < len; l++) {
        for (int32_t i = 0; i < len - l; i++) {
            const int32_t j = i + l;
            m[i * len + j] = DBL_MAX;
            for (int32_t k = i; k < j; k++) {
                // `vertex` (int) operands: the product wraps in 32 bits
                const uint32_t p = (uint32_t)d[i] * (uint32_t)d[k] * (uint32_t)d[j + 1];
                const double cost = m[i * len + k] + m[(k + 1) * len + j] + (double)(int32_t)p;
                if (cost < m[i * len + j]) {
                    m[i * len + j] = cost;
                    split[i * len + j] = k;
                }
            }
        }
    }
}

// SSP_dynamic on device-resident matrices (see file comment).
//
// With `widen` set, products run in uint32 and the chain escalates to uint64
// at the first product whose counts overflow: that product is recomputed in
// uint64 from widened operands (every earlier intermediate is exact, its
// counts having fit), and the rest of the chain continues in uint64.  Leaves
// in uint64 come from `leaf64` when given (the graph's cache), else are
// widened here.
//
// With `sink` set, the final product is computed in blocks of rows of its
// left operand (a row range of a CSR is its row pointers from the range's
// first row on) and every block goes to the sink, then is freed: a result
// larger than the free device memory never exists whole on the device.  The
// block height is the sink's, or chosen so that a block's estimated entries
// (RES estimate of the whole chain, spread evenly over the rows) take at most
// a quarter of the memory left under the budget.  *Cout stays null.
int32_t chain_exec(rmcm_handle *h, rmcm_mat *const *mats, int32_t len, const int32_t *fixed_pairs, rmcm_mat **Cout,
                   rmcm_timings *t, bool widen, const std::function<int32_t(int, rmcm_mat **)> &leaf64,
                   ChainLog *log = nullptr, bool order_given = false, const BlockSink *sink = nullptr) {
    rmcm_timings tm{};
    *Cout = nullptr;
    // slot bookkeeping of the optional log
    std::map<const rmcm_mat *, int> slot_of;
    auto slot = [&](const rmcm_mat *m) -> int {
        auto it = slot_of.find(m);
        if (it != slot_of.end()) return it->second;
        const int id = log->nslots++;
        slot_of[m] = id;
        return id;
    };
    auto log_op = [&](LogOp op) {
        if (log) log->ops.push_back(op);
    };
    auto release = [&](rmcm_mat *m) {
        if (log && m) {
            LogOp op;
            op.kind = LogOp::kFree;
            op.a = slot(m);
            log_op(op);
            slot_of.erase(m);
        }
        mat_release(h, m);
    };
    if (log) {
        log->len = len;
        log->leaves.assign(mats, mats + len);
        log->nslots = len;
        for (int i = 0; i < len; i++) slot_of[mats[i]] = i;
    }
    if (len < 1 || len > 16) return set_error(h, RMCM_EINVAL, "chain length must be 1..16");
    for (int i = 0; i < len; i++) {
        if (!mats[i]) return set_error(h, RMCM_EINVAL, "null matrix in chain");
        if (mats[i]->valtype != mats[0]->valtype) return set_error(h, RMCM_EINVAL, "chain mixes value types");
        if (i + 1 < len && mats[i]->d.cols != mats[i + 1]->d.rows)
            return set_error(h, RMCM_EINVAL, "consecutive matrices do not chain");
    }
    cudaStream_t s = h->stream;
    int32_t cur = mats[0]->valtype;
    widen = widen && cur == RMCM_VAL_U32;
    if (len == 1) {
        // efficient/resmcm.cpp:670-677: the leaf itself is the result (no timed work)
        RMCM_TRY(copy_mat(h, mats[0], Cout));
        RMCM_CUDA(h, cudaStreamSynchronize(s));
        tm.nnz = (*Cout)->d.nnz;
        tm.valtype = cur;
        if (t) *t = tm;
        if (log) {
            log->result = 0;
            log->nnz = tm.nnz;
            log->valtype = cur;
        }
        return RMCM_OK;
    }
    cudaEvent_t *ev = h->ev;
    RMCM_CUDA(h, cudaEventRecord(ev[0], s));
    int32_t pairs[32];
    int32_t rc = RMCM_OK;
    double host_dp_s = -1;
    double est_result = -1;        // RES estimate of the result's nnz (blocked final product)
    int64_t block_next = 0;        // blocked final product: first row not yet delivered
    int64_t block_nnz = 0;
    bool delivered = false;
    int32_t block_rc = RMCM_OK;    // EOVERFLOW kept from a delivered block (fixed value type)
    if (!fixed_pairs && h->order_mode != RMCM_ORDER_RES) {
        // ablation orders: no estimator, order computed on the host
        cudaEventRecord(ev[1], s);
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<int32_t> pl;
        if (h->order_mode == RMCM_ORDER_L2R) {
            pl.resize(2 * (len - 1));
            rmcm_order_l2r(len, pl.data());
        } else {
            std::vector<int64_t> d(len + 1);
            for (int i = 0; i < len; i++) d[i] = mats[i]->d.rows;
            d[len] = mats[len - 1]->d.cols;
            std::vector<int32_t> split;
            std::vector<double> m;
            dense_order(d.data(), len, split, m);
            post_order(split, len, 0, len - 1, pl);
        }
        host_dp_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        memcpy(pairs, pl.data(), sizeof(int32_t) * 2 * (len - 1));
        cudaEventRecord(ev[2], s);
        fixed_pairs = pairs;
    }
    if (order_given && fixed_pairs) {
        // the caller ordered the chain already: no estimator, no DP
        memcpy(pairs, fixed_pairs, sizeof(int32_t) * 2 * (len - 1));
        cudaEventRecord(ev[1], s);
        cudaEventRecord(ev[2], s);
        host_dp_s = 0;
        fixed_pairs = pairs;
    }
    if (fixed_pairs == pairs) {
        // order already known
    } else {
    if (log) {
        LogOp e;
        e.kind = LogOp::kEst;
        log_op(e);
        LogOp d;
        d.kind = LogOp::kDp;
        log_op(d);
    }
    // (a) estimator
    double *c_dev = nullptr;
    char *ord = nullptr;
    const int64_t ord_bytes = 8 * 256 + 4 * 256 + 4 * 64;
    RMCM_TRY(dev_alloc(h, (void **)&c_dev, 8 * 256));
    rc = estimate(h, mats, len, c_dev);
    if (rc == RMCM_OK) rc = dev_alloc(h, (void **)&ord, ord_bytes);
    if (rc != RMCM_OK) {
        dev_free(h, c_dev, 8 * 256);
        return rc;
    }
    cudaEventRecord(ev[1], s);
    // (b) DP + order
    int32_t *pairs_dev = (int32_t *)(ord + 8 * 256 + 4 * 256);
    rc = chain_order_dev(h, c_dev, len, (int32_t *)(ord + 8 * 256), (double *)ord, pairs_dev);
    cudaEventRecord(ev[2], s);
    if (rc == RMCM_OK) {
        if (fixed_pairs) {
            memcpy(pairs, fixed_pairs, sizeof(int32_t) * 2 * (len - 1));
        } else {
            cudaError_t e = cudaMemcpyAsync(h->h_pinned, pairs_dev, sizeof(int32_t) * 2 * (len - 1), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) rc = cuda_error(h, e, "order download");
            else memcpy(pairs, h->h_pinned, sizeof(int32_t) * 2 * (len - 1));
        }
    }
    if (rc == RMCM_OK && sink) {
        // the whole chain's estimated nnz sizes the result's blocks
        cudaError_t e = cudaMemcpyAsync(h->h_pinned, c_dev + (len - 1), sizeof(double), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_error(h, e, "estimate download");
        else memcpy(&est_result, h->h_pinned, sizeof(double));
    }
    dev_free(h, ord, ord_bytes);
    dev_free(h, c_dev, 8 * 256);
    if (rc != RMCM_OK) return rc;
    }
    // validate the pair list against the stack machine before running it
    {
        int depth = 0;
        std::vector<char> used(len, 0);
        for (int p = 0; p < len - 1; p++) {
            const int k = pairs[2 * p], l = pairs[2 * p + 1];
            const int need = (k < 0) + (l < 0);
            if ((k >= 0 && (k >= len || used[k])) || (l >= 0 && (l >= len || used[l])) || k < -1 || l < -1 || depth < need)
                return set_error(h, RMCM_EINVAL, "invalid chain order pair list");
            if (k >= 0) used[k] = 1;
            if (l >= 0) used[l] = 1;
            depth += 1 - need;
        }
        if (depth != 1) return set_error(h, RMCM_EINVAL, "invalid chain order pair list");
    }
    // (c) executor, efficient/resmcm.cpp:709-760
    std::vector<rmcm_mat *> stack;
    std::vector<rmcm_mat *> wide(len, nullptr);     // uint64 leaves widened here
    auto leaf = [&](int i, const rmcm_mat **out) -> int32_t {
        if (cur == mats[i]->valtype) {
            *out = mats[i];
            return RMCM_OK;
        }
        if (leaf64) {
            rmcm_mat *m = nullptr;
            RMCM_TRY(leaf64(i, &m));
            if (log && !slot_of.count(m)) {
                LogOp op;
                op.kind = LogOp::kBind;
                op.c = slot(m);
                op.ext = m;
                log_op(op);
            }
            *out = m;
            return RMCM_OK;
        }
        if (!wide[i]) {
            RMCM_TRY(convert_values(h, mats[i], RMCM_VAL_U64, &wide[i]));
            if (log) {
                LogOp op;
                op.kind = LogOp::kWiden;
                op.a = i;
                op.c = slot(wide[i]);
                log_op(op);
            }
        }
        *out = wide[i];
        return RMCM_OK;
    };
    double spgemm_s = 0;
    for (int p = 0; p < len - 1 && rc == RMCM_OK; p++) {
        const int k = pairs[2 * p], l = pairs[2 * p + 1];
        const int sz = (int)stack.size();
        const rmcm_mat *A = nullptr, *B = nullptr;
        if (k >= 0) rc = leaf(k, &A);
        else A = (l >= 0) ? stack[sz - 1] : stack[sz - 2];
        if (rc == RMCM_OK) {
            if (l >= 0) rc = leaf(l, &B);
            else B = stack[sz - 1];
        }
        if (rc != RMCM_OK) break;
        if (sink && p == len - 2) {
            // the final product, a block of rows of A at a time
            const int64_t rows = A->d.rows;
            int64_t rb = sink->rows_per_block;
            if (rb <= 0) {
                const double row_bytes = est_result > 0 && rows > 0
                                             ? (est_result / (double)rows) * (4.0 + (double)val_bytes(cur)) + 48.0
                                             : 0.0;
                const double room = (double)std::max<int64_t>(h->budget - h->in_use, 0) / 4.0;
                rb = row_bytes > 0 ? (int64_t)std::max(1.0, room / row_bytes) : rows;
            }
            rb = std::max<int64_t>(1, std::min<int64_t>(rb, std::max<int64_t>(rows, 1)));
            bool need_widen = false;
            while (block_next < rows && rc == RMCM_OK) {
                const int64_t r0 = block_next, r1 = std::min(rows, r0 + rb);
                // row view of A: its row pointers from r0 on (entries keep
                // their positions, so nnz stays A's)
                rmcm_mat *view = new rmcm_mat(*A);
                view->d.rowptr = A->d.rowptr + r0;
                view->d.rows = r1 - r0;
                view->d.rowsum = nullptr;
                view->d.info = nullptr;
                view->rowsum = nullptr;
                view->est_long = nullptr;
                view->n_est_long = -1;
                view->xfer_done = nullptr;
                view->graph_owned = true;
                view->bytes = 0;
                cudaEventRecord(ev[3], s);
                rmcm_mat *Cb = nullptr;
                int64_t fl = 0;
                h->abort_on_certain_overflow = widen && cur == RMCM_VAL_U32;
                rc = spgemm(h, view, B, &Cb, &fl, nullptr);
                h->abort_on_certain_overflow = false;
                cudaEventRecord(ev[4], s);
                if (view->rowsum) dev_free(h, view->rowsum, 8 * (view->d.rows + 1) + 8 * view->d.rows);
                delete view;
                if (rc == RMCM_EOVERFLOW && widen && cur == RMCM_VAL_U32 && !Cb) {
                    rc = RMCM_OK;
                    need_widen = true;
                    break;
                }
                if (rc != RMCM_OK) break;
                cudaEventSynchronize(ev[4]);
                spgemm_s += elapsed_s(ev[3], ev[4]);
                const int32_t st = check_status(h);
                if (st == RMCM_EOVERFLOW && widen && cur == RMCM_VAL_U32) {
                    mat_release(h, Cb);
                    need_widen = true;
                    break;
                }
                if (st == RMCM_EOVERFLOW) {
                    Cb->positive = false;
                    block_rc = RMCM_EOVERFLOW;
                } else if (st != RMCM_OK) {
                    mat_release(h, Cb);
                    rc = st;
                    break;
                }
                tm.flops += fl;
                block_nnz += Cb->d.nnz;
                const int32_t urc = sink->fn(sink->user, r0, Cb);
                mat_release(h, Cb);
                if (urc != RMCM_OK) {
                    rc = set_error(h, urc, "the block sink stopped the chain");
                    break;
                }
                block_next = r1;
            }
            if (rc != RMCM_OK) break;
            if (need_widen) {
                // blocks delivered so far fitted uint32 and are exact; the
                // rest of the final product runs in uint64
                cur = RMCM_VAL_U64;
                for (auto &m : stack) {
                    rmcm_mat *w = nullptr;
                    rc = convert_values(h, m, RMCM_VAL_U64, &w);
                    if (rc != RMCM_OK) break;
                    mat_release(h, m);
                    m = w;
                }
                if (rc != RMCM_OK) break;
                p--;
                continue;
            }
            tm.n_products++;
            for (auto *m : stack) mat_release(h, m);
            stack.clear();
            delivered = true;
            break;
        }
        cudaEventRecord(ev[3], s);
        rmcm_mat *C = nullptr;
        int64_t fl = 0;
        h->abort_on_certain_overflow = widen && cur == RMCM_VAL_U32;
        ProductPlan plan;
        plan.mode = log ? 1 : 0;
        rc = spgemm(h, A, B, &C, &fl, log ? &plan : nullptr);
        h->abort_on_certain_overflow = false;
        cudaEventRecord(ev[4], s);
        if (rc == RMCM_EOVERFLOW && widen && cur == RMCM_VAL_U32 && !C) {
            // overflow is certain from the row-sum bound: escalate before computing
            rc = RMCM_OK;
            cur = RMCM_VAL_U64;
            for (auto &m : stack) {
                rmcm_mat *w = nullptr;
                rc = convert_values(h, m, RMCM_VAL_U64, &w);
                if (rc != RMCM_OK) break;
                if (log) {
                    LogOp op;
                    op.kind = LogOp::kWiden;
                    op.a = slot(m);
                    op.c = slot(w);
                    log_op(op);
                }
                release(m);
                m = w;
            }
            if (rc != RMCM_OK) break;
            p--;
            continue;
        }
        if (rc != RMCM_OK) break;
        // one wait for the product and, when it may overflow, its status
        const bool want_status = widen && cur == RMCM_VAL_U32;
        if (want_status) {
            rc = status_fetch(h);
            if (rc == RMCM_OK) {
                const cudaError_t e = cudaStreamSynchronize(s);
                if (e != cudaSuccess) rc = cuda_error(h, e, "chain");
            }
            if (rc != RMCM_OK) {
                mat_release(h, C);
                break;
            }
        } else {
            cudaEventSynchronize(ev[4]);
        }
        spgemm_s += elapsed_s(ev[3], ev[4]);
        if (want_status) {
            const int32_t st = status_eval(h);
            if (st == RMCM_EOVERFLOW) {
                // escalate: drop C, widen the live intermediates, redo this product
                mat_release(h, C);
                cur = RMCM_VAL_U64;
                for (auto &m : stack) {
                    rmcm_mat *w = nullptr;
                    rc = convert_values(h, m, RMCM_VAL_U64, &w);
                    if (rc != RMCM_OK) break;
                    if (log) {
                        LogOp op;
                        op.kind = LogOp::kWiden;
                        op.a = slot(m);
                        op.c = slot(w);
                        log_op(op);
                    }
                    release(m);
                    m = w;
                }
                p--;
                continue;
            }
            if (st != RMCM_OK) {
                mat_release(h, C);
                rc = st;
                break;
            }
        }
        tm.flops += fl;
        tm.n_products++;
        if (log) {
            LogOp op;
            op.kind = LogOp::kSpgemm;
            op.a = slot(A);
            op.b = slot(B);
            op.c = slot(C);
            op.plan = plan;
            log_op(op);
        }
        if (k >= 0 && l >= 0) {
            stack.push_back(C);
        } else if (k >= 0 || l >= 0) {
            release(stack[sz - 1]);
            stack[sz - 1] = C;
        } else {
            release(stack[sz - 1]);
            release(stack[sz - 2]);
            stack.pop_back();
            stack[sz - 2] = C;
        }
    }
    for (auto *m : wide) release(m);
    if (rc != RMCM_OK) {
        for (auto *m : stack) mat_release(h, m);
        return rc;
    }
    cudaEventRecord(ev[5], s);
    RMCM_CUDA(h, cudaEventSynchronize(ev[5]));
    // the ablation orders run no estimator, as efficient/l2r.cpp and naive.cpp
    tm.es_s = host_dp_s >= 0 ? 0.0 : elapsed_s(ev[0], ev[1]);
    tm.dp_s = host_dp_s >= 0 ? host_dp_s : elapsed_s(ev[1], ev[2]);
    tm.spgemm_s = spgemm_s;
    tm.total_s = elapsed_s(ev[0], ev[5]);
    tm.valtype = cur;
    if (delivered) {
        tm.nnz = block_nnz;
        if (t) *t = tm;
        return block_rc;
    }
    *Cout = stack[0];
    tm.nnz = stack[0]->d.nnz;
    if (log) {
        log->result = slot(stack[0]);
        log->nnz = stack[0]->d.nnz;
        log->valtype = cur;
    }
    rc = check_status(h);
    if (rc == RMCM_EOVERFLOW) stack[0]->positive = false;   // wrapped counts may be 0
    if (t) *t = tm;
    return rc;
}

// Issues a chain's logged device work again, reading nothing back.  The
// result's digest goes to digest_dev (when given); the result is freed unless
// `keep`.
int32_t chain_replay(rmcm_handle *h, const ChainLog &log, uint64_t *digest_dev, bool keep, rmcm_mat **out) {
    std::vector<rmcm_mat *> slot(log.nslots, nullptr);
    for (int i = 0; i < log.len; i++) slot[i] = log.leaves[i];
    std::vector<bool> owned(log.nslots, false);
    double *c_dev = nullptr;
    int32_t rc = RMCM_OK;
    for (const LogOp &op : log.ops) {
        switch (op.kind) {
            case LogOp::kEst:
                rc = dev_alloc(h, (void **)&c_dev, 8 * 256);
                if (rc == RMCM_OK) rc = estimate(h, log.leaves.data(), log.len, c_dev);
                break;
            case LogOp::kDp: {
                char *buf = nullptr;
                const int64_t bytes = 8 * 256 + 4 * 256 + 8 * 256 + 4 * 64;
                rc = dev_alloc(h, (void **)&buf, bytes);
                if (rc == RMCM_OK)
                    rc = chain_order_launch(h, c_dev, log.len, (double *)buf, (int32_t *)(buf + 8 * 256),
                                            (double *)(buf + 8 * 256 + 4 * 256), (int32_t *)(buf + 8 * 256 + 4 * 256 + 8 * 256));
                dev_free(h, buf, bytes);
                dev_free(h, c_dev, 8 * 256);
                c_dev = nullptr;
                break;
            }
            case LogOp::kBind:
                slot[op.c] = op.ext;
                break;
            case LogOp::kSpgemm: {
                ProductPlan p = op.plan;
                p.mode = 2;
                rmcm_mat *C = nullptr;
                rc = spgemm(h, slot[op.a], slot[op.b], &C, nullptr, &p);
                slot[op.c] = C;
                owned[op.c] = true;
                break;
            }
            case LogOp::kWiden:
                rc = convert_values(h, slot[op.a], RMCM_VAL_U64, &slot[op.c]);
                owned[op.c] = true;
                break;
            case LogOp::kFree:
                if (owned[op.a]) mat_release(h, slot[op.a]);
                slot[op.a] = nullptr;
                owned[op.a] = false;
                break;
        }
        if (rc != RMCM_OK) break;
    }
    if (c_dev) dev_free(h, c_dev, 8 * 256);
    rmcm_mat *res = log.result >= 0 ? slot[log.result] : nullptr;
    if (rc == RMCM_OK && res && digest_dev) rc = mat_digest_launch(h, res, digest_dev);
    for (int i = 0; i < log.nslots; i++)
        if (owned[i] && slot[i] && slot[i] != res) mat_release(h, slot[i]);
    if (rc != RMCM_OK) {
        if (res && owned[log.result]) mat_release(h, res);
        return rc;
    }
    if (keep && out) *out = res;
    else if (res && owned[log.result]) mat_release(h, res);
    return RMCM_OK;
}

}  // namespace

namespace rmcm {

int32_t leaf_of(rmcm_handle *h, rmcm_graph *g, int32_t src, int32_t sink, int32_t et, int32_t valtype,
                rmcm_mat **out) {
    return get_leaf(h, g, src, sink, et, valtype, out);
}

int32_t path_parse(const char *s, std::vector<int32_t> &vts, std::vector<int32_t> &ets) {
    return parse_path(s, vts, ets);
}

int32_t chain_run_ordered(rmcm_handle *h, rmcm_mat *const *mats, int32_t len, const int32_t *pairs, rmcm_mat **out,
                          rmcm_timings *t, bool widen, const std::function<int32_t(int, rmcm_mat **)> &leaf64) {
    return chain_exec(h, mats, len, pairs, out, t, widen, leaf64, nullptr, true);
}

int32_t chain_plan(rmcm_handle *h, rmcm_mat *const *mats, int32_t len, double *c, int32_t *split, int32_t *pairs,
                   double *es_s, double *dp_s) {
    if (len < 2 || len > 16) return set_error(h, RMCM_EINVAL, "chain_plan: length must be 2..16");
    cudaStream_t s = h->stream;
    char *buf = nullptr;
    const int64_t bytes = 8 * 256 + 8 * 256 + 4 * 256 + 4 * 64;
    RMCM_TRY(dev_alloc(h, (void **)&buf, bytes));
    double *c_dev = (double *)buf;
    double *cost_dev = (double *)(buf + 8 * 256);
    int32_t *split_dev = (int32_t *)(buf + 16 * 256);
    int32_t *pairs_dev = (int32_t *)(buf + 16 * 256 + 4 * 256);
    cudaEventRecord(h->ev[0], s);
    int32_t rc = estimate(h, mats, len, c_dev);
    cudaEventRecord(h->ev[1], s);
    if (rc == RMCM_OK) rc = chain_order_dev(h, c_dev, len, split_dev, cost_dev, pairs_dev);
    cudaEventRecord(h->ev[2], s);
    std::vector<char> host(bytes);
    if (rc == RMCM_OK) {
        cudaError_t e = cudaMemcpyAsync(host.data(), buf, bytes, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_error(h, e, "chain plan download");
    }
    dev_free(h, buf, bytes);
    if (rc != RMCM_OK) return rc;
    if (c) memcpy(c, host.data(), sizeof(double) * len * len);
    if (split) memcpy(split, host.data() + 16 * 256, sizeof(int32_t) * len * len);
    if (pairs) memcpy(pairs, host.data() + 16 * 256 + 4 * 256, sizeof(int32_t) * 2 * (len - 1));
    if (es_s) *es_s = elapsed_s(h->ev[0], h->ev[1]);
    if (dp_s) *dp_s = elapsed_s(h->ev[1], h->ev[2]);
    return RMCM_OK;
}

}  // namespace rmcm

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

RMCM_API const char *rmcm_status_string(int32_t status) {
    switch (status) {
        case RMCM_OK: return "ok";
        case RMCM_EINVAL: return "invalid argument";
        case RMCM_ENOMEM: return "out of device memory budget";
        case RMCM_EOVERFLOW: return "path count overflow";
        case RMCM_ETIMEOUT: return "device wait timed out";
        case RMCM_ECUDA: return "CUDA error";
        case RMCM_EIO: return "I/O error";
        case RMCM_EPARSE: return "parse error";
        case RMCM_EINTERNAL: return "internal invariant violated";
        default: return "unknown status";
    }
}

RMCM_API int32_t rmcm_create(rmcm_handle **out, const rmcm_opts *opts) {
    if (!out) return RMCM_EINVAL;
    *out = nullptr;
    rmcm_handle *h = new rmcm_handle();
    rmcm_opts o{};
    o.valtype = RMCM_VAL_AUTO;
    if (opts) o = *opts;
    h->device = o.device;
    h->valtype = o.valtype;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0 || o.device < 0 || o.device >= ndev) {
        cudaGetLastError();
        delete h;
        return RMCM_ECUDA;
    }
    e = cudaSetDevice(o.device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, o.device);
    if (e == cudaSuccess) {
        if (o.stream) h->stream = (cudaStream_t)o.stream;
        else {
            e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
            h->own_stream = true;
        }
    }
    for (int i = 0; i < 8 && e == cudaSuccess; i++) e = cudaEventCreate(&h->ev[i]);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->aux, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->xfer, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void **)&h->d_status, sizeof(int) * kNumStatus);
    if (e == cudaSuccess) e = cudaMemset(h->d_status, 0, sizeof(int) * kNumStatus);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&h->h_status, sizeof(int) * kNumStatus);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&h->h_pinned, sizeof(int64_t) * 64);
    size_t free_b = 0, total_b = 0;
    if (e == cudaSuccess) e = cudaMemGetInfo(&free_b, &total_b);
    if (e == cudaSuccess) {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, o.device) == cudaSuccess) {
            uint64_t thr = ~0ull;   // keep freed blocks cached in the pool
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        rmcm_destroy(h);
        return RMCM_ECUDA;
    }
    h->budget = o.mem_budget_bytes > 0 ? o.mem_budget_bytes : (int64_t)(0.9 * (double)free_b);
    *out = h;
    return RMCM_OK;
}

RMCM_API int32_t rmcm_destroy(rmcm_handle *h) {
    if (!h) return RMCM_OK;
    while (!h->batches.empty()) rmcm_batch_free(h, *h->batches.begin());
    if (h->xfer) {
        // downloads in flight land first; matrices freed meanwhile go now
        cudaStreamSynchronize(h->xfer);
        for (rmcm_mat *m : h->deferred) mat_release(h, m);
        h->deferred.clear();
    }
    // graphs outliving their handle keep their host arrays only
    for (rmcm_graph *g : h->graphs) {
        for (auto &kv : g->leaves) mat_release(h, kv.second);
        g->leaves.clear();
        g->h = nullptr;
    }
    h->graphs.clear();
    for (auto &r : h->prof)
        for (auto &e : r.ev)
            if (e) cudaEventDestroy(e);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->scratch) dev_free(h, h->scratch, h->scratch_bytes);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->d_status) cudaFree(h->d_status);
    if (h->h_status) cudaFreeHost(h->h_status);
    if (h->h_pinned) cudaFreeHost(h->h_pinned);
    for (auto &e : h->ev)
        if (e) cudaEventDestroy(e);
    if (h->xfer) cudaStreamDestroy(h->xfer);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->aux) cudaStreamDestroy(h->aux);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return RMCM_OK;
}

RMCM_API const char *rmcm_last_error(const rmcm_handle *h) { return h ? h->last_error.c_str() : ""; }

RMCM_API int32_t rmcm_set_stream(rmcm_handle *h, void *stream) {
    if (!h) return RMCM_EINVAL;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    h->own_stream = false;
    h->stream = (cudaStream_t)stream;
    return RMCM_OK;
}

RMCM_API void *rmcm_get_stream(const rmcm_handle *h) { return h ? (void *)h->stream : nullptr; }
RMCM_API int64_t rmcm_mem_in_use(const rmcm_handle *h) { return h ? h->in_use : 0; }
RMCM_API int64_t rmcm_mem_peak(rmcm_handle *h, int32_t reset) {
    if (!h) return 0;
    const int64_t p = h->peak;
    if (reset) h->peak = h->in_use;
    return p;
}
RMCM_API int64_t rmcm_kernel_launches(const rmcm_handle *h) { return h ? h->launches : 0; }

RMCM_API int32_t rmcm_set_profiling(rmcm_handle *h, int32_t level) {
    if (!h || level < 0 || level > 2) return RMCM_EINVAL;
    h->prof_level = level;
    return RMCM_OK;
}

RMCM_API int32_t rmcm_get_product_stats(rmcm_handle *h, rmcm_product_stats *out, int32_t cap, int32_t *count,
                                        int32_t reset) {
    if (!h) return RMCM_EINVAL;
    RMCM_CUDA(h, cudaStreamSynchronize(h->stream));
    const int32_t n = (int32_t)h->prof.size();
    if (count) *count = n;
    for (int32_t i = 0; i < n && out && i < cap; i++) {
        rmcm::ProdRecord &r = h->prof[i];
        float a = 0, b = 0, c = 0;
        if (cudaEventElapsedTime(&a, r.ev[0], r.ev[1]) != cudaSuccess) a = 0;
        if (cudaEventElapsedTime(&b, r.ev[2], r.ev[3]) != cudaSuccess) b = 0;
        if (cudaEventElapsedTime(&c, r.ev[4], r.ev[5]) != cudaSuccess) c = 0;
        float gm = 0;
        if (r.st.gemm_limbs > 0 && cudaEventElapsedTime(&gm, r.ev[6], r.ev[7]) != cudaSuccess) gm = 0;
        cudaGetLastError();   // an unrecorded event must not leak into later launch checks
        r.st.gemm_ms = gm;
        r.st.analyze_ms = a;
        r.st.symbolic_ms = b;
        r.st.numeric_ms = c;
        out[i] = r.st;
    }
    if (reset) {
        for (auto &r : h->prof)
            for (auto &e : r.ev)
                if (e) cudaEventDestroy(e);
        h->prof.clear();
    }
    return RMCM_OK;
}

RMCM_API int32_t rmcm_graph_load_text(rmcm_handle *h, const char *graph_file, const char *vertex_file,
                                      const char *edge_file, rmcm_graph **out) {
    if (!h || !out || !graph_file || !vertex_file || !edge_file) return RMCM_EINVAL;
    *out = nullptr;
    rmcm_graph *g = new rmcm_graph();
    g->h = h;
    int32_t rc = load_text(h, graph_file, vertex_file, edge_file, g);
    if (rc != RMCM_OK) {
        delete g;
        return rc;
    }
    h->graphs.insert(g);
    *out = g;
    return RMCM_OK;
}

RMCM_API int32_t rmcm_graph_from_adjacency(rmcm_handle *h, int64_t n, const int32_t *vtype, const int64_t *adj_ptr,
                                           const int32_t *adj_nbr, const int32_t *adj_et, rmcm_graph **out) {
    if (!h || !out || n < 0 || (n > 0 && (!vtype || !adj_ptr))) return set_error(h, RMCM_EINVAL, "graph: bad arguments");
    *out = nullptr;
    const int64_t m = n > 0 ? adj_ptr[n] : 0;
    if (m > 0 && (!adj_nbr || !adj_et)) return set_error(h, RMCM_EINVAL, "graph: missing adjacency arrays");
    rmcm_graph *g = new rmcm_graph();
    g->h = h;
    g->n = n;
    g->m = m;
    g->vtype.assign(vtype, vtype + n);
    g->adj_ptr.assign(adj_ptr, adj_ptr + n + 1);
    g->adj_nbr.assign(adj_nbr, adj_nbr + m);
    g->adj_et.assign(adj_et, adj_et + m);
    g->max_vt = 0;
    bool ok = adj_ptr[0] == 0;
    for (int64_t v = 0; v < n && ok; v++) {
        ok = vtype[v] >= 0 && vtype[v] <= 1000000 && adj_ptr[v + 1] >= adj_ptr[v];
        g->max_vt = std::max(g->max_vt, vtype[v]);
    }
    for (int64_t q = 0; q < m && ok; q++) ok = adj_nbr[q] >= 0 && adj_nbr[q] < n;
    if (!ok) {
        delete g;
        return set_error(h, RMCM_EINVAL, "graph: vertex type, row pointer or neighbour id out of range");
    }
    graph_finish(g);
    h->graphs.insert(g);
    *out = g;
    return RMCM_OK;
}

RMCM_API int32_t rmcm_graph_free(rmcm_graph *g) {
    if (!g) return RMCM_OK;
    if (g->batches > 0) {
        if (g->h) set_error(g->h, RMCM_EINVAL, "graph_free: free the batches recorded on this graph first");
        return RMCM_EINVAL;
    }
    if (g->h) {
        for (auto &kv : g->leaves) mat_release(g->h, kv.second);
        if (g->h->stream) cudaStreamSynchronize(g->h->stream);
        g->h->graphs.erase(g);
    }
    delete g;
    return RMCM_OK;
}

RMCM_API int32_t rmcm_graph_info(const rmcm_graph *g, int64_t *n, int64_t *m, int32_t *max_vt) {
    if (!g) return RMCM_EINVAL;
    if (n) *n = g->n;
    if (m) *m = g->m;
    if (max_vt) *max_vt = g->max_vt;
    return RMCM_OK;
}

RMCM_API int64_t rmcm_graph_dim(const rmcm_graph *g, int32_t vt) {
    if (!g || vt < 0 || vt > g->max_vt) return 0;
    return g->dims[vt];
}

RMCM_API int32_t rmcm_metapath_parse(const char *s, int32_t *vts, int32_t *ets, int32_t cap, int32_t *len) {
    std::vector<int32_t> v, e;
    int32_t rc = parse_path(s, v, e);
    if (rc != RMCM_OK) return rc;
    if ((int64_t)e.size() > cap) return RMCM_EINVAL;
    if (vts) std::copy(v.begin(), v.end(), vts);
    if (ets) std::copy(e.begin(), e.end(), ets);
    if (len) *len = (int32_t)e.size();
    return RMCM_OK;
}

RMCM_API int32_t rmcm_metapath_format(const int32_t *vts, const int32_t *ets, int32_t len, char *buf, int64_t cap) {
    // MetaPath::toString, efficient/resmcm.cpp:301-308
    if (!vts || (len > 0 && !ets) || len < 0 || !buf || cap <= 0) return RMCM_EINVAL;
    std::string str;
    for (int i = 0; i < len; i++) str += std::to_string(vts[i]) + "-" + std::to_string(ets[i]) + "-";
    str += std::to_string(vts[len]);
    if ((int64_t)str.size() + 1 > cap) return RMCM_EINVAL;
    memcpy(buf, str.c_str(), str.size() + 1);
    return RMCM_OK;
}

RMCM_API int32_t rmcm_leaf(rmcm_handle *h, rmcm_graph *g, int32_t src_vt, int32_t sink_vt, int32_t et,
                           int32_t valtype, rmcm_mat **out) {
    if (!h || !g || !out || (valtype != RMCM_VAL_U32 && valtype != RMCM_VAL_U64)) return RMCM_EINVAL;
    return get_leaf(h, g, src_vt, sink_vt, et, valtype, out);
}

RMCM_API int32_t rmcm_mat_upload(rmcm_handle *h, int64_t rows, int64_t cols, const int64_t *rowptr,
                                 const int32_t *col, const void *val, int32_t valtype, rmcm_mat **out) {
    if (!h || !out || rows < 0 || cols < 0 || cols > INT32_MAX || !rowptr || (valtype != RMCM_VAL_U32 && valtype != RMCM_VAL_U64))
        return set_error(h, RMCM_EINVAL, "upload: bad arguments");
    *out = nullptr;
    const int64_t nnz = rowptr[rows];
    if (rowptr[0] != 0 || nnz < 0 || (nnz > 0 && !col)) return set_error(h, RMCM_EINVAL, "upload: bad row pointer");
    // copy, then validate on the device (rows ascending, columns in range);
    // rows that are not ascending are sorted here and uploaded again
    CsrFlags ck;
    {
        rmcm_mat *m = nullptr;
        RMCM_TRY(upload_csr(h, rows, cols, rowptr, col, val, valtype, &m, &ck));
        if (!ck.bad && !ck.unsorted) {
            if (val) m->positive = !ck.zero;
            m->distinct = !ck.dup;
            *out = m;
            return RMCM_OK;
        }
        mat_release(h, m);
    }
    if (ck.bad) return set_error(h, RMCM_EINVAL, "upload: row pointer not monotone or column out of range");
    const bool positive = !ck.zero;
    int dup = 0;
    std::vector<int32_t> c2(col, col + nnz);
    std::vector<char> v2;
    const int64_t vb = val_bytes(valtype);
    if (val) v2.assign((const char *)val, (const char *)val + vb * nnz);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t r = 0; r < rows; r++) {
        const int64_t a = rowptr[r], b = rowptr[r + 1];
        std::vector<int64_t> idx(b - a);
        for (int64_t q = 0; q < b - a; q++) idx[q] = a + q;
        std::stable_sort(idx.begin(), idx.end(), [&](int64_t x, int64_t y) { return col[x] < col[y]; });
        for (int64_t q = 0; q < b - a; q++) {
            c2[a + q] = col[idx[q]];
            if (val) memcpy(&v2[(a + q) * vb], (const char *)val + idx[q] * vb, vb);
        }
    }
#pragma omp parallel for schedule(dynamic, 4096) reduction(| : dup)
    for (int64_t r = 0; r < rows; r++)
        for (int64_t q = rowptr[r] + 1; q < rowptr[r + 1]; q++) dup |= c2[q] == c2[q - 1];
    int32_t rc = upload_csr(h, rows, cols, rowptr, c2.data(), val ? v2.data() : nullptr, valtype, out, nullptr);
    if (rc == RMCM_OK) {
        if (val) (*out)->positive = positive;
        (*out)->distinct = !dup;
    }
    return rc;
}

RMCM_API int32_t rmcm_mat_info(const rmcm_mat *m, int64_t *rows, int64_t *cols, int64_t *nnz, int32_t *valtype) {
    if (!m) return RMCM_EINVAL;
    if (rows) *rows = m->d.rows;
    if (cols) *cols = m->d.cols;
    if (nnz) *nnz = m->d.nnz;
    if (valtype) *valtype = m->valtype;
    return RMCM_OK;
}

RMCM_API int32_t rmcm_mat_download(rmcm_handle *h, const rmcm_mat *m, int64_t *rowptr, int32_t *col, void *val) {
    if (!h || !m) return RMCM_EINVAL;
    cudaStream_t s = h->stream;
    if (rowptr) RMCM_CUDA(h, cudaMemcpyAsync(rowptr, m->d.rowptr, 8 * (m->d.rows + 1), cudaMemcpyDeviceToHost, s));
    if (col && m->d.nnz) RMCM_CUDA(h, cudaMemcpyAsync(col, m->d.col, 4 * m->d.nnz, cudaMemcpyDeviceToHost, s));
    if (val && m->d.nnz)
        RMCM_CUDA(h, cudaMemcpyAsync(val, m->d.val, val_bytes(m->valtype) * m->d.nnz, cudaMemcpyDeviceToHost, s));
    RMCM_CUDA(h, cudaStreamSynchronize(s));
    return RMCM_OK;
}

namespace {

// Releases deferred matrices whose download has landed (all of them when
// `all`, after the transfer stream has been synchronised).
void release_deferred(rmcm_handle *h, bool all) {
    auto &d = h->deferred;
    size_t keep = 0;
    for (size_t i = 0; i < d.size(); i++) {
        if (all || cudaEventQuery(d[i]->xfer_done) == cudaSuccess) mat_release(h, d[i]);
        else d[keep++] = d[i];
    }
    d.resize(keep);
    cudaGetLastError();   // cudaErrorNotReady from the queries is not an error
}

}  // namespace

RMCM_API int32_t rmcm_mat_free(rmcm_handle *h, rmcm_mat *m) {
    if (!h || !m) return RMCM_EINVAL;
    if (m->graph_owned) return set_error(h, RMCM_EINVAL, "leaf matrices are owned by their graph");
    release_deferred(h, false);
    if (m->xfer_done && cudaEventQuery(m->xfer_done) == cudaErrorNotReady) {
        cudaGetLastError();
        h->deferred.push_back(m);   // released once its download has landed
        return RMCM_OK;
    }
    mat_release(h, m);
    return RMCM_OK;
}

RMCM_API int32_t rmcm_mat_download_async(rmcm_handle *h, rmcm_mat *m, int64_t *rowptr, int32_t *col, void *val) {
    if (!h || !m) return RMCM_EINVAL;
    // the copies start once the work already queued on the handle's stream is done
    RMCM_CUDA(h, cudaEventRecord(h->ev_fork, h->stream));
    RMCM_CUDA(h, cudaStreamWaitEvent(h->xfer, h->ev_fork, 0));
    cudaStream_t x = h->xfer;
    {
        // pinned destinations: SM stores (k_copy_out), so the copy engines stay
        // free for the executor's small read-backs on the handle's stream
        const void *src[3] = {m->d.rowptr, m->d.col, m->d.val};
        void *dst[3] = {rowptr, m->d.nnz ? col : nullptr, m->d.nnz ? val : nullptr};
        const int64_t bytes[3] = {8 * (m->d.rows + 1), 4 * m->d.nnz, val_bytes(m->valtype) * m->d.nnz};
        if (copy_out_launch(src, dst, bytes, x)) {
            h->launches++;
            if (!m->xfer_done) RMCM_CUDA(h, cudaEventCreateWithFlags(&m->xfer_done, cudaEventDisableTiming));
            RMCM_CUDA(h, cudaEventRecord(m->xfer_done, x));
            return RMCM_OK;
        }
    }
    // pieces of at most 8 MB: the executor's small read-backs on the
    // handle's stream get the copy engine between them
    auto copy = [&](void *dst, const void *src, int64_t bytes) -> int32_t {
        constexpr int64_t kPiece = 8LL << 20;
        for (int64_t o = 0; o < bytes; o += kPiece)
            RMCM_CUDA(h, cudaMemcpyAsync((char *)dst + o, (const char *)src + o, std::min(kPiece, bytes - o),
                                         cudaMemcpyDeviceToHost, x));
        return RMCM_OK;
    };
    if (rowptr) RMCM_TRY(copy(rowptr, m->d.rowptr, 8 * (m->d.rows + 1)));
    if (col && m->d.nnz) RMCM_TRY(copy(col, m->d.col, 4 * m->d.nnz));
    if (val && m->d.nnz) RMCM_TRY(copy(val, m->d.val, val_bytes(m->valtype) * m->d.nnz));
    if (!m->xfer_done) RMCM_CUDA(h, cudaEventCreateWithFlags(&m->xfer_done, cudaEventDisableTiming));
    RMCM_CUDA(h, cudaEventRecord(m->xfer_done, x));
    return RMCM_OK;
}

RMCM_API int32_t rmcm_synchronize(rmcm_handle *h) {
    if (!h) return RMCM_EINVAL;
    RMCM_CUDA(h, cudaStreamSynchronize(h->stream));
    RMCM_CUDA(h, cudaStreamSynchronize(h->xfer));
    release_deferred(h, true);
    return RMCM_OK;
}

RMCM_API int32_t rmcm_transfers_wait(rmcm_handle *h) {
    if (!h) return RMCM_EINVAL;
    RMCM_CUDA(h, cudaStreamSynchronize(h->xfer));
    release_deferred(h, true);
    return RMCM_OK;
}

RMCM_API int32_t rmcm_estimate(rmcm_handle *h, rmcm_mat *const *chain, int32_t len, double *c_out) {
    if (!h || !chain || !c_out) return RMCM_EINVAL;
    double *c_dev = nullptr;
    RMCM_TRY(dev_alloc(h, (void **)&c_dev, 8 * 256));
    int32_t rc = estimate(h, chain, len, c_dev);
    if (rc == RMCM_OK) {
        cudaError_t e = cudaMemcpyAsync(c_out, c_dev, sizeof(double) * len * len, cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) rc = cuda_error(h, e, "estimate download");
    }
    dev_free(h, c_dev, 8 * 256);
    return rc;
}

RMCM_API int32_t rmcm_order(rmcm_handle *h, const double *c, int32_t len, int32_t *split, double *cost,
                            int32_t *pairs) {
    if (!h || !c || len < 1 || len > 16) return set_error(h, RMCM_EINVAL, "order: bad arguments");
    char *buf = nullptr;
    const int64_t bytes = 8 * 256 + 4 * 256 + 8 * 256 + 4 * 64;
    RMCM_TRY(dev_alloc(h, (void **)&buf, bytes));
    double *c_dev = (double *)buf;
    int32_t *s_dev = (int32_t *)(buf + 8 * 256);
    double *m_dev = (double *)(buf + 8 * 256 + 4 * 256);
    int32_t *p_dev = (int32_t *)(buf + 8 * 256 + 4 * 256 + 8 * 256);
    cudaStream_t s = h->stream;
    int32_t rc = RMCM_OK;
    cudaError_t e = cudaMemcpyAsync(c_dev, c, sizeof(double) * len * len, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) rc = cuda_error(h, e, "order upload");
    if (rc == RMCM_OK) rc = chain_order_dev(h, c_dev, len, s_dev, m_dev, p_dev);
    if (rc == RMCM_OK) {
        e = cudaSuccess;
        if (split) e = cudaMemcpyAsync(split, s_dev, 4 * len * len, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && cost) e = cudaMemcpyAsync(cost, m_dev, 8 * len * len, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && pairs && len > 1) e = cudaMemcpyAsync(pairs, p_dev, 4 * 2 * (len - 1), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_error(h, e, "order download");
    }
    dev_free(h, buf, bytes);
    return rc;
}

RMCM_API int32_t rmcm_spgemm(rmcm_handle *h, const rmcm_mat *A, const rmcm_mat *B, rmcm_mat **C) {
    if (!h || !C) return RMCM_EINVAL;
    *C = nullptr;
    int32_t rc = spgemm(h, A, B, C, nullptr);
    if (rc != RMCM_OK) return rc;
    rc = check_status(h);
    if (rc == RMCM_EOVERFLOW) (*C)->positive = false;   // wrapped counts may be 0
    if (rc != RMCM_OK && rc != RMCM_EOVERFLOW) {
        mat_release(h, *C);
        *C = nullptr;
    }
    return rc;
}

RMCM_API int32_t rmcm_chain(rmcm_handle *h, rmcm_mat *const *chain, int32_t len, const int32_t *pairs,
                            rmcm_mat **C, rmcm_timings *t) {
    if (!h || !chain || !C) return RMCM_EINVAL;
    int32_t rc = chain_exec(h, chain, len, pairs, C, t, h->valtype == RMCM_VAL_AUTO, nullptr);
    if (rc != RMCM_OK && rc != RMCM_EOVERFLOW && *C) {
        mat_release(h, *C);
        *C = nullptr;
    }
    return rc;
}

RMCM_API int32_t rmcm_run_metapath(rmcm_handle *h, rmcm_graph *g, const char *metapath, rmcm_mat **C,
                                   rmcm_timings *t) {
    if (!h || !g || !metapath) return RMCM_EINVAL;
    if (C) *C = nullptr;
    std::vector<int32_t> vts, ets;
    if (parse_path(metapath, vts, ets) != RMCM_OK)
        return set_error(h, RMCM_EINVAL, std::string("the meta-path is incorrect: ") + metapath);
    const int len = (int)ets.size();
    if (len < 1 || len > 16) return set_error(h, RMCM_EINVAL, "meta-path must have 1..16 edge types");
    const int32_t vt = h->valtype == RMCM_VAL_U64 ? RMCM_VAL_U64 : RMCM_VAL_U32;
    const bool widen = h->valtype == RMCM_VAL_AUTO;
    std::vector<rmcm_mat *> mats(len);
    for (int i = 0; i < len; i++) RMCM_TRY(get_leaf(h, g, vts[i], vts[i + 1], ets[i], vt, &mats[i]));
    auto leaf64 = [&](int i, rmcm_mat **out) { return get_leaf(h, g, vts[i], vts[i + 1], ets[i], RMCM_VAL_U64, out); };
    rmcm_mat *res = nullptr;
    int32_t rc = chain_exec(h, mats.data(), len, nullptr, &res, t, widen, leaf64);
    if (res && (rc == RMCM_OK || rc == RMCM_EOVERFLOW)) {
        if (C) *C = res;
        else mat_release(h, res);
    } else if (res) {
        mat_release(h, res);
    }
    return rc;
}

RMCM_API int32_t rmcm_run_metapath_blocks(rmcm_handle *h, rmcm_graph *g, const char *metapath,
                                          int64_t rows_per_block, rmcm_block_fn fn, void *user, rmcm_timings *t) {
    if (!h || !g || !metapath || !fn) return RMCM_EINVAL;
    std::vector<int32_t> vts, ets;
    if (parse_path(metapath, vts, ets) != RMCM_OK)
        return set_error(h, RMCM_EINVAL, std::string("the meta-path is incorrect: ") + metapath);
    const int len = (int)ets.size();
    if (len < 1 || len > 16) return set_error(h, RMCM_EINVAL, "meta-path must have 1..16 edge types");
    const int32_t vt = h->valtype == RMCM_VAL_U64 ? RMCM_VAL_U64 : RMCM_VAL_U32;
    const bool widen = h->valtype == RMCM_VAL_AUTO;
    std::vector<rmcm_mat *> mats(len);
    for (int i = 0; i < len; i++) RMCM_TRY(get_leaf(h, g, vts[i], vts[i + 1], ets[i], vt, &mats[i]));
    auto leaf64 = [&](int i, rmcm_mat **out) { return get_leaf(h, g, vts[i], vts[i + 1], ets[i], RMCM_VAL_U64, out); };
    if (len == 1) {
        // the leaf is the result: one block
        rmcm_timings tm{};
        tm.nnz = mats[0]->d.nnz;
        tm.valtype = vt;
        const int32_t urc = fn(user, 0, mats[0]);
        if (t) *t = tm;
        return urc == RMCM_OK ? RMCM_OK : set_error(h, urc, "the block sink stopped the chain");
    }
    BlockSink sink;
    sink.rows_per_block = rows_per_block;
    sink.fn = fn;
    sink.user = user;
    rmcm_mat *res = nullptr;
    int32_t rc = chain_exec(h, mats.data(), len, nullptr, &res, t, widen, leaf64, nullptr, false, &sink);
    if (res) mat_release(h, res);
    return rc;
}

RMCM_API int32_t rmcm_mat_digest_rows(rmcm_handle *h, const rmcm_mat *m, int64_t row0, uint64_t *nnz,
                                      uint64_t *digest) {
    if (!h || !m || row0 < 0) return RMCM_EINVAL;
    uint64_t *d = nullptr;
    RMCM_TRY(dev_alloc(h, (void **)&d, 16));
    int32_t rc = mat_digest_launch(h, m, d, row0);
    if (rc == RMCM_OK) {
        cudaError_t e = cudaMemcpyAsync(h->h_pinned, d, 16, cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) rc = cuda_error(h, e, "digest download");
    }
    dev_free(h, d, 16);
    if (rc != RMCM_OK) return rc;
    if (nnz) *nnz = (uint64_t)h->h_pinned[0];
    if (digest) *digest = (uint64_t)h->h_pinned[1];
    return RMCM_OK;
}

RMCM_API int32_t rmcm_set_order_mode(rmcm_handle *h, int32_t mode) {
    if (!h || mode < RMCM_ORDER_RES || mode > RMCM_ORDER_DENSE) return RMCM_EINVAL;
    h->order_mode = mode;
    return RMCM_OK;
}

RMCM_API int32_t rmcm_order_l2r(int32_t len, int32_t *pairs) {
    if (len < 2 || !pairs) return RMCM_EINVAL;
    pairs[0] = 0;
    pairs[1] = 1;
    for (int32_t i = 2; i < len; i++) {
        pairs[2 * (i - 1)] = -1;
        pairs[2 * (i - 1) + 1] = i;
    }
    return RMCM_OK;
}

RMCM_API int32_t rmcm_order_dense(const int64_t *dims_vt, int32_t len, int32_t *split, double *cost, int32_t *pairs) {
    if (!dims_vt || len < 1 || len > 64) return RMCM_EINVAL;
    std::vector<int32_t> sp;
    std::vector<double> m;
    dense_order(dims_vt, len, sp, m);
    if (split) std::copy(sp.begin(), sp.end(), split);
    if (cost) std::copy(m.begin(), m.end(), cost);
    if (pairs && len > 1) {
        std::vector<int32_t> pl;
        post_order(sp, len, 0, len - 1, pl);
        std::copy(pl.begin(), pl.end(), pairs);
    }
    return RMCM_OK;
}

RMCM_API int32_t rmcm_graph_save(const rmcm_graph *g, const char *path) {
    if (!g || !path) return RMCM_EINVAL;
    FILE *f = fopen(path, "wb");
    if (!f) return RMCM_EIO;
    const char magic[8] = {'R', 'M', 'C', 'M', 'H', 'I', 'N', '1'};
    const int64_t hdr[2] = {g->n, g->m};
    const int32_t hdr2[2] = {g->max_vt, 0};
    bool ok = fwrite(magic, 1, 8, f) == 8 && fwrite(hdr, 8, 2, f) == 2 && fwrite(hdr2, 4, 2, f) == 2;
    ok = ok && (g->n == 0 || fwrite(g->vtype.data(), 4, g->n, f) == (size_t)g->n);
    ok = ok && fwrite(g->adj_ptr.data(), 8, g->n + 1, f) == (size_t)(g->n + 1);
    ok = ok && (g->m == 0 || fwrite(g->adj_nbr.data(), 4, g->m, f) == (size_t)g->m);
    ok = ok && (g->m == 0 || fwrite(g->adj_et.data(), 4, g->m, f) == (size_t)g->m);
    ok = (fclose(f) == 0) && ok;
    return ok ? RMCM_OK : RMCM_EIO;
}

RMCM_API int32_t rmcm_graph_load(rmcm_handle *h, const char *path, rmcm_graph **out) {
    if (!h || !path || !out) return RMCM_EINVAL;
    *out = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) return set_error(h, RMCM_EIO, std::string("cannot open ") + path);
    char magic[8];
    int64_t hdr[2];
    int32_t hdr2[2];
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, "RMCMHIN1", 8) != 0 || fread(hdr, 8, 2, f) != 2 ||
        fread(hdr2, 4, 2, f) != 2 || hdr[0] < 0 || hdr[1] < 0) {
        fclose(f);
        return set_error(h, RMCM_EPARSE, std::string("not a graph cache file: ") + path);
    }
    const int64_t n = hdr[0], m = hdr[1];
    std::vector<int32_t> vt(n), nbr(m), et(m);
    std::vector<int64_t> ptr(n + 1);
    bool ok = (n == 0 || fread(vt.data(), 4, n, f) == (size_t)n) && fread(ptr.data(), 8, n + 1, f) == (size_t)(n + 1) &&
              (m == 0 || fread(nbr.data(), 4, m, f) == (size_t)m) && (m == 0 || fread(et.data(), 4, m, f) == (size_t)m);
    fclose(f);
    if (!ok || ptr[n] != m) return set_error(h, RMCM_EPARSE, std::string("truncated graph cache file: ") + path);
    return rmcm_graph_from_adjacency(h, n, vt.data(), ptr.data(), nbr.data(), et.data(), out);
}

RMCM_API int32_t rmcm_graph_global_ids(const rmcm_graph *g, int32_t vt, int32_t *out) {
    if (!g || !out || vt < 0 || vt > g->max_vt) return RMCM_EINVAL;
    std::copy(g->bin_ids.begin() + g->bin_ptr[vt], g->bin_ids.begin() + g->bin_ptr[vt + 1], out);
    return RMCM_OK;
}

RMCM_API int32_t rmcm_mat_save(rmcm_handle *h, const rmcm_mat *m, const char *path) {
    if (!h || !m || !path) return RMCM_EINVAL;
    std::vector<int64_t> rp(m->d.rows + 1);
    std::vector<int32_t> col(std::max<int64_t>(m->d.nnz, 1));
    std::vector<char> val(std::max<int64_t>(m->d.nnz * val_bytes(m->valtype), 1));
    RMCM_TRY(rmcm_mat_download(h, m, rp.data(), col.data(), val.data()));
    FILE *f = fopen(path, "wb");
    if (!f) return set_error(h, RMCM_EIO, std::string("cannot write ") + path);
    const char magic[8] = {'R', 'M', 'C', 'M', 'C', 'S', 'R', '1'};
    const int64_t hdr[3] = {m->d.rows, m->d.cols, m->d.nnz};
    const int32_t hdr2[2] = {m->valtype, 0};
    bool ok = fwrite(magic, 1, 8, f) == 8 && fwrite(hdr, 8, 3, f) == 3 && fwrite(hdr2, 4, 2, f) == 2 &&
              fwrite(rp.data(), 8, rp.size(), f) == rp.size();
    ok = ok && (m->d.nnz == 0 || (fwrite(col.data(), 4, m->d.nnz, f) == (size_t)m->d.nnz &&
                                  fwrite(val.data(), val_bytes(m->valtype), m->d.nnz, f) == (size_t)m->d.nnz));
    ok = (fclose(f) == 0) && ok;
    return ok ? RMCM_OK : set_error(h, RMCM_EIO, std::string("short write to ") + path);
}

RMCM_API int32_t rmcm_estimate_metapath(rmcm_handle *h, rmcm_graph *g, const char *metapath, double *est_nnz) {
    if (!h || !g || !metapath || !est_nnz) return RMCM_EINVAL;
    std::vector<int32_t> vts, ets;
    if (parse_path(metapath, vts, ets) != RMCM_OK)
        return set_error(h, RMCM_EINVAL, std::string("the meta-path is incorrect: ") + metapath);
    const int len = (int)ets.size();
    if (len < 1 || len > 16) return set_error(h, RMCM_EINVAL, "meta-path must have 1..16 edge types");
    std::vector<rmcm_mat *> mats(len);
    for (int i = 0; i < len; i++) RMCM_TRY(get_leaf(h, g, vts[i], vts[i + 1], ets[i], RMCM_VAL_U32, &mats[i]));
    std::vector<double> c(len * len, 0.0);
    RMCM_TRY(rmcm_estimate(h, mats.data(), len, c.data()));
    *est_nnz = c[len - 1];   // c_[len - 1] = c[0][len-1], accuracy/res.cpp:522
    return RMCM_OK;
}

}  // extern "C"

// ===========================================================================
// Batches: many meta-paths over one graph, recorded once and replayed as one
// CUDA graph over concurrent lanes.
// ===========================================================================

struct rmcm_batch {
    rmcm_handle *h = nullptr;
    rmcm_graph *g = nullptr;
    std::vector<std::string> paths;
    std::vector<ChainLog> logs;
    std::vector<int32_t> lane_of;
    std::vector<rmcm_handle *> lanes;
    std::vector<int64_t> scratch_need;      // per lane
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaEvent_t> fork_join;     // 1 fork + one join per lane
    uint64_t *d_digest = nullptr;           // 2 per chain
    uint64_t *h_digest = nullptr;           // pinned mirror
    int64_t launches_per_run = 0;
    int64_t nodes = 0;
    int64_t runs = 0;
    rmcm::FusedBatch *fused = nullptr;      // rmcm_batch_create_fused: everything lives here
};

namespace {

void batch_release(rmcm_batch *b) {
    rmcm_handle *h = b->h;
    if (b->fused) fused_free(h, b->fused);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (auto e : b->fork_join)
        if (e) cudaEventDestroy(e);
    for (rmcm_handle *l : b->lanes) rmcm_destroy(l);
    if (b->d_digest) {
        dev_free(h, b->d_digest, 16 * (int64_t)b->paths.size());
        cudaStreamSynchronize(h->stream);
    }
    if (b->h_digest) cudaFreeHost(b->h_digest);
    if (b->g) b->g->batches--;
    h->batches.erase(b);
    delete b;
}

// Captures every lane's chains into one CUDA graph: a fork event on the
// handle's stream, each lane replaying its chains in order on its own
// stream, a join back, then one copy of all digests to pinned host memory.
int32_t batch_capture(rmcm_batch *b) {
    rmcm_handle *h = b->h;
    const int K = (int)b->lanes.size();
    // scratch is grown outside the capture: a replay never allocates it
    for (int k = 0; k < K; k++) {
        RMCM_TRY(scratch_reserve(b->lanes[k], b->scratch_need[k]));
        RMCM_CUDA(h, cudaStreamSynchronize(b->lanes[k]->stream));
    }
    const int64_t launches0 = [&] {
        int64_t x = 0;
        for (auto *l : b->lanes) x += l->launches;
        return x;
    }();
    RMCM_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int32_t rc = RMCM_OK;
    cudaError_t e = cudaEventRecord(b->fork_join[0], h->stream);
    std::vector<bool> forked(K, false);
    for (int k = 0; k < K && e == cudaSuccess; k++) {
        e = cudaStreamWaitEvent(b->lanes[k]->stream, b->fork_join[0], 0);
        forked[k] = e == cudaSuccess;
    }
    if (e != cudaSuccess) rc = cuda_error(h, e, "batch fork");
    for (size_t i = 0; i < b->logs.size() && rc == RMCM_OK; i++) {
        rmcm_handle *l = b->lanes[b->lane_of[i]];
        rc = chain_replay(l, b->logs[i], b->d_digest + 2 * i, false, nullptr);
        if (rc != RMCM_OK) set_error(h, rc, "batch capture: " + b->paths[i] + ": " + l->last_error);
    }
    for (int k = 0; k < K; k++) {
        if (!forked[k]) continue;
        cudaEventRecord(b->fork_join[1 + k], b->lanes[k]->stream);
        cudaStreamWaitEvent(h->stream, b->fork_join[1 + k], 0);
    }
    if (rc == RMCM_OK) {
        e = cudaMemcpyAsync(b->h_digest, b->d_digest, 16 * b->paths.size(), cudaMemcpyDeviceToHost, h->stream);
        if (e != cudaSuccess) rc = cuda_error(h, e, "batch digest copy");
    }
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(h->stream, &graph);
    if (rc == RMCM_OK && e != cudaSuccess) rc = cuda_error(h, e, "cudaStreamEndCapture");
    if (rc != RMCM_OK) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return rc;
    }
    b->graph = graph;
    e = cudaGraphInstantiate(&b->exec, graph, 0);
    if (e != cudaSuccess) {
        b->exec = nullptr;
        return cuda_error(h, e, "cudaGraphInstantiate");
    }
    size_t nodes = 0;
    cudaGraphGetNodes(graph, nullptr, &nodes);
    b->nodes = (int64_t)nodes;
    int64_t launches1 = 0;
    for (auto *l : b->lanes) launches1 += l->launches;
    b->launches_per_run = launches1 - launches0;
    return RMCM_OK;
}

}  // namespace

RMCM_API int32_t rmcm_set_tuning(rmcm_handle *h, const rmcm_tuning *t) {
    if (!h || !t) return RMCM_EINVAL;
    const int32_t g = t->threads_per_row;
    if (g != 1 && g != 2 && g != 4 && g != 8 && g != 16 && g != 32 && g != 128)
        return set_error(h, RMCM_EINVAL, "tuning: threads_per_row must be 1, 2, 4, 8, 16, 32 or 128");
    if (t->hash_max_flops < 32 || t->hash_max_flops > (1 << 20))
        return set_error(h, RMCM_EINVAL, "tuning: hash_max_flops must be in 32 .. 1048576");
    if (t->dense_ratio < 1) return set_error(h, RMCM_EINVAL, "tuning: dense_ratio must be >= 1");
    if (!(t->hash_load >= 0.1 && t->hash_load <= 0.75))
        return set_error(h, RMCM_EINVAL, "tuning: hash_load must be in 0.1 .. 0.75");
    if (t->warp_max_flops < 0 || t->warp_max_flops > 65536)
        return set_error(h, RMCM_EINVAL, "tuning: warp_max_flops must be in 0 .. 65536");
    if (t->gemm_inv_density < 0 || t->gemm_inv_density > 65536)
        return set_error(h, RMCM_EINVAL, "tuning: gemm_inv_density must be in 0 .. 65536");
    if (t->gemm_min_mflops < 0) return set_error(h, RMCM_EINVAL, "tuning: gemm_min_mflops must be >= 0");
    h->tune.gemm_inv_density = t->gemm_inv_density;
    h->tune.gemm_min_mflops = t->gemm_min_mflops;
    h->tune.threads_per_row = g;
    h->tune.warp_max_flops = t->warp_max_flops;
    h->tune.hash_max_flops = t->hash_max_flops;
    h->tune.dense_ratio = t->dense_ratio;
    h->tune.hash_load = t->hash_load;
    return RMCM_OK;
}

RMCM_API int32_t rmcm_get_tuning(const rmcm_handle *h, rmcm_tuning *t) {
    if (!h || !t) return RMCM_EINVAL;
    t->threads_per_row = h->tune.threads_per_row;
    t->hash_max_flops = h->tune.hash_max_flops;
    t->dense_ratio = h->tune.dense_ratio;
    t->warp_max_flops = h->tune.warp_max_flops;
    t->hash_load = h->tune.hash_load;
    t->gemm_inv_density = h->tune.gemm_inv_density;
    t->gemm_min_mflops = h->tune.gemm_min_mflops;
    return RMCM_OK;
}

RMCM_API int32_t rmcm_batch_create_fused(rmcm_handle *h, rmcm_graph *g, const char *const *metapaths, int32_t count,
                                         rmcm_batch **out) {
    if (!h || !g || !metapaths || count < 1 || !out) return RMCM_EINVAL;
    *out = nullptr;
    if (g->h != h) return set_error(h, RMCM_EINVAL, "batch: the graph belongs to another handle");
    if (h->order_mode != RMCM_ORDER_RES) return set_error(h, RMCM_EINVAL, "batch: only the RES order is batched");
    rmcm_batch *b = new rmcm_batch();
    b->h = h;
    b->g = g;
    g->batches++;
    h->batches.insert(b);
    for (int32_t i = 0; i < count; i++) b->paths.emplace_back(metapaths[i] ? metapaths[i] : "");
    int32_t rc = fused_create(h, g, metapaths, count, &b->fused);
    if (rc != RMCM_OK) {
        const std::string why = h->last_error;
        batch_release(b);
        h->last_error = why;
        return rc;
    }
    *out = b;
    return RMCM_OK;
}

RMCM_API int32_t rmcm_batch_create(rmcm_handle *h, rmcm_graph *g, const char *const *metapaths, int32_t count,
                                   int32_t lanes, rmcm_batch **out) {
    if (!h || !g || !metapaths || count < 1 || !out) return RMCM_EINVAL;
    *out = nullptr;
    if (g->h != h) return set_error(h, RMCM_EINVAL, "batch: the graph belongs to another handle");
    if (h->order_mode != RMCM_ORDER_RES) return set_error(h, RMCM_EINVAL, "batch: only the RES order is batched");
    if (lanes < 1) lanes = 8;
    lanes = std::min(lanes, std::min<int32_t>(count, 64));
    rmcm_batch *b = new rmcm_batch();
    b->h = h;
    b->g = g;
    g->batches++;
    h->batches.insert(b);
    const int32_t vt = h->valtype == RMCM_VAL_U64 ? RMCM_VAL_U64 : RMCM_VAL_U32;
    const bool widen = h->valtype == RMCM_VAL_AUTO;
    const int32_t prof = h->prof_level;
    h->prof_level = 0;
    int32_t rc = RMCM_OK;
    // record pass: every chain once through the ordinary executor
    std::vector<double> cost(count, 0.0);
    for (int32_t i = 0; i < count && rc == RMCM_OK; i++) {
        const char *mp = metapaths[i];
        std::vector<int32_t> vts, ets;
        if (!mp || parse_path(mp, vts, ets) != RMCM_OK) {
            rc = set_error(h, RMCM_EINVAL, std::string("the meta-path is incorrect: ") + (mp ? mp : "(null)"));
            break;
        }
        const int len = (int)ets.size();
        if (len < 1 || len > 16) {
            rc = set_error(h, RMCM_EINVAL, "meta-path must have 1..16 edge types");
            break;
        }
        std::vector<rmcm_mat *> mats(len);
        for (int j = 0; j < len && rc == RMCM_OK; j++) rc = get_leaf(h, g, vts[j], vts[j + 1], ets[j], vt, &mats[j]);
        if (rc != RMCM_OK) break;
        auto leaf64 = [&](int j, rmcm_mat **o) { return get_leaf(h, g, vts[j], vts[j + 1], ets[j], RMCM_VAL_U64, o); };
        b->paths.emplace_back(mp);
        b->logs.emplace_back();
        rmcm_mat *res = nullptr;
        rc = chain_exec(h, mats.data(), len, nullptr, &res, nullptr, widen, leaf64, &b->logs.back());
        if (res) mat_release(h, res);
        if (rc != RMCM_OK) {
            const std::string why = h->last_error;
            rc = set_error(h, rc, "batch record: " + std::string(mp) + ": " + why);
            break;
        }
        for (const LogOp &op : b->logs.back().ops)
            cost[i] += op.kind == LogOp::kSpgemm ? 2e6 + (double)op.plan.flops + 4.0 * (double)op.plan.nnz : 2e5;
    }
    h->prof_level = prof;
    // lanes: longest chains first onto the least-loaded lane
    if (rc == RMCM_OK) {
        rmcm_opts o{};
        o.device = h->device;
        o.valtype = h->valtype;
        o.mem_budget_bytes = h->budget;
        for (int k = 0; k < lanes && rc == RMCM_OK; k++) {
            rmcm_handle *l = nullptr;
            rc = rmcm_create(&l, &o);
            if (rc != RMCM_OK) {
                set_error(h, rc, "batch: could not create a lane");
                break;
            }
            l->tune = h->tune;
            b->lanes.push_back(l);
        }
    }
    if (rc == RMCM_OK) {
        std::vector<int32_t> idx(count);
        for (int32_t i = 0; i < count; i++) idx[i] = i;
        std::stable_sort(idx.begin(), idx.end(), [&](int32_t x, int32_t y) { return cost[x] > cost[y]; });
        std::vector<double> load(lanes, 0.0);
        b->lane_of.assign(count, 0);
        b->scratch_need.assign(lanes, 256);
        for (int32_t i : idx) {
            const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            b->lane_of[i] = k;
            load[k] += cost[i];
            for (const LogOp &op : b->logs[i].ops)
                if (op.kind == LogOp::kSpgemm) b->scratch_need[k] = std::max(b->scratch_need[k], op.plan.scratch_bytes);
        }
        b->fork_join.assign(1 + lanes, nullptr);
        for (auto &e : b->fork_join)
            if (rc == RMCM_OK && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
                rc = set_error(h, RMCM_ECUDA, "batch: event creation failed");
    }
    if (rc == RMCM_OK) rc = dev_alloc(h, (void **)&b->d_digest, 16 * (int64_t)count);
    if (rc == RMCM_OK && cudaMallocHost((void **)&b->h_digest, 16 * (size_t)count) != cudaSuccess) {
        b->h_digest = nullptr;
        rc = set_error(h, RMCM_ECUDA, "batch: pinned digest buffer");
    }
    if (rc == RMCM_OK) {
        RMCM_CUDA(h, cudaStreamSynchronize(h->stream));
        rc = batch_capture(b);
    }
    if (rc != RMCM_OK) {
        const std::string why = h->last_error;
        batch_release(b);
        h->last_error = why;
        return rc;
    }
    *out = b;
    return RMCM_OK;
}

RMCM_API int32_t rmcm_batch_run(rmcm_handle *h, rmcm_batch *b, int64_t *nnz_out, uint64_t *digest_out,
                                double *seconds) {
    if (!h || !b || b->h != h) return RMCM_EINVAL;
    if (b->fused) {
        b->runs++;
        return fused_run(h, b->fused, nnz_out, digest_out, seconds);
    }
    if (!b->exec) return RMCM_EINVAL;
    cudaEvent_t *ev = h->ev;
    RMCM_CUDA(h, cudaEventRecord(ev[6], h->stream));
    RMCM_CUDA(h, cudaGraphLaunch(b->exec, h->stream));
    RMCM_CUDA(h, cudaEventRecord(ev[7], h->stream));
    RMCM_CUDA(h, cudaStreamSynchronize(h->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, ev[6], ev[7]);
    if (seconds) *seconds = ms * 1e-3;
    h->launches += b->launches_per_run;
    b->runs++;
    for (size_t k = 0; k < b->lanes.size(); k++) {
        const int32_t st = check_status(b->lanes[k]);
        if (st != RMCM_OK) return set_error(h, st, "batch run: lane " + std::to_string(k) + ": " + b->lanes[k]->last_error);
    }
    const size_t n = b->paths.size();
    for (size_t i = 0; i < n; i++) {
        if ((int64_t)b->h_digest[2 * i] != b->logs[i].nnz)
            return set_error(h, RMCM_EINTERNAL, "batch run: result size of " + b->paths[i] + " differs from its record");
        if (nnz_out) nnz_out[i] = (int64_t)b->h_digest[2 * i];
        if (digest_out) digest_out[i] = b->h_digest[2 * i + 1];
    }
    return RMCM_OK;
}

RMCM_API int32_t rmcm_batch_info(const rmcm_batch *b, int32_t *count, int32_t *lanes, int64_t *launches_per_run,
                                 int64_t *graph_nodes) {
    if (!b) return RMCM_EINVAL;
    if (b->fused) {
        fused_info(b->fused, count, launches_per_run, graph_nodes);
        if (lanes) *lanes = 1;
        return RMCM_OK;
    }
    if (count) *count = (int32_t)b->paths.size();
    if (lanes) *lanes = (int32_t)b->lanes.size();
    if (launches_per_run) *launches_per_run = b->launches_per_run;
    if (graph_nodes) *graph_nodes = b->nodes;
    return RMCM_OK;
}

RMCM_API int32_t rmcm_batch_free(rmcm_handle *h, rmcm_batch *b) {
    if (!b) return RMCM_OK;
    if (!h || b->h != h) return RMCM_EINVAL;
    cudaStreamSynchronize(h->stream);
    batch_release(b);
    return RMCM_OK;
}

RMCM_API int32_t rmcm_mat_digest(rmcm_handle *h, const rmcm_mat *m, uint64_t *nnz, uint64_t *digest) {
    if (!h || !m) return RMCM_EINVAL;
    uint64_t *d = nullptr;
    RMCM_TRY(dev_alloc(h, (void **)&d, 16));
    int32_t rc = mat_digest_launch(h, m, d);
    if (rc == RMCM_OK) {
        cudaError_t e = cudaMemcpyAsync(h->h_pinned, d, 16, cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) rc = cuda_error(h, e, "digest download");
    }
    dev_free(h, d, 16);
    if (rc != RMCM_OK) return rc;
    if (nnz) *nnz = (uint64_t)h->h_pinned[0];
    if (digest) *digest = (uint64_t)h->h_pinned[1];
    return RMCM_OK;
}
