// Meta-path query server: per-edge-type CSRs resident on the GPU, queries
// admitted by the device bytes their RES estimates predict, and several
// queries in flight at once on concurrent lanes (continuous batching).
//
// The reference answers one meta-path at a time in main() (efficient/
// resmcm.cpp:839-889): estimate (rows_sparse_optimal_matrix_chain_order),
// order, multiply, print.  Each query here takes the same three steps on one
// lane — a worker thread with its own handle, CUDA stream and scratch — so
// a query's arithmetic is exactly that of rmcm_run_metapath.
//
// Admission.  A worker takes the oldest query, runs its estimator and DP on
// its lane, and computes the query's predicted bytes from the estimates:
// every intermediate and the result at 12 bytes per estimated entry (int32
// column + uint64 count) plus 8 bytes per row pointer and 40 bytes per row
// of SpGEMM scratch.  A query whose prediction exceeds the whole budget is
// rejected (RMCM_ENOMEM); one that does not fit the budget left now waits,
// and waiting queries are retried, oldest first, whenever a query finishes
// and returns its bytes.  While a query waits, workers go on admitting
// younger queries that fit, so the device stays busy.
//
// Leaves are built once per graph (all edge types, uint32) on the owning
// handle when the graph is added; uint64 leaves for an escalated chain are
// built on demand under a lock and the owning stream is synchronised before
// any lane reads them.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "internal.h"

using namespace rmcm;

namespace {

struct Query {
    int64_t tag = 0;
    int32_t graph = 0;
    std::string path;
    double t_submit = 0;
    double t_admit = 0;
    // filled by the admission step
    bool planned = false;
    std::vector<int32_t> vts, ets, pairs;
    double est_bytes = 0;
    double es_s = 0, dp_s = 0;
};

}  // namespace

struct rmcm_server {
    rmcm_handle *h = nullptr;
    int64_t budget = 0;
    int64_t reserved = 0;               // predicted bytes of the queries on the GPU
    std::vector<rmcm_graph *> graphs;
    std::vector<rmcm_handle *> lanes;
    std::vector<std::thread> workers;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Query> pending;          // not yet estimated, arrival order
    std::deque<Query> waiting;          // estimated, waiting for bytes, arrival order
    std::deque<rmcm_query_result> done;
    int64_t in_flight = 0;              // queries taken by a worker and not yet done
    int64_t submitted = 0, completed = 0, rejected = 0;
    int64_t peak_reserved = 0;
    int32_t max_running = 0, running = 0;
    bool stop = false;
    std::mutex leaf_mu;                 // leaves map and owning stream
    std::chrono::steady_clock::time_point t0;

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

// Predicted device bytes of a planned chain: every node of the split tree
// (an intermediate or the result) at 12 bytes per estimated entry + row
// pointers + SpGEMM scratch rows.
double predicted_bytes(const std::vector<double> &c, const std::vector<int32_t> &split, const std::vector<int64_t> &dims,
                       int32_t len) {
    double bytes = 0;
    std::vector<std::pair<int, int>> st{{0, len - 1}};
    while (!st.empty()) {
        auto [i, j] = st.back();
        st.pop_back();
        if (i == j) continue;
        const double rows = (double)dims[i];
        bytes += 12.0 * c[i * len + j] + 8.0 * (rows + 1) + 40.0 * rows;
        const int k = split[i * len + j];
        st.push_back({i, k});
        st.push_back({k + 1, j});
    }
    return bytes;
}

int32_t server_leaf(rmcm_server *S, rmcm_graph *g, int32_t src, int32_t sink, int32_t et, int32_t vt, rmcm_mat **out) {
    std::lock_guard<std::mutex> lock(S->leaf_mu);
    int32_t rc = leaf_of(S->h, g, src, sink, et, vt, out);
    if (rc == RMCM_OK && cudaStreamSynchronize(S->h->stream) != cudaSuccess)
        rc = set_error(S->h, RMCM_ECUDA, "leaf build");
    return rc;
}

void finish(rmcm_server *S, const Query &q, int32_t status, int64_t nnz, uint64_t digest, int32_t valtype, int lane,
            double t_done, const std::string &err) {
    rmcm_query_result r{};
    r.tag = q.tag;
    r.status = status;
    r.graph = q.graph;
    r.nnz = nnz;
    r.digest = digest;
    r.t_submit = q.t_submit;
    r.t_admit = q.t_admit;
    r.t_done = t_done;
    r.est_bytes = q.est_bytes;
    r.es_s = q.es_s;
    r.dp_s = q.dp_s;
    r.valtype = valtype;
    r.lane = lane;
    std::snprintf(r.error, sizeof(r.error), "%s", err.c_str());
    S->done.push_back(r);
    S->completed++;
    if (status != RMCM_OK) S->rejected++;
}

// Estimator + DP of a query on lane L; fills q.pairs and q.est_bytes.
int32_t plan_query(rmcm_server *S, rmcm_handle *L, Query &q, std::string &err) {
    if (q.graph < 0 || q.graph >= (int32_t)S->graphs.size()) {
        err = "no such graph";
        return RMCM_EINVAL;
    }
    rmcm_graph *g = S->graphs[q.graph];
    if (path_parse(q.path.c_str(), q.vts, q.ets) != RMCM_OK) {
        err = "the meta-path is incorrect: " + q.path;
        return RMCM_EINVAL;
    }
    const int len = (int)q.ets.size();
    if (len < 1 || len > 16) {
        err = "meta-path must have 1..16 edge types";
        return RMCM_EINVAL;
    }
    std::vector<rmcm_mat *> mats(len);
    std::vector<int64_t> dims(len + 1);
    for (int i = 0; i < len; i++) {
        int32_t rc = server_leaf(S, g, q.vts[i], q.vts[i + 1], q.ets[i], RMCM_VAL_U32, &mats[i]);
        if (rc != RMCM_OK) {
            err = S->h->last_error;
            return rc;
        }
        dims[i] = mats[i]->d.rows;
    }
    dims[len] = mats[len - 1]->d.cols;
    if (len == 1) {
        q.est_bytes = 12.0 * (double)mats[0]->d.nnz + 8.0 * (double)(dims[0] + 1);
        q.planned = true;
        return RMCM_OK;
    }
    std::vector<double> c(len * len);
    std::vector<int32_t> split(len * len);
    q.pairs.assign(2 * (len - 1), 0);
    int32_t rc = chain_plan(L, mats.data(), len, c.data(), split.data(), q.pairs.data(), &q.es_s, &q.dp_s);
    if (rc != RMCM_OK) {
        err = L->last_error;
        return rc;
    }
    q.est_bytes = predicted_bytes(c, split, dims, len);
    q.planned = true;
    return RMCM_OK;
}

// Runs a planned query on lane L; returns nnz / digest / value type.
int32_t run_query(rmcm_server *S, rmcm_handle *L, const Query &q, int64_t *nnz, uint64_t *digest, int32_t *vt,
                  std::string &err) {
    rmcm_graph *g = S->graphs[q.graph];
    const int len = (int)q.ets.size();
    std::vector<rmcm_mat *> mats(len);
    for (int i = 0; i < len; i++) {
        int32_t rc = server_leaf(S, g, q.vts[i], q.vts[i + 1], q.ets[i], RMCM_VAL_U32, &mats[i]);
        if (rc != RMCM_OK) {
            err = S->h->last_error;
            return rc;
        }
    }
    auto leaf64 = [&](int i, rmcm_mat **o) {
        int32_t rc = server_leaf(S, g, q.vts[i], q.vts[i + 1], q.ets[i], RMCM_VAL_U64, o);
        if (rc != RMCM_OK) set_error(L, rc, S->h->last_error);
        return rc;
    };
    rmcm_mat *C = nullptr;
    rmcm_timings t{};
    int32_t rc;
    if (len == 1) {
        C = mats[0];                       // the leaf itself is the result
        rc = RMCM_OK;
    } else {
        rc = chain_run_ordered(L, mats.data(), len, q.pairs.data(), &C, &t, true, leaf64);
    }
    if (rc == RMCM_OK) {
        uint64_t *d = nullptr;
        rc = dev_alloc(L, (void **)&d, 16);
        if (rc == RMCM_OK) rc = mat_digest_launch(L, C, d);
        if (rc == RMCM_OK) {
            cudaError_t e = cudaMemcpyAsync(L->h_pinned, d, 16, cudaMemcpyDeviceToHost, L->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(L->stream);
            if (e != cudaSuccess) rc = cuda_error(L, e, "digest download");
        }
        if (d) dev_free(L, d, 16);
        if (rc == RMCM_OK) {
            *nnz = L->h_pinned[0];
            *digest = (uint64_t)L->h_pinned[1];
            *vt = C->valtype;
        }
    }
    if (C && len > 1) mat_release(L, C);
    if (rc != RMCM_OK) err = L->last_error;
    return rc;
}

void worker_main(rmcm_server *S, int lane) {
    rmcm_handle *L = S->lanes[lane];
    cudaSetDevice(L->device);
    std::unique_lock<std::mutex> lock(S->mu);
    for (;;) {
        // oldest waiting query that fits now, else the oldest unplanned one
        Query q;
        bool have = false;
        for (auto it = S->waiting.begin(); it != S->waiting.end(); ++it) {
            if (S->reserved + (int64_t)it->est_bytes <= S->budget) {
                q = std::move(*it);
                S->waiting.erase(it);
                have = true;
                break;
            }
        }
        if (!have && !S->pending.empty()) {
            q = std::move(S->pending.front());
            S->pending.pop_front();
            have = true;
        }
        if (!have) {
            if (S->stop) return;
            S->cv_work.wait(lock);
            continue;
        }
        S->in_flight++;
        std::string err;
        if (!q.planned) {
            lock.unlock();
            const int32_t rc = plan_query(S, L, q, err);
            lock.lock();
            if (rc != RMCM_OK || q.est_bytes > (double)S->budget) {
                if (rc == RMCM_OK) err = "predicted bytes exceed the server budget";
                finish(S, q, rc != RMCM_OK ? rc : RMCM_ENOMEM, 0, 0, 0, lane, S->now(), err);
                S->in_flight--;
                S->cv_done.notify_all();
                continue;
            }
            if (S->reserved + (int64_t)q.est_bytes > S->budget) {
                // does not fit now: wait for bytes, in arrival order
                auto pos = std::find_if(S->waiting.begin(), S->waiting.end(),
                                        [&](const Query &w) { return w.t_submit > q.t_submit; });
                S->waiting.insert(pos, std::move(q));
                S->in_flight--;
                continue;
            }
        }
        const int64_t bytes = (int64_t)q.est_bytes;
        S->reserved += bytes;
        S->peak_reserved = std::max(S->peak_reserved, S->reserved);
        S->running++;
        S->max_running = std::max(S->max_running, S->running);
        q.t_admit = S->now();
        lock.unlock();
        int64_t nnz = 0;
        uint64_t digest = 0;
        int32_t vt = 0;
        const int32_t rc = run_query(S, L, q, &nnz, &digest, &vt, err);
        lock.lock();
        S->reserved -= bytes;
        S->running--;
        finish(S, q, rc, nnz, digest, vt, lane, S->now(), err);
        S->in_flight--;
        S->cv_done.notify_all();
        S->cv_work.notify_all();   // bytes came back: waiting queries may fit
    }
}

// All (src type, sink type, edge type) triples of a graph's edges.
std::set<std::tuple<int32_t, int32_t, int32_t>> edge_kinds(const rmcm_graph *g) {
    std::set<std::tuple<int32_t, int32_t, int32_t>> kinds;
    for (int64_t u = 0; u < g->n; u++)
        for (int64_t e = g->adj_ptr[u]; e < g->adj_ptr[u + 1]; e++)
            kinds.insert({g->vtype[u], g->vtype[g->adj_nbr[e]], g->adj_et[e]});
    return kinds;
}

}  // namespace

RMCM_API int32_t rmcm_server_create(rmcm_handle *h, const rmcm_server_opts *opts, rmcm_server **out) {
    if (!h || !out) return RMCM_EINVAL;
    *out = nullptr;
    rmcm_server_opts o{};
    if (opts) o = *opts;
    const int lanes = o.lanes > 0 ? std::min(o.lanes, 64) : 8;
    rmcm_server *S = new rmcm_server();
    S->h = h;
    S->budget = o.mem_budget_bytes > 0 ? o.mem_budget_bytes : h->budget;
    S->t0 = std::chrono::steady_clock::now();
    rmcm_opts lo{};
    lo.device = h->device;
    lo.valtype = RMCM_VAL_AUTO;
    lo.mem_budget_bytes = h->budget;
    for (int k = 0; k < lanes; k++) {
        rmcm_handle *L = nullptr;
        int32_t rc = rmcm_create(&L, &lo);
        if (rc != RMCM_OK) {
            for (auto *x : S->lanes) rmcm_destroy(x);
            delete S;
            return set_error(h, rc, "server: could not create a lane");
        }
        L->tune = h->tune;
        S->lanes.push_back(L);
    }
    for (int k = 0; k < lanes; k++) S->workers.emplace_back(worker_main, S, k);
    *out = S;
    return RMCM_OK;
}

RMCM_API int32_t rmcm_server_add_graph(rmcm_server *S, rmcm_graph *g, int32_t *index) {
    if (!S || !g) return RMCM_EINVAL;
    if (g->h != S->h) return set_error(S->h, RMCM_EINVAL, "server: the graph belongs to another handle");
    {
        std::lock_guard<std::mutex> lock(S->leaf_mu);
        for (auto &k : edge_kinds(g)) {
            rmcm_mat *m = nullptr;
            RMCM_TRY(leaf_of(S->h, g, std::get<0>(k), std::get<1>(k), std::get<2>(k), RMCM_VAL_U32, &m));
        }
        RMCM_CUDA(S->h, cudaStreamSynchronize(S->h->stream));
    }
    std::lock_guard<std::mutex> lock(S->mu);
    g->batches++;                          // the graph may not be freed under the server
    S->graphs.push_back(g);
    if (index) *index = (int32_t)S->graphs.size() - 1;
    return RMCM_OK;
}

RMCM_API double rmcm_server_now(const rmcm_server *S) { return S ? S->now() : 0.0; }

RMCM_API int32_t rmcm_server_submit(rmcm_server *S, int32_t graph, const char *metapath, int64_t tag,
                                    double t_arrival) {
    if (!S || !metapath) return RMCM_EINVAL;
    Query q;
    q.tag = tag;
    q.graph = graph;
    q.path = metapath;
    q.t_submit = t_arrival >= 0 ? t_arrival : S->now();
    std::lock_guard<std::mutex> lock(S->mu);
    S->pending.push_back(std::move(q));
    S->submitted++;
    S->cv_work.notify_one();
    return RMCM_OK;
}

RMCM_API int32_t rmcm_server_poll(rmcm_server *S, rmcm_query_result *out, int32_t cap, int32_t *count,
                                  double wait_s) {
    if (!S || !count || (cap > 0 && !out)) return RMCM_EINVAL;
    std::unique_lock<std::mutex> lock(S->mu);
    if (S->done.empty() && wait_s > 0)
        S->cv_done.wait_for(lock, std::chrono::duration<double>(wait_s), [&] { return !S->done.empty(); });
    int32_t n = 0;
    while (n < cap && !S->done.empty()) {
        out[n++] = S->done.front();
        S->done.pop_front();
    }
    *count = n;
    return RMCM_OK;
}

RMCM_API int32_t rmcm_server_drain(rmcm_server *S, double timeout_s) {
    if (!S) return RMCM_EINVAL;
    std::unique_lock<std::mutex> lock(S->mu);
    auto idle = [&] { return S->pending.empty() && S->waiting.empty() && S->in_flight == 0; };
    if (timeout_s > 0) {
        if (!S->cv_done.wait_for(lock, std::chrono::duration<double>(timeout_s), idle)) return RMCM_ETIMEOUT;
    } else {
        S->cv_done.wait(lock, idle);
    }
    return RMCM_OK;
}

RMCM_API int32_t rmcm_server_stats(const rmcm_server *S, rmcm_server_counters *st) {
    if (!S || !st) return RMCM_EINVAL;
    rmcm_server *W = const_cast<rmcm_server *>(S);
    std::lock_guard<std::mutex> lock(W->mu);
    st->submitted = S->submitted;
    st->completed = S->completed;
    st->rejected = S->rejected;
    st->pending = (int64_t)S->pending.size();
    st->waiting = (int64_t)S->waiting.size();
    st->running = S->running;
    st->max_running = S->max_running;
    st->lanes = (int32_t)S->lanes.size();
    st->budget = S->budget;
    st->reserved = S->reserved;
    st->peak_reserved = S->peak_reserved;
    int64_t launches = 0;
    for (auto *L : S->lanes) launches += L->launches;
    st->kernel_launches = launches;
    return RMCM_OK;
}

RMCM_API int32_t rmcm_server_destroy(rmcm_server *S) {
    if (!S) return RMCM_OK;
    {
        std::unique_lock<std::mutex> lock(S->mu);
        S->cv_done.wait(lock, [&] { return S->pending.empty() && S->waiting.empty() && S->in_flight == 0; });
        S->stop = true;
        S->cv_work.notify_all();
    }
    for (auto &t : S->workers) t.join();
    for (auto *L : S->lanes) rmcm_destroy(L);
    for (auto *g : S->graphs) g->batches--;
    delete S;
    return RMCM_OK;
}
