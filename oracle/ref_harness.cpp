// Harness around the reference program efficient/resmcm.cpp (swordzlim/RESMCM_ARI).
//
// TEST INFRASTRUCTURE ONLY.  The recipe in oracle/Makefile compiles the
// reference source file where it lies (its path comes in as REF_RESMCM_CPP),
// renaming its main(), and adds the extern "C" entry points below so the
// tests can call the reference's own classes directly:
//   HeteroGraph (efficient/resmcm.cpp:181-240),
//   DynamicOptimizer::rows_sparse_optimal_matrix_chain_order (:488-541),
//   DynamicOptimizer::get_optimal_chain_order (:563-573),
//   SSP_dynamic (:653-772).
// Nothing of the reference is copied here; the built library lands in
// oracle/_ref/ and is used to pin the C oracle and to make golden fixtures.
#include <cstdint>
#include <cstdlib>
#include <cstring>

#define main resmcm_reference_main
#include REF_RESMCM_CPP
#undef main

namespace {

std::vector<int32_t> local_ids(HeteroGraph *g) {
    std::vector<int32_t> loc(g->n, -1);
    for (int t = 0; t <= g->max_vt; t++) {
        int32_t r = 0;
        for (vertex v : *g->bins[t]) loc[v] = r++;
    }
    return loc;
}

}  // namespace

extern "C" {

void *ref_load(const char *graph, const char *vertex, const char *edge) {
    return new HeteroGraph(graph, vertex, edge);
}

void ref_free(void *h) { delete static_cast<HeteroGraph *>(h); }

void ref_free_buf(void *p) { free(p); }

// Estimates c_, split table s_ and the post-order pair list, with the
// reference's own classes.  Arrays are len*len (c, s) and 2*(len-1) (pairs).
int ref_estimate(void *h, const char *metapath, int threads, double *c_out, int32_t *s_out,
                 int32_t *pairs_out, int32_t *len_out, double *m_out) {
    HeteroGraph *g = static_cast<HeteroGraph *>(h);
    omp_set_num_threads(threads);
    MetaPath path{std::string(metapath)};
    int len = path.pathLen;
    *len_out = len;
    if (len < 2) return 0;
    std::vector<vertex_type> p_vts = path.vertexTypes;
    BoolMatrix **mats = (BoolMatrix **)malloc(len * sizeof(BoolMatrix *));
    for (int i = 0; i < len; i++)
        mats[i] = new BoolMatrix(g->heteGraph, g->vertexTypes, p_vts[i], p_vts[i + 1], path.edgeTypes[i], g->n);
    DynamicOptimizer op;
    op.rows_sparse_optimal_matrix_chain_order(len, mats, g->bins, g->dimensions, &p_vts, g->n);
    for (int q = 0; q < len * len; q++) {
        c_out[q] = op.c_[q];
        s_out[q] = op.s_[q];
        if (m_out) m_out[q] = op.m_[q];
    }
    std::vector<std::pair<int, int>> order;
    op.get_optimal_chain_order(0, len - 1, &order);
    for (size_t q = 0; q < order.size(); q++) {
        pairs_out[2 * q] = order[q].first;
        pairs_out[2 * q + 1] = order[q].second;
    }
    op.free_rows_sparse_optimal_matrix_chain_order();
    for (int i = 0; i < len; i++) delete mats[i];
    free(mats);
    return 0;
}

// Runs SSP_dynamic and exports the result rows of the start type in local
// ids, each row sorted.  *rowptr_out / *col_out are malloc'd (ref_free_buf).
// times: es, dp, spgemm, total (the reference's own globals).
int ref_chain(void *h, const char *metapath, int threads, int64_t *nnz_out, double *times,
              int64_t *rows_out, int64_t **rowptr_out, int32_t **col_out) {
    HeteroGraph *g = static_cast<HeteroGraph *>(h);
    omp_set_num_threads(threads);
    int tnum = omp_get_max_threads();
    t_rows = (long *)calloc(tnum, sizeof(long));
    t_times = (double *)calloc(tnum, sizeof(double));
    es_time = dp_time = spgemm_time = smcm_time = 0;
    MetaPath path{std::string(metapath)};
    BoolMatrix *res = nullptr;
    build_pair(g->heteGraph, res, g->vertexTypes, g->edgeTypes, g->bins, g->dimensions, &path, g->n, g->m);
    times[0] = es_time;
    times[1] = dp_time;
    times[2] = spgemm_time;
    times[3] = smcm_time;
    std::vector<int32_t> loc = local_ids(g);
    std::vector<vertex> &rows = *g->bins[path.vertexTypes[0]];
    int64_t nr = (int64_t)rows.size();
    int64_t *rp = (int64_t *)malloc(sizeof(int64_t) * (nr + 1));
    rp[0] = 0;
    for (int64_t k = 0; k < nr; k++) rp[k + 1] = rp[k] + (int64_t)res->rows[rows[k]]->size();
    int32_t *col = (int32_t *)malloc(sizeof(int32_t) * (rp[nr] ? rp[nr] : 1));
    for (int64_t k = 0; k < nr; k++) {
        std::vector<vertex> &r = *res->rows[rows[k]];
        int32_t *dst = col + rp[k];
        for (size_t q = 0; q < r.size(); q++) dst[q] = loc[r[q]];
        std::sort(dst, dst + r.size());
    }
    *nnz_out = rp[nr];
    *rows_out = nr;
    *rowptr_out = rp;
    *col_out = col;
    res->free_memory();
    delete res;
    free(t_rows);
    free(t_times);
    t_rows = nullptr;
    t_times = nullptr;
    return 0;
}

}  // extern "C"
