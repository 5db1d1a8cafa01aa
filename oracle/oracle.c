/*
 * CPU oracle for the RESMCM sparse-matrix-chain path (plain C + OpenMP).
 *
 * TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the CPU-baseline
 * leg of the benchmark use it as the checker / reference-algorithm timing.
 * The GPU product path never links, loads or calls this file.
 *
 * Every function below names the part of efficient/resmcm.cpp
 * (swordzlim/RESMCM_ARI) whose behaviour it restates.  Deliberate, documented
 * differences from the reference, all on inputs where the reference has
 * undefined behaviour:
 *   - a vertex with no line in graph.txt has no neighbours (the reference
 *     dereferences an uninitialised pointer, efficient/resmcm.cpp:87,389);
 *   - malformed numbers, ids out of range, an odd (nbr, eid) token count or a
 *     repeated vertex line give ORC_EPARSE instead of silent garbage;
 *   - a chain of one matrix reports zero chain time (the reference re-reports
 *     the previous chain's stale smcm_time, efficient/resmcm.cpp:670-677,857).
 *
 * Build with -ffp-contract=off so that no multiply-add is fused: the
 * estimator and DP sums must round exactly like the reference's.
 */
#define _POSIX_C_SOURCE 200809L
#include "oracle.h"

#include <float.h>
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <sys/time.h>

struct orc_graph {
    int64_t n, m;
    int32_t max_vt;
    int32_t *vtype;        /* [n] */
    int64_t *adj_ptr;      /* [n+1] graph.txt order */
    int32_t *adj_nbr;      /* [adj_ptr[n]] */
    int32_t *adj_et;       /* [adj_ptr[n]] edge type of each entry */
    int64_t *dims;         /* [max_vt+1] HeteroGraph::set_dimensions */
    int64_t *bin_ptr;      /* [max_vt+2] HeteroGraph::set_bins, CSR form */
    int32_t *bin_ids;      /* [n] ascending global ids per type */
    int32_t *local;        /* [n] rank of a vertex inside its type bin */
};

/* A matrix over global row ids; rows of other types are empty (the
 * reference's nullptr rows).  vals is only used in counting mode. */
typedef struct {
    int64_t n;
    int64_t *len;
    int32_t **cols;
    uint64_t **vals;
    int32_t row_vt;        /* vertex type whose rows are populated */
    int32_t col_vt;
} rowmat;

struct orc_result {
    const orc_graph *g;
    rowmat *mat;
    int64_t nnz;
    int32_t mode;
};

static double now_s(void) {
    /* gettimeofday, as the reference's timers (efficient/resmcm.cpp:506-517) */
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return (double)tv.tv_sec + (double)tv.tv_usec / 1e6;
}

/* ------------------------------------------------------------------------ */
/* text loader: DataReader, efficient/resmcm.cpp:49-177                     */
/* ------------------------------------------------------------------------ */

static char *slurp(const char *path, size_t *size) {
    FILE *f = fopen(path, "rb");
    if (!f) return NULL;
    if (fseek(f, 0, SEEK_END) != 0) { fclose(f); return NULL; }
    long sz = ftell(f);
    if (sz < 0) { fclose(f); return NULL; }
    rewind(f);
    char *buf = (char *)malloc((size_t)sz + 1);
    if (!buf) { fclose(f); return NULL; }
    size_t got = fread(buf, 1, (size_t)sz, f);
    fclose(f);
    buf[got] = '\0';
    *size = got;
    return buf;
}

/* Lines as getline sees them: a final line without '\n' still counts. */
static int64_t count_lines(const char *b, size_t sz) {
    int64_t n = 0;
    for (size_t i = 0; i < sz; i++) n += (b[i] == '\n');
    if (sz > 0 && b[sz - 1] != '\n') n++;
    return n;
}

/* Parse whitespace-separated integers of one line [p, e).  Returns the
 * number of tokens, -1 on a malformed token. */
static int next_int(const char **pp, const char *e, int64_t *out) {
    const char *p = *pp;
    while (p < e && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\v' || *p == '\f')) p++;
    if (p >= e) { *pp = p; return 0; }
    int neg = 0;
    if (*p == '+' || *p == '-') { neg = (*p == '-'); p++; }
    if (p >= e || *p < '0' || *p > '9') return -1;
    int64_t v = 0;
    while (p < e && *p >= '0' && *p <= '9') {
        v = v * 10 + (*p - '0');
        if (v > ((int64_t)1 << 50)) return -1;
        p++;
    }
    if (p < e && !(*p == ' ' || *p == '\t' || *p == '\r' || *p == '\v' || *p == '\f')) return -1;
    *out = neg ? -v : v;
    *pp = p;
    return 1;
}

static void graph_free_arrays(orc_graph *g) {
    if (!g) return;
    free(g->vtype); free(g->adj_ptr); free(g->adj_nbr); free(g->adj_et);
    free(g->dims); free(g->bin_ptr); free(g->bin_ids); free(g->local);
}

void orc_graph_free(orc_graph *g) {
    graph_free_arrays(g);
    free(g);
}

/* HeteroGraph::set_dimensions / set_bins, efficient/resmcm.cpp:206-222 */
static int graph_finish(orc_graph *g) {
    int32_t nt = g->max_vt + 1;
    g->dims = (int64_t *)calloc((size_t)nt, sizeof(int64_t));
    g->bin_ptr = (int64_t *)calloc((size_t)nt + 1, sizeof(int64_t));
    g->bin_ids = (int32_t *)malloc(sizeof(int32_t) * (size_t)(g->n ? g->n : 1));
    g->local = (int32_t *)malloc(sizeof(int32_t) * (size_t)(g->n ? g->n : 1));
    if (!g->dims || !g->bin_ptr || !g->bin_ids || !g->local) return ORC_ENOMEM;
    for (int64_t v = 0; v < g->n; v++) g->dims[g->vtype[v]]++;
    for (int32_t t = 0; t < nt; t++) g->bin_ptr[t + 1] = g->bin_ptr[t] + g->dims[t];
    int64_t *fill = (int64_t *)calloc((size_t)nt, sizeof(int64_t));
    if (!fill) return ORC_ENOMEM;
    for (int64_t v = 0; v < g->n; v++) {
        int32_t t = g->vtype[v];
        g->local[v] = (int32_t)fill[t];
        g->bin_ids[g->bin_ptr[t] + fill[t]++] = (int32_t)v;
    }
    free(fill);
    return ORC_OK;
}

int orc_graph_load_text(const char *graph, const char *vertex, const char *edge, orc_graph **out) {
    *out = NULL;
    size_t vsz = 0, esz = 0, gsz = 0;
    char *vb = slurp(vertex, &vsz);
    if (!vb) return ORC_EIO;
    char *eb = slurp(edge, &esz);
    if (!eb) { free(vb); return ORC_EIO; }
    char *gb = slurp(graph, &gsz);
    if (!gb) { free(vb); free(eb); return ORC_EIO; }
    int rc = ORC_OK;
    orc_graph *g = (orc_graph *)calloc(1, sizeof(orc_graph));
    int32_t *edge_types = NULL;
    int64_t *cnt = NULL;
    unsigned char *seen = NULL;
    if (!g) { rc = ORC_ENOMEM; goto done; }

    /* n = number of lines of vertex.txt (DataReader ctor, :59-84) */
    g->n = count_lines(vb, vsz);
    g->vtype = (int32_t *)calloc((size_t)(g->n ? g->n : 1), sizeof(int32_t));
    if (!g->vtype) { rc = ORC_ENOMEM; goto done; }
    /* readVertexType, :115-135 */
    {
        const char *p = vb, *end = vb + vsz;
        while (p < end) {
            const char *le = memchr(p, '\n', (size_t)(end - p));
            if (!le) le = end;
            const char *q = p;
            int64_t v, t;
            int a = next_int(&q, le, &v);
            if (a == 1) {
                if (next_int(&q, le, &t) != 1 || v < 0 || v >= g->n || t < 0 || t > 1000000) {
                    rc = ORC_EPARSE; goto done;
                }
                g->vtype[v] = (int32_t)t;
                if (t > g->max_vt) g->max_vt = (int32_t)t;
            } else if (a < 0) { rc = ORC_EPARSE; goto done; }
            p = le + 1;
        }
    }
    /* readEdgeType first pass: m = number of (nbr, eid) pairs, :137-156 */
    {
        const char *p = gb, *end = gb + gsz;
        g->m = 0;
        while (p < end) {
            const char *le = memchr(p, '\n', (size_t)(end - p));
            if (!le) le = end;
            const char *q = p;
            int64_t x;
            int64_t toks = 0;
            int a;
            while ((a = next_int(&q, le, &x)) == 1) toks++;
            if (a < 0) { rc = ORC_EPARSE; goto done; }
            if (toks > 0) {
                if ((toks - 1) % 2 != 0) { rc = ORC_EPARSE; goto done; }
                g->m += (toks - 1) / 2;
            }
            p = le + 1;
        }
    }
    edge_types = (int32_t *)malloc(sizeof(int32_t) * (size_t)(g->m ? g->m : 1));
    if (!edge_types) { rc = ORC_ENOMEM; goto done; }
    for (int64_t e = 0; e < g->m; e++) edge_types[e] = -1;
    /* readEdgeType second pass over edge.txt, :158-173 */
    {
        const char *p = eb, *end = eb + esz;
        while (p < end) {
            const char *le = memchr(p, '\n', (size_t)(end - p));
            if (!le) le = end;
            const char *q = p;
            int64_t e, t;
            int a = next_int(&q, le, &e);
            if (a == 1) {
                if (next_int(&q, le, &t) != 1 || e < 0 || e >= g->m || t < 0) { rc = ORC_EPARSE; goto done; }
                edge_types[e] = (int32_t)t;
            } else if (a < 0) { rc = ORC_EPARSE; goto done; }
            p = le + 1;
        }
    }
    /* readGraph, :86-113 (two passes into CSR form) */
    cnt = (int64_t *)calloc((size_t)g->n + 1, sizeof(int64_t));
    seen = (unsigned char *)calloc((size_t)(g->n ? g->n : 1), 1);
    g->adj_ptr = (int64_t *)calloc((size_t)g->n + 1, sizeof(int64_t));
    g->adj_nbr = (int32_t *)malloc(sizeof(int32_t) * (size_t)(g->m ? g->m : 1));
    g->adj_et = (int32_t *)malloc(sizeof(int32_t) * (size_t)(g->m ? g->m : 1));
    if (!cnt || !seen || !g->adj_ptr || !g->adj_nbr || !g->adj_et) { rc = ORC_ENOMEM; goto done; }
    for (int pass = 0; pass < 2; pass++) {
        const char *p = gb, *end = gb + gsz;
        while (p < end) {
            const char *le = memchr(p, '\n', (size_t)(end - p));
            if (!le) le = end;
            const char *q = p;
            int64_t vid;
            int a = next_int(&q, le, &vid);
            if (a == 1) {
                if (vid < 0 || vid >= g->n) { rc = ORC_EPARSE; goto done; }
                if (pass == 0) {
                    if (seen[vid]) { rc = ORC_EPARSE; goto done; }
                    seen[vid] = 1;
                }
                int64_t nb, eid;
                while (next_int(&q, le, &nb) == 1) {
                    if (next_int(&q, le, &eid) != 1) { rc = ORC_EPARSE; goto done; }
                    if (nb < 0 || nb >= g->n || eid < 0 || eid >= g->m || edge_types[eid] < 0) {
                        rc = ORC_EPARSE; goto done;
                    }
                    if (pass == 0) {
                        cnt[vid]++;
                    } else {
                        int64_t pos = g->adj_ptr[vid] + cnt[vid]++;
                        g->adj_nbr[pos] = (int32_t)nb;
                        g->adj_et[pos] = edge_types[eid];
                    }
                }
            }
            p = le + 1;
        }
        if (pass == 0) {
            for (int64_t v = 0; v < g->n; v++) g->adj_ptr[v + 1] = g->adj_ptr[v] + cnt[v];
            memset(cnt, 0, sizeof(int64_t) * ((size_t)g->n + 1));
        }
    }
    rc = graph_finish(g);
done:
    free(vb); free(eb); free(gb); free(edge_types); free(cnt); free(seen);
    if (rc != ORC_OK) { orc_graph_free(g); g = NULL; }
    *out = g;
    return rc;
}

int orc_graph_from_arrays(int64_t n, const int32_t *vtype, const int64_t *adj_ptr,
                          const int32_t *adj_nbr, const int32_t *adj_et, orc_graph **out) {
    *out = NULL;
    if (n < 0 || (n > 0 && (!vtype || !adj_ptr))) return ORC_EINVAL;
    orc_graph *g = (orc_graph *)calloc(1, sizeof(orc_graph));
    if (!g) return ORC_ENOMEM;
    g->n = n;
    g->m = n ? adj_ptr[n] : 0;
    g->vtype = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n ? n : 1));
    g->adj_ptr = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
    g->adj_nbr = (int32_t *)malloc(sizeof(int32_t) * (size_t)(g->m ? g->m : 1));
    g->adj_et = (int32_t *)malloc(sizeof(int32_t) * (size_t)(g->m ? g->m : 1));
    if (!g->vtype || !g->adj_ptr || !g->adj_nbr || !g->adj_et) { orc_graph_free(g); return ORC_ENOMEM; }
    g->adj_ptr[0] = 0;
    for (int64_t v = 0; v < n; v++) {
        if (vtype[v] < 0 || adj_ptr[v + 1] < adj_ptr[v]) { orc_graph_free(g); return ORC_EINVAL; }
        g->vtype[v] = vtype[v];
        if (vtype[v] > g->max_vt) g->max_vt = vtype[v];
        g->adj_ptr[v + 1] = adj_ptr[v + 1];
    }
    for (int64_t e = 0; e < g->m; e++) {
        if (adj_nbr[e] < 0 || adj_nbr[e] >= n) { orc_graph_free(g); return ORC_EINVAL; }
        g->adj_nbr[e] = adj_nbr[e];
        g->adj_et[e] = adj_et[e];
    }
    int rc = graph_finish(g);
    if (rc != ORC_OK) { orc_graph_free(g); return rc; }
    *out = g;
    return ORC_OK;
}

int64_t orc_graph_n(const orc_graph *g) { return g->n; }
int64_t orc_graph_m(const orc_graph *g) { return g->m; }
int32_t orc_graph_max_vt(const orc_graph *g) { return g->max_vt; }
int64_t orc_graph_dim(const orc_graph *g, int32_t vt) {
    return (vt < 0 || vt > g->max_vt) ? 0 : g->dims[vt];
}

void orc_graph_export(const orc_graph *g, int32_t *vtype, int64_t *adj_ptr, int32_t *adj_nbr, int32_t *adj_et) {
    if (vtype) memcpy(vtype, g->vtype, sizeof(int32_t) * (size_t)g->n);
    if (adj_ptr) memcpy(adj_ptr, g->adj_ptr, sizeof(int64_t) * (size_t)(g->n + 1));
    if (adj_nbr) memcpy(adj_nbr, g->adj_nbr, sizeof(int32_t) * (size_t)g->m);
    if (adj_et) memcpy(adj_et, g->adj_et, sizeof(int32_t) * (size_t)g->m);
}

/* ------------------------------------------------------------------------ */
/* meta-path grammar: MetaPath(string), efficient/resmcm.cpp:269-299         */
/* ------------------------------------------------------------------------ */

int orc_metapath_parse(const char *s, int32_t *vts, int32_t *ets, int32_t cap, int32_t *len) {
    /* Maximal digit runs; every non-digit character closes a number (even
     * when no digit preceded it, which then yields 0), alternating vt, et. */
    int32_t nv = 0, ne = 0, i = 0;
    int64_t num = 0;
    size_t L = strlen(s);
    if (L == 0) return ORC_EPARSE;
    for (size_t q = 0; q < L; q++) {
        char ch = s[q];
        if (ch >= '0' && ch <= '9') {
            num = num * 10 + (ch - '0');
            if (num > 1000000000) return ORC_EPARSE;
        } else {
            if (i % 2 == 0) { if (nv >= cap + 1) return ORC_EINVAL; vts[nv++] = (int32_t)num; }
            else { if (ne >= cap) return ORC_EINVAL; ets[ne++] = (int32_t)num; }
            num = 0;
            i++;
        }
    }
    char last = s[L - 1];
    if (last >= '0' && last <= '9') {
        if (i % 2 == 0) { if (nv >= cap + 1) return ORC_EINVAL; vts[nv++] = (int32_t)num; }
        else { if (ne >= cap) return ORC_EINVAL; ets[ne++] = (int32_t)num; }
        i++;
    }
    if (nv != ne + 1) return ORC_EPARSE;   /* "the meta-path is incorrect" */
    *len = i / 2;
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* matrices                                                                  */
/* ------------------------------------------------------------------------ */

static rowmat *rowmat_new(int64_t n, int32_t row_vt, int32_t col_vt) {
    rowmat *M = (rowmat *)calloc(1, sizeof(rowmat));
    if (!M) return NULL;
    M->n = n;
    M->row_vt = row_vt;
    M->col_vt = col_vt;
    M->len = (int64_t *)calloc((size_t)(n ? n : 1), sizeof(int64_t));
    M->cols = (int32_t **)calloc((size_t)(n ? n : 1), sizeof(int32_t *));
    M->vals = (uint64_t **)calloc((size_t)(n ? n : 1), sizeof(uint64_t *));
    if (!M->len || !M->cols || !M->vals) {
        free(M->len); free(M->cols); free(M->vals); free(M);
        return NULL;
    }
    return M;
}

static void rowmat_free(rowmat *M) {
    if (!M) return;
    for (int64_t i = 0; i < M->n; i++) { free(M->cols[i]); free(M->vals[i]); }
    free(M->len); free(M->cols); free(M->vals);
    free(M);
}

/* BoolMatrix(HIN, vertex_types, source_vt, sink_vt, et, n), :374-396.
 * Rows keep graph.txt order and repeated neighbours. */
static rowmat *leaf_matrix(const orc_graph *g, int32_t src, int32_t sink, int32_t et, int count_mode) {
    rowmat *M = rowmat_new(g->n, src, sink);
    if (!M) return NULL;
    if (src < 0 || src > g->max_vt) return M;
    int64_t b0 = g->bin_ptr[src], b1 = g->bin_ptr[src + 1];
    int fail = 0;
#pragma omp parallel for schedule(dynamic, 1000)
    for (int64_t k = b0; k < b1; k++) {
        int32_t u = g->bin_ids[k];
        int64_t cnt = 0;
        for (int64_t e = g->adj_ptr[u]; e < g->adj_ptr[u + 1]; e++)
            if (g->adj_et[e] == et && g->vtype[g->adj_nbr[e]] == sink) cnt++;
        M->len[u] = cnt;
        M->cols[u] = (int32_t *)malloc(sizeof(int32_t) * (size_t)(cnt ? cnt : 1));
        if (count_mode) M->vals[u] = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(cnt ? cnt : 1));
        if (!M->cols[u] || (count_mode && !M->vals[u])) { fail = 1; continue; }
        int64_t q = 0;
        for (int64_t e = g->adj_ptr[u]; e < g->adj_ptr[u + 1]; e++)
            if (g->adj_et[e] == et && g->vtype[g->adj_nbr[e]] == sink) {
                M->cols[u][q] = g->adj_nbr[e];
                if (count_mode) M->vals[u][q] = 1;
                q++;
            }
    }
    if (fail) { rowmat_free(M); return NULL; }
    return M;
}

int orc_leaf(const orc_graph *g, int32_t src_vt, int32_t sink_vt, int32_t et, int64_t *rowptr, int32_t *col) {
    if (src_vt < 0 || src_vt > g->max_vt || sink_vt < 0 || sink_vt > g->max_vt) return ORC_EINVAL;
    rowmat *M = leaf_matrix(g, src_vt, sink_vt, et, 0);
    if (!M) return ORC_ENOMEM;
    int64_t b0 = g->bin_ptr[src_vt], b1 = g->bin_ptr[src_vt + 1];
    rowptr[0] = 0;
    for (int64_t k = b0; k < b1; k++) {
        int32_t u = g->bin_ids[k];
        rowptr[k - b0 + 1] = rowptr[k - b0] + M->len[u];
        if (col)
            for (int64_t q = 0; q < M->len[u]; q++) col[rowptr[k - b0] + q] = g->local[M->cols[u][q]];
    }
    rowmat_free(M);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* RES estimator: getSparsities :442-452, compute_sparsities :468-485,       */
/* estimator loop of rows_sparse_optimal_matrix_chain_order :506-517         */
/* ------------------------------------------------------------------------ */

static int estimate_core(const orc_graph *g, rowmat **mats, const int32_t *vts, int32_t len,
                         int32_t threads, double *c) {
    int64_t n = g->n;
    memset(c, 0, sizeof(double) * (size_t)len * (size_t)len);
    /* r_[i][j] for the current level i and the previous level i+1 only. */
    double **cur = (double **)calloc((size_t)len, sizeof(double *));
    double **nxt = (double **)calloc((size_t)len, sizeof(double *));
    if (!cur || !nxt) { free(cur); free(nxt); return ORC_ENOMEM; }
    int rc = ORC_OK;
    for (int32_t j = 0; j < len; j++) {
        cur[j] = (double *)calloc((size_t)(n ? n : 1), sizeof(double));
        nxt[j] = (double *)calloc((size_t)(n ? n : 1), sizeof(double));
        if (!cur[j] || !nxt[j]) rc = ORC_ENOMEM;
    }
    double *part = (double *)calloc((size_t)(threads > 0 ? threads : 1), sizeof(double));
    if (!part) rc = ORC_ENOMEM;
    for (int32_t i = len - 1; rc == ORC_OK && i >= 0; i--) {
        rowmat *M = mats[i];
        int32_t rt = vts[i];
        int64_t b0 = g->bin_ptr[rt], b1 = g->bin_ptr[rt + 1];
        /* leaf sparsity: s = |row| / dim(vts[i+1]), capped at 1 */
        int64_t dim_sink = g->dims[vts[i + 1]];
        double *ri = cur[i];
        for (int64_t k = b0; k < b1; k++) {
            int32_t u = g->bin_ids[k];
            double s = (double)M->len[u] / (double)dim_sink;
            ri[u] = s > 1 ? 1 : s;
        }
        for (int32_t j = len - 1; j > i; j--) {
            const double *right = nxt[j];            /* r_[(i+1)*len + j] */
            double *res = cur[j];
            double dim = (double)g->dims[vts[j + 1]];
            if (threads <= 1) {
                double nnz = 0;
                for (int64_t k = b0; k < b1; k++) {
                    int32_t u = g->bin_ids[k];
                    double tmp_rho = 1;
                    for (int64_t q = 0; q < M->len[u]; q++) tmp_rho *= (1 - right[M->cols[u][q]]);
                    double s = 1 - tmp_rho;
                    res[u] = s;
                    nnz += s * dim;
                }
                c[i * len + j] = nnz;
            } else {
                /* static split, partial sums combined in thread order */
                for (int t = 0; t < threads; t++) part[t] = 0;
#pragma omp parallel num_threads(threads)
                {
                    int t = omp_get_thread_num();
                    int nt = omp_get_num_threads();
                    int64_t tot = b1 - b0;
                    int64_t lo = b0 + tot * t / nt, hi = b0 + tot * (t + 1) / nt;
                    double nnz = 0;
                    for (int64_t k = lo; k < hi; k++) {
                        int32_t u = g->bin_ids[k];
                        double tmp_rho = 1;
                        for (int64_t q = 0; q < M->len[u]; q++) tmp_rho *= (1 - right[M->cols[u][q]]);
                        double s = 1 - tmp_rho;
                        res[u] = s;
                        nnz += s * dim;
                    }
                    part[t] = nnz;
                }
                double nnz = 0;
                for (int t = 0; t < threads; t++) nnz += part[t];
                c[i * len + j] = nnz;
            }
        }
        double **sw = cur; cur = nxt; nxt = sw;   /* level i becomes "i+1" */
    }
    for (int32_t j = 0; j < len; j++) { free(cur[j]); free(nxt[j]); }
    free(cur); free(nxt); free(part);
    return rc;
}

static int check_path(const orc_graph *g, const int32_t *vts, int32_t len) {
    if (len < 1) return ORC_EINVAL;
    for (int32_t i = 0; i <= len; i++)
        if (vts[i] < 0 || vts[i] > g->max_vt) return ORC_EINVAL;
    return ORC_OK;
}

int orc_estimate(const orc_graph *g, const int32_t *vts, const int32_t *ets, int32_t len,
                 int32_t threads, double *c_out, double *es_seconds) {
    int rc = check_path(g, vts, len);
    if (rc) return rc;
    if (threads < 1) threads = 1;
    omp_set_num_threads(threads);
    rowmat **mats = (rowmat **)calloc((size_t)len, sizeof(rowmat *));
    if (!mats) return ORC_ENOMEM;
    for (int32_t i = 0; i < len; i++) {
        mats[i] = leaf_matrix(g, vts[i], vts[i + 1], ets[i], 0);
        if (!mats[i]) rc = ORC_ENOMEM;
    }
    double t0 = now_s();
    if (!rc) rc = estimate_core(g, mats, vts, len, threads, c_out);
    if (es_seconds) *es_seconds = now_s() - t0;
    for (int32_t i = 0; i < len; i++) rowmat_free(mats[i]);
    free(mats);
    return rc;
}

/* DP: efficient/resmcm.cpp:519-536.  Costs evaluated in the reference's
 * expression order; strict '<' keeps the smallest k on ties. */
int orc_dp(const double *c, int32_t len, double *m, int32_t *s) {
    if (len < 1) return ORC_EINVAL;
    int32_t sz = len * len;
    double *cc = (double *)malloc(sizeof(double) * (size_t)sz);
    if (!cc) return ORC_ENOMEM;
    memcpy(cc, c, sizeof(double) * (size_t)sz);
    for (int32_t i = 0; i < len; i++) cc[i * len + i] = 0;   /* never set by the estimator */
    memset(m, 0, sizeof(double) * (size_t)sz);
    memset(s, 0, sizeof(int32_t) * (size_t)sz);
    for (int32_t l = 1; l < len; l++) {
        for (int32_t i = 0; i < len - l; i++) {
            int32_t j = i + l;
            m[i * len + j] = DBL_MAX;
            for (int32_t k = i; k < j; k++) {
                double tmp = cc[i * len + k] + cc[(k + 1) * len + j] + cc[i * len + j];
                double cost = m[i * len + k] + m[(k + 1) * len + j] + tmp;
                if (cost < m[i * len + j]) {
                    m[i * len + j] = cost;
                    s[i * len + j] = k;
                }
            }
        }
    }
    free(cc);
    return ORC_OK;
}

/* get_optimal_chain_order, efficient/resmcm.cpp:563-573 */
static int32_t order_rec(const int32_t *s, int32_t len, int32_t i, int32_t j, int32_t *pairs, int32_t *np) {
    if (i == j) return i;
    int32_t k = order_rec(s, len, i, s[i * len + j], pairs, np);
    int32_t l = order_rec(s, len, s[i * len + j] + 1, j, pairs, np);
    pairs[2 * *np] = k;
    pairs[2 * *np + 1] = l;
    (*np)++;
    return -1;
}

int orc_order(const int32_t *s, int32_t len, int32_t *pairs) {
    if (len < 1) return ORC_EINVAL;
    int32_t np = 0;
    order_rec(s, len, 0, len - 1, pairs, &np);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* SpGEMM                                                                    */
/* ------------------------------------------------------------------------ */

/* Boolean Gustavson: row_wise_SpGEMM_based_on_bitmap :586-615 driven by
 * SpGEMM :619-647 (dynamic chunks of ceil(|bins| / (8 tnum)), a per-thread
 * bitmap slice, per-row timing counters). */
static rowmat *spgemm_bool(const orc_graph *g, const rowmat *A, const rowmat *B, unsigned char *bitmap,
                           int32_t tnum, double *t_times, int64_t *t_rows) {
    rowmat *C = rowmat_new(g->n, A->row_vt, B->col_vt);
    if (!C) return NULL;
    int32_t rt = A->row_vt;
    int64_t b0 = g->bin_ptr[rt], b1 = g->bin_ptr[rt + 1];
    int64_t chunk = (int64_t)((b1 - b0 + (int64_t)tnum * 8 - 1) / ((int64_t)tnum * 8));
    if (chunk < 1) chunk = 1;
    int64_t n = g->n;
    int fail = 0;
#pragma omp parallel num_threads(tnum)
    {
        int tid = omp_get_thread_num();
        unsigned char *seen = bitmap + (size_t)tid * (size_t)n;
        int64_t qcap = 1024, qn;
        int32_t *queue = (int32_t *)malloc(sizeof(int32_t) * (size_t)qcap);
        if (!queue) fail = 1;
#pragma omp for schedule(dynamic, chunk)
        for (int64_t k = b0; k < b1; k++) {
            if (!queue) continue;
            double ts = now_s();
            int32_t u = g->bin_ids[k];
            qn = 0;
            for (int64_t a = 0; a < A->len[u]; a++) {
                int32_t w = A->cols[u][a];
                const int32_t *brow = B->cols[w];
                int64_t bl = B->len[w];
                for (int64_t q = 0; q < bl; q++) {
                    int32_t v = brow[q];
                    if (seen[v]) continue;
                    seen[v] = 1;
                    if (qn == qcap) {
                        qcap *= 2;
                        int32_t *nq = (int32_t *)realloc(queue, sizeof(int32_t) * (size_t)qcap);
                        if (!nq) { fail = 1; break; }
                        queue = nq;
                    }
                    queue[qn++] = v;
                }
            }
            int32_t *row = (int32_t *)malloc(sizeof(int32_t) * (size_t)(qn ? qn : 1));
            if (!row) { fail = 1; }
            else memcpy(row, queue, sizeof(int32_t) * (size_t)qn);
            C->cols[u] = row;
            C->len[u] = qn;
            for (int64_t q = 0; q < qn; q++) seen[queue[q]] = 0;
            t_times[tid] += now_s() - ts;
            t_rows[tid] += A->len[u];
        }
        free(queue);
    }
    if (fail) { rowmat_free(C); return NULL; }
    return C;
}

static int cmp_i32(const void *a, const void *b) {
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* Counting Gustavson: exact uint64 path counts, rows sorted ascending.
 * Not in the reference (Boolean); it pins the GPU path's integer values. */
static rowmat *spgemm_count(const orc_graph *g, const rowmat *A, const rowmat *B, int32_t tnum, int *overflow) {
    rowmat *C = rowmat_new(g->n, A->row_vt, B->col_vt);
    if (!C) return NULL;
    int32_t rt = A->row_vt;
    int64_t b0 = g->bin_ptr[rt], b1 = g->bin_ptr[rt + 1];
    int64_t n = g->n;
    int fail = 0, ovf = 0;
#pragma omp parallel num_threads(tnum) reduction(| : ovf)
    {
        uint64_t *acc = (uint64_t *)calloc((size_t)(n ? n : 1), sizeof(uint64_t));
        unsigned char *mark = (unsigned char *)calloc((size_t)(n ? n : 1), 1);
        int64_t qcap = 1024, qn;
        int32_t *queue = (int32_t *)malloc(sizeof(int32_t) * (size_t)qcap);
        if (!acc || !mark || !queue) fail = 1;
#pragma omp for schedule(dynamic, 64)
        for (int64_t k = b0; k < b1; k++) {
            if (!acc || !mark || !queue) continue;
            int32_t u = g->bin_ids[k];
            qn = 0;
            for (int64_t a = 0; a < A->len[u]; a++) {
                int32_t w = A->cols[u][a];
                uint64_t va = A->vals[u][a];
                for (int64_t q = 0; q < B->len[w]; q++) {
                    int32_t v = B->cols[w][q];
                    uint64_t prod, sum;
                    if (__builtin_mul_overflow(va, B->vals[w][q], &prod)) ovf = 1;
                    if (__builtin_add_overflow(acc[v], prod, &sum)) ovf = 1;
                    acc[v] = sum;
                    if (!mark[v]) {
                        mark[v] = 1;
                        if (qn == qcap) {
                            qcap *= 2;
                            int32_t *nq = (int32_t *)realloc(queue, sizeof(int32_t) * (size_t)qcap);
                            if (!nq) { fail = 1; break; }
                            queue = nq;
                        }
                        queue[qn++] = v;
                    }
                }
            }
            qsort(queue, (size_t)qn, sizeof(int32_t), cmp_i32);
            C->cols[u] = (int32_t *)malloc(sizeof(int32_t) * (size_t)(qn ? qn : 1));
            C->vals[u] = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(qn ? qn : 1));
            if (!C->cols[u] || !C->vals[u]) { fail = 1; continue; }
            for (int64_t q = 0; q < qn; q++) {
                int32_t v = queue[q];
                C->cols[u][q] = v;
                C->vals[u][q] = acc[v];
                acc[v] = 0;
                mark[v] = 0;
            }
            C->len[u] = qn;
        }
        free(acc); free(mark); free(queue);
    }
    *overflow |= ovf;
    if (fail) { rowmat_free(C); return NULL; }
    return C;
}

/* ------------------------------------------------------------------------ */
/* chain executor: SSP_dynamic, efficient/resmcm.cpp:653-772                 */
/* ------------------------------------------------------------------------ */

static int chain_impl(const orc_graph *g, const char *metapath, const int32_t *fixed_pairs,
                      int32_t mode, int32_t threads, orc_result **out, orc_times *times) {
    *out = NULL;
    orc_times tm = {0, 0, 0, 0};
    int32_t vts[64], ets[64], len = 0;
    int rc = orc_metapath_parse(metapath, vts, ets, 63, &len);
    if (rc) return rc;
    rc = check_path(g, vts, len);
    if (rc) return rc;
    if (threads < 1) threads = 1;
    omp_set_num_threads(threads);
    int cm = (mode == ORC_MODE_COUNT);

    rowmat *mats[64] = {0};
    for (int32_t i = 0; i < len; i++) {           /* not timed, :664-667 */
        mats[i] = leaf_matrix(g, vts[i], vts[i + 1], ets[i], cm);
        if (!mats[i]) { rc = ORC_ENOMEM; goto fail; }
    }
    orc_result *res = (orc_result *)calloc(1, sizeof(orc_result));
    if (!res) { rc = ORC_ENOMEM; goto fail; }
    res->g = g;
    res->mode = mode;
    if (len == 1) {                                /* :670-677 */
        res->mat = mats[0];
        mats[0] = NULL;
    } else {
        double t_start = now_s();                  /* :679-680 */
        double c[64 * 64], m[64 * 64];
        int32_t s[64 * 64], pairs[2 * 64];
        double e0 = now_s();
        rc = estimate_core(g, mats, vts, len, threads, c);
        tm.es = now_s() - e0;
        if (rc) { free(res); goto fail; }
        double d0 = now_s();
        orc_dp(c, len, m, s);
        tm.dp = now_s() - d0;
        if (fixed_pairs) memcpy(pairs, fixed_pairs, sizeof(int32_t) * 2 * (size_t)(len - 1));
        else orc_order(s, len, pairs);

        unsigned char *bitmap = NULL;              /* :693-700, inside the timed region */
        double *t_times = (double *)calloc((size_t)threads, sizeof(double));
        int64_t *t_rows = (int64_t *)calloc((size_t)threads, sizeof(int64_t));
        if (!cm) {
            bitmap = (unsigned char *)malloc((size_t)threads * (size_t)(g->n ? g->n : 1));
            if (bitmap) {
#pragma omp parallel num_threads(threads)
                {
                    int tid = omp_get_thread_num();
                    memset(bitmap + (size_t)tid * (size_t)g->n, 0, (size_t)g->n);
                }
            }
        }
        if ((!cm && !bitmap) || !t_times || !t_rows) {
            free(bitmap); free(t_times); free(t_rows); free(res);
            rc = ORC_ENOMEM; goto fail;
        }
        rowmat *stack[64] = {0};
        int32_t sp = 0;
        int ovf = 0;
        for (int32_t p = 0; p < len - 1 && !rc; p++) {     /* executor :709-760 */
            int32_t k = pairs[2 * p], l = pairs[2 * p + 1];
            rowmat *A, *B;
            if (k >= 0 && l >= 0) { A = mats[k]; B = mats[l]; }
            else if (k == -1 && l >= 0) { A = stack[sp - 1]; B = mats[l]; }
            else if (k >= 0 && l == -1) { A = mats[k]; B = stack[sp - 1]; }
            else { A = stack[sp - 2]; B = stack[sp - 1]; }
            double s0 = now_s();
            rowmat *C = cm ? spgemm_count(g, A, B, threads, &ovf)
                           : spgemm_bool(g, A, B, bitmap, threads, t_times, t_rows);
            tm.spgemm += now_s() - s0;
            if (!C) { rc = ORC_ENOMEM; break; }
            if (k >= 0 && l >= 0) {
                rowmat_free(mats[k]); mats[k] = NULL;
                rowmat_free(mats[l]); mats[l] = NULL;
                stack[sp++] = C;
            } else if (k == -1 && l >= 0) {
                rowmat_free(mats[l]); mats[l] = NULL;
                rowmat_free(stack[sp - 1]);
                stack[sp - 1] = C;
            } else if (k >= 0 && l == -1) {
                rowmat_free(mats[k]); mats[k] = NULL;
                rowmat_free(stack[sp - 1]);
                stack[sp - 1] = C;
            } else {
                rowmat_free(stack[sp - 1]);
                rowmat_free(stack[sp - 2]);
                stack[sp - 2] = C;
                sp--;
            }
        }
        free(bitmap); free(t_times); free(t_rows);
        if (rc) {
            for (int32_t q = 0; q < sp; q++) rowmat_free(stack[q]);
            free(res);
            goto fail;
        }
        res->mat = stack[0];
        tm.total = now_s() - t_start;              /* :770-771 */
        if (ovf) rc = ORC_EOVERFLOW;
    }
    /* nnz over the rows of the start type, main :859-868 */
    {
        int32_t st = vts[0];
        int64_t nnz = 0;
        for (int64_t k = g->bin_ptr[st]; k < g->bin_ptr[st + 1]; k++) nnz += res->mat->len[g->bin_ids[k]];
        res->nnz = nnz;
    }
    for (int32_t i = 0; i < len; i++) rowmat_free(mats[i]);
    if (times) *times = tm;
    *out = res;
    return rc;
fail:
    for (int32_t i = 0; i < len; i++) rowmat_free(mats[i]);
    if (times) *times = tm;
    return rc;
}

int orc_chain(const orc_graph *g, const char *metapath, int32_t mode, int32_t threads,
              orc_result **out, orc_times *times) {
    return chain_impl(g, metapath, NULL, mode, threads, out, times);
}

int orc_chain_with_order(const orc_graph *g, const char *metapath, const int32_t *pairs,
                         int32_t mode, int32_t threads, orc_result **out, orc_times *times) {
    return chain_impl(g, metapath, pairs, mode, threads, out, times);
}

int64_t orc_result_rows(const orc_result *r) { return r->g->dims[r->mat->row_vt]; }
int64_t orc_result_nnz(const orc_result *r) { return r->nnz; }

int orc_result_export(const orc_result *r, int64_t *rowptr, int32_t *col, uint64_t *val) {
    const orc_graph *g = r->g;
    int32_t rt = r->mat->row_vt;
    int64_t b0 = g->bin_ptr[rt], b1 = g->bin_ptr[rt + 1];
    rowptr[0] = 0;
    for (int64_t k = b0; k < b1; k++) {
        int32_t u = g->bin_ids[k];
        rowptr[k - b0 + 1] = rowptr[k - b0] + r->mat->len[u];
    }
    if (!col) return ORC_OK;
    int fail = 0;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t k = b0; k < b1; k++) {
        int32_t u = g->bin_ids[k];
        int64_t o = rowptr[k - b0], L = r->mat->len[u];
        int32_t *dst = col + o;
        for (int64_t q = 0; q < L; q++) dst[q] = r->mat->cols[u][q];
        if (r->mode == ORC_MODE_BOOL) {
            qsort(dst, (size_t)L, sizeof(int32_t), cmp_i32);
        } else if (val) {
            for (int64_t q = 0; q < L; q++) val[o + q] = r->mat->vals[u][q];
        }
        for (int64_t q = 0; q < L; q++) dst[q] = g->local[dst[q]];
        if (val && r->mode == ORC_MODE_BOOL)
            for (int64_t q = 0; q < L; q++) val[o + q] = 1;
    }
    return fail ? ORC_ENOMEM : ORC_OK;
}

/* splitmix64 output function (Steele, Lea and Flood, OOPSLA 2014). */
static uint64_t mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xBF58476D1CE4E5B9ULL;
    x ^= x >> 27;
    x *= 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

/* Order-free digest of the result in local ids: the sum mod 2^64 over its
 * entries (r, c, v) of mix64(mix64(r * 2^32 + c) + v), v = 1 in Boolean
 * mode.  Not in the reference; it lets a test compare a result of billions
 * of entries with another implementation's without exporting it. */
int orc_result_digest(const orc_result *r, uint64_t *digest) {
    const orc_graph *g = r->g;
    int32_t rt = r->mat->row_vt;
    int64_t b0 = g->bin_ptr[rt], b1 = g->bin_ptr[rt + 1];
    uint64_t acc = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : acc)
    for (int64_t k = b0; k < b1; k++) {
        int32_t u = g->bin_ids[k];
        uint64_t row = (uint64_t)(k - b0) << 32;
        int64_t L = r->mat->len[u];
        for (int64_t q = 0; q < L; q++) {
            uint64_t key = row | (uint64_t)(uint32_t)g->local[r->mat->cols[u][q]];
            uint64_t v = r->mode == ORC_MODE_COUNT ? r->mat->vals[u][q] : 1;
            acc += mix64(mix64(key) + v);
        }
    }
    *digest = acc;
    return ORC_OK;
}

void orc_result_free(orc_result *r) {
    if (!r) return;
    rowmat_free(r->mat);
    free(r);
}
