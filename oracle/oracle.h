/*
 * CPU oracle for the RESMCM sparse-matrix-chain path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the tests, the
 * smoke check and the CPU-baseline leg of the benchmark call it to produce
 * the expected answer (or the reference-algorithm CPU timing).  The GPU
 * product path never links, loads or calls it.
 *
 * It restates, in plain C with OpenMP, the algorithm of the reference program
 * efficient/resmcm.cpp (swordzlim/RESMCM_ARI):
 *   - text loader           DataReader           efficient/resmcm.cpp:49-177
 *   - typed graph, bins     HeteroGraph          efficient/resmcm.cpp:181-240
 *   - meta-path grammar     MetaPath(string)     efficient/resmcm.cpp:269-299
 *   - leaf matrices         BoolMatrix(HIN,...)  efficient/resmcm.cpp:374-396
 *   - leaf sparsity         getSparsities        efficient/resmcm.cpp:442-452
 *   - RES estimator step    compute_sparsities   efficient/resmcm.cpp:468-485
 *   - chain-order DP        rows_sparse_optimal_matrix_chain_order
 *                                                 efficient/resmcm.cpp:488-541
 *   - order extraction      get_optimal_chain_order efficient/resmcm.cpp:563-573
 *   - Boolean Gustavson     row_wise_SpGEMM_based_on_bitmap / SpGEMM
 *                                                 efficient/resmcm.cpp:586-647
 *   - chain executor        SSP_dynamic          efficient/resmcm.cpp:653-772
 * plus a counting Gustavson (exact uint64 path counts with an overflow flag),
 * which the reference does not have (it is Boolean) and which pins the
 * integer values the GPU path produces.
 *
 * Matrices use global vertex ids, as in the reference (n x n with empty rows
 * for vertices of other types); results are exported in per-type local ids
 * (rank of a vertex among the ascending global ids of its type).
 */
#ifndef RESMCM_ORACLE_H
#define RESMCM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_OK = 0, ORC_EINVAL = 1, ORC_ENOMEM = 2, ORC_EOVERFLOW = 3, ORC_EIO = 6, ORC_EPARSE = 7 };
enum { ORC_MODE_BOOL = 0, ORC_MODE_COUNT = 1 };

typedef struct orc_graph orc_graph;
typedef struct orc_result orc_result;

typedef struct {
    double es;      /* estimator seconds  (es_time) */
    double dp;      /* DP seconds         (dp_time) */
    double spgemm;  /* SpGEMM seconds     (spgemm_time) */
    double total;   /* chain seconds      (smcm_time) */
} orc_times;

int orc_graph_load_text(const char *graph, const char *vertex, const char *edge, orc_graph **out);
int orc_graph_from_arrays(int64_t n, const int32_t *vtype, const int64_t *adj_ptr,
                          const int32_t *adj_nbr, const int32_t *adj_et, orc_graph **out);
void orc_graph_free(orc_graph *g);
int64_t orc_graph_n(const orc_graph *g);
int64_t orc_graph_m(const orc_graph *g);
int32_t orc_graph_max_vt(const orc_graph *g);
int64_t orc_graph_dim(const orc_graph *g, int32_t vt);
/* Export the parsed adjacency (graph.txt order) and vertex types. */
void orc_graph_export(const orc_graph *g, int32_t *vtype, int64_t *adj_ptr, int32_t *adj_nbr, int32_t *adj_et);

int orc_metapath_parse(const char *s, int32_t *vts, int32_t *ets, int32_t cap, int32_t *len);

/* Leaf matrix M = BoolMatrix(HIN, vt, src, sink, et) in local ids.
 * rowptr: dims[src]+1, col: caller sizes it from a first call with col == NULL. */
int orc_leaf(const orc_graph *g, int32_t src_vt, int32_t sink_vt, int32_t et,
             int64_t *rowptr, int32_t *col);

/* Estimator: c_out[len*len] (row-major c_[i*len+j]); with threads == 1 the
 * sums follow the reference's sequential order exactly. */
int orc_estimate(const orc_graph *g, const int32_t *vts, const int32_t *ets, int32_t len,
                 int32_t threads, double *c_out, double *es_seconds);
/* DP over c (c_[i*len+i] ignored, treated as 0 like the reference's memset). */
int orc_dp(const double *c, int32_t len, double *m_out, int32_t *s_out);
/* Post-order (k,l) pair list, -1 = "top of the temporary stack". */
int orc_order(const int32_t *s, int32_t len, int32_t *pairs);

/* Whole chain (SSP_dynamic).  mode: ORC_MODE_BOOL runs the reference's
 * Boolean bitmap Gustavson (rows in discovery order); ORC_MODE_COUNT runs
 * the counting Gustavson (sorted rows, uint64 values).  Returns ORC_EOVERFLOW
 * (result kept, values invalid) if a uint64 count overflowed. */
int orc_chain(const orc_graph *g, const char *metapath, int32_t mode, int32_t threads,
              orc_result **out, orc_times *times);
/* Same chain with a caller-fixed order (pairs as produced by orc_order). */
int orc_chain_with_order(const orc_graph *g, const char *metapath, const int32_t *pairs,
                         int32_t mode, int32_t threads, orc_result **out, orc_times *times);
int64_t orc_result_rows(const orc_result *r);
int64_t orc_result_nnz(const orc_result *r);
/* Export in local ids with each row sorted ascending; val may be NULL. */
int orc_result_export(const orc_result *r, int64_t *rowptr, int32_t *col, uint64_t *val);
/* Order-free digest of the result (local ids): sum mod 2^64 of
 * mix64(mix64(row * 2^32 + col) + value), value 1 in Boolean mode. */
int orc_result_digest(const orc_result *r, uint64_t *digest);
void orc_result_free(orc_result *r);

#ifdef __cplusplus
}
#endif
#endif
