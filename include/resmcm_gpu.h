/*
 * resmcm_gpu.h — C ABI of the GB300 (sm_103a) sparse-matrix-chain engine.
 *
 * Drop-in for the RESMCM chain path of efficient/resmcm.cpp
 * (swordzlim/RESMCM_ARI): RES row-wise sparsity estimator → chain-order DP →
 * Gustavson SpGEMM chain.  The reference has no library boundary; its seam is
 * the function SSP_dynamic (efficient/resmcm.cpp:653-772) called by
 * build_pair (:774-779) from main (:782-895).  Each entry point below names
 * the reference interface it replaces.
 *
 * Conventions
 *   - Every function returns an rmcm_status (0 = RMCM_OK); no C++ exception
 *     crosses the boundary.  rmcm_last_error() gives a message for the last
 *     failing call on a handle.
 *   - Plain pointers and sizes only.  Host arrays are caller-owned; device
 *     matrices (rmcm_mat) are owned by the handle that made them and freed
 *     with rmcm_mat_free (leaf matrices are owned by their graph).
 *   - Vertex ids inside matrices are per-type LOCAL ids: the rank of a vertex
 *     among the ascending global ids of its type (the order of
 *     HeteroGraph::bins, efficient/resmcm.cpp:214-222).  Rows of every matrix
 *     have ascending column indices.
 *   - Work is issued on the handle's CUDA stream (rmcm_set_stream).  Calls
 *     that return host data synchronise that stream.
 *   - A handle is not thread-safe; use one handle per host thread.
 */
#ifndef RESMCM_GPU_H
#define RESMCM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define RMCM_API __attribute__((visibility("default")))
#else
#define RMCM_API
#endif

typedef enum rmcm_status {
    RMCM_OK = 0,
    RMCM_EINVAL = 1,        /* bad argument, shape mismatch, bad meta-path */
    RMCM_ENOMEM = 2,        /* device memory budget or device allocation exhausted */
    RMCM_EOVERFLOW = 3,     /* a path count exceeded the value type (structure still exact) */
    RMCM_ETIMEOUT = 4,      /* a bounded device wait gave up */
    RMCM_ECUDA = 5,         /* CUDA runtime error */
    RMCM_EIO = 6,           /* file could not be read */
    RMCM_EPARSE = 7,        /* malformed input file */
    RMCM_EINTERNAL = 8      /* a device-side invariant check failed */
} rmcm_status;

typedef enum rmcm_valtype {
    RMCM_VAL_U32 = 0,       /* uint32 path counts */
    RMCM_VAL_U64 = 1,       /* uint64 path counts */
    RMCM_VAL_AUTO = 2       /* uint32, re-run in uint64 if a count overflows */
} rmcm_valtype;

typedef enum rmcm_order_mode {
    RMCM_ORDER_RES = 0,     /* RES estimates + DP (efficient/resmcm.cpp) */
    RMCM_ORDER_L2R = 1,     /* left to right, no estimator (efficient/l2r.cpp:725-727) */
    RMCM_ORDER_DENSE = 2    /* DP over dense dimensions, no estimator (efficient/naive.cpp:506-523) */
} rmcm_order_mode;

typedef struct rmcm_handle rmcm_handle;
typedef struct rmcm_graph rmcm_graph;
typedef struct rmcm_mat rmcm_mat;
typedef struct rmcm_batch rmcm_batch;
typedef struct rmcm_server rmcm_server;

typedef struct rmcm_opts {
    int32_t device;            /* CUDA device ordinal */
    int32_t valtype;           /* rmcm_valtype used by rmcm_run_metapath / rmcm_chain */
    int64_t mem_budget_bytes;  /* 0 = 90% of the device memory free at create time */
    void *stream;              /* cudaStream_t to use; NULL = the handle creates one */
} rmcm_opts;

/* Times of one chain, with the region definitions of the reference's timers
 * (efficient/resmcm.cpp:18-21): es = estimator (:506-517), dp = DP (:519-538),
 * spgemm = sum of the products (:620-645), total = whole chain after the
 * leaf matrices exist (:679-771).  Seconds. */
typedef struct rmcm_timings {
    double total_s;
    double spgemm_s;
    double dp_s;
    double es_s;
    int64_t nnz;               /* result nnz (Boolean structure size) */
    int64_t flops;             /* sum over the products of the multiply-adds */
    int32_t valtype;           /* value type the result was computed in */
    int32_t n_products;
} rmcm_timings;

/* Per-product record kept while profiling is on (rmcm_set_profiling,
 * rmcm_get_product_stats).
 * Bytes are the algorithmic (compulsory) bytes of C = A*B: with ip = 8
 * (row pointers) and iv = value bytes, bytes_a = (rows+1)*ip + nnz_a*(4+iv),
 * bytes_b_touched = sum over the distinct columns c of A of
 * (2*ip + |B[c]|*(4+iv)), bytes_c = (rows+1)*ip + nnz_c*(4+iv). */
typedef struct rmcm_product_stats {
    int64_t rows, inner, cols;          /* A is rows x inner, B is inner x cols */
    int64_t nnz_a, nnz_b, nnz_c, flops;
    int64_t touched_rows;               /* distinct columns of A (B rows read); level 2 only */
    int64_t touched_nnz;                /* entries of those B rows; level 2 only */
    int64_t bytes_a, bytes_b_touched, bytes_c;   /* level 2 only */
    double analyze_ms, symbolic_ms, numeric_ms;  /* CUDA-event times on the handle's stream; symbolic_ms
                                                    includes the setup after the analysis (temporaries,
                                                    packing, the tensor-core part, split preparation) */
    int32_t valtype;
    int32_t bin_rows[8];                /* rows per bin: tiny, hash512, hash2k, hash8k, dense, rank, micro, warp */
    int32_t gemm_limbs;                 /* limb pairs (A x B) of the tensor-core GEMM (0: no GEMM part) */
    int64_t gemm_inner;                 /* inner indices multiplied by that GEMM */
    double gemm_ms;                     /* CUDA-event time of its GEMM calls */
} rmcm_product_stats;

/* ---- handle -------------------------------------------------------------- */
RMCM_API const char *rmcm_status_string(int32_t status);
RMCM_API int32_t rmcm_create(rmcm_handle **out, const rmcm_opts *opts);
RMCM_API int32_t rmcm_destroy(rmcm_handle *h);
RMCM_API const char *rmcm_last_error(const rmcm_handle *h);
RMCM_API int32_t rmcm_set_stream(rmcm_handle *h, void *stream);
RMCM_API void *rmcm_get_stream(const rmcm_handle *h);
/* Bytes of device memory currently held by matrices and scratch. */
RMCM_API int64_t rmcm_mem_in_use(const rmcm_handle *h);
/* Largest rmcm_mem_in_use since the handle was created or the last reset
 * (reset != 0 restarts it from the current use). */
RMCM_API int64_t rmcm_mem_peak(rmcm_handle *h, int32_t reset);
/* Number of kernels this handle has launched so far. */
RMCM_API int64_t rmcm_kernel_launches(const rmcm_handle *h);
/* Profiling of SpGEMM products: 0 off, 1 CUDA-event times, 2 times and
 * algorithmic byte counts (adds a small kernel and a sync per product). */
RMCM_API int32_t rmcm_set_profiling(rmcm_handle *h, int32_t level);
/* Copies up to cap records (oldest first) of the products run since the
 * last reset; *count = records available.  reset != 0 drops them after the
 * copy.  Synchronises the handle's stream. */
RMCM_API int32_t rmcm_get_product_stats(rmcm_handle *h, rmcm_product_stats *out, int32_t cap, int32_t *count,
                                        int32_t reset);

/* ---- typed graph: replaces DataReader + HeteroGraph, efficient/resmcm.cpp:49-240 ---- */
/* Reads vertex.txt (vid vt), edge.txt (eid et) and graph.txt (vid (nbr eid)*). */
RMCM_API int32_t rmcm_graph_load_text(rmcm_handle *h, const char *graph_file, const char *vertex_file,
                                      const char *edge_file, rmcm_graph **out);
/* Same graph from arrays: vtype[n], adjacency adj_ptr[n+1] / adj_nbr[m] / adj_et[m]
 * (global ids, graph.txt order, adj_et = edge TYPE of each entry). */
RMCM_API int32_t rmcm_graph_from_adjacency(rmcm_handle *h, int64_t n, const int32_t *vtype,
                                           const int64_t *adj_ptr, const int32_t *adj_nbr,
                                           const int32_t *adj_et, rmcm_graph **out);
RMCM_API int32_t rmcm_graph_free(rmcm_graph *g);
RMCM_API int32_t rmcm_graph_info(const rmcm_graph *g, int64_t *n, int64_t *m, int32_t *max_vt);
/* Vertices of type vt (HeteroGraph::dimensions, efficient/resmcm.cpp:206-212). */
RMCM_API int64_t rmcm_graph_dim(const rmcm_graph *g, int32_t vt);

/* ---- meta-path: replaces MetaPath(string) / toString, efficient/resmcm.cpp:269-308 ---- */
/* vts needs cap+1 slots, ets cap slots; *len = number of edge types (matrices). */
RMCM_API int32_t rmcm_metapath_parse(const char *s, int32_t *vts, int32_t *ets, int32_t cap, int32_t *len);
RMCM_API int32_t rmcm_metapath_format(const int32_t *vts, const int32_t *ets, int32_t len, char *buf,
                                      int64_t cap);

/* ---- matrices ------------------------------------------------------------ */
/* Leaf matrix of one edge type: replaces BoolMatrix(HIN, vt, src, sink, et, n),
 * efficient/resmcm.cpp:374-396.  Rows = vertices of type src, columns =
 * vertices of type sink, one entry (value 1) per adjacency entry of edge type
 * et whose neighbour has type sink; repeated neighbours stay separate entries.
 * Device resident and cached in the graph (owned by it; do not free). */
RMCM_API int32_t rmcm_leaf(rmcm_handle *h, rmcm_graph *g, int32_t src_vt, int32_t sink_vt, int32_t et,
                           int32_t valtype, rmcm_mat **out);
/* Upload a CSR from host memory (rowptr[rows+1], col[nnz], val[nnz] of
 * valtype or NULL for all ones).  The arrays are checked on the device after
 * the copy (row pointers non-decreasing and within nnz, columns in
 * [0, cols): RMCM_EINVAL otherwise).  Rows need not be sorted: a matrix with
 * an unsorted row is sorted on the host (stable, values follow their
 * columns) and copied again. */
RMCM_API int32_t rmcm_mat_upload(rmcm_handle *h, int64_t rows, int64_t cols, const int64_t *rowptr,
                                 const int32_t *col, const void *val, int32_t valtype, rmcm_mat **out);
RMCM_API int32_t rmcm_mat_info(const rmcm_mat *m, int64_t *rows, int64_t *cols, int64_t *nnz,
                               int32_t *valtype);
/* Copy a device matrix to host arrays (rowptr[rows+1], col[nnz], val[nnz]);
 * any pointer may be NULL to skip that array. */
RMCM_API int32_t rmcm_mat_download(rmcm_handle *h, const rmcm_mat *m, int64_t *rowptr, int32_t *col,
                                   void *val);
RMCM_API int32_t rmcm_mat_free(rmcm_handle *h, rmcm_mat *m);
/* Asynchronous download (no reference counterpart: the reference keeps its
 * results in host memory): the same copies as rmcm_mat_download, issued on
 * the handle's transfer stream once the work already queued on its stream is
 * done, so a result can travel to the host while the next chain computes.
 * The host buffers (pinned memory for full speed) must stay valid until
 * rmcm_transfers_wait returns; rmcm_mat_free may be called at once — the
 * matrix is released when its download has landed. */
RMCM_API int32_t rmcm_mat_download_async(rmcm_handle *h, rmcm_mat *m, int64_t *rowptr, int32_t *col, void *val);
/* Waits for every asynchronous download of the handle. */
RMCM_API int32_t rmcm_transfers_wait(rmcm_handle *h);
/* Waits for all work of the handle (its stream and its transfer stream).
 * Matrices made on one handle may be read by another handle's operations
 * once this has returned (a loader thread can upload the next chain on its
 * own handle while this one multiplies). */
RMCM_API int32_t rmcm_synchronize(rmcm_handle *h);

/* ---- stage (a): RES estimator ---------------------------------------------
 * Replaces the estimator loop of rows_sparse_optimal_matrix_chain_order
 * (efficient/resmcm.cpp:506-517) with getSparsities (:442-452) and
 * compute_sparsities (:468-485).  c_out[len*len] receives c_[i*len+j]
 * (estimated nnz of M_i..M_j, j > i; 0 elsewhere) in FP64. */
RMCM_API int32_t rmcm_estimate(rmcm_handle *h, rmcm_mat *const *chain, int32_t len, double *c_out);

/* ---- stage (b): chain-order DP --------------------------------------------
 * Replaces the DP of rows_sparse_optimal_matrix_chain_order
 * (efficient/resmcm.cpp:519-536) and get_optimal_chain_order (:563-573).
 * Runs as one warp on the device, 2 <= len <= 16.  split/cost are len*len
 * (may be NULL); pairs[2*(len-1)] receives the post-order (k,l) list where -1
 * means "the top of the temporary stack". */
RMCM_API int32_t rmcm_order(rmcm_handle *h, const double *c, int32_t len, int32_t *split, double *cost,
                            int32_t *pairs);

/* ---- stage (c): Gustavson SpGEMM ------------------------------------------
 * Replaces SpGEMM / row_wise_SpGEMM_based_on_bitmap (efficient/resmcm.cpp:586-647).
 * C = A*B with exact integer path counts in A's value type; C's rows are
 * sorted.  Returns RMCM_EOVERFLOW (C kept) if a count overflowed. */
RMCM_API int32_t rmcm_spgemm(rmcm_handle *h, const rmcm_mat *A, const rmcm_mat *B, rmcm_mat **C);

/* ---- (a)+(b)+(c): one chain -----------------------------------------------
 * Replaces SSP_dynamic (efficient/resmcm.cpp:653-772) on matrices that are
 * already device resident.  The chain's matrices are not modified.  When
 * pairs is non-NULL it overrides the DP's order (same encoding as rmcm_order). */
RMCM_API int32_t rmcm_chain(rmcm_handle *h, rmcm_mat *const *chain, int32_t len, const int32_t *pairs,
                            rmcm_mat **C, rmcm_timings *t);

/* ---- whole meta-path over a graph -----------------------------------------
 * build_pair + nnz count of main (efficient/resmcm.cpp:774-779, :859-868):
 * leaf matrices (cached in the graph), then rmcm_chain.  C may be NULL, in
 * which case the result is freed after its nnz is taken. */
RMCM_API int32_t rmcm_run_metapath(rmcm_handle *h, rmcm_graph *g, const char *metapath, rmcm_mat **C,
                                   rmcm_timings *t);

/* ---- whole meta-path, result delivered in blocks of rows ------------------
 * The executor of SSP_dynamic (efficient/resmcm.cpp:702-760) and the nnz
 * count of main (:859-868), for results too large to hold on the device: the
 * chain runs as rmcm_run_metapath, except that its final product is computed
 * a block of rows at a time (rows of its left operand) and each block is
 * handed to fn as a device matrix (rows block_rows x the result's columns,
 * row pointers from 0, valid only during the call; row0 = the block's first
 * row in the result), then freed.  rows_per_block 0 lets the library choose:
 * a block's RES-estimated entries take at most a quarter of the device
 * memory left under the handle's budget.  A non-OK return from fn stops the
 * chain with that status.  t->nnz is the sum over the blocks.  In AUTO mode
 * blocks that fit uint32 are delivered as uint32 and, after the first block
 * that overflows, the rest as uint64 (each block's values are exact). */
typedef int32_t (*rmcm_block_fn)(void *user, int64_t row0, const rmcm_mat *block);
RMCM_API int32_t rmcm_run_metapath_blocks(rmcm_handle *h, rmcm_graph *g, const char *metapath,
                                          int64_t rows_per_block, rmcm_block_fn fn, void *user, rmcm_timings *t);

/* Order used by rmcm_run_metapath / rmcm_chain when no pair list is given.
 * The ablation orders of the reference's l2r and naive programs skip the
 * estimator (es time 0), exactly as those programs do. */
RMCM_API int32_t rmcm_set_order_mode(rmcm_handle *h, int32_t mode);
/* Left-to-right pair list (0,1), (-1,2), ..., (-1,len-1): efficient/l2r.cpp:725-727. */
RMCM_API int32_t rmcm_order_l2r(int32_t len, int32_t *pairs);
/* DP of efficient/naive.cpp:506-523 over dims_vt[len+1] (the vertex counts
 * of the meta-path's types): cost(i,k,j) = m[i][k] + m[k+1][j] +
 * d[i]*d[k]*d[j+1], the product taken in 32-bit two's-complement int
 * arithmetic as the reference's `vertex` (int) operands do, then widened to
 * double; strict '<' keeps the smallest k.  split/cost may be NULL. */
RMCM_API int32_t rmcm_order_dense(const int64_t *dims_vt, int32_t len, int32_t *split, double *cost,
                                  int32_t *pairs);

/* ---- graph cache and result sinks -----------------------------------------
 * Binary form of a typed graph (vertex types and typed adjacency), so a graph
 * parsed once from text loads in one read: "RMCMHIN1", n, m, max_vt, then
 * vtype[n] int32, adj_ptr[n+1] int64, adj_nbr[m] int32, adj_et[m] int32
 * (little endian). */
RMCM_API int32_t rmcm_graph_save(const rmcm_graph *g, const char *path);
RMCM_API int32_t rmcm_graph_load(rmcm_handle *h, const char *path, rmcm_graph **out);
/* Global vertex ids of the vertices of type vt in local-id order (ascending;
 * the order of HeteroGraph::bins).  out needs rmcm_graph_dim(g, vt) slots. */
RMCM_API int32_t rmcm_graph_global_ids(const rmcm_graph *g, int32_t vt, int32_t *out);
/* A matrix to a binary file: "RMCMCSR1", rows, cols, nnz (int64), valtype
 * (int32), 4 bytes padding, rowptr[rows+1] int64, col[nnz] int32,
 * val[nnz] uint32 or uint64. */
RMCM_API int32_t rmcm_mat_save(rmcm_handle *h, const rmcm_mat *m, const char *path);

/* Estimated nnz of the whole chain, c_[0][len-1]: the estimator-only program
 * accuracy/res.cpp (final_result_estimate :564-600, output :698). */
RMCM_API int32_t rmcm_estimate_metapath(rmcm_handle *h, rmcm_graph *g, const char *metapath,
                                        double *est_nnz);

/* ---- SpGEMM tunables --------------------------------------------------------
 * Row binning of every product on this handle (none changes a result):
 *   threads_per_row  rows of at most 32 products: 32 = a warp per row;
 *                    1, 2, 4, 8 or 16 = that many lanes per row for rows of at
 *                    most that many products (the others a warp each);
 *                    128 = a 128-thread CTA per row (512-slot hash bin)
 *   hash_max_flops   rows with more products leave the hash bins for the
 *                    dense / rank bins (32 .. 1048576)
 *   dense_ratio      a row whose products x dense_ratio reach the output
 *                    width goes to the dense bin (>= 1)
 *   warp_max_flops   rows of an output at most 2048 columns wide with more
 *                    products than the short-row bins take and at most this
 *                    many get a warp each with a window of its own
 *                    (0 .. 65536; 0 = none)
 *   hash_load        hash tables get at least min(products, width) / load
 *                    slots (0.1 .. 0.75)
 *   gemm_inv_density products whose rows all take the single-pass dense path
 *                    (uint32 or uint64, positive, no row able to overflow):
 *                    inner indices with (A column count / rows) x
 *                    (B row length / cols) >= 1 / gemm_inv_density are
 *                    multiplied as dense FP16 GEMMs on the tensor cores
 *                    (exact: values in limbs, partial sums below 2^24, see
 *                    dense_gemm.cu); 0 = never (0 .. 65536)
 *   gemm_min_mflops  products with fewer multiply-adds (millions) never try
 *                    it (>= 0)
 * Defaults: 4, 4096, 16, 2048, 0.5, 512, 512.  A batch keeps the values it
 * was created with (its recorded products never use the GEMM). */
typedef struct rmcm_tuning {
    int32_t threads_per_row;
    int32_t hash_max_flops;
    int32_t dense_ratio;
    int32_t warp_max_flops;
    double hash_load;
    int32_t gemm_inv_density;
    int32_t gemm_min_mflops;
} rmcm_tuning;
RMCM_API int32_t rmcm_set_tuning(rmcm_handle *h, const rmcm_tuning *t);
RMCM_API int32_t rmcm_get_tuning(const rmcm_handle *h, rmcm_tuning *t);

/* ---- batches ---------------------------------------------------------------
 * Many meta-paths over one graph, each computed exactly as rmcm_run_metapath
 * computes it (RES estimate, DP order, SpGEMM chain, uint32 with escalation
 * in AUTO mode).  The reference runs its meta-paths one after another in
 * main() (efficient/resmcm.cpp:839-889); a batch runs them all at once.
 * rmcm_batch_create runs every path once through the ordinary executor and
 * records each device step with the sizes it read back, then captures the
 * whole set into one CUDA graph over `lanes` concurrent streams (<= 0: 8),
 * longest chains first onto the least-loaded lane.  rmcm_batch_run launches
 * that graph: every estimate, order and product is computed again on the
 * device with no host round trip, and per path the result nnz and an
 * order-free digest of the result (rmcm_mat_digest) come back.  The result
 * matrices themselves are freed inside the graph.  A product whose replayed
 * size differs from its record returns RMCM_EINTERNAL.  The graph's leaves
 * must stay loaded: rmcm_graph_free fails while a batch uses the graph, and
 * rmcm_destroy frees the handle's batches.  Only RMCM_ORDER_RES is batched. */
RMCM_API int32_t rmcm_batch_create(rmcm_handle *h, rmcm_graph *g, const char *const *metapaths,
                                   int32_t count, int32_t lanes, rmcm_batch **out);
/* nnz_out[count], digest_out[count] may be NULL; seconds = device time of
 * the graph launch (CUDA events on the handle's stream). */
/* The same batch in fused launches: the estimator levels of every chain
 * (one launch per level step over all chains), the DP of every chain (one
 * launch), then "waves": wave w multiplies the w-th product of every chain
 * that has one as ONE SpGEMM of block-diagonal operands (the chains' left
 * operands stacked, their columns shifted onto their chains' stacked right
 * operands).  Recorded once, captured as one CUDA graph; rmcm_batch_run,
 * _info (lanes = 1) and _free apply.  Replaces the per-path loop of main
 * (efficient/resmcm.cpp:834-889); results equal rmcm_run_metapath's. */
RMCM_API int32_t rmcm_batch_create_fused(rmcm_handle *h, rmcm_graph *g, const char *const *metapaths,
                                         int32_t count, rmcm_batch **out);
RMCM_API int32_t rmcm_batch_run(rmcm_handle *h, rmcm_batch *b, int64_t *nnz_out, uint64_t *digest_out,
                                double *seconds);
RMCM_API int32_t rmcm_batch_info(const rmcm_batch *b, int32_t *count, int32_t *lanes,
                                 int64_t *launches_per_run, int64_t *graph_nodes);
RMCM_API int32_t rmcm_batch_free(rmcm_handle *h, rmcm_batch *b);
/* nnz and an entry-order-free 64-bit digest of a matrix: the sum mod 2^64
 * over entries (r, c, v) of f(f(r * 2^32 + c) + v), f the splitmix64 output
 * function.  Equal matrices give equal digests.  Synchronises the stream. */
RMCM_API int32_t rmcm_mat_digest(rmcm_handle *h, const rmcm_mat *m, uint64_t *nnz, uint64_t *digest);
/* rmcm_mat_digest of m taken as rows row0.. of a larger matrix: the digests of
 * a result's blocks (rmcm_run_metapath_blocks) add up, mod 2^64, to the
 * digest of the whole result.  No counterpart in the reference. */
RMCM_API int32_t rmcm_mat_digest_rows(rmcm_handle *h, const rmcm_mat *m, int64_t row0, uint64_t *nnz,
                                      uint64_t *digest);

/* ---- query server ------------------------------------------------------------
 * A request loop over resident graphs: the reference's per-meta-path steps
 * (main(), efficient/resmcm.cpp:839-889: estimate, order, multiply) run for
 * many queries at once on `lanes` worker threads, each with its own stream.
 * A query is admitted when the device bytes its RES estimates predict (12
 * bytes per estimated entry of every intermediate and of the result, plus
 * row pointers and scratch) fit the budget left; one predicted above the
 * whole budget completes with RMCM_ENOMEM; one that does not fit yet waits
 * and is retried oldest first as bytes come back, while younger queries that
 * fit go ahead.  Every query's result equals rmcm_run_metapath's in AUTO
 * mode; a completed query reports its nnz and rmcm_mat_digest, and its
 * result is freed.  Graphs are added before their queries are submitted and
 * cannot be freed while the server lives; the owning handle must not be
 * used by another thread meanwhile.  Times are seconds on the server clock
 * (rmcm_server_now). */
typedef struct rmcm_server_opts {
    int32_t lanes;                  /* worker lanes (<= 0: 8) */
    int32_t reserved;
    int64_t mem_budget_bytes;       /* admission budget (<= 0: the handle's) */
} rmcm_server_opts;
typedef struct rmcm_query_result {
    int64_t tag;                    /* the caller's tag from rmcm_server_submit */
    int32_t status;                 /* RMCM_OK or the error */
    int32_t graph;
    int64_t nnz;
    uint64_t digest;
    double t_submit, t_admit, t_done;
    double est_bytes;               /* predicted device bytes used for admission */
    double es_s, dp_s;              /* estimator and DP device time */
    int32_t valtype;                /* value type of the result */
    int32_t lane;
    char error[128];
} rmcm_query_result;
typedef struct rmcm_server_stats {
    int64_t submitted, completed, rejected, pending, waiting;
    int32_t running, max_running;
    int32_t lanes, reserved_;
    int64_t budget, reserved, peak_reserved, kernel_launches;
} rmcm_server_counters;
RMCM_API int32_t rmcm_server_create(rmcm_handle *h, const rmcm_server_opts *opts, rmcm_server **out);
/* Builds the graph's uint32 leaves of every edge kind; *index names it in submit. */
RMCM_API int32_t rmcm_server_add_graph(rmcm_server *s, rmcm_graph *g, int32_t *index);
RMCM_API double rmcm_server_now(const rmcm_server *s);
/* Queues a query; t_arrival >= 0 stamps its arrival (server clock) instead of now. */
RMCM_API int32_t rmcm_server_submit(rmcm_server *s, int32_t graph, const char *metapath, int64_t tag,
                                    double t_arrival);
/* Completed queries, oldest first; waits up to wait_s for the first. */
RMCM_API int32_t rmcm_server_poll(rmcm_server *s, rmcm_query_result *out, int32_t cap, int32_t *count,
                                  double wait_s);
/* Waits until no query is queued, waiting or running (timeout_s <= 0: no limit). */
RMCM_API int32_t rmcm_server_drain(rmcm_server *s, double timeout_s);
RMCM_API int32_t rmcm_server_stats(const rmcm_server *s, rmcm_server_counters *st);
/* Drains, stops the workers and frees the lanes. */
RMCM_API int32_t rmcm_server_destroy(rmcm_server *s);

/* ---- RES estimator that allocates nothing --------------------------------
 * No counterpart in the reference.  For callers that may not allocate device
 * memory when they need an estimate (a host framework that owns all device
 * memory through its own pool, a serving loop that forbids allocation after
 * start-up): same estimates as
 * rmcm_estimate, computed from caller-owned device CSR arrays of the chain
 * (rows[i] x cols[i], rowptr[i] with rows[i]+1 int64 entries, col[i] int32
 * column indices; cols[i] == rows[i+1]) into the host array c_out[len*len].
 * It calls no allocating routine: its temporaries live in a fixed 32 MiB
 * device array that every GPU which loads this library holds until the
 * process exits, so a chain fits when 2*8*len*max(rows) bytes plus about
 * 0.2 MiB stay within 32 MiB (len <= 16); larger chains return RMCM_EINVAL
 * before anything is launched.  The first call on a device looks the array
 * up (make that first call before any stream capture).  All calls share the
 * array: calls that overlap on the GPU race, so issue them one after
 * another.  Copies the estimates to c_out and synchronises `stream` (NULL =
 * the default stream) before it returns. */
RMCM_API int32_t rmcm_estimate_noalloc(int32_t len, const int64_t *rows, const int64_t *cols,
                                       const int64_t *const *rowptr, const int32_t *const *col, double *c_out,
                                       void *stream);

#ifdef __cplusplus
}
#endif
#endif /* RESMCM_GPU_H */
