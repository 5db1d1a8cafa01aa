// Harness around the reference program efficient/naive.cpp (swordzlim/RESMCM_ARI).
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles the reference source
// where it lies (path in REF_NAIVE_CPP) with its main() renamed, and this
// entry point runs its DynamicOptimizer::rows_sparse_optimal_matrix_chain_order
// (efficient/naive.cpp:488-530), whose DP reads only the type dimensions,
// and its get_optimal_chain_order.  Used to pin the dense-order DP.
#include <cstdint>
#include <cstdlib>

#define main naive_reference_main
#include REF_NAIVE_CPP
#undef main

extern "C" int ref_naive_order(const int32_t *dims_by_type, int32_t ntypes, const int32_t *vts, int32_t len,
                               int32_t *split_out, double *m_out, int32_t *pairs_out) {
    std::vector<vertex> dims(dims_by_type, dims_by_type + ntypes);
    std::vector<vertex_type> p_vts(vts, vts + len + 1);
    DynamicOptimizer op;
    op.rows_sparse_optimal_matrix_chain_order(len, nullptr, nullptr, dims.data(), &p_vts, 0);
    for (int q = 0; q < len * len; q++) {
        split_out[q] = op.s_[q];
        m_out[q] = op.m_[q];
    }
    std::vector<std::pair<int, int>> order;
    op.get_optimal_chain_order(0, len - 1, &order);
    for (size_t q = 0; q < order.size(); q++) {
        pairs_out[2 * q] = order[q].first;
        pairs_out[2 * q + 1] = order[q].second;
    }
    return 0;
}
