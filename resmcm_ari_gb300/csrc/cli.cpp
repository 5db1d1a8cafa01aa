// resmcm_gpu — drop-in for the reference program efficient/resmcm.
//
//   resmcm_gpu THREADS ITERATIONS GRAPH VERTEX EDGE METAPATHS OUTPUT
//
// Same seven positional arguments as main() of efficient/resmcm.cpp
// (:782-802), same inputs, and the same appended output line per meta-path
// (:879-888):
//   <meta-path> <result nnz> <total time> <spgemm time> <dp time> <estimation time>
// with the times averaged over ITERATIONS and printed with the default
// ostream formatting (6 significant digits).  THREADS sets the host threads
// used by the graph loader and leaf builder; the chain itself runs on GPU 0
// (override with RESMCM_GPU_DEVICE).  Unlike the reference, missing arguments
// are an error instead of hard-coded developer paths, and a line that fails
// prints the status and continues with the next meta-path.
#include <omp.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "resmcm_gpu.h"

int main(int argc, char **argv) {
    if (argc != 8) {
        std::cerr << "usage: resmcm_gpu THREADS ITERATIONS GRAPH VERTEX EDGE METAPATHS OUTPUT" << std::endl;
        return 2;
    }
    const int threads = std::stoi(argv[1]);
    const double iterations = std::stod(argv[2]);
    const std::string graph = argv[3], vertex = argv[4], edge = argv[5], mpfile = argv[6], out = argv[7];
    if (threads > 0) omp_set_num_threads(threads);
    std::cout << "******************** input parameters ***************************" << std::endl;
    std::cout << "*\t# of thread:" << omp_get_max_threads() << std::endl;
    std::cout << "*\t# of iteration:" << iterations << std::endl;
    std::cout << "*\tthe input graph file:" << graph << std::endl;
    std::cout << "*\tthe input vertex file:" << vertex << std::endl;
    std::cout << "*\tthe input edge file:" << edge << std::endl;
    std::cout << "*\tthe input meta-path:" << mpfile << std::endl;
    std::cout << "*\tthe output file:" << out << std::endl;
    std::cout << "*****************************************************************" << std::endl;

    rmcm_opts opts{};
    opts.valtype = RMCM_VAL_AUTO;
    if (const char *d = std::getenv("RESMCM_GPU_DEVICE")) opts.device = std::atoi(d);
    rmcm_handle *h = nullptr;
    int32_t rc = rmcm_create(&h, &opts);
    if (rc != RMCM_OK) {
        std::cerr << "resmcm_gpu: cannot open the GPU: " << rmcm_status_string(rc) << std::endl;
        return 1;
    }
    rmcm_graph *g = nullptr;
    rc = rmcm_graph_load_text(h, graph.c_str(), vertex.c_str(), edge.c_str(), &g);
    if (rc != RMCM_OK) {
        std::cerr << "resmcm_gpu: " << rmcm_status_string(rc) << ": " << rmcm_last_error(h) << std::endl;
        rmcm_destroy(h);
        return 1;
    }
    int64_t n = 0, m = 0;
    rmcm_graph_info(g, &n, &m, nullptr);
    std::cout << "*\tthe number of vertex is: " << n << "." << std::endl;
    std::cout << "*\tthe number of edge is: " << m << "." << std::endl;

    // read_metapathesN, efficient/resmcm.cpp:339-357: first token of each line
    std::vector<std::string> paths;
    {
        std::ifstream in(mpfile);
        if (!in) {
            std::cerr << "resmcm_gpu: cannot open " << mpfile << std::endl;
            rmcm_graph_free(g);
            rmcm_destroy(h);
            return 1;
        }
        std::string line;
        while (std::getline(in, line)) {
            std::istringstream buf(line);
            std::string tok;
            if (buf >> tok) paths.push_back(tok);
        }
    }
    int failures = 0;
    for (const std::string &p : paths) {
        int32_t vts[17], ets[16], len = 0;
        if (rmcm_metapath_parse(p.c_str(), vts, ets, 16, &len) != RMCM_OK) {
            std::cerr << "the meta-path is incorrect: " << p << std::endl;
            failures++;
            continue;
        }
        char name[512];
        rmcm_metapath_format(vts, ets, len, name, sizeof(name));
        double cost = 0, t_spgemm = 0, t_dp = 0, t_es = 0;
        int64_t nnz = 0;
        bool ok = true;
        for (int i = 0; i < iterations; i++) {
            rmcm_timings t{};
            rc = rmcm_run_metapath(h, g, p.c_str(), nullptr, &t);
            if (rc != RMCM_OK) {
                std::cerr << "resmcm_gpu: " << name << ": " << rmcm_status_string(rc) << ": " << rmcm_last_error(h)
                          << std::endl;
                ok = false;
                break;
            }
            t_es += t.es_s / iterations;
            t_dp += t.dp_s / iterations;
            t_spgemm += t.spgemm_s / iterations;
            cost += t.total_s / iterations;
            if (i % 20 == 0) {
                nnz = t.nnz;
                std::cout << "time cost of spgemm in " << i << "-th process: " << t.spgemm_s << "s" << std::endl;
                std::cout << "time cost of :" << i << "th process: " << t.total_s << "s" << std::endl;
                std::cout << i << "th m: " << nnz << std::endl;
            }
        }
        if (!ok) {
            failures++;
            continue;
        }
        std::cout << "time cost of spgemm: " << t_spgemm << "s" << std::endl;
        std::cout << "time cost:" << cost << "s" << std::endl;
        std::ofstream o(out, std::ios::out | std::ios::app);
        o << name << " " << nnz << " " << cost << " " << t_spgemm << " " << t_dp << " " << t_es << std::endl;
    }
    rmcm_graph_free(g);
    rmcm_destroy(h);
    return failures ? 1 : 0;
}
