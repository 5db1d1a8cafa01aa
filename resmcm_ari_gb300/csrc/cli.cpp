// resmcm_gpu — drop-in for the reference program efficient/resmcm.
//
//   resmcm_gpu THREADS ITERATIONS GRAPH VERTEX EDGE METAPATHS OUTPUT [--flags]
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
//
// Optional flags (none changes the arithmetic):
//   --order=res|l2r|dense   chain order: RES estimates + DP (default), left to
//                           right (efficient/l2r.cpp) or the dense-dimension DP
//                           (efficient/naive.cpp)
//   --estimate-only         write "<meta-path> <estimated nnz>" lines, the
//                           output of accuracy/res.cpp (:698), and multiply nothing
//   --valtype=auto|u32|u64  path-count type (auto: uint32, uint64 on overflow)
//   --cache=FILE            binary graph cache: read FILE if it exists, else
//                           parse the text files and write FILE
//   --save-result=DIR       write each result matrix to DIR/<meta-path>.csr
//   --row-counts=DIR        write "<vertex id> <row size>" per start vertex to
//                           DIR/<meta-path>.cnt (BoolMatrix::write_graph_cnt,
//                           efficient/resmcm.cpp:398-410)
#include <omp.h>
#include <sys/stat.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "resmcm_gpu.h"

namespace {

bool starts_with(const std::string &s, const std::string &p) { return s.compare(0, p.size(), p) == 0; }

bool file_exists(const std::string &p) {
    struct stat st;
    return stat(p.c_str(), &st) == 0;
}

}  // namespace

int main(int argc, char **argv) {
    std::vector<std::string> pos;
    std::string order = "res", valtype = "auto", cache, save_dir, cnt_dir;
    bool estimate_only = false;
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        if (starts_with(a, "--order=")) order = a.substr(8);
        else if (a == "--estimate-only") estimate_only = true;
        else if (starts_with(a, "--valtype=")) valtype = a.substr(10);
        else if (starts_with(a, "--cache=")) cache = a.substr(8);
        else if (starts_with(a, "--save-result=")) save_dir = a.substr(14);
        else if (starts_with(a, "--row-counts=")) cnt_dir = a.substr(13);
        else if (starts_with(a, "--")) {
            std::cerr << "resmcm_gpu: unknown flag " << a << std::endl;
            return 2;
        } else pos.push_back(a);
    }
    if (pos.size() != 7) {
        std::cerr << "usage: resmcm_gpu THREADS ITERATIONS GRAPH VERTEX EDGE METAPATHS OUTPUT [--order=res|l2r|dense]"
                     " [--estimate-only] [--valtype=auto|u32|u64] [--cache=FILE] [--save-result=DIR]"
                     " [--row-counts=DIR]"
                  << std::endl;
        return 2;
    }
    const int threads = std::stoi(pos[0]);
    const double iterations = std::stod(pos[1]);
    const std::string graph = pos[2], vertex = pos[3], edge = pos[4], mpfile = pos[5], out = pos[6];
    int32_t order_mode = RMCM_ORDER_RES;
    if (order == "l2r") order_mode = RMCM_ORDER_L2R;
    else if (order == "dense") order_mode = RMCM_ORDER_DENSE;
    else if (order != "res") {
        std::cerr << "resmcm_gpu: --order must be res, l2r or dense" << std::endl;
        return 2;
    }
    int32_t vt_mode = RMCM_VAL_AUTO;
    if (valtype == "u32") vt_mode = RMCM_VAL_U32;
    else if (valtype == "u64") vt_mode = RMCM_VAL_U64;
    else if (valtype != "auto") {
        std::cerr << "resmcm_gpu: --valtype must be auto, u32 or u64" << std::endl;
        return 2;
    }
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
    opts.valtype = vt_mode;
    if (const char *d = std::getenv("RESMCM_GPU_DEVICE")) opts.device = std::atoi(d);
    rmcm_handle *h = nullptr;
    int32_t rc = rmcm_create(&h, &opts);
    if (rc != RMCM_OK) {
        std::cerr << "resmcm_gpu: cannot open the GPU: " << rmcm_status_string(rc) << std::endl;
        return 1;
    }
    rmcm_set_order_mode(h, order_mode);
    rmcm_graph *g = nullptr;
    if (!cache.empty() && file_exists(cache)) {
        rc = rmcm_graph_load(h, cache.c_str(), &g);
    } else {
        rc = rmcm_graph_load_text(h, graph.c_str(), vertex.c_str(), edge.c_str(), &g);
        if (rc == RMCM_OK && !cache.empty() && rmcm_graph_save(g, cache.c_str()) != RMCM_OK)
            std::cerr << "resmcm_gpu: could not write the graph cache " << cache << std::endl;
    }
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
        if (estimate_only) {
            // accuracy/res.cpp: main :612-705, line :698
            double est = 0;
            rc = rmcm_estimate_metapath(h, g, p.c_str(), &est);
            if (rc != RMCM_OK) {
                std::cerr << "resmcm_gpu: " << name << ": " << rmcm_status_string(rc) << ": " << rmcm_last_error(h)
                          << std::endl;
                failures++;
                continue;
            }
            std::ofstream o(out, std::ios::out | std::ios::app);
            o << name << " " << est << std::endl;
            continue;
        }
        double cost = 0, t_spgemm = 0, t_dp = 0, t_es = 0;
        int64_t nnz = 0;
        bool ok = true;
        for (int i = 0; i < iterations; i++) {
            rmcm_timings t{};
            const bool keep = i == 0 && (!save_dir.empty() || !cnt_dir.empty());
            rmcm_mat *C = nullptr;
            rc = rmcm_run_metapath(h, g, p.c_str(), keep ? &C : nullptr, &t);
            if (rc != RMCM_OK) {
                std::cerr << "resmcm_gpu: " << name << ": " << rmcm_status_string(rc) << ": " << rmcm_last_error(h)
                          << std::endl;
                if (C) rmcm_mat_free(h, C);
                ok = false;
                break;
            }
            if (C) {
                if (!save_dir.empty() && rmcm_mat_save(h, C, (save_dir + "/" + name + ".csr").c_str()) != RMCM_OK)
                    std::cerr << "resmcm_gpu: could not save the result of " << name << std::endl;
                if (!cnt_dir.empty()) {
                    int64_t rows = 0;
                    rmcm_mat_info(C, &rows, nullptr, nullptr, nullptr);
                    std::vector<int64_t> rp(rows + 1);
                    std::vector<int32_t> gid(rows);
                    rmcm_mat_download(h, C, rp.data(), nullptr, nullptr);
                    rmcm_graph_global_ids(g, vts[0], gid.data());
                    std::ofstream cf(cnt_dir + "/" + name + ".cnt");
                    for (int64_t r = 0; r < rows; r++) cf << gid[r] << " " << (rp[r + 1] - rp[r]) << "\n";
                }
                rmcm_mat_free(h, C);
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
