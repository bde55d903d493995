// hhl -- command line of the GB300 engine, a drop-in for the reference CLIs
// (shared_memory/hhl.cpp:16-79 and distributed_memory/hhl.cpp:15-94) on top
// of the C ABI in chl.h.
//
//   -g <graph>   graph file (DIMACS / METIS / SNAP / edge list)
//   -o <order>   order file
//   -l <labels>  write labels (reference text layout)
//   -s <sf>      superstep label budget sf*N (default: chosen from the
//                graph, 32 heavy-tailed / 1024 road-like; labels are the same)
//   -p <threads> accepted for compatibility (the GPU decides its own)
//   -paraPLL     accepted, ignored (as in the reference)
//   -ps <ratio>  PLaNT -> pruned phase switch ratio (default 1024)
//   -cb, -ft, -b accepted, ignored (the distributed CLI parses them too)
//   -qm <mode>   run queries after the build and print one distance per
//                line (modes 0-5 all answer on this GPU)
//   -rq <file>   query pairs `u v` per line (default: 1,000,000 pairs from
//                rand() % N, as distributed_memory/query.hpp:43-51)
//   --gpu-mode hybrid|gll|plant, --gpu-first <roots>,
//   --gpu-growth <factor>, --gpu-verbose
#include <chl.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

int main(int argc, char **argv) {
    // echo the command line (shared_memory/hhl.cpp:28-32)
    for (int i = 0; i < argc; ++i) printf("%s ", argv[i]);
    std::cout << std::endl;

    const char *graph_path = nullptr, *order_path = nullptr, *label_path = nullptr, *query_path = nullptr;
    chl_build_opts opts;
    chl_build_opts_default(&opts);
    opts.verbose = 1;
    int query_mode = -1;
    for (int i = 0; i < argc; ++i) {
        const bool has = i + 1 < argc;
        if (!strcmp(argv[i], "-g") && has) graph_path = argv[i + 1];
        else if (!strcmp(argv[i], "-o") && has) order_path = argv[i + 1];
        else if (!strcmp(argv[i], "-l") && has) label_path = argv[i + 1];
        else if (!strcmp(argv[i], "-s") && has) opts.sf = atof(argv[i + 1]);
        else if (!strcmp(argv[i], "-ps") && has) opts.ps = atof(argv[i + 1]);
        else if (!strcmp(argv[i], "-qm") && has) query_mode = atoi(argv[i + 1]);
        else if (!strcmp(argv[i], "-rq") && has) query_path = argv[i + 1];
        else if (!strcmp(argv[i], "--gpu-mode") && has) {
            std::string m = argv[i + 1];
            opts.mode = m == "gll" ? CHL_MODE_GLL : m == "plant" ? CHL_MODE_PLANT : CHL_MODE_HYBRID;
        } else if (!strcmp(argv[i], "--gpu-first") && has) {
            opts.first_superstep = (uint32_t)atol(argv[i + 1]);
        } else if (!strcmp(argv[i], "--gpu-growth") && has) {
            opts.growth = atof(argv[i + 1]);
        } else if (!strcmp(argv[i], "--gpu-verbose")) {
            opts.verbose = 2;
        }
    }
    if (!order_path) {
        std::cout << "ERROR: couldn't open order file named (none)" << std::endl;
        return 1;
    }
    uint32_t *order = nullptr, n = 0;
    int st = chl_order_load(order_path, &order, &n);
    if (st == CHL_ERR_IO) {
        std::cout << "ERROR: couldn't open order file named " << order_path << std::endl;
        return 1;
    }
    if (st != CHL_OK) {
        std::cerr << "bad order file " << order_path << ": " << chl_last_error() << std::endl;
        return 1;
    }
    chl_graph *g = nullptr;
    if (!graph_path || chl_graph_load_gpu(graph_path, 0, &g, nullptr) != CHL_OK) {
        std::cerr << "Unable to read graph from raw " << (graph_path ? graph_path : "(none)") << std::endl;
        return 1;
    }
    std::cerr << "Order size: " << n << " |V|: " << chl_graph_n(g) << std::endl;
    chl_labels *L = nullptr;
    st = chl_build(g, order, n, &opts, &L);
    if (st != CHL_OK) {
        std::cerr << "build failed: " << chl_status_str(st) << " (" << chl_last_error() << ")" << std::endl;
        return 1;
    }
    if (label_path && chl_labels_write(L, label_path) != CHL_OK) {
        std::cerr << "cannot write labels to " << label_path << std::endl;
        return 1;
    }
    if (query_mode >= 0 || query_path) {
        std::vector<uint32_t> pairs;
        if (query_path) {
            uint32_t *q = nullptr;
            size_t k = 0;
            if (chl_query_load(query_path, &q, &k) != CHL_OK) {
                std::cerr << "cannot read queries " << query_path << std::endl;
                return 1;
            }
            pairs.assign(q, q + 2 * k);
            chl_order_free(q);
        } else {
            const size_t k = 1000000;
            pairs.resize(2 * k);
            for (size_t i = 0; i < k; ++i) {
                pairs[2 * i] = (uint32_t)(rand() % n);
                pairs[2 * i + 1] = (uint32_t)(rand() % n);
            }
        }
        const size_t k = pairs.size() / 2;
        std::vector<int32_t> dist(k);
        st = chl_query_batch(L, pairs.data(), k, dist.data(), nullptr);
        if (st != CHL_OK) {
            std::cerr << "query failed: " << chl_last_error() << std::endl;
            return 1;
        }
        std::string out;
        out.reserve(k * 8);
        for (size_t i = 0; i < k; ++i) {
            out += std::to_string(dist[i]);
            out += '\n';
        }
        fwrite(out.data(), 1, out.size(), stdout);
    }
    chl_labels_free(L);
    chl_graph_free(g);
    chl_order_free(order);
    return 0;
}
