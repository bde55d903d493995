// Test harness compiled against the reference's own shared_memory headers:
// reads a graph and an order file the way shared_memory/hhl.cpp:34-62 does,
// runs hl::run_paraPLL with hhl's arguments (label_limit = sf * N,
// shared_memory/hhl.cpp:65) and prints the digest (chl_digest.h) of the
// labeling it built instead of writing the label file, so builds whose
// label files would be many GB can still be compared with the reference.
// Usage: ref_digest <graph> <order> <threads> [sf=32]
// Output: the reference's own summary lines, then
//         "digest <16 hex> n <n> total <entries> avg <avg label>".
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "labeling.hpp"
#include "ordering.hpp"
#include "akiba.hpp"
#include "dijkstra.hpp"
#include "omp.h"

#include "chl_digest.h"

int main(int argc, char **argv) {
    if (argc < 4) return 2;
    hl::Graph g;
    if (!g.read(argv[1])) {
        printf("FAIL graph\n");
        return 1;
    }
    std::vector<unsigned int> order;
    if (!hl::Order::read(argv[2], order)) {
        printf("FAIL order\n");
        return 1;
    }
    const unsigned threads = (unsigned)atoi(argv[3]);
    const int sf = argc > 4 ? atoi(argv[4]) : 32;
    const unsigned N = order.size();
    hl::Labeling *labeling = new hl::Labeling(N);
    hl::Labeling *local = new hl::Labeling(N);
    std::vector<unsigned int> revMap(N);
    for (unsigned i = 0; i < N; ++i) revMap[order[i]] = i;
    hl::run_paraPLL(&g, order, revMap, *local, *labeling, threads, (size_t)sf * N, false);
    delete local;

    uint64_t digest = chd_head(N);
    uint64_t total = 0;
    for (unsigned v = 0; v < N; ++v) {
        for (int side = 0; side < 2; ++side) {
            const std::vector<hl::Vertex> &hv = labeling->label_v[v][side];
            const std::vector<hl::Distance> &dv = labeling->label_d[v][side];
            const uint64_t base = chd_list_base(2ull * v + (uint64_t)side);
            digest += chd_list_term(base, hv.size());
            for (size_t j = 0; j < hv.size(); ++j)
                digest += chd_entry_term(base, j, (uint32_t)hv[j], (uint32_t)dv[j]);
            total += hv.size();
        }
    }
    printf("digest %016" PRIx64 " n %u total %" PRIu64 " avg %.6f\n", digest, N, total,
           N ? (double)total / N / 2 : 0.0);
    return 0;
}
