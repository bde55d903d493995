// Test harness compiled against the reference's own graph.hpp
// (shared_memory/graph.hpp): reads a graph with hl::Graph::read and prints
// the adjacency it built, so the product's parsers can be pinned to it.
// Usage: graphdump <graph> [undirected 0/1]
// Output: "n m" then per vertex v two lines "v side count (head len)*".
#include <cstdio>
#include <cstdlib>
#include "graph.hpp"

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    hl::Graph g;
    bool und = argc > 2 && atoi(argv[2]) != 0;
    if (!g.read(argv[1], und)) {
        printf("FAIL\n");
        return 0;
    }
    printf("%u %zu\n", g.get_n(), g.get_m());
    for (hl::Vertex v = 0; v < g.get_n(); ++v) {
        for (int side = 0; side < 2; ++side) {
            hl::Graph::arc_iterator b = g.begin(v, side == 1), e = g.end(v, side == 1);
            printf("%u %d %ld", v, side, (long)(e - b));
            for (hl::Graph::arc_iterator a = b; a < e; ++a) printf(" %u %d", (unsigned)a->head, a->length);
            printf("\n");
        }
    }
    return 0;
}
