// Test harness compiled against the reference's own labeling.hpp
// (shared_memory/labeling.hpp): reads a label file with Labeling::read,
// answers the `u v` pairs of a query file with Labeling::query, one
// distance per line, and optionally re-writes the labels with
// Labeling::write.
// Usage: labelquery <labels> <pairs> [rewrite-path]
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "labeling.hpp"

int main(int argc, char **argv) {
    if (argc < 3) return 2;
    hl::Labeling L;
    if (!L.read(argv[1])) {
        printf("FAIL\n");
        return 0;
    }
    FILE *f = fopen(argv[2], "r");
    if (!f) return 3;
    unsigned u, v;
    while (fscanf(f, "%u %u", &u, &v) == 2) printf("%d\n", L.query(u, v));
    fclose(f);
    if (argc > 3) L.write(argv[3]);
    return 0;
}
