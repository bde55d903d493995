// Host-side graph ingestion: the four text parsers, the reference's arc
// de-duplication / direction merge, seeded generators and a DIMACS writer.
//
// Parsing rules follow hl::Graph (shared_memory/graph.hpp):
//   read()          :327-335  DIMACS, then METIS, then SNAP, then edge list
//   read_dimacs     :168-189  `p sp n m`, `a u v w` (1-based), `c` comments
//   read_metis      :211-256  METIS with fmt/ncon header
//   read_snap       :262-282  `# Nodes: n Edges: m` header, `u v` 0-based
//   read_edgelist   :284-308  `u v w` 0-based, n = number of distinct ids
//   add_tmp_arc     :156-162  bounds check, arc + mirrored reverse arc
//   init_arcs       :103-153  dedup keeping the shortest, merge fwd/rev arcs
// The arc lists of every vertex come out in the reference's order: arcs with
// only the reverse flag, then bidirectional arcs, then forward-only arcs,
// each group by (head, length).
#include "chl_internal.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <set>
#include <unordered_set>

namespace chl {

struct TmpArc {
    uint32_t u;
    uint32_t head;   // 30-bit in the reference's Arc; n < 2^30 is enforced
    int32_t len;
    uint8_t fwd, rev;
};

// cmp_by_direction (shared_memory/graph.hpp:91-100)
static inline bool cmp_dir(const TmpArc &x, const TmpArc &y) {
    if (x.u != y.u) return x.u < y.u;
    if (x.rev != y.rev) return x.rev > y.rev;      // reverse arcs first
    if (x.fwd != y.fwd) return x.fwd < y.fwd;      // then non-forward first
    if (x.head != y.head) return x.head < y.head;
    return x.len < y.len;
}
// cmp_by_head (shared_memory/graph.hpp:81-88)
static inline bool cmp_head(const TmpArc &x, const TmpArc &y) {
    if (x.u != y.u) return x.u < y.u;
    if (x.head != y.head) return x.head < y.head;
    return x.len < y.len;
}

void graph_fill_stats(chl_graph *g) {
    int32_t mn = kInfty, mx = 0;
    bool unit = true;
    for (int s = 0; s < 2; ++s) {
        for (int32_t l : g->len[s]) {
            mn = std::min(mn, l);
            mx = std::max(mx, l);
            if (l != 1) unit = false;
        }
    }
    if (mn == kInfty) mn = 1;
    g->min_len = mn;
    g->max_len = mx;
    g->unit = unit;
    g->symmetric = (g->off[0] == g->off[1] && g->head[0] == g->head[1] &&
                    g->len[0] == g->len[1]);
}

// init_arcs: de-duplicate, merge, and lay out per-vertex arc lists.
static void init_arcs(chl_graph *g, std::vector<TmpArc> &a) {
    const uint32_t n = g->n;
    if (!a.empty()) {
        std::sort(a.begin(), a.end(), cmp_dir);
        size_t i = 0;
        for (size_t j = 1; j < a.size(); ++j) {
            if (a[i].u == a[j].u && a[i].head == a[j].head &&
                a[i].fwd == a[j].fwd && a[i].rev == a[j].rev)
                continue;
            if (++i < j) a[i] = a[j];
        }
        a.resize(i + 1);
        std::sort(a.begin(), a.end(), cmp_head);
        i = 0;
        for (size_t j = 1; j < a.size(); ++j) {
            if (a[i].u == a[j].u && a[i].head == a[j].head &&
                a[i].len == a[j].len) {
                a[i].fwd |= a[j].fwd;
                a[i].rev |= a[j].rev;
                continue;
            }
            if (++i < j) a[i] = a[j];
        }
        a.resize(i + 1);
        std::sort(a.begin(), a.end(), cmp_dir);
    }
    for (int s = 0; s < 2; ++s) {
        g->off[s].assign((size_t)n + 1, 0);
        g->head[s].clear();
        g->len[s].clear();
    }
    // side 1 = forward (out) arcs, side 0 = reverse (in) arcs
    for (const TmpArc &t : a) {
        if (t.fwd) g->off[1][t.u + 1]++;
        if (t.rev) g->off[0][t.u + 1]++;
    }
    for (int s = 0; s < 2; ++s) {
        for (uint32_t v = 0; v < n; ++v) g->off[s][v + 1] += g->off[s][v];
        g->head[s].resize(g->off[s][n]);
        g->len[s].resize(g->off[s][n]);
    }
    std::vector<uint64_t> pos0(g->off[0].begin(), g->off[0].end() - 1);
    std::vector<uint64_t> pos1(g->off[1].begin(), g->off[1].end() - 1);
    for (const TmpArc &t : a) {
        if (t.fwd) {
            uint64_t p = pos1[t.u]++;
            g->head[1][p] = t.head;
            g->len[1][p] = t.len;
        }
        if (t.rev) {
            uint64_t p = pos0[t.u]++;
            g->head[0][p] = t.head;
            g->len[0][p] = t.len;
        }
    }
    a.clear();
    a.shrink_to_fit();
    graph_fill_stats(g);
}

// add_tmp_arc (shared_memory/graph.hpp:156-162).  u and v arrive already
// converted to the unsigned Vertex type, as in the reference.
static bool add_tmp_arc(chl_graph *g, long long n, std::vector<TmpArc> &tmp,
                        uint32_t u, uint32_t v, int32_t w, bool undirected) {
    if ((long long)u >= n || (long long)v >= n) return false;
    tmp.push_back(TmpArc{u, v, w, 1, (uint8_t)undirected});
    tmp.push_back(TmpArc{v, u, w, (uint8_t)undirected, 1});
    g->m += 1 + (undirected ? 1 : 0);
    return true;
}

static bool read_dimacs(FILE *file, bool undirected, chl_graph *g,
                        std::vector<TmpArc> &tmp, long long &n) {
    char buf[512];
    long long u, v, w, m;
    bool inited = false;
    while (fgets(buf, sizeof(buf), file) != NULL) {
        size_t L = strlen(buf);
        if (L == 0 || buf[L - 1] != '\n') {
            if (buf[0] != 'c') return false;
            while (!feof(file) && fgetc(file) != '\n') {}
        } else if (buf[0] == 'p') {
            if (inited) return false;
            inited = true;
            if (sscanf(buf, "p sp %lld %lld", &n, &m) != 2) return false;
        } else if (buf[0] == 'a') {
            if (sscanf(buf, "a %lld %lld %lld", &u, &v, &w) != 3) return false;
            if (!add_tmp_arc(g, n, tmp, (uint32_t)(u - 1), (uint32_t)(v - 1),
                             (int32_t)w, undirected))
                return false;
        } else if (buf[0] == 'c') {
            continue;
        } else {
            return false;
        }
    }
    return true;
}

// character sources of the METIS reader: the file, or a buffer (whose end
// reads as EOF)
struct FileChars {
    FILE *f;
    int get() { return fgetc(f); }
};
struct BufChars {
    const char *p, *e;
    bool hit_end;
    int get() {
        if (p < e) return (int)(unsigned char)*p++;
        hit_end = true;
        return EOF;
    }
};

template <class Chars>
static bool metis_parse(Chars &src, bool undirected, chl_graph *g, std::vector<TmpArc> &tmp, long long &n) {
    int c, i = 0, fmt = 0, ncon = 0, skip = 0;
    long long elem = 0;
    uint32_t v = 0, head = 0xFFFFFFFFu;
    // The reference never clears its `newline` flag, so a '%' anywhere
    // starts a comment that runs to the end of the line.
    const bool newline = true;
    bool inelem = false;
    (void)ncon;
    do {
        c = src.get();
        if (newline && c == '%') {
            while (c != '\n' && c != EOF) c = src.get();
        } else if (c != EOF && isdigit(c)) {
            inelem = true;
            elem = elem * 10 + c - '0';
        } else if (c == EOF || isspace(c)) {
            if (inelem) {
                if (v == 0) {
                    if (i == 0) {
                        n = elem;
                    } else if (i == 1) {
                        /* m */
                    } else if (i == 2) {
                        if ((elem % 10 > 1) || ((elem / 10) % 10 > 1) || elem > 111)
                            return false;
                        fmt = (int)elem;
                        skip = (fmt >= 100) + (fmt % 100 >= 10);
                    } else if (i == 3) {
                        if (fmt % 100 < 10) return false;
                        ncon = (int)elem;
                        skip = (fmt >= 100) + ncon;
                    } else {
                        return false;
                    }
                } else if (i >= skip) {
                    if (fmt % 10 == 1) {
                        if ((i - skip) % 2 == 0) {
                            head = (uint32_t)(elem - 1);
                        } else if (!add_tmp_arc(g, n, tmp, v - 1, head,
                                                (int32_t)elem, undirected)) {
                            return false;
                        }
                    } else if (!add_tmp_arc(g, n, tmp, v - 1, (uint32_t)(elem - 1),
                                            1, undirected)) {
                        return false;
                    }
                }
                ++i;
                elem = 0;
                inelem = false;
            }
            if (c == '\n' || (!newline && c == EOF)) {
                if (v > 0 && (i < skip || (fmt % 10 == 1 && (i - skip) % 2 == 1)))
                    return false;
                ++v;
                i = 0;
            }
        } else {
            return false;
        }
    } while (c != EOF);
    return true;
}

static bool read_metis(FILE *file, bool undirected, chl_graph *g,
                       std::vector<TmpArc> &tmp, long long &n) {
    FileChars src{file};
    return metis_parse(src, undirected, g, tmp, n);
}

// true when the METIS reader returns false before it has read past
// buf[0, len): it reads characters in order and never revisits a verdict, so
// it rejects any file that starts with these bytes at the same character
// (false: no verdict from this prefix)
bool metis_rejects_prefix(const char *buf, size_t len) {
    chl_graph g;
    std::vector<TmpArc> tmp;
    long long n = 0;
    BufChars src{buf, buf + len, false};
    return !metis_parse(src, false, &g, tmp, n) && !src.hit_end;
}

static bool read_snap(FILE *file, bool undirected, chl_graph *g,
                      std::vector<TmpArc> &tmp, long long &n) {
    char buf[512];
    long long u, v, m;
    bool inited = false;
    while (fgets(buf, sizeof(buf), file)) {
        size_t L = strlen(buf);
        if (buf[0] == '#') {
            if (sscanf(buf, "# Nodes: %lld Edges: %lld", &n, &m) == 2) {
                if (inited) return false;
                inited = true;
            }
            for (int ch = L ? buf[L - 1] : EOF; ch != '\n' && ch != EOF; ch = fgetc(file)) {}
        } else {
            if ((L == 0 || buf[L - 1] != '\n') && !feof(file)) return false;
            if (sscanf(buf, "%lld %lld", &u, &v) != 2) return false;
            if (!add_tmp_arc(g, n, tmp, (uint32_t)u, (uint32_t)v, 1, undirected))
                return false;
        }
    }
    return true;
}

// The reference counts distinct ids as n and indexes per-vertex arrays by
// the raw ids; ids outside [0, n) are undefined behaviour there and are
// rejected here.
static bool read_edgelist(FILE *file, bool undirected, chl_graph *g,
                          std::vector<TmpArc> &tmp, long long &n) {
    char buf[512];
    long long u, v, w;
    std::set<long long> nodes;
    while (fgets(buf, sizeof(buf), file)) {
        size_t L = strlen(buf);
        if ((L == 0 || buf[L - 1] != '\n') && !feof(file)) return false;
        if (sscanf(buf, "%lld %lld %lld", &u, &v, &w) != 3) return false;
        tmp.push_back(TmpArc{(uint32_t)u, (uint32_t)v, (int32_t)w, 1, (uint8_t)undirected});
        tmp.push_back(TmpArc{(uint32_t)v, (uint32_t)u, (int32_t)w, (uint8_t)undirected, 1});
        g->m += 1 + (undirected ? 1 : 0);
        if (nodes.insert(u).second) n++;
        if (nodes.insert(v).second) n++;
    }
    for (const TmpArc &t : tmp)
        if ((long long)t.u >= n || (long long)t.head >= n) return false;
    return true;
}

static int finish(chl_graph *g, long long n, std::vector<TmpArc> &tmp) {
    if (n < 0 || n >= (1ll << 30)) {
        set_error("graph has too many vertices (the arc head field is 30 bits)");
        return CHL_ERR_INVALID;
    }
    g->n = (uint32_t)n;
    init_arcs(g, tmp);
    return CHL_OK;
}

int graph_from_undirected_unique(uint32_t n, std::vector<uint64_t> &uv,
                                 std::vector<int32_t> &w, chl_graph **out) {
    // Equivalent to reading a DIMACS file that lists every undirected edge
    // {u, v} once in each direction: init_arcs merges the two arcs at each
    // endpoint into one bidirectional arc, so both lists equal the neighbour
    // list sorted by (head, length).
    chl_graph *g = new (std::nothrow) chl_graph();
    if (!g) return CHL_ERR_OOM;
    g->n = n;
    g->m = 2 * (uint64_t)uv.size();
    std::vector<uint64_t> &off = g->off[1];
    off.assign((size_t)n + 1, 0);
    for (uint64_t e : uv) {
        off[(uint32_t)(e >> 32) + 1]++;
        off[(uint32_t)e + 1]++;
    }
    for (uint32_t v = 0; v < n; ++v) off[v + 1] += off[v];
    std::vector<uint64_t> pos(off.begin(), off.end() - 1);
    std::vector<uint64_t> key(off[n]);
    for (size_t k = 0; k < uv.size(); ++k) {
        uint32_t a = (uint32_t)(uv[k] >> 32), b = (uint32_t)uv[k];
        key[pos[a]++] = ((uint64_t)b << 32) | (uint32_t)w[k];
        key[pos[b]++] = ((uint64_t)a << 32) | (uint32_t)w[k];
    }
    g->head[1].resize(off[n]);
    g->len[1].resize(off[n]);
    for (uint32_t v = 0; v < n; ++v) {
        std::sort(key.begin() + off[v], key.begin() + off[v + 1]);
        for (uint64_t p = off[v]; p < off[v + 1]; ++p) {
            g->head[1][p] = (uint32_t)(key[p] >> 32);
            g->len[1][p] = (int32_t)(uint32_t)key[p];
        }
    }
    g->off[0] = g->off[1];
    g->head[0] = g->head[1];
    g->len[0] = g->len[1];
    graph_fill_stats(g);
    *out = g;
    return CHL_OK;
}

}  // namespace chl

using namespace chl;

extern "C" int chl_graph_load(const char *path, int undirected, chl_graph **out) {
    if (!path || !out) return CHL_ERR_INVALID;
    FILE *file = fopen(path, "r");
    if (!file) {
        set_error(std::string("cannot open graph file ") + path);
        return CHL_ERR_IO;
    }
    typedef bool (*parser_t)(FILE *, bool, chl_graph *, std::vector<TmpArc> &, long long &);
    const parser_t parsers[4] = {read_dimacs, read_metis, read_snap, read_edgelist};
    for (int p = 0; p < 4; ++p) {
        chl_graph *g = new (std::nothrow) chl_graph();
        if (!g) {
            fclose(file);
            return CHL_ERR_OOM;
        }
        std::vector<TmpArc> tmp;
        long long n = 0;
        bool ok = parsers[p](file, undirected != 0, g, tmp, n);
        if (ok) {
            fclose(file);
            int st = finish(g, n, tmp);
            if (st != CHL_OK) {
                delete g;
                return st;
            }
            *out = g;
            return CHL_OK;
        }
        delete g;
        rewind(file);
    }
    fclose(file);
    set_error(std::string("no parser accepts graph file ") + path);
    return CHL_ERR_FORMAT;
}

extern "C" int chl_graph_from_arcs(uint32_t n, size_t k, const uint32_t *src,
                                   const uint32_t *dst, const int32_t *len,
                                   int undirected, chl_graph **out) {
    if (!out || (k && (!src || !dst || !len))) return CHL_ERR_INVALID;
    chl_graph *g = new (std::nothrow) chl_graph();
    if (!g) return CHL_ERR_OOM;
    std::vector<TmpArc> tmp;
    tmp.reserve(2 * k);
    for (size_t i = 0; i < k; ++i) {
        if (!add_tmp_arc(g, n, tmp, src[i], dst[i], len[i], undirected != 0)) {
            delete g;
            set_error("arc endpoint out of range");
            return CHL_ERR_INVALID;
        }
    }
    int st = finish(g, n, tmp);
    if (st != CHL_OK) {
        delete g;
        return st;
    }
    *out = g;
    return CHL_OK;
}

extern "C" int chl_graph_from_csr(uint32_t n, const uint64_t *off, const uint32_t *head,
                                  const int32_t *len, int undirected, chl_graph **out) {
    if (!out || !off) return CHL_ERR_INVALID;
    if (off[0] != 0) {
        set_error("CSR offsets must start at 0");
        return CHL_ERR_INVALID;
    }
    for (uint32_t v = 0; v < n; ++v)
        if (off[v + 1] < off[v]) {
            set_error("CSR offsets must not decrease");
            return CHL_ERR_INVALID;
        }
    const uint64_t k = off[n];
    if (k && (!head || !len)) return CHL_ERR_INVALID;
    std::vector<uint32_t> src;
    try {
        src.resize(k);
    } catch (...) {
        return CHL_ERR_OOM;
    }
    for (uint32_t v = 0; v < n; ++v)
        for (uint64_t e = off[v]; e < off[v + 1]; ++e) src[e] = v;
    return chl_graph_from_arcs(n, k, src.data(), head, len, undirected, out);
}

extern "C" int chl_graph_write_dimacs(const chl_graph *g, const char *path) {
    if (!g || !path) return CHL_ERR_INVALID;
    FILE *f = fopen(path, "w");
    if (!f) return CHL_ERR_IO;
    std::vector<char> buf(1 << 20);
    setvbuf(f, buf.data(), _IOFBF, buf.size());
    fprintf(f, "p sp %u %llu\n", g->n, (unsigned long long)g->off[1][g->n]);
    for (uint32_t v = 0; v < g->n; ++v)
        for (uint64_t p = g->off[1][v]; p < g->off[1][v + 1]; ++p)
            fprintf(f, "a %u %u %d\n", v + 1, g->head[1][p] + 1, g->len[1][p]);
    bool bad = ferror(f) != 0;
    if (fclose(f) != 0) bad = true;
    return bad ? CHL_ERR_IO : CHL_OK;
}

extern "C" uint32_t chl_graph_n(const chl_graph *g) { return g ? g->n : 0; }
extern "C" uint64_t chl_graph_m(const chl_graph *g) { return g ? g->m : 0; }
extern "C" uint64_t chl_graph_out_arcs(const chl_graph *g) {
    return g ? g->off[1][g->n] : 0;
}
extern "C" int chl_graph_symmetric(const chl_graph *g) { return g && g->symmetric; }

extern "C" uint32_t chl_graph_degree(const chl_graph *g, uint32_t v) {
    if (!g || v >= g->n) return 0;
    return (uint32_t)((g->off[1][v + 1] - g->off[1][v]) + (g->off[0][v + 1] - g->off[0][v]));
}

extern "C" int chl_graph_degrees(const chl_graph *g, int forward, uint32_t *deg) {
    if (!g || !deg) return CHL_ERR_INVALID;
    const int s = forward ? 1 : 0;
    for (uint32_t v = 0; v < g->n; ++v) deg[v] = (uint32_t)(g->off[s][v + 1] - g->off[s][v]);
    return CHL_OK;
}

extern "C" int chl_graph_export(const chl_graph *g, int forward, uint64_t *off, uint32_t *head,
                                int32_t *len) {
    if (!g || !off) return CHL_ERR_INVALID;
    const int s = forward ? 1 : 0;
    std::copy(g->off[s].begin(), g->off[s].end(), off);
    if (head) std::copy(g->head[s].begin(), g->head[s].end(), head);
    if (len) std::copy(g->len[s].begin(), g->len[s].end(), len);
    return CHL_OK;
}

extern "C" int chl_graph_arcs(const chl_graph *g, uint32_t v, int forward,
                              uint32_t *heads, int32_t *lens, uint32_t cap,
                              uint32_t *cnt) {
    if (!g || v >= g->n || !cnt) return CHL_ERR_INVALID;
    int s = forward ? 1 : 0;
    uint64_t b = g->off[s][v], e = g->off[s][v + 1];
    *cnt = (uint32_t)(e - b);
    if (heads || lens) {
        if (cap < e - b) return CHL_ERR_INVALID;
        for (uint64_t p = b; p < e; ++p) {
            if (heads) heads[p - b] = g->head[s][p];
            if (lens) lens[p - b] = g->len[s][p];
        }
    }
    return CHL_OK;
}

extern "C" void chl_graph_free(chl_graph *g) {
    if (!g) return;
    graph_release_device(g);
    delete g;
}

// ------------------------------------------------------------ generators
//
// Road-like grid.  Vertex (r, c) has id r*cols + c.  Grid edges are listed
// row by row: (r,c)-(r,c+1) then (r,c)-(r+1,c); each gets a length uniform
// in [wmin, wmax] in that listing order.  round(del_frac * E) edges are
// deleted (partial Fisher-Yates), the largest connected component is kept
// (ties: the one holding the smallest id) and renumbered in id order, then
// floor(diag_frac * n) diagonal shortcuts (r,c)-(r+-1,c+-1) between distinct
// kept vertices are added, then `highways` edges between kept vertices
// 2..hw_steps grid steps apart (dr uniform in [-s, s], dc uniform in the
// remaining Manhattan budget), length llround(hw_factor * steps).
extern "C" int chl_gen_grid(uint32_t rows, uint32_t cols, double del_frac,
                            double diag_frac, int32_t wmin, int32_t wmax,
                            uint32_t highways, uint32_t hw_steps, double hw_factor,
                            uint64_t seed, chl_graph **out) {
    if (!out || rows == 0 || cols == 0 || wmin < 1 || wmax < wmin ||
        (uint64_t)rows * cols >= (1ull << 30) || del_frac < 0 || del_frac >= 1)
        return CHL_ERR_INVALID;
    Rng rng(seed);
    const uint64_t N0 = (uint64_t)rows * cols;
    struct E { uint32_t a, b; int32_t w; };
    std::vector<E> edges;
    edges.reserve(2 * N0);
    for (uint32_t r = 0; r < rows; ++r)
        for (uint32_t c = 0; c < cols; ++c) {
            uint32_t id = r * cols + c;
            if (c + 1 < cols) edges.push_back({id, id + 1, 0});
            if (r + 1 < rows) edges.push_back({id, id + cols, 0});
        }
    for (E &e : edges) e.w = wmin + (int32_t)rng.below((uint64_t)(wmax - wmin) + 1);
    const uint64_t E0 = edges.size();
    const uint64_t ndel = (uint64_t)llround(del_frac * (double)E0);
    for (uint64_t k = 0; k < ndel && k < E0; ++k) {
        uint64_t j = k + rng.below(E0 - k);
        std::swap(edges[k], edges[j]);
    }
    edges.erase(edges.begin(), edges.begin() + std::min(ndel, E0));
    // largest connected component (union-find)
    std::vector<uint32_t> par(N0);
    for (uint64_t i = 0; i < N0; ++i) par[i] = (uint32_t)i;
    auto find = [&](uint32_t x) {
        while (par[x] != x) {
            par[x] = par[par[x]];
            x = par[x];
        }
        return x;
    };
    for (const E &e : edges) {
        uint32_t a = find(e.a), b = find(e.b);
        if (a != b) par[std::max(a, b)] = std::min(a, b);
    }
    std::vector<uint32_t> sz(N0, 0);
    for (uint64_t i = 0; i < N0; ++i) sz[find((uint32_t)i)]++;
    uint32_t best = 0;
    for (uint64_t i = 0; i < N0; ++i)
        if (sz[i] > sz[best]) best = (uint32_t)i;
    std::vector<uint32_t> newid(N0, 0xFFFFFFFFu);
    std::vector<uint32_t> oldid;
    for (uint64_t i = 0; i < N0; ++i)
        if (find((uint32_t)i) == best) {
            newid[i] = (uint32_t)oldid.size();
            oldid.push_back((uint32_t)i);
        }
    const uint32_t n = (uint32_t)oldid.size();
    std::vector<uint64_t> uv;
    std::vector<int32_t> w;
    std::unordered_set<uint64_t> present;
    auto key = [](uint32_t a, uint32_t b) {
        if (a > b) std::swap(a, b);
        return ((uint64_t)a << 32) | b;
    };
    for (const E &e : edges) {
        if (newid[e.a] == 0xFFFFFFFFu) continue;
        uint64_t k = key(newid[e.a], newid[e.b]);
        uv.push_back(k);
        w.push_back(e.w);
        present.insert(k);
    }
    // diagonal shortcuts
    const uint64_t ndiag = (uint64_t)std::floor(diag_frac * (double)n);
    uint64_t added = 0, tries = 0;
    while (added < ndiag && tries < 64 * (ndiag + 16)) {
        ++tries;
        uint32_t x = oldid[rng.below(n)];
        uint32_t dir = (uint32_t)rng.below(4);
        int r = (int)(x / cols), c = (int)(x % cols);
        int r2 = r + ((dir & 1) ? 1 : -1), c2 = c + ((dir & 2) ? 1 : -1);
        int32_t len = wmin + (int32_t)rng.below((uint64_t)(wmax - wmin) + 1);
        if (r2 < 0 || c2 < 0 || r2 >= (int)rows || c2 >= (int)cols) continue;
        uint32_t y = (uint32_t)r2 * cols + (uint32_t)c2;
        if (newid[y] == 0xFFFFFFFFu) continue;
        uint64_t k = key(newid[x], newid[y]);
        if (present.count(k)) continue;
        present.insert(k);
        uv.push_back(k);
        w.push_back(len);
        ++added;
    }
    // highways
    added = 0;
    tries = 0;
    const int S = (int)hw_steps;
    while (S >= 2 && added < highways && tries < 64 * ((uint64_t)highways + 16)) {
        ++tries;
        uint32_t x = oldid[rng.below(n)];
        int dr = (int)rng.below(2 * (uint64_t)S + 1) - S;
        int rem = S - std::abs(dr);
        int dc = (int)rng.below(2 * (uint64_t)rem + 1) - rem;
        int steps = std::abs(dr) + std::abs(dc);
        if (steps < 2) continue;
        int r2 = (int)(x / cols) + dr, c2 = (int)(x % cols) + dc;
        if (r2 < 0 || c2 < 0 || r2 >= (int)rows || c2 >= (int)cols) continue;
        uint32_t y = (uint32_t)r2 * cols + (uint32_t)c2;
        if (newid[y] == 0xFFFFFFFFu) continue;
        uint64_t k = key(newid[x], newid[y]);
        if (present.count(k)) continue;
        present.insert(k);
        uv.push_back(k);
        w.push_back((int32_t)llround(hw_factor * steps));
        ++added;
    }
    return graph_from_undirected_unique(n, uv, w, out);
}

// RMAT: edge k (k = 0 .. ef*2^scale-1) descends `scale` levels; level l uses
// the l-th draw of the counter-based stream seeded with mix64(seed ^ k*C).
// Quadrant: x < a -> (0,0); x < a+b -> (0,1); x < a+b+c -> (1,0); else (1,1),
// the bit of u first.  Self loops dropped, {u,v} symmetrised and
// de-duplicated; unit lengths.
extern "C" int chl_gen_rmat(uint32_t scale, uint32_t ef, double a, double b,
                            double c, uint64_t seed, chl_graph **out) {
    if (!out || scale == 0 || scale > 29 || ef == 0) return CHL_ERR_INVALID;
    const uint64_t n = 1ull << scale;
    const uint64_t M = (uint64_t)ef * n;
    std::vector<uint64_t> uv(M);
    const double ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(static)
    for (long long k = 0; k < (long long)M; ++k) {
        Rng r(mix64(seed ^ ((uint64_t)k * 0xD1B54A32D192ED03ull)));
        uint64_t u = 0, v = 0;
        for (uint32_t l = 0; l < scale; ++l) {
            double x = r.unit();
            uint64_t bu, bv;
            if (x < a) { bu = 0; bv = 0; }
            else if (x < ab) { bu = 0; bv = 1; }
            else if (x < abc) { bu = 1; bv = 0; }
            else { bu = 1; bv = 1; }
            u = (u << 1) | bu;
            v = (v << 1) | bv;
        }
        if (u == v) {
            uv[k] = ~0ull;
        } else {
            if (u > v) std::swap(u, v);
            uv[k] = (u << 32) | v;
        }
    }
    std::sort(uv.begin(), uv.end());
    uv.erase(std::unique(uv.begin(), uv.end()), uv.end());
    if (!uv.empty() && uv.back() == ~0ull) uv.pop_back();
    std::vector<int32_t> w(uv.size(), 1);
    return graph_from_undirected_unique((uint32_t)n, uv, w, out);
}
