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

// add_tmp_arc (shared_memory/graph.hpp:156-162): the arc and its mirrored
// reverse record, after a bounds check of the (already 32-bit) endpoints.
static bool add_tmp_arc(chl_graph *g, long long n, std::vector<TmpArc> &tmp,
                        uint32_t u, uint32_t v, int32_t w, bool undirected) {
    if ((long long)u >= n || (long long)v >= n) return false;
    tmp.push_back(TmpArc{u, v, w, 1, (uint8_t)undirected});
    tmp.push_back(TmpArc{v, u, w, (uint8_t)undirected, 1});
    g->m += 1 + (undirected ? 1 : 0);
    return true;
}

// ---------------------------------------------------------------- text input
//
// The reference reads its formats with stdio: fgets into a 512-byte buffer
// examined with strlen and sscanf (DIMACS, SNAP, edge lists), or fgetc
// (METIS).  Here the file is a byte span and Text hands out exactly what
// those calls would see, so the accept / reject decision and every value
// match the reference byte for byte, including long lines (fgets returns
// them in 511-byte pieces), NUL bytes (strlen stops there) and a last line
// without a newline (fgets stops at the end of the input and sets feof).
struct Text {
    const unsigned char *p, *e;
    bool at_eof = false;   // a read has tried to go past the last byte (feof)

    // fgets(buf, 512): up to 511 bytes, through the first newline.  `vis` is
    // strlen(buf); false when nothing is left.
    struct Piece {
        const char *s;
        size_t vis;
    };
    bool piece(Piece &pc) {
        if (p >= e) {
            at_eof = true;
            return false;
        }
        const unsigned char *q = p;
        size_t k = 0;
        bool nl = false;
        while (k < 511 && q < e) {
            ++k;
            if (*q++ == '\n') {
                nl = true;
                break;
            }
        }
        if (!nl && k < 511) at_eof = true;   // stopped by the end of the input
        pc.s = (const char *)p;
        pc.vis = 0;
        while (pc.vis < k && pc.s[pc.vis] != '\0') ++pc.vis;
        p = q;
        return true;
    }
    // fgetc: a byte, or EOF
    int get() {
        if (p >= e) {
            at_eof = true;
            return EOF;
        }
        return *p++;
    }
    // fgetc until a newline (consumed) or the end
    void rest_of_line() {
        for (int c = get(); c != '\n' && c != EOF; c = get()) {}
    }
};

static inline bool ends_line(const Text::Piece &pc) { return pc.vis > 0 && pc.s[pc.vis - 1] == '\n'; }

// sscanf on s[0, len) with a format of literal bytes, ' ' (any run of white
// space, possibly empty) and 'D' (a %lld conversion: white space, optional
// sign, at least one digit; out-of-range values saturate as strtoll's do).
// Returns the number of conversions before the first mismatch.
static int scan_fmt(const char *s, size_t len, const char *fmt, long long *out) {
    size_t k = 0;
    int got = 0;
    auto space = [&](size_t at) { return at < len && isspace((unsigned char)s[at]); };
    for (const char *f = fmt; *f; ++f) {
        if (*f == ' ') {
            while (space(k)) ++k;
        } else if (*f == 'D') {
            while (space(k)) ++k;
            bool neg = false;
            if (k < len && (s[k] == '+' || s[k] == '-')) neg = s[k++] == '-';
            const size_t d0 = k;
            unsigned long long mag = 0;
            bool over = false;
            const unsigned long long lim = neg ? 9223372036854775808ull : 9223372036854775807ull;
            for (; k < len && s[k] >= '0' && s[k] <= '9'; ++k) {
                const unsigned dig = (unsigned)(s[k] - '0');
                if (!over && mag <= (lim - dig) / 10) mag = mag * 10 + dig;
                else over = true;
            }
            if (k == d0) return got;
            if (over) mag = lim;
            out[got++] = neg ? (long long)(0ull - mag) : (long long)mag;
        } else {
            if (k >= len || s[k] != *f) return got;
            ++k;
        }
    }
    return got;
}

// DIMACS (shared_memory/graph.hpp:168-189): `p sp n m` once, `a u v w` with
// 1-based ids, `c` comments; a piece that does not end its line (long line,
// or the last line without a newline) is allowed only as a comment, whose
// remainder is skipped.
static bool parse_dimacs(Text &t, bool undirected, chl_graph *g, std::vector<TmpArc> &tmp, long long &n) {
    bool have_p = false;
    Text::Piece pc;
    long long v[3];
    while (t.piece(pc)) {
        const char c0 = pc.vis ? pc.s[0] : '\0';
        if (!ends_line(pc)) {
            if (c0 != 'c') return false;
            if (!t.at_eof) t.rest_of_line();
            continue;
        }
        switch (c0) {
        case 'c':
            break;
        case 'p':
            if (have_p || scan_fmt(pc.s, pc.vis, "p sp D D", v) != 2) return false;
            have_p = true;
            n = v[0];
            break;
        case 'a':
            if (scan_fmt(pc.s, pc.vis, "a D D D", v) != 3 ||
                !add_tmp_arc(g, n, tmp, (uint32_t)(v[0] - 1), (uint32_t)(v[1] - 1), (int32_t)v[2], undirected))
                return false;
            break;
        default:
            return false;
        }
    }
    return true;
}

// SNAP (shared_memory/graph.hpp:262-282): `#` lines are comments (their
// remainder skipped), one of them may be the `# Nodes: n Edges: m` header;
// every other line holds `u v` (0-based, length 1) and must end with a
// newline unless it is the last.
static bool parse_snap(Text &t, bool undirected, chl_graph *g, std::vector<TmpArc> &tmp, long long &n) {
    bool have_header = false;
    Text::Piece pc;
    long long v[2];
    while (t.piece(pc)) {
        if (pc.vis && pc.s[0] == '#') {
            // sscanf stores each conversion as it succeeds: a comment that
            // matches only up to the vertex count still sets n
            const int got = scan_fmt(pc.s, pc.vis, "# Nodes: D Edges: D", v);
            if (got >= 1) n = v[0];
            if (got == 2) {
                if (have_header) return false;
                have_header = true;
            }
            if (!ends_line(pc)) t.rest_of_line();
            continue;
        }
        if (!ends_line(pc) && !t.at_eof) return false;
        if (scan_fmt(pc.s, pc.vis, "D D", v) != 2 ||
            !add_tmp_arc(g, n, tmp, (uint32_t)v[0], (uint32_t)v[1], 1, undirected))
            return false;
    }
    return true;
}

// Edge list (shared_memory/graph.hpp:284-308): `u v w` per line (0-based),
// n = the number of distinct ids.  The reference indexes its arrays by the
// raw ids, so ids outside [0, n) are undefined behaviour there; they are
// rejected here.
static bool parse_edgelist(Text &t, bool undirected, chl_graph *g, std::vector<TmpArc> &tmp, long long &n) {
    std::set<long long> ids;
    Text::Piece pc;
    long long v[3];
    while (t.piece(pc)) {
        if (!ends_line(pc) && !t.at_eof) return false;
        if (scan_fmt(pc.s, pc.vis, "D D D", v) != 3) return false;
        tmp.push_back(TmpArc{(uint32_t)v[0], (uint32_t)v[1], (int32_t)v[2], 1, (uint8_t)undirected});
        tmp.push_back(TmpArc{(uint32_t)v[1], (uint32_t)v[0], (int32_t)v[2], (uint8_t)undirected, 1});
        g->m += 1 + (undirected ? 1 : 0);
        ids.insert(v[0]);
        ids.insert(v[1]);
    }
    n = (long long)ids.size();
    for (const TmpArc &a : tmp)
        if ((long long)a.u >= n || (long long)a.head >= n) return false;
    return true;
}

// METIS (shared_memory/graph.hpp:211-256), in two stages.  The lexer turns
// bytes into numbers and line ends: digits accumulate into a number (with
// wrap-around, as the reference's long long does), white space ends it, a
// newline also ends the line, '%' starts a comment that swallows everything
// through the next newline -- that newline ends no line, and a number may go
// on after it -- and any other byte rejects the file.  The end of the input
// ends a pending number but no line, except inside a comment, where the
// pending number is dropped.
// The interpreter reads line 0 as the header `n m [fmt [ncon]]` (fmt's
// digits each 0 or 1, fmt <= 111; ncon only when fmt's tens digit is 1) and
// line v > 0 as the arcs of vertex v - 1 after `skip` leading numbers (vertex
// size and weights): heads (1-based), each followed by a length when fmt's
// ones digit is 1.  A line short of its leading numbers, or with a head but
// no length, rejects the file.
struct MetisInterp {
    bool undirected;
    chl_graph *g;
    std::vector<TmpArc> &tmp;
    long long &n;
    uint32_t line = 0;
    int idx = 0;          // numbers seen on this line
    long long fmt = 0;
    int skip = 0;
    uint32_t head = 0xFFFFFFFFu;

    bool number(long long x) {
        if (line == 0) {
            switch (idx) {
            case 0:
                n = x;
                break;
            case 1:
                break;   // the arc count is not used
            case 2:
                if (x % 10 > 1 || (x / 10) % 10 > 1 || x > 111) return false;
                fmt = x;
                skip = (fmt >= 100) + (fmt % 100 >= 10);
                break;
            case 3:
                if (fmt % 100 < 10) return false;
                skip = (int)((fmt >= 100) + x);
                break;
            default:
                return false;
            }
        } else if (idx >= skip) {
            const bool weighted = fmt % 10 == 1;
            if (weighted && (idx - skip) % 2 == 0) {
                head = (uint32_t)(x - 1);
            } else if (!add_tmp_arc(g, n, tmp, line - 1, weighted ? head : (uint32_t)(x - 1),
                                    weighted ? (int32_t)x : 1, undirected)) {
                return false;
            }
        }
        ++idx;
        return true;
    }
    bool end_line() {
        if (line > 0 && (idx < skip || (fmt % 10 == 1 && (idx - skip) % 2 == 1))) return false;
        ++line;
        idx = 0;
        return true;
    }
};

// Runs the METIS lexer over t; true if the file is accepted.  *stopped_early
// (may be NULL) tells whether a rejection came before the end of the input.
static bool parse_metis(Text &t, MetisInterp &in, bool *stopped_early) {
    unsigned long long acc = 0;
    bool pending = false;
    if (stopped_early) *stopped_early = false;
    auto reject = [&]() {
        if (stopped_early) *stopped_early = !t.at_eof;
        return false;
    };
    while (true) {
        const int c = t.get();
        if (c == '%') {
            int d;
            do d = t.get(); while (d != '\n' && d != EOF);
            if (d == EOF) return true;   // a pending number is dropped
            continue;
        }
        if (c >= '0' && c <= '9') {
            acc = acc * 10 + (unsigned)(c - '0');
            pending = true;
            continue;
        }
        if (c != EOF && !isspace(c)) return reject();
        if (pending) {
            if (!in.number((long long)acc)) return reject();
            acc = 0;
            pending = false;
        }
        if (c == EOF) return true;
        if (c == '\n' && !in.end_line()) return reject();
    }
}

// true when the METIS reader rejects a file that starts with buf[0, len)
// before reading past it (its verdict is then final for the whole file)
bool metis_rejects_prefix(const char *buf, size_t len) {
    chl_graph g;
    std::vector<TmpArc> tmp;
    long long n = 0;
    Text t{(const unsigned char *)buf, (const unsigned char *)buf + len};
    MetisInterp in{false, &g, tmp, n};
    bool early = false;
    return !parse_metis(t, in, &early) && early;
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
    FILE *file = fopen(path, "rb");
    if (!file) {
        set_error(std::string("cannot open graph file ") + path);
        return CHL_ERR_IO;
    }
    std::vector<unsigned char> bytes;
    {
        unsigned char chunk[1 << 16];
        size_t k;
        while ((k = fread(chunk, 1, sizeof(chunk), file)) > 0) bytes.insert(bytes.end(), chunk, chunk + k);
        const bool bad = ferror(file) != 0;
        fclose(file);
        if (bad) {
            set_error(std::string("cannot read graph file ") + path);
            return CHL_ERR_IO;
        }
    }
    // hl::Graph::read (shared_memory/graph.hpp:327-335): each reader in turn
    // from the start of the file, the first that accepts it wins
    const unsigned char *b = bytes.data(), *e = bytes.data() + bytes.size();
    for (int fmt = 0; fmt < 4; ++fmt) {
        chl_graph *g = new (std::nothrow) chl_graph();
        if (!g) return CHL_ERR_OOM;
        std::vector<TmpArc> tmp;
        long long n = 0;
        Text t{b, e};
        bool ok;
        if (fmt == 0) {
            ok = parse_dimacs(t, undirected != 0, g, tmp, n);
        } else if (fmt == 1) {
            MetisInterp in{undirected != 0, g, tmp, n};
            ok = parse_metis(t, in, nullptr);
        } else if (fmt == 2) {
            ok = parse_snap(t, undirected != 0, g, tmp, n);
        } else {
            ok = parse_edgelist(t, undirected != 0, g, tmp, n);
        }
        if (ok) {
            int st = finish(g, n, tmp);
            if (st != CHL_OK) {
                delete g;
                return st;
            }
            *out = g;
            return CHL_OK;
        }
        delete g;
    }
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
