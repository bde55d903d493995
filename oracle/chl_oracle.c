/*
 * chl_oracle.c -- CPU restatement of the reference's canonical hub labeling
 * path.  TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the CPU
 * baseline leg of bench.py load this library as the checker / baseline.
 * The product (plant_gb300) never links or calls it.
 *
 * Every function names the reference code it restates (paths relative to
 * the qingdo/plant project root).  Parity of this restatement is pinned
 * against the reference itself (oracle/_ref, built from the reference
 * sources by oracle/Makefile) by tests/test_oracle_pin.py and by the golden
 * fixtures under tests/golden/.
 */
#include <limits.h>
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "chl_digest.h"

#define INFTY INT_MAX

/* ------------------------------------------------------------- graph */

/* Adjacency after init_arcs (shared_memory/graph.hpp:103-153): CSR per
 * direction, side 1 = forward (out) arcs, side 0 = reverse (in) arcs. */
typedef struct {
    uint32_t n;
    uint64_t *off[2];
    uint32_t *head[2];
    int32_t *len[2];
} og_graph;

typedef struct {
    uint32_t u, head;
    int32_t len;
    uint8_t fwd, rev;
} og_tmp;

static int cmp_dir(const void *pa, const void *pb) {
    const og_tmp *x = pa, *y = pb;
    if (x->u != y->u) return x->u < y->u ? -1 : 1;
    if (x->rev != y->rev) return x->rev > y->rev ? -1 : 1;
    if (x->fwd != y->fwd) return x->fwd < y->fwd ? -1 : 1;
    if (x->head != y->head) return x->head < y->head ? -1 : 1;
    if (x->len != y->len) return x->len < y->len ? -1 : 1;
    return 0;
}
static int cmp_head(const void *pa, const void *pb) {
    const og_tmp *x = pa, *y = pb;
    if (x->u != y->u) return x->u < y->u ? -1 : 1;
    if (x->head != y->head) return x->head < y->head ? -1 : 1;
    if (x->len != y->len) return x->len < y->len ? -1 : 1;
    /* order of equal (u, head, len) is immaterial: flags are OR-merged */
    return 0;
}

/* init_arcs: dedup keeping the shortest arc per (u, head, fwd, rev), merge
 * equal-length forward/reverse arcs, lay out per-vertex lists. */
static og_graph *og_finalize(uint32_t n, og_tmp *a, size_t na) {
    og_graph *g = calloc(1, sizeof(og_graph));
    g->n = n;
    if (na) {
        size_t i = 0, j;
        qsort(a, na, sizeof(og_tmp), cmp_dir);
        for (j = 1; j < na; ++j) {
            if (a[i].u == a[j].u && a[i].head == a[j].head && a[i].fwd == a[j].fwd &&
                a[i].rev == a[j].rev)
                continue;
            if (++i < j) a[i] = a[j];
        }
        na = i + 1;
        qsort(a, na, sizeof(og_tmp), cmp_head);
        i = 0;
        for (j = 1; j < na; ++j) {
            if (a[i].u == a[j].u && a[i].head == a[j].head && a[i].len == a[j].len) {
                a[i].fwd |= a[j].fwd;
                a[i].rev |= a[j].rev;
                continue;
            }
            if (++i < j) a[i] = a[j];
        }
        na = i + 1;
        qsort(a, na, sizeof(og_tmp), cmp_dir);
    }
    for (int s = 0; s < 2; ++s) {
        g->off[s] = calloc((size_t)n + 1, sizeof(uint64_t));
    }
    for (size_t k = 0; k < na; ++k) {
        if (a[k].fwd) g->off[1][a[k].u + 1]++;
        if (a[k].rev) g->off[0][a[k].u + 1]++;
    }
    for (int s = 0; s < 2; ++s) {
        for (uint32_t v = 0; v < n; ++v) g->off[s][v + 1] += g->off[s][v];
        g->head[s] = malloc((g->off[s][n] + 1) * sizeof(uint32_t));
        g->len[s] = malloc((g->off[s][n] + 1) * sizeof(int32_t));
    }
    uint64_t *pos[2];
    for (int s = 0; s < 2; ++s) {
        pos[s] = malloc(((size_t)n + 1) * sizeof(uint64_t));
        memcpy(pos[s], g->off[s], ((size_t)n + 1) * sizeof(uint64_t));
    }
    for (size_t k = 0; k < na; ++k) {
        for (int s = 0; s < 2; ++s) {
            if (s == 1 ? a[k].fwd : a[k].rev) {
                uint64_t p = pos[s][a[k].u]++;
                g->head[s][p] = a[k].head;
                g->len[s][p] = a[k].len;
            }
        }
    }
    free(pos[0]);
    free(pos[1]);
    return g;
}

/* Graph::read_dimacs (shared_memory/graph.hpp:168-189) with
 * undirected = false, as the hhl CLI calls it.  Returns NULL if the file is
 * not a DIMACS graph. */
og_graph *og_read_dimacs(const char *path) {
    FILE *f = fopen(path, "r");
    if (!f) return NULL;
    char buf[512];
    long long u, v, w, m, n = 0;
    int inited = 0, ok = 1;
    size_t na = 0, cap = 1024;
    og_tmp *a = malloc(cap * sizeof(og_tmp));
    while (fgets(buf, sizeof(buf), f)) {
        size_t L = strlen(buf);
        if (L == 0 || buf[L - 1] != '\n') {
            if (buf[0] != 'c') { ok = 0; break; }
            while (!feof(f) && fgetc(f) != '\n') {}
        } else if (buf[0] == 'p') {
            if (inited) { ok = 0; break; }
            inited = 1;
            if (sscanf(buf, "p sp %lld %lld", &n, &m) != 2) { ok = 0; break; }
        } else if (buf[0] == 'a') {
            if (sscanf(buf, "a %lld %lld %lld", &u, &v, &w) != 3) { ok = 0; break; }
            uint32_t uu = (uint32_t)(u - 1), vv = (uint32_t)(v - 1);
            if ((long long)uu >= n || (long long)vv >= n) { ok = 0; break; }
            if (na + 2 > cap) {
                cap *= 2;
                a = realloc(a, cap * sizeof(og_tmp));
            }
            a[na++] = (og_tmp){uu, vv, (int32_t)w, 1, 0};
            a[na++] = (og_tmp){vv, uu, (int32_t)w, 0, 1};
        } else if (buf[0] == 'c') {
            continue;
        } else {
            ok = 0;
            break;
        }
    }
    fclose(f);
    if (!ok) {
        free(a);
        return NULL;
    }
    og_graph *g = og_finalize((uint32_t)n, a, na);
    free(a);
    return g;
}

/* Graph from arrays of arcs (add_arc with undirected=false, then finalize). */
og_graph *og_from_arcs(uint32_t n, size_t k, const uint32_t *src, const uint32_t *dst,
                       const int32_t *len) {
    og_tmp *a = malloc((2 * k + 1) * sizeof(og_tmp));
    for (size_t i = 0; i < k; ++i) {
        a[2 * i] = (og_tmp){src[i], dst[i], len[i], 1, 0};
        a[2 * i + 1] = (og_tmp){dst[i], src[i], len[i], 0, 1};
    }
    og_graph *g = og_finalize(n, a, 2 * k);
    free(a);
    return g;
}

uint32_t og_n(const og_graph *g) { return g->n; }
uint64_t og_arcs(const og_graph *g, int side) { return g->off[side][g->n]; }
/* copy CSR of one side out (off: n+1, head/len: arcs) */
void og_export(const og_graph *g, int side, uint64_t *off, uint32_t *head, int32_t *len) {
    memcpy(off, g->off[side], ((size_t)g->n + 1) * sizeof(uint64_t));
    memcpy(head, g->head[side], g->off[side][g->n] * sizeof(uint32_t));
    memcpy(len, g->len[side], g->off[side][g->n] * sizeof(int32_t));
}

void og_free(og_graph *g) {
    if (!g) return;
    for (int s = 0; s < 2; ++s) {
        free(g->off[s]);
        free(g->head[s]);
        free(g->len[s]);
    }
    free(g);
}

/* ------------------------------------------------- workload generators */
/* Restatements of the package's own seeded generators (chl_gen_grid and
 * chl_gen_rmat; the reference has none: its datasets are external files), so
 * the CPU baseline can build the benchmark's graphs without loading the
 * product library.  Same splitmix64 stream, same draws in the same order,
 * same edge lists; the graph is then built as a DIMACS file listing every
 * undirected edge in both directions would be (og_from_arcs = init_arcs). */

typedef struct {
    uint64_t s;
} og_rng;
static inline uint64_t og_rng_next(og_rng *r) {
    r->s += 0x9E3779B97F4A7C15ull;
    uint64_t z = r->s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static inline uint64_t og_rng_below(og_rng *r, uint64_t range) { return og_rng_next(r) % range; }
static inline double og_rng_unit(og_rng *r) { return (double)(og_rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }
static inline uint64_t og_mix_seed(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* open-addressing set of undirected edge keys (min << 32 | max) */
typedef struct {
    uint64_t *t;
    uint64_t mask;
} og_eset;
static void eset_init(og_eset *e, uint64_t expect) {
    uint64_t c = 1024;
    while (c < 2 * expect + 16) c <<= 1;
    e->t = malloc(c * sizeof(uint64_t));
    memset(e->t, 0xFF, c * sizeof(uint64_t));
    e->mask = c - 1;
}
/* 1 if inserted, 0 if present */
static int eset_add(og_eset *e, uint64_t k) {
    uint64_t h = og_mix_seed(k) & e->mask;
    while (e->t[h] != ~0ull) {
        if (e->t[h] == k) return 0;
        h = (h + 1) & e->mask;
    }
    e->t[h] = k;
    return 1;
}
static inline uint64_t ekey(uint32_t a, uint32_t b) {
    if (a > b) {
        uint32_t t = a;
        a = b;
        b = t;
    }
    return ((uint64_t)a << 32) | b;
}

static uint32_t uf_find(uint32_t *par, uint32_t x) {
    while (par[x] != x) {
        par[x] = par[par[x]];
        x = par[x];
    }
    return x;
}

static og_graph *og_from_edges(uint32_t n, const uint64_t *uv, const int32_t *w, size_t k) {
    uint32_t *src = malloc((k + 1) * sizeof(uint32_t)), *dst = malloc((k + 1) * sizeof(uint32_t));
    for (size_t i = 0; i < k; ++i) {
        src[i] = (uint32_t)(uv[i] >> 32);
        dst[i] = (uint32_t)uv[i];
    }
    /* both directions of every edge, as a DIMACS file listing each twice */
    og_tmp *a = malloc((4 * k + 1) * sizeof(og_tmp));
    for (size_t i = 0; i < k; ++i) {
        a[4 * i] = (og_tmp){src[i], dst[i], w[i], 1, 0};
        a[4 * i + 1] = (og_tmp){dst[i], src[i], w[i], 0, 1};
        a[4 * i + 2] = (og_tmp){dst[i], src[i], w[i], 1, 0};
        a[4 * i + 3] = (og_tmp){src[i], dst[i], w[i], 0, 1};
    }
    og_graph *g = og_finalize(n, a, 4 * k);
    free(a);
    free(src);
    free(dst);
    return g;
}

/* chl_gen_grid: rows x cols 4-neighbour grid, del_frac of its edges deleted,
 * largest component kept, floor(diag_frac * n) diagonal shortcuts, then
 * `highways` edges of length round(hw_factor * Manhattan steps) between
 * vertices at most hw_steps apart.  NULL on invalid arguments. */
og_graph *og_gen_grid(uint32_t rows, uint32_t cols, double del_frac, double diag_frac, int32_t wmin,
                      int32_t wmax, uint32_t highways, uint32_t hw_steps, double hw_factor, uint64_t seed) {
    if (rows == 0 || cols == 0 || wmin < 1 || wmax < wmin || (uint64_t)rows * cols >= (1ull << 30) ||
        del_frac < 0 || del_frac >= 1)
        return NULL;
    og_rng rng = {seed};
    const uint64_t N0 = (uint64_t)rows * cols;
    typedef struct {
        uint32_t a, b;
        int32_t w;
    } E;
    E *edges = malloc((2 * N0 + 1) * sizeof(E));
    uint64_t E0 = 0;
    for (uint32_t r = 0; r < rows; ++r)
        for (uint32_t c = 0; c < cols; ++c) {
            uint32_t id = r * cols + c;
            if (c + 1 < cols) edges[E0++] = (E){id, id + 1, 0};
            if (r + 1 < rows) edges[E0++] = (E){id, id + cols, 0};
        }
    for (uint64_t k = 0; k < E0; ++k) edges[k].w = wmin + (int32_t)og_rng_below(&rng, (uint64_t)(wmax - wmin) + 1);
    uint64_t ndel = (uint64_t)llround(del_frac * (double)E0);
    if (ndel > E0) ndel = E0;
    for (uint64_t k = 0; k < ndel; ++k) {
        uint64_t j = k + og_rng_below(&rng, E0 - k);
        E t = edges[k];
        edges[k] = edges[j];
        edges[j] = t;
    }
    uint32_t *par = malloc(N0 * sizeof(uint32_t));
    for (uint64_t i = 0; i < N0; ++i) par[i] = (uint32_t)i;
    for (uint64_t k = ndel; k < E0; ++k) {
        uint32_t a = uf_find(par, edges[k].a), b = uf_find(par, edges[k].b);
        if (a != b) {
            if (a > b) par[a] = b;
            else par[b] = a;
        }
    }
    uint32_t *sz = calloc(N0, sizeof(uint32_t));
    for (uint64_t i = 0; i < N0; ++i) sz[uf_find(par, (uint32_t)i)]++;
    uint32_t best = 0;
    for (uint64_t i = 0; i < N0; ++i)
        if (sz[i] > sz[best]) best = (uint32_t)i;
    uint32_t *newid = malloc(N0 * sizeof(uint32_t)), *oldid = malloc(N0 * sizeof(uint32_t));
    uint32_t n = 0;
    for (uint64_t i = 0; i < N0; ++i) {
        newid[i] = 0xFFFFFFFFu;
        if (uf_find(par, (uint32_t)i) == best) {
            newid[i] = n;
            oldid[n++] = (uint32_t)i;
        }
    }
    const uint64_t ndiag = (uint64_t)floor(diag_frac * (double)n);
    const uint64_t cap = (E0 - ndel) + ndiag + highways + 1;
    uint64_t *uv = malloc(cap * sizeof(uint64_t));
    int32_t *w = malloc(cap * sizeof(int32_t));
    size_t k = 0;
    og_eset present;
    eset_init(&present, cap);
    for (uint64_t e = ndel; e < E0; ++e) {
        if (newid[edges[e].a] == 0xFFFFFFFFu) continue;
        uint64_t key = ekey(newid[edges[e].a], newid[edges[e].b]);
        uv[k] = key;
        w[k++] = edges[e].w;
        eset_add(&present, key);
    }
    uint64_t added = 0, tries = 0;
    while (added < ndiag && tries < 64 * (ndiag + 16)) {
        ++tries;
        uint32_t x = oldid[og_rng_below(&rng, n)];
        uint32_t dir = (uint32_t)og_rng_below(&rng, 4);
        int r = (int)(x / cols), c = (int)(x % cols);
        int r2 = r + ((dir & 1) ? 1 : -1), c2 = c + ((dir & 2) ? 1 : -1);
        int32_t len = wmin + (int32_t)og_rng_below(&rng, (uint64_t)(wmax - wmin) + 1);
        if (r2 < 0 || c2 < 0 || r2 >= (int)rows || c2 >= (int)cols) continue;
        uint32_t y = (uint32_t)r2 * cols + (uint32_t)c2;
        if (newid[y] == 0xFFFFFFFFu) continue;
        uint64_t key = ekey(newid[x], newid[y]);
        if (!eset_add(&present, key)) continue;
        uv[k] = key;
        w[k++] = len;
        ++added;
    }
    added = 0;
    tries = 0;
    const int S = (int)hw_steps;
    while (S >= 2 && added < highways && tries < 64 * ((uint64_t)highways + 16)) {
        ++tries;
        uint32_t x = oldid[og_rng_below(&rng, n)];
        int dr = (int)og_rng_below(&rng, 2 * (uint64_t)S + 1) - S;
        int rem = S - abs(dr);
        int dc = (int)og_rng_below(&rng, 2 * (uint64_t)rem + 1) - rem;
        int steps = abs(dr) + abs(dc);
        if (steps < 2) continue;
        int r2 = (int)(x / cols) + dr, c2 = (int)(x % cols) + dc;
        if (r2 < 0 || c2 < 0 || r2 >= (int)rows || c2 >= (int)cols) continue;
        uint32_t y = (uint32_t)r2 * cols + (uint32_t)c2;
        if (newid[y] == 0xFFFFFFFFu) continue;
        uint64_t key = ekey(newid[x], newid[y]);
        if (!eset_add(&present, key)) continue;
        uv[k] = key;
        w[k++] = (int32_t)llround(hw_factor * steps);
        ++added;
    }
    og_graph *g = og_from_edges(n, uv, w, k);
    free(present.t);
    free(uv);
    free(w);
    free(newid);
    free(oldid);
    free(sz);
    free(par);
    free(edges);
    return g;
}

static int cmp_u64(const void *pa, const void *pb) {
    const uint64_t x = *(const uint64_t *)pa, y = *(const uint64_t *)pb;
    return x < y ? -1 : (x > y);
}

/* chl_gen_rmat: 2^scale vertices, ef * 2^scale edge draws with quadrant
 * probabilities (a, b, c, 1 - a - b - c), draw k from its own stream seeded
 * by mix(seed ^ k * 0xD1B54A32D192ED03); self loops and duplicates dropped,
 * unit lengths. */
og_graph *og_gen_rmat(uint32_t scale, uint32_t ef, double a, double b, double c, uint64_t seed) {
    if (scale == 0 || scale > 29 || ef == 0) return NULL;
    const uint64_t n = 1ull << scale, M = (uint64_t)ef * n;
    uint64_t *uv = malloc(M * sizeof(uint64_t));
    const double ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(static)
    for (long long k = 0; k < (long long)M; ++k) {
        og_rng r = {og_mix_seed(seed ^ ((uint64_t)k * 0xD1B54A32D192ED03ull))};
        uint64_t u = 0, v = 0;
        for (uint32_t l = 0; l < scale; ++l) {
            double x = og_rng_unit(&r);
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
            if (u > v) {
                uint64_t t = u;
                u = v;
                v = t;
            }
            uv[k] = (u << 32) | v;
        }
    }
    qsort(uv, M, sizeof(uint64_t), cmp_u64);
    size_t k = 0;
    for (uint64_t i = 0; i < M; ++i) {
        if (uv[i] == ~0ull) break;
        if (k == 0 || uv[k - 1] != uv[i]) uv[k++] = uv[i];
    }
    int32_t *w = malloc((k + 1) * sizeof(int32_t));
    for (size_t i = 0; i < k; ++i) w[i] = 1;
    og_graph *g = og_from_edges((uint32_t)n, uv, w, k);
    free(w);
    free(uv);
    return g;
}

/* ------------------------------------------------------------- labels */

typedef struct {
    uint32_t *h;
    int32_t *d;
    uint32_t n, cap;
} ol_list;

/* Labeling (shared_memory/labeling.hpp:45-54): lists[2v + side]. */
typedef struct {
    uint32_t n;
    ol_list *l;
} ol_labels;

static ol_labels *ol_new(uint32_t n) {
    ol_labels *L = malloc(sizeof(ol_labels));
    L->n = n;
    L->l = calloc(2 * (size_t)n + 1, sizeof(ol_list));
    return L;
}

static inline void ol_push(ol_list *x, uint32_t h, int32_t d) {
    if (x->n == x->cap) {
        x->cap = x->cap ? 2 * x->cap : 4;
        x->h = realloc(x->h, x->cap * sizeof(uint32_t));
        x->d = realloc(x->d, x->cap * sizeof(int32_t));
    }
    x->h[x->n] = h;
    x->d[x->n] = d;
    x->n++;
}

static void ol_clear(ol_labels *L) {
    for (size_t x = 0; x < 2 * (size_t)L->n; ++x) L->l[x].n = 0;
}

void ol_free(ol_labels *L) {
    if (!L) return;
    for (size_t x = 0; x < 2 * (size_t)L->n; ++x) {
        free(L->l[x].h);
        free(L->l[x].d);
    }
    free(L->l);
    free(L);
}

uint64_t ol_total(const ol_labels *L) {
    uint64_t t = 0;
    for (size_t x = 0; x < 2 * (size_t)L->n; ++x) t += L->l[x].n;
    return t;
}

/* Labeling::get_avg (shared_memory/labeling.hpp:153-158) */
double ol_avg(const ol_labels *L) { return (double)ol_total(L) / L->n / 2; }

/* export as CSR over index 2v+side */
void ol_export(const ol_labels *L, uint64_t *off, uint32_t *hub, int32_t *dist) {
    uint64_t p = 0;
    off[0] = 0;
    for (size_t x = 0; x < 2 * (size_t)L->n; ++x) {
        for (uint32_t k = 0; k < L->l[x].n; ++k, ++p) {
            hub[p] = L->l[x].h[k];
            dist[p] = L->l[x].d[k];
        }
        off[x + 1] = p;
    }
}

ol_labels *ol_import(uint32_t n, const uint64_t *off, const uint32_t *hub, const int32_t *dist) {
    ol_labels *L = ol_new(n);
    for (size_t x = 0; x < 2 * (size_t)n; ++x)
        for (uint64_t k = off[x]; k < off[x + 1]; ++k) ol_push(&L->l[x], hub[k], dist[k]);
    return L;
}

/* Digest (chl_digest.h) of the content Labeling::write would emit
 * (shared_memory/labeling.hpp:167-183): n, then every list 2v + side. */
uint64_t ol_digest(const ol_labels *L) {
    uint64_t dg = chd_head(L->n);
    for (size_t x = 0; x < 2 * (size_t)L->n; ++x) {
        const uint64_t base = chd_list_base(x);
        dg += chd_list_term(base, L->l[x].n);
        for (uint32_t k = 0; k < L->l[x].n; ++k) dg += chd_entry_term(base, k, L->l[x].h[k], (uint32_t)L->l[x].d[k]);
    }
    return dg;
}

/* Digest of an order (rank -> vertex), as written by Order::write
 * (shared_memory/ordering.hpp:37-49). */
uint64_t og_order_digest(const uint32_t *order, uint32_t n) {
    uint64_t dg = chd_head(n);
    for (uint32_t i = 0; i < n; ++i) dg += chd_order_term(i, order[i]);
    return dg;
}

/* Labeling::write (shared_memory/labeling.hpp:167-183) */
int ol_write(const ol_labels *L, const char *path) {
    FILE *f = fopen(path, "w");
    if (!f) return 1;
    fprintf(f, "%u\n", L->n);
    for (uint32_t v = 0; v < L->n; ++v)
        for (int s = 0; s < 2; ++s) {
            const ol_list *x = &L->l[2 * (size_t)v + s];
            fprintf(f, "%u", x->n);
            for (uint32_t k = 0; k < x->n; ++k) fprintf(f, " %u %d", x->h[k], x->d[k]);
            fputc('\n', f);
        }
    return fclose(f) != 0;
}

/* Labeling::query (shared_memory/labeling.hpp:56-65), f = true:
 * merge L(u,1) with L(v,0). */
int32_t ol_query(const ol_labels *L, uint32_t u, uint32_t v) {
    const ol_list *a = &L->l[2 * (size_t)u + 1], *b = &L->l[2 * (size_t)v];
    int64_t r = INFTY;
    uint32_t i = 0, j = 0;
    while (i < a->n && j < b->n) {
        if (a->h[i] == b->h[j]) {
            int64_t s = (int64_t)a->d[i++] + b->d[j++];
            if (s < r) r = s;
        } else if (a->h[i] < b->h[j]) {
            ++i;
        } else {
            ++j;
        }
    }
    return (int32_t)r;
}

/* batchLocalQuery (distributed_memory/query_funcs.hpp:23-30) */
void ol_query_batch(const ol_labels *L, const uint32_t *pairs, size_t k, int32_t *out, int threads) {
#pragma omp parallel for num_threads(threads) schedule(dynamic, 2 * threads)
    for (long long i = 0; i < (long long)k; ++i) out[i] = ol_query(L, pairs[2 * i], pairs[2 * i + 1]);
}

/* ------------------------------------------------------ heap + dijkstra */

/* KHeap<Vertex, Distance, 4> (shared_memory/kheap.hpp:33-89) */
typedef struct {
    uint32_t size;
    uint32_t *heap;
    uint32_t *pos;   /* UINT32_MAX = not in heap */
    int32_t *key;
} oh_heap;

static void oh_init(oh_heap *h, uint32_t n) {
    h->size = 0;
    h->heap = malloc(((size_t)n + 1) * sizeof(uint32_t));
    h->pos = malloc(((size_t)n + 1) * sizeof(uint32_t));
    h->key = malloc(((size_t)n + 1) * sizeof(int32_t));
    for (uint32_t i = 0; i < n; ++i) h->pos[i] = UINT32_MAX;
}
static void oh_free(oh_heap *h) {
    free(h->heap);
    free(h->pos);
    free(h->key);
}
static inline void oh_swap(oh_heap *h, uint32_t i, uint32_t j) {
    uint32_t a = h->heap[i], b = h->heap[j];
    h->heap[i] = b;
    h->heap[j] = a;
    h->pos[b] = i;
    h->pos[a] = j;
}
static inline uint32_t oh_kid(const oh_heap *h, uint32_t i) {
    uint32_t c0 = i * 4 + 1, m = 0;
    for (uint32_t j = 1; j < 4 && c0 + j < h->size; ++j)
        if (h->key[h->heap[c0 + j]] < h->key[h->heap[c0 + m]]) m = j;
    return c0 + m;
}
static inline void oh_fix(oh_heap *h, uint32_t i) {
    uint32_t c;
    while (i * 4 + 1 < h->size && h->key[h->heap[i]] > h->key[h->heap[(c = oh_kid(h, i))]]) {
        oh_swap(h, i, c);
        i = c;
    }
    while (i > 0 && h->key[h->heap[i]] < h->key[h->heap[(i - 1) / 4]]) {
        oh_swap(h, i, (i - 1) / 4);
        i = (i - 1) / 4;
    }
}
static inline void oh_update(oh_heap *h, uint32_t v, int32_t k) {
    if (h->pos[v] == UINT32_MAX) {
        h->pos[v] = h->size++;
        h->heap[h->pos[v]] = v;
    }
    h->key[v] = k;
    oh_fix(h, h->pos[v]);
}
static inline uint32_t oh_pop(oh_heap *h) {
    uint32_t v = h->heap[0];
    uint32_t p = h->pos[v];
    if (p < --h->size) {
        oh_swap(h, p, h->size);
        oh_fix(h, p);
    }
    h->pos[v] = UINT32_MAX;
    return v;
}
static void oh_clear(oh_heap *h) {
    for (uint32_t i = 0; i < h->size; ++i) h->pos[h->heap[i]] = UINT32_MAX;
    h->size = 0;
}

/* Dijkstra::run (shared_memory/dijkstra.hpp:83-95): dist[] for all vertices
 * (INT_MAX if unreachable), forward = 1 follows out-arcs. */
void og_dijkstra(const og_graph *g, uint32_t src, int forward, int32_t *dist) {
    oh_heap h;
    oh_init(&h, g->n);
    for (uint32_t i = 0; i < g->n; ++i) dist[i] = INFTY;
    dist[src] = 0;
    oh_update(&h, src, 0);
    const int s = forward ? 1 : 0;
    while (h.size) {
        uint32_t u = oh_pop(&h);
        int32_t d = dist[u];
        for (uint64_t a = g->off[s][u]; a < g->off[s][u + 1]; ++a) {
            int32_t dd = d + g->len[s][a];
            uint32_t w = g->head[s][a];
            if (dd < dist[w]) {
                dist[w] = dd;
                oh_update(&h, w, dd);
            }
        }
    }
    oh_free(&h);
}

/* ------------------------------------------------------------ GLL */

/* Per-thread state of hl::Akiba (shared_memory/akiba.hpp:42-63 and
 * BasicDijkstra shared_memory/dijkstra.hpp:34-72). */
typedef struct {
    oh_heap q;
    int32_t *distance;
    uint8_t *is_dirty;
    uint32_t *dirty;
    uint32_t ndirty;
    int32_t *label_tmp;
    uint8_t *is_dirty_tmp;
    uint32_t *dirty_tmp;
    uint32_t ndirty_tmp;
} o_akiba;

static void ak_init(o_akiba *a, uint32_t n) {
    oh_init(&a->q, n);
    a->distance = malloc((size_t)n * sizeof(int32_t));
    a->label_tmp = malloc((size_t)n * sizeof(int32_t));
    for (uint32_t i = 0; i < n; ++i) a->distance[i] = a->label_tmp[i] = INFTY;
    a->is_dirty = calloc(n, 1);
    a->is_dirty_tmp = calloc(n, 1);
    a->dirty = malloc(((size_t)n + 1) * sizeof(uint32_t));
    a->dirty_tmp = malloc(((size_t)n + 1) * sizeof(uint32_t));
    a->ndirty = a->ndirty_tmp = 0;
}
static void ak_free(o_akiba *a) {
    oh_free(&a->q);
    free(a->distance);
    free(a->label_tmp);
    free(a->is_dirty);
    free(a->is_dirty_tmp);
    free(a->dirty);
    free(a->dirty_tmp);
}
static inline void ak_update(o_akiba *a, uint32_t v, int32_t d) {
    a->distance[v] = d;
    oh_update(&a->q, v, d);
    if (!a->is_dirty[v]) {
        a->dirty[a->ndirty++] = v;
        a->is_dirty[v] = 1;
    }
}
static inline void ak_update_tmp(o_akiba *a, uint32_t h, int32_t d) {
    a->label_tmp[h] = d;
    if (!a->is_dirty_tmp[h]) {
        a->dirty_tmp[a->ndirty_tmp++] = h;
        a->is_dirty_tmp[h] = 1;
    }
}
static void ak_clear(o_akiba *a) {
    oh_clear(&a->q);
    for (uint32_t i = 0; i < a->ndirty; ++i) {
        a->distance[a->dirty[i]] = INFTY;
        a->is_dirty[a->dirty[i]] = 0;
    }
    a->ndirty = 0;
    for (uint32_t i = 0; i < a->ndirty_tmp; ++i) {
        a->label_tmp[a->dirty_tmp[i]] = INFTY;
        a->is_dirty_tmp[a->dirty_tmp[i]] = 0;
    }
    a->ndirty_tmp = 0;
}

static inline void spin_lock(volatile uint8_t *l) {
    while (!__sync_bool_compare_and_swap(l, 0, 1)) {}
}
static inline void spin_unlock(volatile uint8_t *l) {
    __sync_synchronize();
    *l = 0;
}

/* Akiba::iteration_gll (shared_memory/akiba.hpp:65-125). */
/* glob_lim: only global entries with hub < glob_lim exist (UINT32_MAX in a
 * build; a replay reads a complete labeling as the committed state of an
 * earlier superstep). */
static uint32_t iteration_gll(o_akiba *a, const og_graph *g, uint32_t i, int forward,
                              volatile uint8_t *lck, const uint32_t *order, const uint32_t *rev,
                              const ol_labels *glob, ol_labels *loc, uint32_t glob_lim) {
    ak_clear(a);
    uint32_t v = order[i];
    uint32_t lcknum = (forward ? 1 : 0) + v * 2;
    uint32_t label_count = 0;
    ak_update(a, v, 0);
    spin_lock(&lck[lcknum]);
    {
        ol_list *x = &loc->l[2 * (size_t)v + forward];
        for (uint32_t k = 0; k < x->n; ++k) {
            if (x->h[k] > i) continue;
            ak_update_tmp(a, x->h[k], x->d[k]);
        }
    }
    spin_unlock(&lck[lcknum]);
    {
        const ol_list *x = &glob->l[2 * (size_t)v + forward];
        for (uint32_t k = 0; k < x->n && x->h[k] < glob_lim; ++k) ak_update_tmp(a, x->h[k], x->d[k]);
    }
    const int s = forward ? 1 : 0;
    while (a->q.size) {
        uint32_t u = oh_pop(&a->q);
        int32_t d = a->distance[u];
        if (rev[u] < i) continue;
        {
            const ol_list *x = &glob->l[2 * (size_t)u + !forward];
            for (uint32_t k = 0; k < x->n && x->h[k] < glob_lim; ++k) {
                uint32_t hub = x->h[k];
                if (hub > i) continue;
                if (a->label_tmp[hub] != INFTY && a->label_tmp[hub] + x->d[k] <= d) goto pruned;
            }
        }
        lcknum = (forward ? 0 : 1) + u * 2;
        spin_lock(&lck[lcknum]);
        {
            ol_list *x = &loc->l[2 * (size_t)u + !forward];
            for (uint32_t k = 0; k < x->n; ++k) {
                uint32_t hub = x->h[k];
                if (hub > i) continue;
                if (a->label_tmp[hub] != INFTY && a->label_tmp[hub] + x->d[k] <= d) {
                    spin_unlock(&lck[lcknum]);
                    goto pruned;
                }
            }
            ol_push(x, i, d);
        }
        spin_unlock(&lck[lcknum]);
        label_count++;
        for (uint64_t e = g->off[s][u]; e < g->off[s][u + 1]; ++e) {
            int32_t dd = d + g->len[s][e];
            uint32_t w = g->head[s][e];
            if (dd < a->distance[w]) ak_update(a, w, dd);
        }
    pruned:;
    }
    return label_count;
}

typedef struct {
    uint32_t h;
    int32_t d;
} o_pair;
static int cmp_pair(const void *pa, const void *pb) {
    const o_pair *x = pa, *y = pb;
    if (x->h != y->h) return x->h < y->h ? -1 : 1;
    if (x->d != y->d) return x->d < y->d ? -1 : 1;
    return 0;
}

/* Labeling::clean_cover (shared_memory/labeling.hpp:78-88) */
static int clean_cover(const ol_labels *L, uint32_t u, uint32_t v, int f, int32_t d, uint32_t hub_order) {
    const ol_list *a = &L->l[2 * (size_t)u + f], *b = &L->l[2 * (size_t)v + !f];
    uint32_t i = 0, j = 0;
    while (i < a->n && j < b->n) {
        if (a->h[i] >= hub_order || b->h[j] >= hub_order) return 0;
        if (a->h[i] == b->h[j]) {
            if (d >= a->d[i++] + b->d[j++]) return 1;
        } else if (a->h[i] < b->h[j]) {
            ++i;
        } else {
            ++j;
        }
    }
    return 0;
}

/* run_paraPLL (shared_memory/akiba.hpp:132-217): supersteps of label_limit
 * labels, sort, clean, append to the global labeling.  Returns the labels;
 * *secs gets the reference's "total time" (labeling + sort + clean). */
ol_labels *og_gll_steps(const og_graph *g, const uint32_t *order, uint32_t N, int threads,
                        uint64_t label_limit, double *secs, uint32_t max_steps, uint32_t *nsteps,
                        uint32_t *step_end, double *step_secs);

ol_labels *og_gll(const og_graph *g, const uint32_t *order, uint32_t N, int threads,
                  uint64_t label_limit, double *secs) {
    return og_gll_steps(g, order, N, threads, label_limit, secs, 0, NULL, NULL, NULL);
}

/* The same build, recording its supersteps: superstep k covers the roots
 * [step_end[k-1], step_end[k]) (step_end[-1] = 0) and took step_secs[k]
 * (labeling + sort + clean); at most max_steps are recorded, *nsteps gets
 * the count (which may exceed max_steps). */
ol_labels *og_gll_steps(const og_graph *g, const uint32_t *order, uint32_t N, int threads,
                        uint64_t label_limit, double *secs, uint32_t max_steps, uint32_t *nsteps,
                        uint32_t *step_end, double *step_secs) {
    ol_labels *glob = ol_new(N), *loc = ol_new(N);
    volatile uint8_t *lck = calloc(2 * (size_t)N + 2, 1);
    uint32_t *rev = malloc((size_t)N * sizeof(uint32_t));
    for (uint32_t i = 0; i < N; ++i) rev[order[i]] = i;
    o_akiba *ak = malloc(sizeof(o_akiba) * threads);
    for (int t = 0; t < threads; ++t) ak_init(&ak[t], g->n);
    double lt = 0, st = 0, ct = 0;
    uint32_t cnt = 0;
    if (nsteps) *nsteps = 0;
    while (cnt < 2 * N) {
        uint64_t label_sum = 0;
        ol_clear(loc);
        double ls = omp_get_wtime();
#pragma omp parallel for num_threads(threads) schedule(static, 1)
        for (int th = 0; th < threads; ++th) {
            uint64_t label_sum_thread = 0;
            while (1) {
                uint32_t r = __sync_fetch_and_add(&cnt, 2);
                if (r >= 2 * N) {
                    __sync_fetch_and_add(&label_sum, label_sum_thread);
                    break;
                }
                uint32_t root = r / 2;
                int side = (r % 2) == 1;
                label_sum_thread += iteration_gll(&ak[th], g, root, side, lck, order, rev, glob, loc, UINT32_MAX);
                side = (r % 2) == 0;
                label_sum_thread += iteration_gll(&ak[th], g, root, side, lck, order, rev, glob, loc, UINT32_MAX);
                if (label_sum_thread > N / 32) {
                    if (__sync_fetch_and_add(&label_sum, label_sum_thread) >= label_limit - label_sum_thread)
                        break;
                    label_sum_thread = 0;
                }
            }
        }
        double le = omp_get_wtime();
        lt += le - ls;
        /* Labeling::sort (shared_memory/labeling.hpp:222-256) */
#pragma omp parallel num_threads(threads)
        {
            o_pair *tmp = NULL;
            uint32_t tcap = 0;
#pragma omp for schedule(dynamic, 64)
            for (long long x = 0; x < 2 * (long long)N; ++x) {
                ol_list *l = &loc->l[x];
                if (l->n < 2) continue;
                if (l->n > tcap) {
                    tcap = l->n;
                    tmp = realloc(tmp, tcap * sizeof(o_pair));
                }
                for (uint32_t k = 0; k < l->n; ++k) tmp[k] = (o_pair){l->h[k], l->d[k]};
                qsort(tmp, l->n, sizeof(o_pair), cmp_pair);
                for (uint32_t k = 0; k < l->n; ++k) {
                    l->h[k] = tmp[k].h;
                    l->d[k] = tmp[k].d;
                }
            }
            free(tmp);
        }
        double se = omp_get_wtime();
        st += se - le;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 64)
        for (long long vi = 0; vi < (long long)N; ++vi) {
            for (int side = 0; side < 2; ++side) {
                ol_list *l = &loc->l[2 * vi + side];
                for (uint32_t k = 0; k < l->n; ++k) {
                    uint32_t hub_order = l->h[k];
                    uint32_t hub = order[hub_order];
                    int32_t hd = l->d[k];
                    if (!clean_cover(loc, (uint32_t)vi, hub, side, hd, hub_order))
                        ol_push(&glob->l[2 * vi + side], hub_order, hd);
                }
            }
        }
        const double ce = omp_get_wtime();
        ct += ce - se;
        if (nsteps) {
            if (*nsteps < max_steps) {
                step_end[*nsteps] = cnt / 2 < N ? cnt / 2 : N;
                step_secs[*nsteps] = ce - ls;
            }
            ++*nsteps;
        }
    }
    if (secs) *secs = lt + st + ct;
    for (int t = 0; t < threads; ++t) ak_free(&ak[t]);
    free(ak);
    free(rev);
    free((void *)lck);
    ol_free(loc);
    return glob;
}

/* Sequential PLL trace: the work model of the build roofline.  Roots in
 * rank order, one at a time, both sides as iteration_gll does them
 * (shared_memory/akiba.hpp:65-125), every label committed at once, so each
 * tree prunes with the complete labels of all higher-ranked hubs.  Counts
 * what this sequential algorithm reads and writes:
 *   out[0] settled vertices (popped with rank >= i)
 *   out[1] label entries scanned by prune tests (up to the first witness)
 *   out[2] arcs relaxed (out-arcs of the unpruned vertices)
 *   out[3] labels written
 *   out[4] algorithmic bytes = 8 * (out[1] + out[2] + out[3])
 *   out[5] whole lists of the settled vertices (sum of |L_<i(u, !f)|)
 *   out[6] out-arcs of the settled vertices
 *   out[7] the build roofline's bytes: 8 * (out[5] + out[6] + out[3])
 * The labels are the canonical labels (the same as og_gll's). */
void og_pll_trace(const og_graph *g, const uint32_t *order, uint32_t N, uint64_t *out) {
    ol_labels *L = ol_new(N);
    uint32_t *rev = malloc((size_t)N * sizeof(uint32_t));
    for (uint32_t i = 0; i < N; ++i) rev[order[i]] = i;
    o_akiba ak;
    ak_init(&ak, g->n);
    uint64_t settled = 0, reads = 0, arcs = 0, labels = 0, lists = 0, outdeg = 0;
    for (uint32_t i = 0; i < N; ++i) {
        const uint32_t v = order[i];
        for (int forward = 0; forward < 2; ++forward) {
            const int s = forward ? 1 : 0;
            ak_clear(&ak);
            ak_update(&ak, v, 0);
            {
                const ol_list *x = &L->l[2 * (size_t)v + forward];
                for (uint32_t k = 0; k < x->n; ++k) ak_update_tmp(&ak, x->h[k], x->d[k]);
            }
            while (ak.q.size) {
                const uint32_t u = oh_pop(&ak.q);
                const int32_t d = ak.distance[u];
                if (rev[u] < i) continue;
                ++settled;
                ol_list *x = &L->l[2 * (size_t)u + !forward];
                lists += x->n;
                outdeg += g->off[s][u + 1] - g->off[s][u];
                int pruned = 0;
                for (uint32_t k = 0; k < x->n; ++k) {
                    ++reads;
                    const uint32_t hub = x->h[k];
                    if (ak.label_tmp[hub] != INFTY && ak.label_tmp[hub] + x->d[k] <= d) {
                        pruned = 1;
                        break;
                    }
                }
                if (pruned) continue;
                ol_push(x, i, d);
                ++labels;
                for (uint64_t e = g->off[s][u]; e < g->off[s][u + 1]; ++e) {
                    ++arcs;
                    const int32_t dd = d + g->len[s][e];
                    const uint32_t w = g->head[s][e];
                    if (dd < ak.distance[w]) ak_update(&ak, w, dd);
                }
            }
        }
    }
    out[0] = settled;
    out[1] = reads;
    out[2] = arcs;
    out[3] = labels;
    out[4] = 8 * (reads + arcs + labels);
    out[5] = lists;
    out[6] = outdeg;
    out[7] = 8 * (lists + outdeg + labels);
    ak_free(&ak);
    free(rev);
    ol_free(L);
}

/* ------------------------------------------------- superstep replay */
/* Re-runs roots [r_begin, r_end) of one superstep of og_gll_steps with the
 * state that superstep had: the committed labels are the complete labeling's
 * entries with hub < s_begin (the superstep's first root: labels of
 * committed hubs are final, and the complete labeling holds exactly them),
 * the local labels start empty; then Labeling::sort and the clean pass
 * (shared_memory/akiba.hpp:152-208) over the replayed roots' labels.  The
 * CPU baseline times replays of sampled root ranges of every superstep to
 * estimate a whole build's time without re-running it. */
typedef struct {
    const og_graph *g;
    const uint32_t *order;
    uint32_t N;
    int threads;
    const ol_labels *complete;
    ol_labels *loc;
    ol_labels *sink;   /* receives the kept labels, as the global labeling does */
    volatile uint8_t *lck;
    uint32_t *rev;
    o_akiba *ak;
} og_replay;

og_replay *og_replay_new(const og_graph *g, const uint32_t *order, uint32_t N, int threads,
                         const ol_labels *complete) {
    og_replay *c = calloc(1, sizeof(og_replay));
    c->g = g;
    c->order = order;
    c->N = N;
    c->threads = threads;
    c->complete = complete;
    c->loc = ol_new(N);
    c->sink = ol_new(N);
    c->lck = calloc(2 * (size_t)N + 2, 1);
    c->rev = malloc((size_t)N * sizeof(uint32_t));
    for (uint32_t i = 0; i < N; ++i) c->rev[order[i]] = i;
    c->ak = malloc(sizeof(o_akiba) * threads);
    for (int t = 0; t < threads; ++t) ak_init(&c->ak[t], g->n);
    return c;
}

void og_replay_free(og_replay *c) {
    if (!c) return;
    for (int t = 0; t < c->threads; ++t) ak_free(&c->ak[t]);
    free(c->ak);
    free(c->rev);
    free((void *)c->lck);
    ol_free(c->loc);
    ol_free(c->sink);
    free(c);
}

/* Labels kept by the clean pass; *secs = labeling + sort + clean time. */
uint64_t og_replay_run(og_replay *c, uint32_t s_begin, uint32_t r_begin, uint32_t r_end, double *secs) {
    const uint32_t N = c->N;
    const int threads = c->threads;
    ol_labels *loc = c->loc;
    ol_clear(loc);
    /* the kept labels are appended to the sink's lists, emptied but with
     * their capacity kept from earlier replays (as a running build's global
     * lists keep theirs) */
    ol_clear(c->sink);
    uint32_t cnt = 2 * r_begin;
    const uint32_t lim = 2 * (r_end < N ? r_end : N);
    const double t0 = omp_get_wtime();
#pragma omp parallel for num_threads(threads) schedule(static, 1)
    for (int th = 0; th < threads; ++th) {
        while (1) {
            uint32_t r = __sync_fetch_and_add(&cnt, 2);
            if (r >= lim) break;
            uint32_t root = r / 2;
            iteration_gll(&c->ak[th], c->g, root, 0, c->lck, c->order, c->rev, c->complete, loc, s_begin);
            iteration_gll(&c->ak[th], c->g, root, 1, c->lck, c->order, c->rev, c->complete, loc, s_begin);
        }
    }
#pragma omp parallel num_threads(threads)
    {
        o_pair *tmp = NULL;
        uint32_t tcap = 0;
#pragma omp for schedule(dynamic, 64)
        for (long long x = 0; x < 2 * (long long)N; ++x) {
            ol_list *l = &loc->l[x];
            if (l->n < 2) continue;
            if (l->n > tcap) {
                tcap = l->n;
                tmp = realloc(tmp, tcap * sizeof(o_pair));
            }
            for (uint32_t k = 0; k < l->n; ++k) tmp[k] = (o_pair){l->h[k], l->d[k]};
            qsort(tmp, l->n, sizeof(o_pair), cmp_pair);
            for (uint32_t k = 0; k < l->n; ++k) {
                l->h[k] = tmp[k].h;
                l->d[k] = tmp[k].d;
            }
        }
        free(tmp);
    }
    uint64_t kept = 0;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 64) reduction(+ : kept)
    for (long long vi = 0; vi < (long long)N; ++vi)
        for (int side = 0; side < 2; ++side) {
            const ol_list *l = &loc->l[2 * vi + side];
            for (uint32_t k = 0; k < l->n; ++k)
                if (!clean_cover(loc, (uint32_t)vi, c->order[l->h[k]], side, l->d[k], l->h[k])) {
                    ol_push(&c->sink->l[2 * vi + side], l->h[k], l->d[k]);
                    kept++;
                }
        }
    if (secs) *secs = omp_get_wtime() - t0;
    return kept;
}

/* ------------------------------------------------------------ PLaNT */

/* Akiba::plant (distributed_memory/akiba.hpp:52-104) without common-label
 * pruning, with BasicDijkstra::update_wo_prune's tie rule
 * (distributed_memory/dijkstra.hpp:56-78).  parent[] holds 1 for "no
 * higher-ranked vertex on the path", 0 for "via hub", UINT32_MAX unseen.
 * Appends labels to L (side !forward of each labelled vertex); returns the
 * label count, *tree_size the popped count. */
static uint32_t plant_tree(o_akiba *a, uint32_t *parent, const og_graph *g, uint32_t i, int forward,
                           const uint32_t *order, const uint32_t *rev, ol_labels *L, uint32_t *tree_size) {
    ak_clear(a);
    for (uint32_t k = 0; k < a->ndirty; ++k) parent[a->dirty[k]] = UINT32_MAX;
    uint32_t v = order[i];
    uint32_t label_count = 0, tsize = 0;
    int64_t queue_left = 1;
    ak_update(a, v, 0);
    parent[v] = 1;
    const int s = forward ? 1 : 0;
    while (a->q.size) {
        uint32_t u = oh_pop(&a->q);
        tsize++;
        int via_hub = parent[u] == 0 || rev[u] < i;
        if (!via_hub) queue_left--;
        int32_t d = a->distance[u];
        if (!via_hub) {
            ol_push(&L->l[2 * (size_t)u + !forward], i, d);
            label_count++;
        }
        for (uint64_t e = g->off[s][u]; e < g->off[s][u + 1]; ++e) {
            int32_t dd = d + g->len[s][e];
            uint32_t w = g->head[s][e];
            uint32_t p = (via_hub || rev[w] < i) ? 0 : 1;
            if (dd <= a->distance[w]) {
                /* update_wo_prune */
                int32_t prev = a->distance[w];
                uint32_t pp = parent[w];
                if (dd < prev) {
                    ak_update(a, w, dd);
                    parent[w] = p;
                    if (pp != 1 && p == 1) queue_left++;
                    else if (pp == 1 && p == 0) queue_left--;
                } else if (pp == 1 && p == 0) {
                    parent[w] = 0;
                    queue_left--;
                }
            }
        }
        if (queue_left == 0) break;
    }
    /* reset parent flags of everything touched */
    for (uint32_t k = 0; k < a->ndirty; ++k) parent[a->dirty[k]] = UINT32_MAX;
    *tree_size = tsize;
    return label_count;
}

/* PLaNT over every root, both sides (labels exact, no cleaning), then
 * Labeling::sort.  tree_sizes/label_counts (optional, n entries) receive the
 * per-root sums over both sides, as run() uses for the phase switch
 * (distributed_memory/akiba.hpp:291-297). */
ol_labels *og_plant_all(const og_graph *g, const uint32_t *order, uint32_t N, uint32_t *tree_sizes,
                        uint32_t *label_counts) {
    ol_labels *L = ol_new(N);
    uint32_t *rev = malloc((size_t)N * sizeof(uint32_t));
    for (uint32_t i = 0; i < N; ++i) rev[order[i]] = i;
    o_akiba a;
    ak_init(&a, g->n);
    uint32_t *parent = malloc((size_t)g->n * sizeof(uint32_t));
    for (uint32_t k = 0; k < g->n; ++k) parent[k] = UINT32_MAX;
    for (uint32_t i = 0; i < N; ++i) {
        uint32_t t1 = 0, t2 = 0;
        uint32_t l1 = plant_tree(&a, parent, g, i, 1, order, rev, L, &t1);
        uint32_t l2 = plant_tree(&a, parent, g, i, 0, order, rev, L, &t2);
        if (tree_sizes) tree_sizes[i] = t1 + t2;
        if (label_counts) label_counts[i] = l1 + l2;
    }
    ak_free(&a);
    free(parent);
    free(rev);
    return L;   /* lists are already ascending: roots are taken in rank order */
}

/* --------------------------------------------------- canonical checker */

/* Brute force check of the canonical labeling definition on a small graph:
 * (rank(h), d) in L(v, side) iff no vertex w with rank(w) < rank(h) lies on
 * a shortest path between v and h (side 1: v -> h, side 0: h -> v), and d is
 * that distance.  Returns the number of mismatching (v, side, h) triples. */
uint64_t og_canonical_check(const og_graph *g, const uint32_t *order, const ol_labels *L) {
    const uint32_t n = g->n;
    int32_t *D = malloc((size_t)n * n * sizeof(int32_t));   /* D[a*n+b] = d(a -> b) */
    for (uint32_t a = 0; a < n; ++a) og_dijkstra(g, a, 1, D + (size_t)a * n);
    uint32_t *rev = malloc((size_t)n * sizeof(uint32_t));
    for (uint32_t i = 0; i < n; ++i) rev[order[i]] = i;
    uint64_t bad = 0;
    int32_t *expect = malloc((size_t)n * sizeof(int32_t));
    for (uint32_t v = 0; v < n; ++v)
        for (int side = 0; side < 2; ++side) {
            for (uint32_t r = 0; r < n; ++r) expect[r] = -1;
            for (uint32_t r = 0; r < n; ++r) {
                uint32_t h = order[r];
                int32_t dvh = side ? D[(size_t)v * n + h] : D[(size_t)h * n + v];
                if (dvh == INFTY) continue;
                int ok = 1;
                for (uint32_t w = 0; w < n && ok; ++w) {
                    if (rev[w] >= r) continue;
                    int32_t a1 = side ? D[(size_t)v * n + w] : D[(size_t)h * n + w];
                    int32_t a2 = side ? D[(size_t)w * n + h] : D[(size_t)w * n + v];
                    if (a1 != INFTY && a2 != INFTY && (int64_t)a1 + a2 == dvh) ok = 0;
                }
                if (ok) expect[r] = dvh;
            }
            const ol_list *x = &L->l[2 * (size_t)v + side];
            uint32_t k = 0;
            for (uint32_t r = 0; r < n; ++r) {
                int has = k < x->n && x->h[k] == r;
                if (expect[r] >= 0) {
                    if (!has || x->d[k] != expect[r]) bad++;
                } else if (has) {
                    bad++;
                }
                if (has) k++;
            }
        }
    free(expect);
    free(rev);
    free(D);
    return bad;
}

/* ------------------------------------------------------------ orders */

static inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static inline uint64_t tie_key(uint64_t seed, uint32_t v) {
    return mix64(seed * 0x9E3779B97F4A7C15ull + (uint64_t)v);
}

typedef struct {
    uint64_t k1, k2;
    uint32_t v;
} o_okey;
static int cmp_okey(const void *pa, const void *pb) {
    const o_okey *x = pa, *y = pb;
    if (x->k1 != y->k1) return x->k1 > y->k1 ? -1 : 1;   /* primary key descending */
    if (x->k2 != y->k2) return x->k2 < y->k2 ? -1 : 1;   /* tie key ascending */
    return x->v < y->v ? -1 : (x->v > y->v);
}

/* Degree order: Graph::get_degree(v) (shared_memory/graph.hpp:324) descending,
 * ties by the seeded permutation tie_key(seed, v) ascending. */
void og_degree_order(const og_graph *g, uint64_t seed, uint32_t *order) {
    o_okey *k = malloc((size_t)g->n * sizeof(o_okey));
    for (uint32_t v = 0; v < g->n; ++v) {
        uint64_t deg = (g->off[1][v + 1] - g->off[1][v]) + (g->off[0][v + 1] - g->off[0][v]);
        k[v] = (o_okey){deg, tie_key(seed, v), v};
    }
    qsort(k, g->n, sizeof(o_okey), cmp_okey);
    for (uint32_t i = 0; i < g->n; ++i) order[i] = k[i].v;
    free(k);
}

/* Sources of the sampled betweenness: draws mix64(seed + j) % n, j = 0, 1,
 * ..., skipping repeats, until `count` distinct vertices. */
void og_bc_sources(uint32_t n, uint32_t count, uint64_t seed, uint32_t *src) {
    uint8_t *seen = calloc(n, 1);
    uint32_t c = 0;
    for (uint64_t j = 0; c < count && c < n; ++j) {
        uint32_t s = (uint32_t)(mix64(seed + j) % n);
        if (seen[s]) continue;
        seen[s] = 1;
        src[c++] = s;
    }
    free(seen);
}

/* Brandes dependencies from each source over forward shortest paths, with
 * a fixed summation order: sigma[w] sums its in-arc predecessors in
 * in-adjacency order; delta[v] sums its out-arc successors in out-adjacency
 * order; bc[v] adds sources in list order.  All in binary64 without fused
 * multiply-add, so a GPU restatement can match it bit for bit. */
typedef struct {
    int32_t *dist;
    double *sigma, *delta;
    uint32_t *seq;
    uint32_t ns;
    oh_heap h;
} og_bc_ws;

/* Dependencies delta_s[v] of one source s (forward shortest paths). */
static void bc_one(const og_graph *g, uint32_t s, og_bc_ws *w) {
    const uint32_t n = g->n;
    int32_t *dist = w->dist;
    double *sigma = w->sigma, *delta = w->delta;
    uint32_t *seq = w->seq;
    for (uint32_t v = 0; v < n; ++v) dist[v] = INFTY;
    dist[s] = 0;
    oh_update(&w->h, s, 0);
    uint32_t ns = 0;
    while (w->h.size) {
        uint32_t u = oh_pop(&w->h);
        seq[ns++] = u;
        for (uint64_t e = g->off[1][u]; e < g->off[1][u + 1]; ++e) {
            int32_t dd = dist[u] + g->len[1][e];
            uint32_t x = g->head[1][e];
            if (dd < dist[x]) {
                dist[x] = dd;
                oh_update(&w->h, x, dd);
            }
        }
    }
    for (uint32_t k = 0; k < ns; ++k) {
        uint32_t x = seq[k];
        if (x == s) {
            sigma[x] = 1.0;
            continue;
        }
        double acc = 0.0;
        for (uint64_t e = g->off[0][x]; e < g->off[0][x + 1]; ++e) {
            uint32_t u = g->head[0][e];
            if (dist[u] != INFTY && dist[u] + g->len[0][e] == dist[x]) acc = acc + sigma[u];
        }
        sigma[x] = acc;
    }
    for (uint32_t k = ns; k-- > 0;) {
        uint32_t v = seq[k];
        double acc = 0.0;
        for (uint64_t e = g->off[1][v]; e < g->off[1][v + 1]; ++e) {
            uint32_t x = g->head[1][e];
            if (dist[x] != INFTY && dist[v] + g->len[1][e] == dist[x]) {
                double q = sigma[v] / sigma[x];
                double t = 1.0 + delta[x];
                acc = acc + q * t;
            }
        }
        delta[v] = acc;
    }
    w->ns = ns;
}

/* Brandes dependencies from each source over forward shortest paths, with
 * a fixed summation order: sigma[w] sums its in-arc predecessors in
 * in-adjacency order; delta[v] sums its out-arc successors in out-adjacency
 * order; bc[v] adds sources in list order.  All in binary64 without fused
 * multiply-add, so a GPU restatement can match it bit for bit.  Sources run
 * in parallel in groups of `threads`; their dependencies are added to bc in
 * source order, so the result does not depend on the thread count. */
void og_betweenness(const og_graph *g, const uint32_t *src, uint32_t count, double *bc) {
    const uint32_t n = g->n;
    int threads = omp_get_max_threads();
    if (threads < 1) threads = 1;
    if ((uint32_t)threads > count && count > 0) threads = (int)count;
    og_bc_ws *ws = calloc((size_t)threads, sizeof(og_bc_ws));
    for (int t = 0; t < threads; ++t) {
        ws[t].dist = malloc((size_t)n * sizeof(int32_t));
        ws[t].sigma = malloc((size_t)n * sizeof(double));
        ws[t].delta = malloc((size_t)n * sizeof(double));
        ws[t].seq = malloc((size_t)n * sizeof(uint32_t));
        oh_init(&ws[t].h, n);
    }
    for (uint32_t v = 0; v < n; ++v) bc[v] = 0.0;
    for (uint32_t j0 = 0; j0 < count; j0 += (uint32_t)threads) {
        const int cnt = (int)((count - j0) < (uint32_t)threads ? (count - j0) : (uint32_t)threads);
#pragma omp parallel for num_threads(cnt) schedule(static, 1)
        for (int t = 0; t < cnt; ++t) bc_one(g, src[j0 + (uint32_t)t], &ws[t]);
        for (int t = 0; t < cnt; ++t) {
            const uint32_t s = src[j0 + (uint32_t)t];
            const uint32_t *seq = ws[t].seq;
            const double *delta = ws[t].delta;
            const int64_t ns = ws[t].ns;
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < ns; ++k) {
                const uint32_t v = seq[k];
                if (v != s) bc[v] = bc[v] + delta[v];
            }
        }
    }
    for (int t = 0; t < threads; ++t) {
        oh_free(&ws[t].h);
        free(ws[t].dist);
        free(ws[t].sigma);
        free(ws[t].delta);
        free(ws[t].seq);
    }
    free(ws);
}

/* Betweenness order: bc descending, ties by tie_key(seed, v) ascending. */
void og_betweenness_order(const og_graph *g, uint32_t count, uint64_t seed, uint32_t *order) {
    const uint32_t n = g->n;
    uint32_t *src = malloc((size_t)(count ? count : 1) * sizeof(uint32_t));
    if (count > n) count = n;
    og_bc_sources(n, count, seed, src);
    double *bc = malloc((size_t)n * sizeof(double));
    og_betweenness(g, src, count, bc);
    o_okey *k = malloc((size_t)n * sizeof(o_okey));
    for (uint32_t v = 0; v < n; ++v) {
        uint64_t bits;
        memcpy(&bits, &bc[v], 8);   /* non-negative doubles order as integers */
        k[v] = (o_okey){bits, tie_key(seed, v), v};
    }
    qsort(k, n, sizeof(o_okey), cmp_okey);
    for (uint32_t i = 0; i < n; ++i) order[i] = k[i].v;
    free(k);
    free(bc);
    free(src);
}
