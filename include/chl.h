/*
 * chl.h - C ABI of the GB300 canonical hub labeling (CHL) engine.
 *
 * The reference (qingdo/plant) exposes its construction and query path as a
 * header-only C++ API in namespace `hl` plus the `hhl` command line.  Every
 * entry point below replaces one piece of that API; the comment above each
 * one names the reference interface it stands in for (file:line, relative to
 * the reference project root).
 *
 * Conventions
 *  - Every function returns an int status (CHL_OK on success).  No function
 *    calls exit() or abort(); bad input is reported as CHL_ERR_FORMAT or
 *    CHL_ERR_INVALID, unreadable files as CHL_ERR_IO.
 *  - Vertex ids are uint32, 0-based.  Hubs stored in labels are RANKS (the
 *    position of the hub vertex in the order), exactly as in the reference's
 *    label file.  Distances are non-negative int32; "no path" is reported as
 *    CHL_INFTY (2147483647), the reference's `infty`.
 *  - Handles are opaque and owned by the caller; free them with chl_*_free.
 *    Mutating calls on one handle must not run concurrently.
 *    chl_query_batch may run concurrently on distinct streams.
 *  - The engine runs on the current CUDA device.  There is no CPU fallback:
 *    if no device is usable, GPU entry points return CHL_ERR_CUDA.
 */
#ifndef CHL_H
#define CHL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CHL_INFTY 2147483647

enum chl_status {
    CHL_OK = 0,
    CHL_ERR_IO = 1,       /* file cannot be opened / read / written          */
    CHL_ERR_FORMAT = 2,   /* no parser accepts the file                      */
    CHL_ERR_OOM = 3,      /* host or device allocation failed                */
    CHL_ERR_TIMEOUT = 4,  /* a bounded device wait gave up                   */
    CHL_ERR_INVALID = 5,  /* bad argument (null, out of range, inconsistent) */
    CHL_ERR_CUDA = 6      /* a CUDA runtime call failed / no device          */
};

typedef struct chl_graph chl_graph;
typedef struct chl_labels chl_labels;
typedef struct chl_server chl_server;
typedef struct chl_gnn chl_gnn;

/* Human-readable text for a status code (static storage). */
const char *chl_status_str(int status);
/* Text of the last CUDA / device-side error seen by this thread. */
const char *chl_last_error(void);

/* ------------------------------------------------------------------ graph */

/* Replaces hl::Graph::read(char*, bool undirected)
 * (shared_memory/graph.hpp:327-335): tries DIMACS, METIS, SNAP, then the
 * `u v w` edge list, with the same acceptance rules, and builds adjacency
 * with the same duplicate / direction merge as Graph::init_arcs
 * (shared_memory/graph.hpp:103-153). */
int chl_graph_load(const char *path, int undirected, chl_graph **out);

/* Replaces hl::Graph::read (shared_memory/graph.hpp:327-335) like
 * chl_graph_load, with DIMACS, SNAP and edge-list files parsed and their arc
 * lists built on the GPU (the reference's line rules and init_arcs, :168-189,
 * :262-282, :284-308 and :103-153; the host picks the reader the reference
 * would end up with).  Files those rules reject, and METIS files, go through
 * the host parsers.  *parsed_on_gpu (may be NULL) tells which path ran. */
int chl_graph_load_gpu(const char *path, int undirected, chl_graph **out,
                       int *parsed_on_gpu);
/* Replaces hl::Graph::set_n + add_arc + finalize
 * (shared_memory/graph.hpp:349-353): builds a graph from k arcs
 * (src[i] -> dst[i], length len[i]); when `undirected` is non-zero every arc
 * is also added in the opposite direction, as add_tmp_arc does. */
int chl_graph_from_arcs(uint32_t n, size_t k, const uint32_t *src,
                        const uint32_t *dst, const int32_t *len,
                        int undirected, chl_graph **out);
/* The same from an out-arc CSR: the arcs of v are head[off[v] .. off[v+1])
 * with lengths len[...]; off has n + 1 non-decreasing entries from 0.  The
 * arc lists are the ones chl_graph_from_arcs builds from those arcs (the
 * init_arcs merge, shared_memory/graph.hpp:103-153). */
int chl_graph_from_csr(uint32_t n, const uint64_t *off, const uint32_t *head,
                       const int32_t *len, int undirected, chl_graph **out);

/* Replaces hl::Graph::write (shared_memory/graph.hpp:338-343) for the
 * forward arcs; used to hand generated graphs to other tools. */
int chl_graph_write_dimacs(const chl_graph *g, const char *path);

/* Replaces Graph::get_n / get_m (shared_memory/graph.hpp:313-314). */
uint32_t chl_graph_n(const chl_graph *g);
uint64_t chl_graph_m(const chl_graph *g);
/* Number of distinct forward (out) arcs after init_arcs merging. */
uint64_t chl_graph_out_arcs(const chl_graph *g);
/* 1 if the in-adjacency equals the out-adjacency (an undirected graph). */
int chl_graph_symmetric(const chl_graph *g);
/* Replaces Graph::get_degree(v) (shared_memory/graph.hpp:324): out + in. */
uint32_t chl_graph_degree(const chl_graph *g, uint32_t v);
/* Copy out the adjacency of v in direction `forward` (1 = out-arcs, as
 * Graph::begin(v, true)); returns the count in *cnt.  heads/lens may be
 * NULL to query the count. */
int chl_graph_arcs(const chl_graph *g, uint32_t v, int forward,
                   uint32_t *heads, int32_t *lens, uint32_t cap,
                   uint32_t *cnt);
/* Per-vertex arc counts of one direction (forward = 1: out-arcs). */
int chl_graph_degrees(const chl_graph *g, int forward, uint32_t *deg);
/* Copy one direction's adjacency as CSR: off has n+1 entries; head/len
 * have chl_graph_out_arcs (forward) or the in-arc count entries; head/len
 * may be NULL. */
int chl_graph_export(const chl_graph *g, int forward, uint64_t *off, uint32_t *head,
                     int32_t *len);
/* Keep a device copy of the adjacency in the graph handle, so builds start
 * with their input resident in HBM (no counterpart: the reference is CPU
 * only).  chl_graph_free releases it. */
int chl_graph_to_device(chl_graph *g);
int chl_graph_release_device(chl_graph *g);
void chl_graph_free(chl_graph *g);

/* Seeded synthetic generators (no reference counterpart; they stand in for
 * the missing public datasets).  Both return an undirected graph built as
 * if its DIMACS file (both arc directions listed) had been read.
 *   grid: rows x cols 4-neighbour grid, `del_frac` of edges deleted, largest
 *         component kept, `diag_frac` x n diagonal shortcuts, lengths
 *         uniform in [wmin, wmax], plus `highways` long edges between
 *         vertices at most `hw_steps` grid steps apart with length
 *         round(hw_factor x Manhattan distance).
 *   rmat: 2^scale vertices, ef * 2^scale edges drawn with quadrant
 *         probabilities (a, b, c, 1-a-b-c), symmetrised, self loops and
 *         duplicates removed, unit lengths. */
int chl_gen_grid(uint32_t rows, uint32_t cols, double del_frac,
                 double diag_frac, int32_t wmin, int32_t wmax,
                 uint32_t highways, uint32_t hw_steps, double hw_factor,
                 uint64_t seed, chl_graph **out);
int chl_gen_rmat(uint32_t scale, uint32_t ef, double a, double b, double c,
                 uint64_t seed, chl_graph **out);

/* ------------------------------------------------------------------ order */

/* Replaces hl::Order::read (shared_memory/ordering.hpp:52-67): first value
 * n, then n vertex ids; order[i] is the vertex of rank i.  *order is
 * allocated with malloc; free it with chl_order_free. */
int chl_order_load(const char *path, uint32_t **order, uint32_t *n);
/* Replaces hl::Order::write (shared_memory/ordering.hpp:37-49). */
int chl_order_write(const char *path, const uint32_t *order, uint32_t n);
void chl_order_free(uint32_t *order);

/* GPU plain orderings.  The reference takes its order from outside tools
 * (distributed_memory/degree.cpp:62-67 for degree; an external betweenness
 * tool for road graphs).  Both write n = chl_graph_n(g) entries to `order`.
 *   degree: degree descending, ties broken by a seeded random permutation.
 *   betweenness: Brandes dependencies summed over `sources` seeded source
 *   vertices (forward shortest paths), descending, same tie break. */
int chl_order_degree(const chl_graph *g, uint64_t seed, uint32_t *order);
int chl_order_betweenness(const chl_graph *g, uint32_t sources,
                          uint64_t seed, uint32_t *order);

/* ------------------------------------------------------------------ build */

enum chl_build_mode {
    CHL_MODE_HYBRID = 0, /* PLaNT trees until the tree/label ratio passes ps,
                            then pruned supersteps                       */
    CHL_MODE_GLL = 1,    /* pruned supersteps from the first root        */
    CHL_MODE_PLANT = 2   /* PLaNT trees only, pruned by committed labels */
};

typedef struct chl_build_opts {
    int32_t mode;         /* chl_build_mode                                  */
    double sf;            /* superstep label budget factor (hhl -s), 0 = auto
                             (32 on heavy-tailed graphs, 1024 otherwise)  */
    double ps;            /* phase switch ratio tree/label (hhl -ps), 0 =
                             auto: 1024 (the reference's default) on road-
                             like graphs, 8 on heavy-tailed ones          */
    int32_t autotune;     /* 1: schedule options left at 0 come from the
                             tuned-schedule table for the graph's class
                             (chl_graph_class; $CHL_SCHEDULES or
                             tuned_schedules.txt beside the library), the
                             rest from graph statistics                    */
    int32_t use_graphs;   /* 1: capture the per-superstep kernel chain in a
                             CUDA graph                                       */
    int32_t verbose;      /* 1: print the reference's summary line            */
    uint32_t first_superstep; /* roots in the first superstep, 0 = auto       */
    double growth;        /* superstep growth factor, 0 = auto                */
    uint32_t max_warps;   /* cap on concurrent trees, 0 = auto                */
    uint32_t root_limit;  /* > 0: build the trees of ranks < root_limit only
                             (the labels of those hubs, which are final;
                             used to time schedules on a prefix)            */
    int32_t superstep_extend; /* while a superstep's trees run, idle warps
                             take up to this many times its nominal roots
                             (0 auto: 4 on road-like graphs, off on heavy-
                             tailed ones; 1 off)                            */
    uint32_t label_cap;   /* new-label buffer entries per superstep: 0 auto
                             (the label budget plus sides * n per tree still
                             running when it is spent, within a quarter of
                             free memory).  A superstep that overflows it is
                             re-run with exactly the room it needed.        */
    int32_t queue_split;  /* near/far queue: 0 auto (road-like graphs: a
                             tree's queue above 1024 vertices is split, about
                             256 kept near; heavy-tailed ones: off), 1 off,
                             q > 1: split above q (about q / 4 near)        */
    uint32_t window_target; /* trees of a superstep with no committed labels
                             (the first) are searched label-correcting in
                             distance windows of about this many vertices:
                             0 auto (1024 on heavy-tailed graphs, off on
                             road-like ones), 1 off (batched settle rounds) */
    uint32_t window_warps; /* warps building one such tree: 0 auto (8 on
                             heavy-tailed graphs, else 4), 1, 2, 4 or 8     */
    uint32_t reserved[1];
} chl_build_opts;

/* Fill opts with the defaults (hybrid, sf auto, ps auto, autotune on,
 * commit chain captured in a CUDA graph). */
void chl_build_opts_default(chl_build_opts *opts);

typedef struct chl_build_stats {
    double build_ms;       /* device time of the whole build (CUDA events)  */
    double tree_ms;        /* tree kernels                                  */
    double sort_ms;        /* 0: the sort is timed within commit_ms         */
    double commit_ms;      /* sort, clean and merge of each superstep's new
                              labels into the committed label arrays      */
    double h2d_ms;         /* graph/order upload                            */
    uint64_t labels;       /* total label entries (both sides)              */
    uint64_t visits;       /* vertices settled over all trees               */
    uint64_t label_reads;  /* label entries read by prune tests             */
    uint64_t arcs;         /* arcs relaxed                                  */
    uint32_t supersteps;
    uint32_t plant_roots;  /* roots built as un-pruned PLaNT trees          */
    uint64_t tree_launches;
    uint64_t kernel_launches;
    double avg_label;
} chl_build_stats;

/* Replaces hl::run_paraPLL (shared_memory/akiba.hpp:132-217) and the hybrid
 * hl::run (distributed_memory/akiba.hpp:190-510): builds canonical labels of
 * g for `order` (n ranks, n must equal chl_graph_n(g)).  The result lives in
 * device memory. */
int chl_build(const chl_graph *g, const uint32_t *order, uint32_t n,
              const chl_build_opts *opts, chl_labels **out);
/* The graph's class in the tuned-schedule table (no reference counterpart):
 * "sym|dir-n2^<log2 n>-deg<mean out-degree>-skewheavy|flat", the key under
 * which plant_gb300/autotune.py stores the schedule it measured fastest for
 * graphs of that kind, and which chl_build with opts->autotune reads. */
int chl_graph_class(const chl_graph *g, char *buf, size_t cap);
/* Statistics of the build that produced `l`. */
int chl_build_get_stats(const chl_labels *l, chl_build_stats *stats);

/* ----------------------------------------------------------------- labels */

/* Replaces hl::Labeling::write (shared_memory/labeling.hpp:167-183):
 * byte-identical text layout. */
int chl_labels_write(const chl_labels *l, const char *path);
/* Replaces hl::Labeling::read (shared_memory/labeling.hpp:186-208); the
 * labels are uploaded to the device. */
int chl_labels_read(const char *path, chl_labels **out);
/* Binary CSR twin of the label file (no reference counterpart): header
 * "CHLLBL01", u32 n, u32 symmetric, u64 entries, u64 lists, then u64
 * offsets[lists + 1] and (u32 hub, u32 dist) entries, little-endian; lists
 * are v (symmetric) or 2v + side.  Streamed from / to device memory. */
int chl_labels_save(const chl_labels *l, const char *path);
/* Load a binary label file into device memory; CHL_ERR_FORMAT if the header,
 * offsets or lists (ascending hubs < n, distances >= 0) are invalid. */
int chl_labels_load(const char *path, chl_labels **out);
/* Replaces Labeling::get_avg (shared_memory/labeling.hpp:153-158). */
double chl_avg_label(const chl_labels *l);
uint32_t chl_labels_n(const chl_labels *l);
uint64_t chl_labels_total(const chl_labels *l);
/* Copy out L(v, side): hub ranks and distances, ascending by hub.  Either
 * array may be NULL to query the size in *cnt. */
int chl_labels_get(const chl_labels *l, uint32_t v, int side, uint32_t *hubs,
                   int32_t *dists, uint32_t cap, uint32_t *cnt);
/* sizes[2v+side] = |L(v, side)| (2n entries). */
int chl_labels_list_sizes(const chl_labels *l, uint32_t *sizes);
/* Copy all labels to host CSR arrays: off has 2n+1 entries (index 2v+side),
 * hubs/dists have chl_labels_total entries. */
int chl_labels_export(const chl_labels *l, uint64_t *off, uint32_t *hubs,
                      int32_t *dists);
/* Build a labels handle from host CSR arrays (same layout as export). */
int chl_labels_import(uint32_t n, const uint64_t *off, const uint32_t *hubs,
                      const int32_t *dists, chl_labels **out);
/* Per-vertex hub frequency: freq[v] = number of label entries (both sides)
 * whose hub is rank(v).  Training target of the learned ranking. */
int chl_labels_hub_freq(const chl_labels *l, const uint32_t *order,
                        uint32_t *freq);
/* Label digest (no counterpart in the reference): a position-dependent
 * 64-bit fingerprint, computed on the device, of the content that
 * hl::Labeling::write (shared_memory/labeling.hpp:167-183) puts in a label
 * file -- n, then every list 2v + side with its size and (hub, dist) entries
 * in order.  Each item adds one SplitMix64-mixed term modulo 2^64:
 *   M(n + C_N) + sum_i M(B_i ^ size_i) + sum_ij M(B_i ^ M(j + C_E) ^ (hub << 32 | dist)),
 *   B_i = M(i + C_L), C_N = 0x243F6A8885A308D3, C_L = 0x13198A2E03707344,
 *   C_E = 0xA4093822299F31D0, M(z) = the SplitMix64 finaliser.
 * Lets a caller compare a build with a reference labeling without writing
 * its many-GB text file. */
int chl_labels_digest(const chl_labels *l, uint64_t *digest);
void chl_labels_free(chl_labels *l);

/* ------------------------------------------------------------------ query */

/* Replaces hl::Labeling::query(u, v, f=true)
 * (shared_memory/labeling.hpp:56-65) over a batch, as batchLocalQuery does
 * (distributed_memory/query_funcs.hpp:23-30): out[i] = d(pairs[2i] ->
 * pairs[2i+1]), CHL_INFTY if the labels share no hub.  pairs/out are HOST
 * pointers (copied in and out on `stream`, a cudaStream_t or NULL). */
int chl_query_batch(const chl_labels *l, const uint32_t *pairs, size_t k,
                    int32_t *out, void *stream);
/* Allocation-free variant of chl_query_batch (no counterpart in the
 * reference).  For callers that cannot let a library allocate device memory:
 * processes whose HBM is already divided up by their own pool allocator, and
 * latency-critical request loops that cannot afford cudaMalloc/cudaFree and
 * their implicit synchronisation.  Same inputs, outputs and answers as
 * chl_query_batch, but the pairs and answers are staged through one
 * file-scope device array of CHL_NOALLOC_MAX_PAIRS pairs (12 MiB, held by
 * every GPU that loads the library until exit); larger k is rejected with
 * CHL_ERR_INVALID.  The labels must already be resident on the device (any
 * build, chl_query_batch or chl_server_create makes them so), else
 * CHL_ERR_INVALID.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress); make that first call before any stream
 * capture.  All calls share the array: calls whose work overlaps on the GPU
 * race.  Synchronises `stream` before returning. */
#define CHL_NOALLOC_MAX_PAIRS (1u << 20)
int chl_query_batch_noalloc(const chl_labels *l, const uint32_t *pairs, size_t k,
                            int32_t *out, void *stream);
/* Same, with DEVICE pointers; returns after the launch (asynchronous). */
int chl_query_batch_device(const chl_labels *l, const uint32_t *d_pairs,
                           size_t k, int32_t *d_out, void *stream);
/* Device-resident query benchmark (no reference counterpart): k uniform
 * pairs generated on the device (hot > 0: each pair drawn from a fixed set
 * of `hot` seeded pairs), `iters` timed launches of the batch query kernel
 * (CUDA events on its own stream); returns the mean ms per launch and the
 * algorithmic bytes of one launch (8 B per label entry of both lists, plus
 * the 8-byte pair and 4-byte answer). */
int chl_query_bench(const chl_labels *l, size_t k, uint64_t seed, int iters, uint32_t hot,
                    double *ms_per_iter, uint64_t *bytes_per_iter);
/* Replaces hl::generate_query (distributed_memory/query.hpp:43-51) with a
 * seeded generator: k uniform pairs over [0, range). */
int chl_query_generate(uint32_t *pairs, size_t k, uint32_t range,
                       uint64_t seed);
/* Replaces hl::load_query (distributed_memory/query.hpp:18-32): `u v` per
 * line.  *pairs is malloc'ed (free with chl_order_free). */
int chl_query_load(const char *path, uint32_t **pairs, size_t *k);

/* ----------------------------------------------------------------- server */

/* Continuous-batching query server (no reference counterpart; its
 * single-node limit is query mode 1, distributed_memory/query.hpp:82-91).
 * Requests are admitted while slots and device memory allow, merged into
 * one launch per cycle, and completed asynchronously. */
typedef struct chl_server_opts {
    uint32_t max_inflight_pairs; /* device slots for pairs (admission bound) */
    uint32_t max_requests;       /* request table size                       */
    uint32_t max_batch_pairs;    /* pairs merged into one launch             */
    uint32_t reserved[5];
} chl_server_opts;

void chl_server_opts_default(chl_server_opts *opts);
int chl_server_create(const chl_labels *l, const chl_server_opts *opts,
                      chl_server **out);
/* Submit k pairs (host memory, copied at admission).  Returns CHL_OK and a
 * request id, or CHL_ERR_OOM if the request can never fit. Blocks while the
 * server is full: admitted pairs that are not yet answered hold 12 bytes of
 * staging each, up to max_inflight_pairs, and unclaimed requests hold one of
 * max_requests entries.  A request's pairs are released as soon as its
 * answers are complete, whether or not they have been collected. */
int chl_server_submit(chl_server *s, const uint32_t *pairs, size_t k,
                      uint64_t *req_id);
/* Wait for request `req_id`; copies its k answers into out and releases
 * its entry.  timeout_ms < 0 waits forever; CHL_ERR_TIMEOUT if it expires.
 * CHL_ERR_INVALID if the server is freed while the caller waits. */
int chl_server_wait(chl_server *s, uint64_t req_id, int32_t *out,
                    double timeout_ms, double *latency_ms);
/* Callers currently blocked in chl_server_submit (waiting for admission)
 * or chl_server_wait (no counterpart in the reference; for monitoring). */
int chl_server_blocked(chl_server *s, uint32_t *callers);
/* Totals since creation: launches, pairs answered, requests completed. */
int chl_server_stats(chl_server *s, uint64_t *launches, uint64_t *pairs,
                     uint64_t *requests);
/* Stops the server: callers blocked in chl_server_submit or chl_server_wait
 * return CHL_ERR_INVALID, requests not yet launched are dropped, launches in
 * flight are finished, then everything is released.  No call may start on
 * the handle once chl_server_free has been called. */
void chl_server_free(chl_server *s);

/* ------------------------------------------------------- learned ranking */

/* Message-passing ranking network (no reference counterpart; the reference
 * reads its vertex order from a file, shared_memory/hhl.cpp:36-37).
 * x_v = standardised [log1p deg, log1p 2-hop degree sum, sampled clustering];
 * h_0 = relu(x W_0 + b_0); h_l = relu([h_{l-1}, mean_{out-nbrs} h_{l-1}] W_l
 * + b_l) for l = 1..layers (BF16 tensor-core GEMMs, FP32 accumulation);
 * score = h_L w + b.  Parameters are FP32, layout W_0[3x64] b_0[64] |
 * per layer W_l[128x64] b_l[64] | w[64] b[1]. */
int chl_gnn_create(uint32_t layers, uint64_t seed, chl_gnn **out);
size_t chl_gnn_param_count(const chl_gnn *m);
int chl_gnn_get_params(const chl_gnn *m, float *out);
int chl_gnn_set_params(chl_gnn *m, const float *in);
/* The n x 3 standardised input features (row-major). */
int chl_gnn_features(const chl_graph *g, uint64_t seed, float *x);
/* n scores (higher = more central). */
int chl_gnn_predict(chl_gnn *m, const chl_graph *g, uint64_t seed, float *score);
/* Mean squared error to target[n] and its gradient (param_count floats,
 * may be NULL). */
int chl_gnn_grad(chl_gnn *m, const chl_graph *g, uint64_t seed, const float *target,
                 double *loss, float *grads);
/* One Adam step (beta 0.9/0.999, eps 1e-8) on the gradient of chl_gnn_grad. */
int chl_gnn_train_step(chl_gnn *m, const chl_graph *g, uint64_t seed, const float *target,
                       float lr, double *loss);
/* Order (rank -> vertex) by score descending, ties by the seeded tie key
 * of chl_order_degree. */
int chl_gnn_order(chl_gnn *m, const chl_graph *g, uint64_t seed, uint32_t *order);
void chl_gnn_free(chl_gnn *m);

#ifdef __cplusplus
}
#endif

#endif /* CHL_H */
