// Canonical hub label construction on one GPU.
//
// Reference path being replaced:
//   hl::run_paraPLL            shared_memory/akiba.hpp:132-217  (GLL supersteps)
//   hl::Akiba::iteration_gll   shared_memory/akiba.hpp:65-125   (pruned Dijkstra)
//   hl::Akiba::plant           distributed_memory/akiba.hpp:52-104 (PLaNT tree)
//   BasicDijkstra::update_wo_prune distributed_memory/dijkstra.hpp:56-78
//   hl::run (hybrid switch)    distributed_memory/akiba.hpp:290-336, 479-480
//   Labeling::sort / clean_cover shared_memory/labeling.hpp:222-256, 78-88
//
// Design (one process, one GPU):
//  * Roots are taken in rank order in supersteps.  A persistent kernel runs
//    one tree per warp; warps pull roots from a device counter until the
//    superstep's label budget (sf * n, the reference's label_limit) is spent.
//  * Every tree prunes only against labels committed by EARLIER supersteps
//    (read-only during the kernel), so a superstep's output does not depend
//    on warp scheduling.
//  * PLaNT trees track the "via a higher-ranked vertex" flag exactly as
//    update_wo_prune does and emit canonical labels directly; GLL trees skip
//    higher-ranked vertices and emit a superset that the clean kernel
//    filters with the reference's clean_cover rule.
//  * New labels are sorted by (vertex, side, hub) with a stable radix sort
//    and merged into the committed CSR (double-buffered) in one pass; a
//    second copy of every list, ordered by (distance, hub), is merged too.
//  * The tree kernel (batch_kernel) settles vertices in batches by the IN
//    criterion from a near/far queue and prunes with one 16-entry item of
//    the distance-ordered lists per lane against a shared-memory hash of the
//    root's label.
#include "chl_dev.cuh"

#include <algorithm>
#include <chrono>
#include <type_traits>
#include <cmath>
#include <cstring>
#include <vector>

namespace chl {

namespace {

constexpr uint32_t kInf = 0xFFFFFFFFu;
constexpr int kWarpsPerBlock = 4;
#ifndef CHL_PHASE_TIMING
#define CHL_PHASE_TIMING 0              // 1: per-phase clock64 counters (diagnostic builds)
#endif
constexpr bool kPhaseTiming = CHL_PHASE_TIMING != 0;
// batched settle code-shape switches (for A/B measurements)
#ifndef CHL_SCAN_CHUNKS
#define CHL_SCAN_CHUNKS 4    // 32-entry frontier chunks per scan step
#endif
#ifndef CHL_SMEM_CAP_KB
#define CHL_SMEM_CAP_KB 112  // dynamic shared memory per block, at most (2 blocks per SM)
#endif
#ifndef CHL_BATCH_MIN_BLOCKS
#define CHL_BATCH_MIN_BLOCKS 0   // batched settle launch bound (0: compiler's choice;
                                 // 1 measured slower: more registers, fewer warps)
#endif
#ifndef CHL_RELAX_PRECHECK
#define CHL_RELAX_PRECHECK 1   // read a key before its atomicMin; skip the atomic when it cannot lower it
#endif
#ifndef CHL_RELAX_CHUNKS
#define CHL_RELAX_CHUNKS 3   // 32-arc chunks per relax step
#endif

struct BuildCtl {
    unsigned long long next_root;   // root fetch counter (absolute rank)
    unsigned long long nlab;        // labels emitted this superstep
    unsigned long long visits;
    unsigned long long label_reads;
    unsigned long long arcs;
    unsigned long long n_keep;      // labels surviving the clean pass
    unsigned int overflow;
    unsigned int err;               // 1: distance overflow, 2: workspace bound
    unsigned int max_dist;          // largest distance of a label emitted this superstep
    unsigned int reserved_;
    unsigned long long max_ratio_num;  // (tree, labels) of the worst root
    unsigned long long max_ratio_den;
    unsigned long long running;     // trees of the nominal root range in progress
    unsigned long long close_at;    // first root refused after the extension closed
    unsigned long long cyc[10];     // per-phase SM cycles summed over warps (diagnostics; [8]: prune
                                    // item selection, part of [2]; [9]: selection passes, a count)
    unsigned long long cnt[4];      // frontier entries scanned, rounds, settle calls, far pile entries read
};

struct TreeArgs {
    uint32_t n;
    int sides;                      // 1: symmetric graph, one label side stored
    const uint64_t *g_off[2];       // [f]: arcs traversed by trees of side f
    const uint4 *g_farc[2];         // (head, length, rank[head], win[head]) per arc
    const uint2 *g_fhead[2];        // (head, rank[head]) per arc, unit lengths
    const uint32_t *order;
    const uint32_t *rank;
    const uint64_t *l_off;          // committed labels, index lidx(v, side)
    const uint2 *l_ent;             // entries ordered by hub
    const uint2 *l_dent;            // the same entries ordered by (distance, hub)
    uint32_t r0, r_end;
    uint32_t r_hard;                // roots past r_end taken while nominal trees run
    unsigned long long budget;
    int hub_bits;
    uint64_t *out_key;
    uint32_t *out_val;
    unsigned long long out_cap;
    uint32_t *tree_size;            // per root (index r - r0), sides summed
    uint32_t *tree_labels;
    uint32_t *ws_key;               // per warp slot, n keys each (64-bit on weighted graphs)
    uint32_t *ws_vis;
    uint32_t *ws_front;             // per warp slot: queue, next queue, far pile
    uint32_t *ws_win;               // window kernel: 6 n words per tree (block)
    BuildCtl *ctl;
    uint32_t hash_slots;            // root hash table slots (a power of two)
    uint32_t hash_shift;            // 32 - log2(hash_slots)
    uint32_t near_on;               // queue size that starts the near/far split (0: never)
    uint32_t near_target;           // near entries aimed at per refill
};

// Phase-timing clock: with CHL_PHASE_TIMING it is also a compiler memory
// barrier, so loads and stores are not moved across phase boundaries (a
// stall is charged to the phase that uses the value); otherwise 0.
__device__ __forceinline__ long long phase_clock() {
    if (!kPhaseTiming) return 0;
    long long t;
    asm volatile("mov.u64 %0, %%clock64;" : "=l"(t)::"memory");
    return t;
}

__device__ __forceinline__ uint32_t lidx(uint32_t v, int side, int sides) {
    return sides == 1 ? v : 2 * v + (uint32_t)side;
}

// ------------------------------------------------------ batch tree kernel
//
// One tree per warp, settled in batches.  A queued vertex v is final (its
// distance AND its via flag) once d(v) < dmin + win(v), where dmin is the
// smallest queued distance and win(v) the shortest arc into v: every
// predecessor p on a shortest path then has d(p) <= d(v) - win(v) < dmin and
// is already settled (the IN criterion of Crauser et al.).  All qualifying
// vertices are settled together:
//   * the queue is an unordered array scanned by the whole warp; a long
//     queue is split at a distance threshold into a near part, scanned
//     every round, and a far pile, read only when the near part runs out;
//   * prune tests are flattened to (vertex, 16-entry chunk) items taken
//     chunk-major, one per lane (default; 32- and 64-entry items in lane
//     groups, and one lane group per vertex, are options); with the
//     distance-ordered lists a vertex's remaining items are dropped once a
//     chunk passes d(r, u);
//   * the arcs of the batch are flattened over the lanes and relaxed with
//     atomicMin on the packed (distance, via) key.
// With unit lengths a batch is exactly one BFS level.  Relaxations from a
// batch cannot improve a batch vertex, so batch order never matters.
#ifndef CHL_KBATCH
#define CHL_KBATCH 256
#endif
constexpr int kBatch = CHL_KBATCH;   // settled vertices buffered per warp (<= 256: item packing)

constexpr int kEmit = 64;   // labels staged per warp before an append

__host__ __device__ constexpr size_t batch_smem_per_warp(uint32_t hash_slots) {
    return ((size_t)8 * kBatch + (size_t)8 * hash_slots + (size_t)4 * (8 * kBatch + 1) + 8 +
            (size_t)12 * kEmit + 15) &
           ~(size_t)15;
}

// The root's committed label as an open-addressing hash table in shared
// memory (linear probing, load <= 1/2), so the up to 8 lookups of a lane are
// independent instead of a chain of dependent binary-search probes.  Entries
// beyond the table's half capacity (the highest hubs) stay in the global
// sorted list and are searched there.  Slot = hub << 32 | dist; ~0 = empty
// (hub 0xFFFFFFFF never occurs: hubs are ranks < n < 2^32).
constexpr uint64_t kSlotEmpty = ~0ull;

__device__ __forceinline__ uint32_t slot_of(uint32_t h, uint32_t shift) { return (h * 0x9E3779B1u) >> shift; }

struct RootHash {
    const uint64_t *tab;
    uint32_t mask;      // table slots - 1
    uint32_t Th;        // entries hashed (the first Th of the list)
    uint32_t hlast;     // hub of entry Th - 1 (0 if Th == 0)
    const uint2 *g;     // whole list in global memory
    uint32_t R;
    // lookup of h; *dist set when found
    __device__ __forceinline__ bool find_tail(uint32_t h, uint32_t &dist) const {
        uint32_t lo = Th, hi = R;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(&g[mid].x) < h) lo = mid + 1;
            else hi = mid;
        }
        if (lo < R) {
            const uint2 e = __ldg(&g[lo]);
            if (e.x == h) {
                dist = e.y;
                return true;
            }
        }
        return false;
    }
};

// Work-conserving supersteps.  A superstep's nominal roots are [r0, r_end);
// while any nominal tree is still running, idle warps take further roots up
// to r_hard instead of waiting (a superstep is as long as its largest tree,
// which one warp builds).  The processed roots stay one contiguous range:
// the warp that ends the last running nominal tree sets kClosed in the fetch
// counter with one atomicOr, and every fetch returning a value with kClosed
// set is refused; close_at records the first refused rank.  Any consecutive
// root range per superstep gives the same labels: trees prune only against
// the labels of earlier supersteps.
constexpr unsigned long long kClosed = 1ull << 62;

__device__ __forceinline__ uint32_t sat_add(uint32_t x, uint32_t y) {
    const uint32_t z = x + y;
    return z < x ? 0xFFFFFFFFu : z;
}

__device__ __forceinline__ uint32_t fetch_root(const TreeArgs &a, bool &nominal) {
    nominal = false;
    const unsigned long long used = *(volatile unsigned long long *)&a.ctl->nlab;
    // no new tree once the budget is spent, or once the label buffer is full
    // (the superstep's range is then re-run with a larger buffer)
    if (used >= a.budget || used >= a.out_cap) return kInf;
    const unsigned long long t = atomicAdd(&a.ctl->next_root, 1ull);
    if (t & kClosed) return kInf;
    if (t < a.r_end) {
        atomicAdd(&a.ctl->running, 1ull);
        nominal = true;
        return (uint32_t)t;
    }
    return t < a.r_hard ? (uint32_t)t : kInf;
}

__device__ __forceinline__ void finish_root(const TreeArgs &a, bool nominal) {
    if (!nominal || a.r_hard <= a.r_end) return;
    if (atomicAdd(&a.ctl->running, ~0ull) == 1ull &&
        (*(volatile unsigned long long *)&a.ctl->next_root & ~kClosed) >= a.r_end) {
        const unsigned long long old = atomicOr(&a.ctl->next_root, kClosed);
        if (!(old & kClosed)) a.ctl->close_at = old;
    }
}

template <bool UNIT, bool PLANT>
__global__ void __launch_bounds__(kWarpsPerBlock * 32, CHL_BATCH_MIN_BLOCKS)
batch_kernel(TreeArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t lane = lane_id(), wib = threadIdx.x >> 5;
    const uint32_t slot = blockIdx.x * kWarpsPerBlock + wib;
    unsigned char *base = smem + wib * batch_smem_per_warp(a.hash_slots);
    uint64_t *s_ba = (uint64_t *)base;                 // arc begin of batch vertex
    uint64_t *s_tab = s_ba + kBatch;                   // root label hash table
    uint32_t *s_bv = (uint32_t *)(s_tab + a.hash_slots);   // batch vertex
    uint32_t *s_bk = s_bv + kBatch;                    // batch key
    uint32_t *s_bp = s_bk + kBatch;                    // 1: pruned or skipped
    uint32_t *s_bx = s_bp + kBatch;                    // arc prefix (kBatch + 1)
    uint32_t *s_tl = s_bx + kBatch + 1;                // batch indices still to test
    uint32_t *s_bl = s_tl + kBatch;                    // label list length
    uint32_t *s_nch = s_bl + kBatch;                   // label list chunks
    uint32_t *s_as = s_nch + kBatch;                   // next chunk to test, per batch vertex
    uint64_t *s_ek = (uint64_t *)(((uintptr_t)(s_as + kBatch) + 7) & ~(uintptr_t)7);   // staged label keys
    uint32_t *s_ev = (uint32_t *)(s_ek + kEmit);       // staged label distances

    // A vertex's key (distance * 2 + not-via).  On weighted graphs it shares
    // a 64-bit word with win(v), the shortest arc into v (key in the high
    // half, so atomicMin orders by key): the frontier scan gets both with
    // one load.  Unit lengths have win(v) = 1 and 32-bit keys.
    using KeyW = typename std::conditional<UNIT, uint32_t, unsigned long long>::type;
    KeyW *key = (KeyW *)a.ws_key + (size_t)slot * a.n;
    constexpr KeyW kKeyNone = (KeyW)~(KeyW)0;
    uint32_t *vis = a.ws_vis + (size_t)slot * a.n;
    // queue as two arrays: a round reads `front` and writes the vertices it
    // keeps, and those its relaxations add, to `fnext`; then they swap
    uint32_t *front = a.ws_front + (size_t)slot * 3 * a.n;
    uint32_t *fnext = front + a.n;
    // far pile of the near/far queue (see the round loop)
    uint32_t *pile = fnext + a.n;
    unsigned long long c_vis = 0, c_reads = 0, c_arcs = 0;
    long long cyc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};   // phase cycles (diagnostics)
    unsigned long long dcnt[4] = {0, 0, 0, 0};      // scanned, rounds, settles, far pile entries
    const long long k_start = phase_clock();

    // emitted labels are staged in shared memory and appended to the new
    // label arrays kEmit at a time (one atomic per flush instead of one
    // per settle round)
    uint32_t n_emit = 0;
    uint32_t d_hi = 0;   // largest distance this lane has written
    auto flush_labels = [&]() {
        __syncwarp();
        if (n_emit) {
            unsigned long long b = 0;
            if (lane == 0) b = atomicAdd(&a.ctl->nlab, (unsigned long long)n_emit);
            b = __shfl_sync(kFull, b, 0);
            for (uint32_t k = lane; k < n_emit; k += 32) {
                const unsigned long long p = b + k;
                d_hi = max(d_hi, s_ev[k]);
                if (p < a.out_cap) {
                    a.out_key[p] = s_ek[k];
                    a.out_val[p] = s_ev[k];
                } else {
                    a.ctl->overflow = 1;
                }
            }
        }
        n_emit = 0;
        __syncwarp();
    };
    for (uint32_t k = lane; k < a.hash_slots; k += 32) s_tab[k] = kSlotEmpty;
    __syncwarp();
    while (true) {
        uint32_t r = kInf;
        bool r_nominal = false;
        if (lane == 0) r = fetch_root(a, r_nominal);
        r = __shfl_sync(kFull, r, 0);
        r_nominal = __shfl_sync(kFull, r_nominal ? 1u : 0u, 0) != 0;
        if (r == kInf) break;
        uint32_t t_size = 0, t_lab = 0;
        const uint32_t v = a.order[r];
        for (int sd = 0; sd < a.sides; ++sd) {
            const long long tr0 = phase_clock();
            const int f = (a.sides == 1) ? 1 : sd;
            const uint64_t *goff = a.g_off[f];
            const uint4 *farc = a.g_farc[f];
            const uint2 *fhead = a.g_fhead[f];
            // label entries the prune tests scan: the distance-ordered copy
            const uint2 *lscan = a.l_dent;
            const uint32_t ridx = lidx(v, f, a.sides);
            const uint64_t rb = a.l_off[ridx], re = a.l_off[ridx + 1];
            const uint32_t R = (uint32_t)(re - rb);
            RootHash rhash;
            rhash.tab = s_tab;
            rhash.mask = a.hash_slots - 1;
            rhash.g = a.l_ent + rb;
            rhash.R = R;
            rhash.hlast = 0;
            rhash.Th = min(R, a.hash_slots / 2);
            for (uint32_t k = lane; k < rhash.Th; k += 32) {
                const uint2 e = a.l_ent[rb + k];
                const uint64_t val = ((uint64_t)e.x << 32) | e.y;
                uint32_t sl = slot_of(e.x, a.hash_shift);
                while (atomicCAS((unsigned long long *)&s_tab[sl], (unsigned long long)kSlotEmpty,
                                 (unsigned long long)val) != (unsigned long long)kSlotEmpty)
                    sl = (sl + 1) & rhash.mask;
            }
            if (rhash.Th) rhash.hlast = a.l_ent[rb + rhash.Th - 1].x;
            // Prune test of one lane's 16 consecutive entries of the
            // distance-ordered L(u) against the hashed root label.  vm marks the entries that belong to the list;
            // an entry beyond d(r, u) witnesses nothing and, the list being
            // in distance order, marks the list exhausted.
            auto test16d = [&](const uint4 (&q)[8], uint32_t vm, uint32_t gdj, bool &exhausted) -> bool {
                bool hit = false;
                uint64_t v[16];
                uint32_t sl[16];
                uint32_t pend = 0;
#pragma unroll
                for (int t = 0; t < 16; ++t) {
                    const uint32_t hh = (t & 1) ? q[t >> 1].z : q[t >> 1].x;
                    const uint32_t dd = (t & 1) ? q[t >> 1].w : q[t >> 1].y;
                    const bool in = (vm >> t) & 1u;
                    v[t] = kSlotEmpty;
                    sl[t] = 0;
                    if (in && dd > gdj) exhausted = true;
                    if (in && dd <= gdj && rhash.Th && hh <= rhash.hlast) {
                        sl[t] = slot_of(hh, a.hash_shift);
                        v[t] = s_tab[sl[t]];
                        pend |= 1u << t;
                    }
                }
                if (rhash.Th < R) {
                    // hubs past the hashed prefix: binary search of the rest
#pragma unroll
                    for (int t = 0; t < 16; ++t) {
                        const uint32_t hh = (t & 1) ? q[t >> 1].z : q[t >> 1].x;
                        const uint32_t dd = (t & 1) ? q[t >> 1].w : q[t >> 1].y;
                        if (((vm >> t) & 1u) && dd <= gdj && !(rhash.Th && hh <= rhash.hlast)) {
                            uint32_t dr;
                            if (rhash.find_tail(hh, dr) && dr + dd <= gdj) hit = true;
                        }
                    }
                }
#pragma unroll
                for (int t = 0; t < 16; ++t) {
                    if (!(pend >> t & 1u)) continue;
                    const uint32_t hh = (t & 1) ? q[t >> 1].z : q[t >> 1].x;
                    const uint32_t dd = (t & 1) ? q[t >> 1].w : q[t >> 1].y;
                    uint64_t w = v[t];
                    uint32_t z = sl[t];
                    while (w != kSlotEmpty && (uint32_t)(w >> 32) != hh) {
                        z = (z + 1) & rhash.mask;
                        w = s_tab[z];
                    }
                    if (w != kSlotEmpty && (uint32_t)w + dd <= gdj) hit = true;
                }
                return hit;
            };
            if (lane == 0) {
                __stcg(&key[v], UNIT ? (KeyW)1u : (KeyW)((1ull << 32) | 1u));   // win 1 admits the root
                vis[0] = v;
                front[0] = v;
            }
            __syncwarp();
            cyc[5] += phase_clock() - tr0;
            uint32_t nvis = 1, nf = 1, nn = 0;   // queue sizes in front and fnext
            // Near/far queue.  A large queue is split at a threshold thr:
            // keys below it are queued in front/fnext and scanned every
            // round, the rest in the far pile, read only when the near
            // vertices run out.  thr == kInf: no split (all queued near).
            uint32_t npile = 0;         // far pile entries (stale ones included)
            uint32_t thr = kInf;
            uint32_t pmin = kInf;       // per lane: lower bound of the live far keys
            uint32_t delta = 0;         // threshold step (0: choose at the next refill)
            int ql = 1;
            uint32_t dmin = 0;          // smallest queued distance (exact, see below)
            bool stop = false;
            uint32_t nb = 0;            // vertices in the smem batch

            // Settle the batch held in smem: prune tests, labels, relaxations.
            // New vertices are appended to fnext; every key decrease of
            // a queued vertex lowers dnext, so dnext is the exact minimum of
            // the queue after the round.
            uint32_t dnext = kInf;
            auto settle = [&]() {
                long long tc0 = phase_clock();
                if (kPhaseTiming) dcnt[2]++;
                t_size += nb;
                int nv_batch = 0;
                for (uint32_t j = lane; j < nb; j += 32) {
                    const uint32_t kx = s_bk[j];
                    const uint32_t rx = __ldg(&a.rank[s_bv[j]]);   // batch vertices only, not every scanned one
                    uint32_t skip;
                    if (PLANT) {
                        nv_batch += (int)(kx & 1u);
                        // a committed vertex (rank < r0) always has a committed
                        // witness: pruned without reading its labels
                        skip = rx < a.r0 ? 1u : 0u;
                    } else {
                        skip = rx < r ? 1u : 0u;   // iteration_gll :92
                    }
                    s_bp[j] = skip;
                }
                if (PLANT) ql -= __reduce_add_sync(kFull, nv_batch);
                __syncwarp();
                long long tc1 = phase_clock();
                cyc[1] += tc1 - tc0;
                if (R > 0) {
                    // Prune tests as (vertex, 16-entry chunk) items, one per
                    // lane and step.  The vertices still under test wait in a
                    // circular queue (s_tl, kBatch entries): a step takes up
                    // to 32 from its front -- with fewer than 32, each gets
                    // several consecutive chunks -- and puts back at the end
                    // those with no witness yet whose list has not passed
                    // d(r, u).  Each vertex gets about one chunk per trip
                    // through the queue (chunk-major order), and no step
                    // looks at a vertex that is already decided.
                    uint32_t nq = 0;
                    for (uint32_t j0 = 0; j0 < nb; j0 += 32) {
                        const uint32_t j = j0 + lane;
                        const bool t = j < nb && s_bp[j] == 0;
                        const uint32_t m = __ballot_sync(kFull, t);
                        if (t) {
                            s_tl[nq + __popc(m & lanemask_lt())] = j;
                            const uint32_t xu = lidx(s_bv[j], 1 - f, a.sides);
                            const uint64_t lb = a.l_off[xu], le = a.l_off[xu + 1];
                            s_ba[j] = lb;
                            s_bl[j] = (uint32_t)(le - lb);
                            s_nch[j] = (uint32_t)((le - (lb & ~1ull) + 15) >> 4);
                            s_as[j] = 0;   // next chunk to test
                        }
                        nq += __popc(m);
                    }
                    __syncwarp();
                    uint32_t qh = 0, nread = 0;
                    while (nq > 0) {
                        const long long tsel = phase_clock();
                        if (kPhaseTiming) cyc[9]++;
                        const uint32_t t = min(nq, 32u);
                        // lane -> (vertex of the queue front, chunk)
                        const uint32_t vi = lane % t;
                        const uint32_t lj = s_tl[(qh + vi) % (uint32_t)kBatch];
                        const uint32_t c = s_as[lj] + lane / t;
                        const bool act = c < s_nch[lj];
                        cyc[8] += phase_clock() - tsel;
                        // one 16-entry item per lane (8 loads of one 128-byte
                        // line in flight per lane)
                        bool hit = false, exhausted = false;
                        if (act) {
                            const uint64_t glb = s_ba[lj];
                            const uint64_t gle = glb + s_bl[lj];
                            const uint32_t gdj = s_bk[lj] >> 1;
                            const uint64_t e0 = (glb & ~1ull) + 16ull * c;
                            // entries [lo, hi) of the 16 belong to the list: lo
                            // is 1 only in chunk 0 of an odd start, and an
                            // active item has e0 < gle
                            const uint32_t lo = (uint32_t)(glb - min(glb, e0));
                            const uint64_t span = gle - e0;
                            const uint32_t hi = span < 16 ? (uint32_t)span : 16u;
                            const uint32_t vm = ((1u << hi) - 1u) & ~((1u << lo) - 1u);
                            uint4 q[8];
#pragma unroll
                            for (int u = 0; u < 8; ++u) {
                                q[u] = make_uint4(0, 0, 0, 0);
                                if ((vm >> (2 * u)) & 3u) q[u] = *(const uint4 *)(lscan + e0 + 2 * u);
                            }
                            hit = test16d(q, vm, gdj, exhausted);
                            nread += 16;
                        }
                        if (hit) s_bp[lj] = 1;
                        else if (exhausted) atomicOr(&s_bp[lj], 2u);
                        __syncwarp();
                        // the front t vertices leave the queue; those still
                        // undecided with chunks left go back at the end
                        bool back = false;
                        uint32_t bj = 0;
                        if (lane < t) {
                            bj = lj;   // vi == lane here
                            const uint32_t taken = 32u / t + (lane < 32u % t ? 1u : 0u);
                            const uint32_t nc = s_as[bj] + taken;
                            s_as[bj] = nc;
                            back = s_bp[bj] == 0 && nc < s_nch[bj];
                        }
                        const uint32_t bm = __ballot_sync(kFull, back);
                        qh = (qh + t) % (uint32_t)kBatch;
                        nq -= t;
                        if (back) s_tl[(qh + nq + __popc(bm & lanemask_lt())) % (uint32_t)kBatch] = bj;
                        nq += __popc(bm);
                        __syncwarp();
                    }
                    c_reads += nread;
                    __syncwarp();
                }
                long long tc2 = phase_clock();
                cyc[2] += tc2 - tc1;
                for (uint32_t j0 = 0; j0 < nb; j0 += 32) {
                    const uint32_t j = j0 + lane;
                    bool emit = false;
                    uint32_t xu = 0, dj = 0;
                    if (j < nb && (s_bp[j] & 1u) == 0) {
                        const uint32_t kx = s_bk[j];
                        emit = !PLANT || (kx & 1u);
                        xu = lidx(s_bv[j], 1 - f, a.sides);
                        dj = kx >> 1;
                    }
                    const uint32_t em = __ballot_sync(kFull, emit);
                    if (em) {
                        // labels go through the warp's shared staging buffer
                        if (n_emit + 32 > (uint32_t)kEmit) flush_labels();
                        if (emit) {
                            const uint32_t at = n_emit + __popc(em & lanemask_lt());
                            s_ek[at] = ((uint64_t)xu << a.hub_bits) | (uint64_t)(r - a.r0);
                            s_ev[at] = dj;
                        }
                        n_emit += __popc(em);
                        t_lab += __popc(em);
                    }
                }
                long long tc3 = phase_clock();
                cyc[3] += tc3 - tc2;
                // arcs of the batch flattened over the lanes: the vertices
                // with arcs are compacted (s_tl[k] = batch index, s_bx[k] =
                // first flattened arc), so the owner of arc t0 + lane is the
                // window's first owner plus the vertex starts inside the
                // window below the lane (one OR-reduction, no search)
                uint32_t total = 0, ncomp = 0;
                for (uint32_t j0 = 0; j0 < nb; j0 += 32) {
                    const uint32_t j = j0 + lane;
                    uint32_t deg = 0;
                    if (j < nb && (s_bp[j] & 1u) == 0) {
                        const uint32_t x = s_bv[j];
                        const uint64_t ab = goff[x];
                        deg = (uint32_t)(goff[x + 1] - ab);
                        s_ba[j] = ab;
                    }
                    uint32_t incl = deg;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t y = __shfl_up_sync(kFull, incl, o);
                        if (lane >= (uint32_t)o) incl += y;
                    }
                    const uint32_t nem = __ballot_sync(kFull, deg > 0);
                    if (deg > 0) {
                        const uint32_t k = ncomp + __popc(nem & lanemask_lt());
                        s_tl[k] = j;
                        s_bx[k] = total + incl - deg;
                    }
                    total += __shfl_sync(kFull, incl, 31);
                    ncomp += __popc(nem);
                }
                if (lane == 0) s_bx[ncomp] = total;
                __syncwarp();
                c_arcs += total;
                uint32_t cur = 0;   // compacted owner of arc t0
                // owner (compacted index) of arc t0 + lane
                auto owner = [&](uint32_t t0) -> uint32_t {
                    if (cur + 1 < ncomp && s_bx[cur + 1] <= t0) ++cur;
                    uint32_t bit = 0;
                    const uint32_t kk = cur + 1 + lane;
                    if (kk < ncomp) {
                        const uint32_t st = s_bx[kk];
                        if (st < t0 + 32) bit = 1u << (st - t0);
                    }
                    const uint32_t starts = __reduce_or_sync(kFull, bit);
                    const uint32_t upto = lane == 31 ? kFull : ((2u << lane) - 1u);
                    const uint32_t own = cur + (uint32_t)__popc(starts & upto);
                    cur += (uint32_t)__popc(starts);
                    return own;
                };
                // CHL_RELAX_CHUNKS 32-arc chunks per step: their arc loads and
                // atomics are issued together (three measured best on the
                // 1024-square grid and RMAT-20: 3.43 -> 3.31 s and 2.06 ->
                // 1.90 s against two)
                constexpr int RC = CHL_RELAX_CHUNKS;
                int dql = 0;   // this lane's change of the queued not-via count
                for (uint32_t t0 = 0; t0 < total; t0 += 32 * RC) {
                    uint32_t w[RC], nk[RC], old[RC], kxs[RC], len[RC], rk[RC], wn[RC];
                    bool act[RC], upd[RC];
#pragma unroll
                    for (int c = 0; c < RC; ++c) {
                        w[c] = 0;
                        nk[c] = 0;
                        old[c] = kInf;
                        kxs[c] = 0;
                        len[c] = 0;
                        rk[c] = 0;
                        wn[c] = 1;
                        act[c] = false;
                        upd[c] = false;
                    }
#pragma unroll
                    for (int c = 0; c < RC; ++c) {
                        const uint32_t tc = t0 + 32u * c;
                        const uint32_t own = tc < total ? owner(tc) : 0u;
                        const uint32_t t = tc + lane;
                        if (t < total) {
                            const uint32_t lo = s_tl[own];
                            const uint64_t e = s_ba[lo] + (t - s_bx[own]);
                            if (UNIT) {
                                const uint2 hr = fhead[e];
                                w[c] = hr.x;
                                rk[c] = hr.y;
                                len[c] = 1;
                            } else {
                                const uint4 hl = farc[e];
                                w[c] = hl.x;
                                len[c] = hl.y;
                                rk[c] = hl.z;
                                wn[c] = hl.w;
                            }
                            kxs[c] = s_bk[lo];
                            act[c] = true;
                        }
                    }
                    uint32_t nv[RC];
                    KeyW pre[RC];   // the key word before the atomic (keys only decrease)
#pragma unroll
                    for (int c = 0; c < RC; ++c) {
                        nv[c] = (!PLANT || ((kxs[c] & 1u) && rk[c] >= r)) ? 1u : 0u;
                        pre[c] = (CHL_RELAX_PRECHECK && act[c]) ? __ldcg(&key[w[c]]) : kKeyNone;
                    }
#pragma unroll
                    for (int c = 0; c < RC; ++c) {
                        if (!act[c]) continue;
                        const uint64_t dd64 = (uint64_t)(kxs[c] >> 1) + len[c];
                        if (dd64 < 0x7FFFFFFFull) {
                            nk[c] = (uint32_t)dd64 * 2u + nv[c];
                            const uint32_t pk = UNIT ? (uint32_t)pre[c] : (uint32_t)((unsigned long long)pre[c] >> 32);
                            if (pk <= nk[c]) {
                                old[c] = pk;   // no decrease: no atomic
                            } else if (UNIT) {
                                old[c] = (uint32_t)atomicMin(&key[w[c]], (KeyW)nk[c]);
                            } else {
                                const unsigned long long o64 =
                                    atomicMin(&key[w[c]], (KeyW)(((unsigned long long)nk[c] << 32) | wn[c]));
                                old[c] = (uint32_t)(o64 >> 32);
                            }
                            upd[c] = nk[c] < old[c];
                            if (upd[c]) dnext = min(dnext, nk[c] >> 1);
                        } else {
                            a.ctl->err = 1;   // the reference asserts dd < infty
                        }
                    }
#pragma unroll
                    for (int c = 0; c < RC; ++c) {
                        const bool fresh = upd[c] && old[c] == kInf;
                        // queued near: a new key below thr, or a far vertex
                        // whose key drops below it (its far entry goes stale)
                        const uint32_t dk = nk[c] >> 1;
                        const bool to_near = upd[c] && dk < thr && (old[c] == kInf || (old[c] >> 1) >= thr);
                        const uint32_t fm = __ballot_sync(kFull, to_near);
                        if (to_near) {
                            const uint32_t o = __popc(fm & lanemask_lt());
                            if (nn + o < a.n) fnext[nn + o] = w[c];
                            else a.ctl->err = 2;
                        }
                        nn = min(nn + __popc(fm), a.n);
                        const uint32_t vm = thr == kInf ? fm : __ballot_sync(kFull, fresh);
                        if (fresh) {
                            const uint32_t o = __popc(vm & lanemask_lt());
                            if (nvis + o < a.n) vis[nvis + o] = w[c];
                            else a.ctl->err = 2;
                        }
                        nvis = min(nvis + __popc(vm), a.n);
                        if (thr != kInf) {
                            if (upd[c] && dk >= thr) pmin = min(pmin, dk);
                            const bool to_far = fresh && dk >= thr;
                            const uint32_t pm = __ballot_sync(kFull, to_far);
                            if (to_far) {
                                const uint32_t o = __popc(pm & lanemask_lt());
                                if (npile + o < a.n) pile[npile + o] = w[c];
                                else a.ctl->err = 2;
                            }
                            npile = min(npile + __popc(pm), a.n);
                        }
                        if (PLANT && upd[c]) dql += (int)(nk[c] & 1u) - (old[c] == kInf ? 0 : (int)(old[c] & 1u));
                    }
                }
                if (PLANT) ql += __reduce_add_sync(kFull, dql);
                __syncwarp();
                nb = 0;
                if (PLANT && ql == 0) stop = true;   // plant :95 early exit
                cyc[4] += phase_clock() - tc3;
            };

            // Refill the (empty) near queue from the far pile: entries whose
            // key is below the old threshold are stale (their vertex was
            // queued near and is settled), entries below the new threshold
            // thr = (their minimum) + delta move near, the rest stay,
            // compacted in place.  From the second pass on the minimum is
            // exact, so a refill takes at most two passes.
            auto refill = [&]() {
                const long long tf0 = phase_clock();
                uint32_t lo = __reduce_min_sync(kFull, pmin);
                if (delta == 0) {
                    // first refill of the split: delta for about near_target
                    // entries, taking the keys as spread evenly over [min, max]
                    uint32_t mn = kInf, mx = 0;
                    for (uint32_t i = lane; i < npile; i += 32) {
                        const uint32_t k = (uint32_t)(__ldcg(&key[pile[i]]) >> (UNIT ? 1 : 33));
                        mn = min(mn, k);
                        mx = max(mx, k);
                    }
                    mn = __reduce_min_sync(kFull, mn);
                    mx = __reduce_max_sync(kFull, mx);
                    lo = mn;
                    uint64_t d = (uint64_t)(mx - min(mn, mx)) * a.near_target / max(npile, 1u);
                    if (d < 1) d = 1;
                    if (d > 0x7FFFFFFFull) d = 0x7FFFFFFFull;
                    delta = (uint32_t)d;
                    if (kPhaseTiming) dcnt[3] += npile;
                }
                for (int pass = 0; pass < 4 && nf == 0 && npile > 0; ++pass) {
                    const uint32_t t_old = thr;
                    thr = sat_add(lo, delta);
                    uint32_t keep = 0, moved = 0, kmin = kInf, nmin = kInf;
                    if (kPhaseTiming) dcnt[3] += npile;
                    for (uint32_t b0 = 0; b0 < npile; b0 += 32) {
                        const uint32_t i = b0 + lane;
                        const bool valid = i < npile;
                        const uint32_t x = valid ? pile[i] : 0u;
                        const uint32_t k = valid ? (uint32_t)(__ldcg(&key[x]) >> (UNIT ? 1 : 33)) : kInf;
                        const bool live = valid && k >= t_old;
                        const bool nr = live && k < thr;
                        const bool kp = live && !nr;
                        const uint32_t nm = __ballot_sync(kFull, nr);
                        const uint32_t km = __ballot_sync(kFull, kp);
                        // every lane has read its entry (ballots above), and
                        // a kept entry moves only to a lower index
                        if (nr) {
                            front[moved + __popc(nm & lanemask_lt())] = x;
                            nmin = min(nmin, k);
                        }
                        if (kp) {
                            pile[keep + __popc(km & lanemask_lt())] = x;
                            kmin = min(kmin, k);
                        }
                        moved += __popc(nm);
                        keep += __popc(km);
                    }
                    __syncwarp();
                    npile = keep;
                    nf = moved;
                    lo = __reduce_min_sync(kFull, kmin);
                    dmin = __reduce_min_sync(kFull, nmin);   // far keys are >= thr
                    pmin = lane == 0 ? lo : kInf;
                    if (moved < a.near_target / 4) delta = delta < 0x40000000u ? 2u * delta : 0x7FFFFFFFu;
                    else if (moved > 4 * a.near_target) delta = max(delta / 2, 1u);
                }
                if (nf == 0 && npile > 0) a.ctl->err = 2;   // not reached: see above
                cyc[0] += phase_clock() - tf0;
            };

            while ((nf > 0 || npile > 0) && !stop) {
                if (nf == 0) {
                    refill();
                    if (nf == 0) break;
                }
                // One round: walk the queue once.  Vertices with
                // d < dmin + win are final and go to the batch (settled
                // whenever it fills); the rest go to fnext, where the
                // round's relaxations add new vertices (which cannot
                // qualify in this round: their d >= dmin + win).
                const uint32_t nf0 = nf;
                nn = 0;
                dnext = kInf;
                if (kPhaseTiming) {
                    dcnt[0] += nf0;
                    dcnt[1]++;
                }
                // several 32-entry chunks per step: their loads are issued
                // together
                auto classify = [&](bool valid, uint32_t x, uint32_t kx, uint32_t wx) {
                    const bool take = valid && (uint64_t)(kx >> 1) < (uint64_t)dmin + wx;
                    const uint32_t tm = __ballot_sync(kFull, take);
                    if (take) {
                        const uint32_t at = nb + __popc(tm & lanemask_lt());
                        s_bv[at] = x;
                        s_bk[at] = kx;
                    }
                    nb += __popc(tm);
                    const bool kp = valid && !take;
                    const uint32_t km = __ballot_sync(kFull, kp);
                    if (kp) {
                        fnext[nn + __popc(km & lanemask_lt())] = x;
                        dnext = min(dnext, kx >> 1);
                    }
                    nn += __popc(km);
                };
                for (uint32_t b0 = 0; b0 < nf0 && !stop; b0 += 32 * CHL_SCAN_CHUNKS) {
                    if (nb > (uint32_t)kBatch - 32 * CHL_SCAN_CHUNKS) settle();
                    if (stop) break;
                    const long long ts0 = phase_clock();
                    bool vv[CHL_SCAN_CHUNKS];
                    uint32_t xx[CHL_SCAN_CHUNKS], kk[CHL_SCAN_CHUNKS], ww[CHL_SCAN_CHUNKS];
#pragma unroll
                    for (int c = 0; c < CHL_SCAN_CHUNKS; ++c) {
                        const uint32_t i = b0 + 32 * c + lane;
                        vv[c] = i < nf0;
                        xx[c] = vv[c] ? front[i] : 0u;
                    }
#pragma unroll
                    for (int c = 0; c < CHL_SCAN_CHUNKS; ++c) {
                        const KeyW k = vv[c] ? __ldcg(&key[xx[c]]) : kKeyNone;
                        kk[c] = UNIT ? (uint32_t)k : (uint32_t)((unsigned long long)k >> 32);
                        // unit lengths: every queued vertex but the root has an
                        // in-arc of length 1, and 1 also admits the root
                        ww[c] = UNIT ? 1u : (uint32_t)k;
                    }
                    __syncwarp();
#pragma unroll
                    for (int c = 0; c < CHL_SCAN_CHUNKS; ++c) classify(vv[c], xx[c], kk[c], ww[c]);
                    __syncwarp();
                    cyc[0] += phase_clock() - ts0;
                }
                if (nb && !stop) settle();
                if (stop) break;
                __syncwarp();
                {
                    uint32_t *t = front;
                    front = fnext;
                    fnext = t;
                }
                nf = nn;
                dmin = __reduce_min_sync(kFull, dnext);
                if (thr == kInf && nf > a.near_on && a.near_on) {
                    // the queue grew large: all of it goes to the far pile,
                    // and the next refill splits it
                    uint32_t *t = pile;
                    pile = front;
                    front = t;
                    npile = nf;
                    nf = 0;
                    thr = 0;
                    delta = 0;
                }
            }
            c_vis += t_size;
            const long long tz0 = phase_clock();
            for (uint32_t k = lane; k < nvis; k += 32) __stcg(&key[vis[k]], kKeyNone);
            for (uint32_t k = lane; k < a.hash_slots; k += 32) s_tab[k] = kSlotEmpty;
            cyc[6] += phase_clock() - tz0;
            __syncwarp();
        }
        flush_labels();
        if (lane == 0) {
            a.tree_size[r - a.r0] = t_size;
            a.tree_labels[r - a.r0] = t_lab;
            finish_root(a, r_nominal);
        }
    }
    d_hi = __reduce_max_sync(kFull, d_hi);
    if (lane == 0) {
        atomicAdd(&a.ctl->visits, c_vis);
        atomicAdd(&a.ctl->arcs, c_arcs);
        if (d_hi) atomicMax(&a.ctl->max_dist, d_hi);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c_reads += __shfl_xor_sync(kFull, c_reads, o);
    if (lane == 0) {
        atomicAdd(&a.ctl->label_reads, c_reads);
        if (kPhaseTiming) {
            cyc[7] = phase_clock() - k_start;   // whole residency of the warp
#pragma unroll
            for (int i = 0; i < 10; ++i) atomicAdd(&a.ctl->cyc[i], (unsigned long long)cyc[i]);
#pragma unroll
            for (int i = 0; i < 4; ++i) atomicAdd(&a.ctl->cnt[i], dcnt[i]);
        }
    }
}

// ------------------------------------------------------ window kernel
//
// Trees of a superstep with no committed labels (the first one) cannot be
// pruned by labels, so a vertex need not be final before it is expanded:
// such trees are searched label-correcting in distance windows [t, thr), as
// delta-stepping does.  Every member of the window is relaxed; a member whose
// key drops is relaxed again in the next pass, until a pass changes no key
// below thr.  Then every key below thr is final -- it is the minimum over all
// paths, and every other queued key is at least thr -- so the window's labels
// are emitted from the final keys, and the next window, [thr, lo + delta),
// is taken from the far pile (lo its smallest live key; delta starts at the
// spread of the root's neighbours' distances and is halved or doubled after
// each window so that a window holds about near_target vertices).  Keys carry PLaNT's via flag
// (distance * 2 + not-via), and a flag change is a key decrease, so relaxing
// again on every decrease keeps the flags exact; PLaNT's early exit
// (distributed_memory/akiba.hpp:95) is tested at window boundaries, where the
// count of queued not-via keys is exact.  GLL trees (iteration_gll) skip
// expanding and labelling vertices ranked above the root.
//
// A block of TW warps builds one tree: the warps split each pass's members
// and the pile, and append to the tree's lists through shared counters (the
// order of members and pile entries never matters).  Per tree, in the
// window workspace (6 n words): key, touched vertices, members, the key each
// member was last relaxed with, and the far pile double-buffered for the
// block-parallel refill.
constexpr int kWinBatch = 256;   // members relaxed per warp batch

struct WinShared {
    uint32_t root, nominal;
    uint32_t nm;        // members of the window
    uint32_t npile;     // entries of the current pile
    uint32_t npile2;    // entries written to the other pile by a refill
    uint32_t nvis;      // touched vertices
    uint32_t thr;       // window end (exclusive)
    uint32_t delta;     // window width (0: choose at the first refill)
    uint32_t lo;        // lower bound of the live far keys
    uint32_t kmin, kmax;
    uint32_t changed;
    uint32_t psel;      // which pile buffer is current
    int ql;             // queued not-via keys (PLaNT)
    uint32_t dnv;       // largest distance of a not-via member so far (PLaNT)
    uint32_t t_size, t_lab;
    uint32_t err;
};

__host__ __device__ constexpr size_t window_smem_per_warp() {
    return ((size_t)8 * kWinBatch + (size_t)4 * (4 * kWinBatch + 1) + 8 + (size_t)12 * kEmit + 15) & ~(size_t)15;
}
__host__ __device__ constexpr size_t window_smem(int tw) {
    return ((sizeof(WinShared) + 15) & ~(size_t)15) + (size_t)tw * window_smem_per_warp();
}

template <bool UNIT, bool PLANT, int TW>
__global__ void __launch_bounds__(TW * 32)
window_kernel(TreeArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    WinShared &sh = *(WinShared *)smem;
    const uint32_t tid = threadIdx.x, lane = lane_id(), wib = tid >> 5;
    unsigned char *base = smem + ((sizeof(WinShared) + 15) & ~(size_t)15) + wib * window_smem_per_warp();
    uint64_t *s_ba = (uint64_t *)base;                 // arc begin of batch vertex
    uint32_t *s_bv = (uint32_t *)(s_ba + kWinBatch);   // batch vertex
    uint32_t *s_bk = s_bv + kWinBatch;                 // batch key
    uint32_t *s_bx = s_bk + kWinBatch;                 // arc prefix (kWinBatch + 1)
    uint32_t *s_tl = s_bx + kWinBatch + 1;             // batch index of each vertex with arcs
    uint64_t *s_ek = (uint64_t *)(((uintptr_t)(s_tl + kWinBatch) + 7) & ~(uintptr_t)7);   // staged label keys
    uint32_t *s_ev = (uint32_t *)(s_ek + kEmit);       // staged label distances

    uint32_t *key = a.ws_win + (size_t)blockIdx.x * 6 * a.n;
    uint32_t *vis = key + a.n;
    uint32_t *memb = vis + a.n;      // window members
    uint32_t *mkey = memb + a.n;     // key a member was last relaxed with
    uint32_t *piles = mkey + a.n;    // two far piles
    unsigned long long c_vis = 0, c_arcs = 0;

    uint32_t n_emit = 0;
    uint32_t d_hi = 0;   // largest distance this lane has written
    auto flush_labels = [&]() {
        __syncwarp();
        if (n_emit) {
            unsigned long long b = 0;
            if (lane == 0) b = atomicAdd(&a.ctl->nlab, (unsigned long long)n_emit);
            b = __shfl_sync(kFull, b, 0);
            for (uint32_t k = lane; k < n_emit; k += 32) {
                const unsigned long long p = b + k;
                d_hi = max(d_hi, s_ev[k]);
                if (p < a.out_cap) {
                    a.out_key[p] = s_ek[k];
                    a.out_val[p] = s_ev[k];
                } else {
                    a.ctl->overflow = 1;
                }
            }
        }
        n_emit = 0;
        __syncwarp();
    };
    // warp-wide append of the lanes with `take` to a list with a shared
    // counter; returns this lane's index (only meaningful where take)
    auto append_at = [&](bool take, uint32_t *counter) -> uint32_t {
        const uint32_t m = __ballot_sync(kFull, take);
        uint32_t b = 0;
        if (m && lane == 0) b = atomicAdd(counter, (uint32_t)__popc(m));
        b = __shfl_sync(kFull, b, 0);
        return b + __popc(m & lanemask_lt());
    };

    while (true) {
        if (tid == 0) {
            bool nom = false;
            sh.root = fetch_root(a, nom);
            sh.nominal = nom ? 1u : 0u;
            sh.t_size = 0;
            sh.t_lab = 0;
        }
        __syncthreads();
        const uint32_t r = sh.root;
        if (r == kInf) break;
        const uint32_t v = a.order[r];
        for (int sd = 0; sd < a.sides; ++sd) {
            const int f = (a.sides == 1) ? 1 : sd;
            const uint64_t *goff = a.g_off[f];
            const uint4 *farc = a.g_farc[f];
            const uint2 *fhead = a.g_fhead[f];
            if (tid == 0) {
                __stcg(&key[v], 1u);
                vis[0] = v;
                memb[0] = v;
                mkey[0] = kInf;
                sh.nm = 1;
                sh.npile = 0;
                sh.nvis = 1;
                sh.thr = 1;          // the first window holds the root alone
                sh.delta = 0;
                sh.lo = kInf;
                sh.psel = 0;
                sh.ql = 1;
                sh.dnv = 0;
                sh.err = 0;
            }
            __syncthreads();
            uint32_t pmin = kInf;    // per lane: lower bound of far keys set since the last refill
            bool changed = false;

            // Relax the warp's nb batch vertices (arcs flattened over the lanes).
            auto relax = [&](uint32_t nb, uint32_t thr, uint32_t *pile) {
                uint32_t total = 0, ncomp = 0;
                for (uint32_t j0 = 0; j0 < nb; j0 += 32) {
                    const uint32_t j = j0 + lane;
                    uint32_t deg = 0;
                    if (j < nb) {
                        const uint32_t x = s_bv[j];
                        const uint64_t ab = goff[x];
                        deg = (uint32_t)(goff[x + 1] - ab);
                        s_ba[j] = ab;
                    }
                    uint32_t incl = deg;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t y = __shfl_up_sync(kFull, incl, o);
                        if (lane >= (uint32_t)o) incl += y;
                    }
                    const uint32_t nem = __ballot_sync(kFull, deg > 0);
                    if (deg > 0) {
                        const uint32_t k = ncomp + __popc(nem & lanemask_lt());
                        s_tl[k] = j;
                        s_bx[k] = total + incl - deg;
                    }
                    total += __shfl_sync(kFull, incl, 31);
                    ncomp += __popc(nem);
                }
                if (lane == 0) s_bx[ncomp] = total;
                __syncwarp();
                c_arcs += total;
                uint32_t cur = 0;
                auto owner = [&](uint32_t t0) -> uint32_t {
                    if (cur + 1 < ncomp && s_bx[cur + 1] <= t0) ++cur;
                    uint32_t bit = 0;
                    const uint32_t kk = cur + 1 + lane;
                    if (kk < ncomp) {
                        const uint32_t st = s_bx[kk];
                        if (st < t0 + 32) bit = 1u << (st - t0);
                    }
                    const uint32_t starts = __reduce_or_sync(kFull, bit);
                    const uint32_t upto = lane == 31 ? kFull : ((2u << lane) - 1u);
                    const uint32_t own = cur + (uint32_t)__popc(starts & upto);
                    cur += (uint32_t)__popc(starts);
                    return own;
                };
                int dql = 0;
                // WC 32-arc chunks per step: their arc loads and atomics are
                // issued together
                constexpr int WC = CHL_RELAX_CHUNKS;
                for (uint32_t t0 = 0; t0 < total; t0 += 32 * WC) {
                    uint32_t w[WC], nk[WC], old[WC], kxs[WC], len[WC], rk[WC];
                    bool act[WC], upd[WC];
#pragma unroll
                    for (int c = 0; c < WC; ++c) {
                        w[c] = 0;
                        nk[c] = 0;
                        old[c] = kInf;
                        kxs[c] = 0;
                        len[c] = 0;
                        rk[c] = 0;
                        act[c] = false;
                        upd[c] = false;
                    }
#pragma unroll
                    for (int c = 0; c < WC; ++c) {
                        const uint32_t tc = t0 + 32u * c;
                        const uint32_t own = tc < total ? owner(tc) : 0u;
                        const uint32_t t = tc + lane;
                        if (t < total) {
                            const uint32_t lo = s_tl[own];
                            const uint64_t e = s_ba[lo] + (t - s_bx[own]);
                            if (UNIT) {
                                const uint2 hr = fhead[e];
                                w[c] = hr.x;
                                rk[c] = hr.y;
                                len[c] = 1;
                            } else {
                                const uint4 hl = farc[e];
                                w[c] = hl.x;
                                len[c] = hl.y;
                                rk[c] = hl.z;
                            }
                            kxs[c] = s_bk[lo];
                            act[c] = true;
                        }
                    }
                    uint32_t pre[WC];   // the key before the atomic (keys only decrease)
#pragma unroll
                    for (int c = 0; c < WC; ++c) pre[c] = (CHL_RELAX_PRECHECK && act[c]) ? __ldcg(&key[w[c]]) : kInf;
#pragma unroll
                    for (int c = 0; c < WC; ++c) {
                        if (!act[c]) continue;
                        const uint32_t nv = (!PLANT || ((kxs[c] & 1u) && rk[c] >= r)) ? 1u : 0u;
                        const uint64_t dd64 = (uint64_t)(kxs[c] >> 1) + len[c];
                        if (dd64 < 0x7FFFFFFFull) {
                            nk[c] = (uint32_t)dd64 * 2u + nv;
                            old[c] = pre[c] <= nk[c] ? pre[c] : atomicMin(&key[w[c]], nk[c]);
                            upd[c] = nk[c] < old[c];
                        } else {
                            a.ctl->err = 1;   // the reference asserts dd < infty
                        }
                    }
#pragma unroll
                    for (int c = 0; c < WC; ++c) {
                        const uint32_t dk = nk[c] >> 1;
                        const bool fresh = upd[c] && old[c] == kInf;
                        const bool in_win = upd[c] && dk < thr;
                        changed |= in_win;
                        // a new member: first touched inside the window, or a far
                        // vertex whose key drops into it (its far entry goes stale)
                        const bool join = in_win && (old[c] == kInf || (old[c] >> 1) >= thr);
                        const uint32_t jo = append_at(join, &sh.nm);
                        if (join) {
                            if (jo < a.n) {
                                memb[jo] = w[c];
                                mkey[jo] = kInf;
                            } else {
                                sh.err = 2;
                            }
                        }
                        const uint32_t vo = append_at(fresh, &sh.nvis);
                        if (fresh) {
                            if (vo < a.n) vis[vo] = w[c];
                            else sh.err = 2;
                        }
                        if (upd[c] && dk >= thr) pmin = min(pmin, dk);
                        const bool to_far = fresh && dk >= thr;
                        const uint32_t po = append_at(to_far, &sh.npile);
                        if (to_far) {
                            if (po < a.n) pile[po] = w[c];
                            else sh.err = 2;
                        }
                        if (PLANT && upd[c]) dql += (int)(nk[c] & 1u) - (old[c] == kInf ? 0 : (int)(old[c] & 1u));
                    }
                }
                if (PLANT) {
                    dql = __reduce_add_sync(kFull, dql);
                    if (lane == 0 && dql) atomicAdd(&sh.ql, dql);
                }
                __syncwarp();
            };

            while (true) {
                // passes over the window's members until no key below thr drops
                while (true) {
                    const uint32_t thr = sh.thr;
                    uint32_t *pile = piles + (size_t)sh.psel * a.n;
                    const uint32_t pass_n = sh.nm;
                    changed = false;
                    uint32_t nb = 0;
                    for (uint32_t b0 = wib * 32; b0 < pass_n; b0 += 32 * TW) {
                        const uint32_t i = b0 + lane;
                        bool need = false;
                        uint32_t x = 0, k = 0;
                        if (i < pass_n) {
                            x = memb[i];
                            k = __ldcg(&key[x]);
                            if (k != mkey[i]) {
                                mkey[i] = k;
                                // GLL trees do not expand vertices ranked above the root
                                need = PLANT || __ldg(&a.rank[x]) >= r;
                            }
                        }
                        const uint32_t bm = __ballot_sync(kFull, need);
                        if (need) {
                            const uint32_t at = nb + __popc(bm & lanemask_lt());
                            s_bv[at] = x;
                            s_bk[at] = k;
                        }
                        nb += __popc(bm);
                        __syncwarp();
                        if (nb > (uint32_t)kWinBatch - 32) {
                            relax(nb, thr, pile);
                            nb = 0;
                        }
                    }
                    if (nb) relax(nb, thr, pile);
                    __syncthreads();   // (a) every member counter and key update is done
                    if (tid == 0) sh.changed = 0;
                    __syncthreads();
                    if (__any_sync(kFull, changed) && lane == 0) sh.changed = 1;
                    __syncthreads();
                    if (!sh.changed) break;
                }
                // the window is final: its labels, from the final keys
                const uint32_t nm = sh.nm;
                int nv_final = 0;
                uint32_t lab = 0, dnv = 0;
                for (uint32_t b0 = wib * 32; b0 < nm; b0 += 32 * TW) {
                    const uint32_t i = b0 + lane;
                    bool emit = false;
                    uint32_t x = 0, k = 0;
                    if (i < nm) {
                        x = memb[i];
                        k = __ldcg(&key[x]);
                        if (PLANT) {
                            nv_final += (int)(k & 1u);
                            emit = (k & 1u) != 0;
                            if (emit) dnv = max(dnv, k >> 1);
                        } else {
                            emit = __ldg(&a.rank[x]) >= r;   // iteration_gll :92
                        }
                    }
                    const uint32_t em = __ballot_sync(kFull, emit);
                    if (em) {
                        if (n_emit + 32 > (uint32_t)kEmit) flush_labels();
                        if (emit) {
                            const uint32_t at = n_emit + __popc(em & lanemask_lt());
                            s_ek[at] = ((uint64_t)lidx(x, 1 - f, a.sides) << a.hub_bits) | (uint64_t)(r - a.r0);
                            s_ev[at] = k >> 1;
                        }
                        n_emit += __popc(em);
                        lab += __popc(em);
                    }
                }
                if (PLANT) {
                    nv_final = __reduce_add_sync(kFull, nv_final);
                    dnv = __reduce_max_sync(kFull, dnv);
                }
                const uint32_t pmin_w = __reduce_min_sync(kFull, pmin);
                pmin = kInf;
                if (lane == 0) {
                    if (PLANT && nv_final) atomicAdd(&sh.ql, -nv_final);
                    if (PLANT && dnv) atomicMax(&sh.dnv, dnv);
                    if (lab) atomicAdd(&sh.t_lab, lab);
                    if (pmin_w != kInf) atomicMin(&sh.lo, pmin_w);
                }
                __syncthreads();   // (b) ql, lo final for this window
                if (PLANT && sh.ql == 0) break;   // plant :95 early exit (all queued keys are via)
                __syncthreads();   // every thread has read ql
                if (tid == 0) {
                    sh.t_size += nm;
                    sh.nm = 0;
                    sh.kmin = kInf;
                    sh.kmax = 0;
                    // the width follows the size of the window just finished
                    if (sh.delta) {
                        if (nm > 2 * a.near_target) sh.delta = max(sh.delta / 2, 1u);
                        else if (nm < a.near_target / 2) sh.delta = sh.delta < 0x40000000u ? 2u * sh.delta : 0x7FFFFFFFu;
                    }
                }
                __syncthreads();
                if (sh.delta == 0) {
                    // first refill: the spread of the root's neighbours'
                    // distances (then adapted window by window)
                    const uint32_t np = sh.npile;
                    const uint32_t *pile = piles + (size_t)sh.psel * a.n;
                    uint32_t mn = kInf, mx = 0;
                    for (uint32_t i = tid; i < np; i += 32 * TW) {
                        const uint32_t k = __ldcg(&key[pile[i]]) >> 1;
                        mn = min(mn, k);
                        mx = max(mx, k);
                    }
                    mn = __reduce_min_sync(kFull, mn);
                    mx = __reduce_max_sync(kFull, mx);
                    if (lane == 0) {
                        atomicMin(&sh.kmin, mn);
                        atomicMax(&sh.kmax, mx);
                    }
                    __syncthreads();
                    if (tid == 0 && np > 0) {
                        sh.lo = sh.kmin;
                        sh.delta = max(sh.kmax - min(sh.kmin, sh.kmax), 1u);
                    }
                    __syncthreads();
                }
                // next window from the far pile: entries below the old
                // threshold are stale (they joined a window), entries below
                // the new one join, the rest move to the other pile buffer
                for (int pass = 0; pass < 4; ++pass) {
                    if (sh.nm != 0 || sh.npile == 0) break;
                    const uint32_t t_old = sh.thr;
                    const uint32_t thr = sat_add(sh.lo, sh.delta);
                    const uint32_t np = sh.npile;
                    const uint32_t *src = piles + (size_t)sh.psel * a.n;
                    uint32_t *dst = piles + (size_t)(sh.psel ^ 1u) * a.n;
                    __syncthreads();   // (d) every thread has read the window state
                    if (tid == 0) {
                        sh.npile2 = 0;
                        sh.kmin = kInf;
                    }
                    __syncthreads();
                    uint32_t kmin = kInf;
                    for (uint32_t b0 = wib * 32; b0 < np; b0 += 32 * TW) {
                        const uint32_t i = b0 + lane;
                        const bool valid = i < np;
                        const uint32_t x = valid ? src[i] : 0u;
                        const uint32_t k = valid ? (__ldcg(&key[x]) >> 1) : kInf;
                        const bool live = valid && k >= t_old;
                        const bool nr = live && k < thr;
                        const bool kp = live && !nr;
                        const uint32_t mo = append_at(nr, &sh.nm);
                        if (nr) {
                            memb[mo] = x;
                            mkey[mo] = kInf;
                        }
                        const uint32_t ko = append_at(kp, &sh.npile2);
                        if (kp) {
                            dst[ko] = x;
                            kmin = min(kmin, k);
                        }
                    }
                    kmin = __reduce_min_sync(kFull, kmin);
                    if (lane == 0 && kmin != kInf) atomicMin(&sh.kmin, kmin);
                    __syncthreads();   // (e) the refill pass is complete
                    if (tid == 0) {
                        sh.thr = thr;
                        sh.psel ^= 1u;
                        sh.npile = sh.npile2;
                        sh.lo = sh.kmin;
                    }
                    __syncthreads();
                }
                if (sh.nm == 0) {
                    if (sh.npile > 0 && tid == 0) a.ctl->err = 2;   // not reached: lo is exact from the second pass on
                    break;
                }
            }
            __syncthreads();
            if (sh.err && tid == 0) a.ctl->err = 2;
            if (PLANT && sh.nm) {
                // the early exit ended the tree inside this window: count its
                // members no farther than the last not-via vertex, the ones
                // the reference's Dijkstra pops before it stops
                // (distributed_memory/akiba.hpp:69-95)
                const uint32_t nm = min(sh.nm, a.n), dl = sh.dnv;
                uint32_t c = 0;
                for (uint32_t i = tid; i < nm; i += 32 * TW) c += (__ldcg(&key[memb[i]]) >> 1) <= dl ? 1u : 0u;
                c = __reduce_add_sync(kFull, c);
                if (lane == 0 && c) atomicAdd(&sh.t_size, c);
            }
            __syncthreads();
            const uint32_t nvis = min(sh.nvis, a.n);
            for (uint32_t k = tid; k < nvis; k += 32 * TW) __stcg(&key[vis[k]], kInf);
            __syncthreads();
        }
        flush_labels();
        if (tid == 0) {
            c_vis += sh.t_size;
            a.tree_size[r - a.r0] = sh.t_size;
            a.tree_labels[r - a.r0] = sh.t_lab;
            finish_root(a, sh.nominal != 0);
        }
        __syncthreads();
    }
    d_hi = __reduce_max_sync(kFull, d_hi);
    if (lane == 0) {
        atomicAdd(&a.ctl->visits, c_vis);
        atomicAdd(&a.ctl->arcs, c_arcs);
        if (d_hi) atomicMax(&a.ctl->max_dist, d_hi);
    }
}

using TreeKernel = void (*)(TreeArgs);

template <bool UNIT, bool PLANT>
TreeKernel window_kernel_tw(uint32_t tw) {
    switch (tw) {
    case 1: return window_kernel<UNIT, PLANT, 1>;
    case 2: return window_kernel<UNIT, PLANT, 2>;
    case 8: return window_kernel<UNIT, PLANT, 8>;
    default: return window_kernel<UNIT, PLANT, 4>;
    }
}

TreeKernel window_kernel_for(bool unit, bool plant, uint32_t tw) {
    if (unit) return plant ? window_kernel_tw<true, true>(tw) : window_kernel_tw<true, false>(tw);
    return plant ? window_kernel_tw<false, true>(tw) : window_kernel_tw<false, false>(tw);
}

__global__ void fat_arcs(uint64_t m, const uint2 *arc, const uint32_t *rank, const uint32_t *win, uint4 *out) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 a = arc[e];
        out[e] = make_uint4(a.x, a.y, rank[a.x], win[a.x]);
    }
}

__global__ void fat_heads(uint64_t m, const uint32_t *head, const uint32_t *rank, uint2 *out) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t h = head[e];
        out[e] = make_uint2(h, rank[h]);
    }
}

// ---------------------------------------------------------- commit chain

// Count new labels per label list (sorted keys).
__global__ void count_keys(const uint64_t *keys, const unsigned long long *d_n,
                           unsigned long long cap, int hub_bits, uint32_t *cnt) {
    unsigned long long n = *d_n;
    if (n > cap) n = cap;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < n; i += (unsigned long long)gridDim.x * blockDim.x)
        atomicAdd(&cnt[keys[i] >> hub_bits], 1u);
}

// GLL clean (shared_memory/akiba.hpp:197-208 with Labeling::clean_cover,
// shared_memory/labeling.hpp:78-88): a new label (h, d) of list (u, s) is
// dropped if some hub h' < h appears in both the new L(u, s) and the new
// L(order[h], !s) with d' + d'' <= d.  Only this superstep's labels take
// part; earlier labels were already used for pruning.
__global__ void clean_mark(const uint64_t *keys, const uint32_t *vals,
                           const unsigned long long *d_n, unsigned long long cap,
                           int hub_bits, uint32_t r0, const uint64_t *pre,
                           const uint32_t *order, const uint32_t *rank, int sides,
                           uint32_t *keep) {
    unsigned long long n = *d_n;
    if (n > cap) n = cap;
    const uint64_t mask = (1ull << hub_bits) - 1;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < n; i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        const uint32_t x = (uint32_t)(k >> hub_bits);
        const uint32_t hrel = (uint32_t)(k & mask);
        const uint32_t d = vals[i];
        const uint32_t hv = order[r0 + hrel];
        uint32_t y;
        if (sides == 1) {
            y = hv;
        } else {
            const uint32_t s = x & 1u;
            y = 2 * hv + (1u - s);
        }
        uint64_t a = pre[x], ae = pre[x + 1];
        uint64_t b = pre[y], be = pre[y + 1];
        bool covered = false;
        while (a < ae && b < be) {
            const uint32_t ha = (uint32_t)(keys[a] & mask), hb = (uint32_t)(keys[b] & mask);
            if (ha >= hrel || hb >= hrel) break;
            if (ha == hb) {
                if (vals[a] + vals[b] <= d) {
                    covered = true;
                    break;
                }
                ++a;
                ++b;
            } else if (ha < hb) {
                ++a;
            } else {
                ++b;
            }
        }
        keep[i] = covered ? 0u : 1u;
    }
}

__global__ void compact_kept(const uint64_t *kin, const uint32_t *vin, const uint32_t *keep,
                             const uint64_t *kpre, const unsigned long long *d_n,
                             unsigned long long cap, uint64_t *kout, uint32_t *vout,
                             unsigned long long *d_nkeep) {
    unsigned long long n = *d_n;
    if (n > cap) n = cap;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < n; i += (unsigned long long)gridDim.x * blockDim.x) {
        if (keep[i]) {
            const uint64_t p = kpre[i];
            kout[p] = kin[i];
            vout[p] = vin[i];
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *d_nkeep = kpre[cap];
}

// new_off[x] = old_off[x] + pre[x]  (pre = exclusive scan of new counts)
__global__ void merge_offsets(const uint64_t *old_off, const uint64_t *pre, uint64_t *new_off,
                              uint32_t nl) {
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x <= nl; x += gridDim.x * blockDim.x)
        new_off[x] = old_off[x] + pre[x];
}

// Copy every committed list to its new position (one warp per list).
__global__ void copy_old_lists(const uint64_t *old_off, const uint2 *old_ent,
                               const uint64_t *new_off, uint2 *new_ent, uint32_t nl) {
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t x = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); x < nl; x += warps) {
        const uint64_t b = old_off[x], e = old_off[x + 1], nb = new_off[x];
        for (uint64_t k = b + lane_id(); k < e; k += 32) new_ent[nb + (k - b)] = old_ent[k];
    }
}

// Append the sorted new labels behind each list's committed part.
__global__ void place_new(const uint64_t *keys, const uint32_t *vals,
                          const unsigned long long *d_n, unsigned long long cap, int hub_bits,
                          uint32_t r0, const uint64_t *pre, const uint64_t *old_off,
                          const uint64_t *new_off, uint2 *new_ent) {
    unsigned long long n = *d_n;
    if (n > cap) n = cap;
    const uint64_t mask = (1ull << hub_bits) - 1;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < n; i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        const uint32_t x = (uint32_t)(k >> hub_bits);
        const uint64_t dst = new_off[x] + (old_off[x + 1] - old_off[x]) + (i - pre[x]);
        new_ent[dst] = make_uint2(r0 + (uint32_t)(k & mask), vals[i]);
    }
}

// ---- distance-ordered copy of the committed labels (prune tests only)
// Lists in the same CSR offsets, entries ordered by (distance, hub): an
// entry (h, dd) of L(u) can only witness d(r, u) if dd <= d(r, u), so a
// prune test stops at the first chunk whose entries all exceed d(r, u).

__device__ __forceinline__ bool ent_less(uint2 a, uint2 b) { return a.y < b.y || (a.y == b.y && a.x < b.x); }

// new labels sorted by (list, hub) -> keys (list << 32 | dist), values hub
__global__ void dist_keys(const uint64_t *keys, const uint32_t *vals, const unsigned long long *d_n,
                          unsigned long long cap, int hub_bits, int dist_bits, uint32_t r0, uint64_t *k2,
                          uint32_t *v2) {
    unsigned long long n = *d_n;
    if (n > cap) n = cap;
    const uint64_t mask = (1ull << hub_bits) - 1;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        k2[i] = ((k >> hub_bits) << dist_bits) | vals[i];
        v2[i] = r0 + (uint32_t)(k & mask);
    }
}

// Merge, per list, the committed distance-ordered entries with the new ones
// (sorted by (list, dist) in k2/v2, the distance in k2's low dist_bits bits,
// the list's run at [pre[x], pre[x+1])).
// One warp per list; every entry's final slot is its rank in the other run
// (binary search) plus its own index.  Ties in distance order by hub.
__global__ void merge_dist_lists(const uint64_t *old_off, const uint2 *old_ent, const uint64_t *new_off,
                                 const uint64_t *pre, const uint64_t *k2, const uint32_t *v2, uint2 *out,
                                 uint32_t nl, int dist_bits) {
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    const uint64_t dmask = (1ull << dist_bits) - 1;
    for (uint32_t x = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); x < nl; x += warps) {
        const uint64_t ob = old_off[x], oe = old_off[x + 1], nb = new_off[x];
        const uint64_t pb = pre[x], pe = pre[x + 1];
        const uint64_t no = oe - ob, nn = pe - pb;
        for (uint64_t i = lane_id(); i < no; i += 32) {
            const uint2 e = old_ent[ob + i];
            uint64_t lo = 0, hi = nn;   // new entries before e
            while (lo < hi) {
                const uint64_t mid = (lo + hi) >> 1;
                const uint2 m = make_uint2(v2[pb + mid], (uint32_t)(k2[pb + mid] & dmask));
                if (ent_less(m, e)) lo = mid + 1;
                else hi = mid;
            }
            out[nb + i + lo] = e;
        }
        for (uint64_t t = lane_id(); t < nn; t += 32) {
            const uint2 e = make_uint2(v2[pb + t], (uint32_t)(k2[pb + t] & dmask));
            uint64_t lo = 0, hi = no;   // old entries before e
            while (lo < hi) {
                const uint64_t mid = (lo + hi) >> 1;
                if (ent_less(old_ent[ob + mid], e)) lo = mid + 1;
                else hi = mid;
            }
            out[nb + t + lo] = e;
        }
    }
}

// Largest tree/label ratio over the superstep's roots (hybrid switch rule,
// distributed_memory/akiba.hpp:297-303), kept as an exact fraction.
__global__ void ratio_max(const uint32_t *tsize, const uint32_t *tlab, const unsigned long long *next_root,
                          uint32_t r0, uint32_t r_end, BuildCtl *ctl) {
    unsigned long long r1 = *next_root;
    if (r1 > r_end) r1 = r_end;
    const uint32_t cnt = (uint32_t)(r1 - r0);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        // pack ratio as a double's bits (positive doubles order like integers)
        const double ratio = tlab[i] ? (double)tsize[i] / (double)tlab[i] : 1e300;
        atomicMax(&ctl->max_ratio_num, (unsigned long long)__double_as_longlong(ratio));
    }
}

// Longest label list (sizes the root-label staging of the next superstep).
__global__ void max_list_len(const uint64_t *off, uint32_t nl, unsigned long long *out) {
    unsigned long long mx = 0;
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < nl; x += gridDim.x * blockDim.x)
        mx = max(mx, (unsigned long long)(off[x + 1] - off[x]));
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(kFull, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, mx);
}

// max and sum of per-root tree sizes of a superstep (diagnostics)
__global__ void tree_stats(const uint32_t *tsize, uint32_t cnt, unsigned long long *out2) {
    unsigned long long mx = 0, sm = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        mx = max(mx, (unsigned long long)tsize[i]);
        sm += tsize[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        mx = max(mx, __shfl_xor_sync(kFull, mx, o));
        sm += __shfl_xor_sync(kFull, sm, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&out2[0], mx);
        atomicAdd(&out2[1], sm);
    }
}

inline int bits_for(uint64_t x) {   // bits needed to represent values < x
    int b = 0;
    while (b < 64 && (1ull << b) < x) ++b;
    return b < 1 ? 1 : b;
}

template <typename T>
int dalloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error(std::string("device allocation failed: ") + cudaGetErrorString(e));
        return CHL_ERR_OOM;
    }
    return CHL_OK;
}

struct DevGraph {
    uint64_t *off[2] = {nullptr, nullptr};
    uint2 *arc[2] = {nullptr, nullptr};
    uint32_t *head[2] = {nullptr, nullptr};
    uint32_t *win[2] = {nullptr, nullptr};   // shortest arc into v, per direction
    void release() {
        // side 1 may alias side 0 (symmetric graphs): free each buffer once
        if (off[1] != off[0]) cudaFree(off[1]);
        if (arc[1] != arc[0]) cudaFree(arc[1]);
        if (head[1] != head[0]) cudaFree(head[1]);
        if (win[1] != win[0]) cudaFree(win[1]);
        cudaFree(off[0]);
        cudaFree(arc[0]);
        cudaFree(head[0]);
        cudaFree(win[0]);
        for (int s = 0; s < 2; ++s) {
            off[s] = nullptr;
            arc[s] = nullptr;
            head[s] = nullptr;
            win[s] = nullptr;
        }
    }
};

int upload_graph(const chl_graph *g, DevGraph &dg, cudaStream_t st) {
    const int nsides = g->symmetric ? 1 : 2;
    for (int s = 0; s < nsides; ++s) {
        const int src = g->symmetric ? 1 : s;
        const uint64_t m = g->off[src][g->n];
        int rc = dalloc(&dg.off[s], (size_t)g->n + 1);
        if (rc) return rc;
        CHL_CUDA(cudaMemcpyAsync(dg.off[s], g->off[src].data(), ((size_t)g->n + 1) * 8,
                                 cudaMemcpyHostToDevice, st));
        if (g->unit) {
            rc = dalloc(&dg.head[s], m);
            if (rc) return rc;
            CHL_CUDA(cudaMemcpyAsync(dg.head[s], g->head[src].data(), m * 4,
                                     cudaMemcpyHostToDevice, st));
        } else {
            std::vector<uint2> pk(m);
            for (uint64_t i = 0; i < m; ++i)
                pk[i] = make_uint2(g->head[src][i], (uint32_t)g->len[src][i]);
            rc = dalloc(&dg.arc[s], m);
            if (rc) return rc;
            CHL_CUDA(cudaMemcpy(dg.arc[s], pk.data(), m * 8, cudaMemcpyHostToDevice));
        }
    }
    for (int s = 0; s < nsides; ++s) {
        const int src = g->symmetric ? 1 : s;
        std::vector<uint32_t> w(g->n, 0x7FFFFFFFu);
        const uint64_t m = g->off[src][g->n];
        for (uint64_t i = 0; i < m; ++i) {
            const uint32_t h = g->head[src][i];
            w[h] = std::min<uint32_t>(w[h], (uint32_t)g->len[src][i]);
        }
        int rc = dalloc(&dg.win[s], (size_t)g->n);
        if (rc) return rc;
        CHL_CUDA(cudaMemcpy(dg.win[s], w.data(), (size_t)g->n * 4, cudaMemcpyHostToDevice));
    }
    if (nsides == 1) {
        dg.off[1] = dg.off[0];
        dg.arc[1] = dg.arc[0];
        dg.head[1] = dg.head[0];
        dg.win[1] = dg.win[0];
    }
    return CHL_OK;
}

}  // namespace

void graph_release_device(chl_graph *g) {
    if (g && g->dev) {
        DevGraph *d = (DevGraph *)g->dev;
        d->release();
        delete d;
        g->dev = nullptr;
    }
}

namespace {

struct Build {
    // sizes
    uint32_t n = 0;
    int sides = 1;
    uint32_t nl = 0;       // number of label lists on the device
    int hub_bits = 0;
    int key_bits = 0;
    // device buffers
    DevGraph own;                   // graph uploaded for this build only
    const DevGraph *dg = nullptr;
    uint32_t *order = nullptr, *rank = nullptr;
    uint64_t *off_a = nullptr, *off_b = nullptr;
    uint2 *ent_a = nullptr, *ent_b = nullptr;
    uint64_t ent_cap_a = 0, ent_cap_b = 0;
    uint2 *dent_a = nullptr, *dent_b = nullptr;   // (distance, hub)-ordered copies
    uint64_t dent_cap_a = 0, dent_cap_b = 0;
    uint64_t *nk0 = nullptr, *nk1 = nullptr;
    uint32_t *nv0 = nullptr, *nv1 = nullptr;
    uint64_t new_cap = 0;
    uint32_t *cnt = nullptr;
    uint64_t *pre = nullptr;
    uint32_t *keep = nullptr;
    uint64_t *kpre = nullptr;
    uint32_t *tsize = nullptr, *tlab = nullptr;
    uint32_t *ws_all = nullptr;   // tree workspace (both kernels' layouts)
    uint32_t *ws_key = nullptr, *ws_vis = nullptr, *ws_front = nullptr;   // batch_kernel views
    uint32_t win_trees = 0, win_tw = 4;   // window_kernel: trees (blocks) and warps per tree
    int ws_layout = 0;   // 1: batch_kernel keys all INF, 2: window_kernel keys all INF
    BuildCtl *ctl = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    cudaStream_t st = nullptr;
    uint32_t warps = 0;   // warps the schedule is sized for
    uint32_t slots = 0;   // warp slots launched by batch_kernel
    uint32_t hash_max = 2048;                // largest root hash table (slots)
    uint4 *farc[2] = {nullptr, nullptr};     // (head, length, rank[head], win[head]) per arc
    uint2 *fhead[2] = {nullptr, nullptr};    // (head, rank[head]) per arc, unit lengths
    cudaGraphExec_t commit_exec = nullptr;   // captured commit chain
    uint64_t graph_launches = 0;

    ~Build() {
        if (commit_exec) cudaGraphExecDestroy(commit_exec);
        if (farc[1] != farc[0]) cudaFree(farc[1]);
        if (fhead[1] != fhead[0]) cudaFree(fhead[1]);
        cudaFree(farc[0]);
        cudaFree(fhead[0]);
        own.release();
        cudaFree(order);
        cudaFree(rank);
        cudaFree(off_a);
        cudaFree(off_b);
        cudaFree(ent_a);
        cudaFree(ent_b);
        cudaFree(dent_a);
        cudaFree(dent_b);
        cudaFree(nk0);
        cudaFree(nk1);
        cudaFree(nv0);
        cudaFree(nv1);
        cudaFree(cnt);
        cudaFree(pre);
        cudaFree(keep);
        cudaFree(kpre);
        cudaFree(tsize);
        cudaFree(tlab);
        cudaFree(ws_all);
        cudaFree(ctl);
        cudaFree(tmp);
        if (st) cudaStreamDestroy(st);
    }
};

// New-label buffers with room for `need` entries (their contents are dead
// between supersteps).  An overflowed superstep counts every label it tried
// to append, so its re-run needs exactly that many: no doubling.
int grow_new(Build &b, uint64_t need) {
    if (need <= b.new_cap) return CHL_OK;
    const uint64_t cap = need;
    cudaFree(b.nk0);
    cudaFree(b.nk1);
    cudaFree(b.nv0);
    cudaFree(b.nv1);
    cudaFree(b.keep);
    cudaFree(b.kpre);
    b.nk0 = b.nk1 = nullptr;
    b.nv0 = b.nv1 = nullptr;
    b.keep = nullptr;
    b.kpre = nullptr;
    int rc;
    if ((rc = dalloc(&b.nk0, cap)) || (rc = dalloc(&b.nk1, cap)) || (rc = dalloc(&b.nv0, cap)) ||
        (rc = dalloc(&b.nv1, cap)) || (rc = dalloc(&b.keep, cap)) || (rc = dalloc(&b.kpre, cap + 1)))
        return rc;
    b.new_cap = cap;
    size_t need_tmp = std::max(radix_tmp_bytes(), scan_tmp_bytes(std::max<uint64_t>(cap, b.nl)));
    if (need_tmp > b.tmp_bytes) {
        cudaFree(b.tmp);
        b.tmp = nullptr;
        if ((rc = dalloc((char **)&b.tmp, need_tmp))) return rc;
        b.tmp_bytes = need_tmp;
    }
    return CHL_OK;
}

int ensure_ent(uint2 **p, uint64_t *cap, uint64_t need) {
    if (need <= *cap) return CHL_OK;
    uint64_t c = std::max<uint64_t>(need, *cap + *cap / 2);
    cudaFree(*p);
    *p = nullptr;
    // 4 spare entries: the prune test reads 16-byte pairs of entries
    int rc = dalloc(p, c + 4);
    if (rc) return rc;
    *cap = c;
    return CHL_OK;
}

}  // namespace

// Host orchestration of one build.
int build_labels(const chl_graph *g, const uint32_t *order_h, uint32_t n,
                 const chl_build_opts *opts_in, chl_labels **out) {
    chl_build_opts opts;
    if (opts_in) opts = *opts_in;
    else chl_build_opts_default(&opts);
    if (g && opts.autotune) apply_tuned_schedule(g, opts);
    if (!g || !order_h || !out || n != g->n) {
        set_error("order size must equal the number of graph vertices");
        return CHL_ERR_INVALID;
    }
    if (g->min_len < 1) {
        set_error("arc lengths must be positive (the reference asserts dd > d)");
        return CHL_ERR_INVALID;
    }
    // order must be a permutation
    std::vector<uint32_t> rank_h(n, kInf);
    for (uint32_t i = 0; i < n; ++i) {
        if (order_h[i] >= n || rank_h[order_h[i]] != kInf) {
            set_error("order is not a permutation of the vertex ids");
            return CHL_ERR_INVALID;
        }
        rank_h[order_h[i]] = i;
    }
    auto t_wall0 = std::chrono::steady_clock::now();
    Build b;
    b.n = n;
    b.sides = g->symmetric ? 1 : 2;
    b.nl = g->symmetric ? n : 2 * n;
    b.hub_bits = bits_for(std::max<uint64_t>(n, 2));
    b.key_bits = b.hub_bits + bits_for((uint64_t)b.nl + 1);
    if (b.key_bits > 64) return CHL_ERR_INVALID;
    CHL_CUDA(cudaStreamCreateWithFlags(&b.st, cudaStreamNonBlocking));
    cudaEvent_t ev0, ev1, ev_a, ev_b, ev_up;
    CHL_CUDA(cudaEventCreate(&ev_up));
    CHL_CUDA(cudaEventCreate(&ev0));
    CHL_CUDA(cudaEventCreate(&ev1));
    CHL_CUDA(cudaEventCreate(&ev_a));
    CHL_CUDA(cudaEventCreate(&ev_b));
    struct EvGuard {
        cudaEvent_t e[5];
        ~EvGuard() {
            for (auto x : e) cudaEventDestroy(x);
        }
    } evg{{ev0, ev1, ev_a, ev_b, ev_up}};

    CHL_CUDA(cudaEventRecord(ev0, b.st));
    int rc;
    if (g->dev) {
        b.dg = (const DevGraph *)g->dev;
    } else {
        if ((rc = upload_graph(g, b.own, b.st))) return rc;
        b.dg = &b.own;
    }
    if ((rc = dalloc(&b.order, n)) || (rc = dalloc(&b.rank, n))) return rc;
    CHL_CUDA(cudaMemcpyAsync(b.order, order_h, (size_t)n * 4, cudaMemcpyHostToDevice, b.st));
    CHL_CUDA(cudaMemcpyAsync(b.rank, rank_h.data(), (size_t)n * 4, cudaMemcpyHostToDevice, b.st));
    CHL_CUDA(cudaEventRecord(ev_up, b.st));

    // committed label CSR (double buffered)
    if ((rc = dalloc(&b.off_a, (size_t)b.nl + 1)) || (rc = dalloc(&b.off_b, (size_t)b.nl + 1)))
        return rc;
    CHL_CUDA(cudaMemsetAsync(b.off_a, 0, ((size_t)b.nl + 1) * 8, b.st));
    if ((rc = ensure_ent(&b.ent_a, &b.ent_cap_a, 1)) || (rc = ensure_ent(&b.dent_a, &b.dent_cap_a, 1))) return rc;
    if ((rc = dalloc(&b.cnt, (size_t)b.nl + 1)) || (rc = dalloc(&b.pre, (size_t)b.nl + 2))) return rc;
    CHL_CUDA(cudaMemsetAsync(b.cnt, 0, ((size_t)b.nl + 1) * 4, b.st));
    if ((rc = dalloc(&b.tsize, n)) || (rc = dalloc(&b.tlab, n))) return rc;
    if ((rc = dalloc(&b.ctl, 1))) return rc;
    if ((rc = grow_new(b, opts.label_cap ? (uint64_t)opts.label_cap : std::max<uint64_t>(4ull * n, 1u << 20))))
        return rc;

    // heavy-tailed degree distribution: the largest out-degree above 32
    // times the mean (scale-free graphs); bounded-degree (road-like)
    // otherwise.  Several schedule defaults below depend on it.
    bool heavy_tail = false;
    {
        uint64_t maxdeg = 0;
        for (uint32_t v = 0; v < n; ++v) maxdeg = std::max<uint64_t>(maxdeg, g->off[1][v + 1] - g->off[1][v]);
        const double avgdeg = n ? (double)g->off[1][n] / n : 0.0;
        heavy_tail = maxdeg > 32.0 * std::max(1.0, avgdeg);
    }
    // workspace: one slot per resident warp
    const int sms = device_sms();
    const bool unit = g->unit;
    size_t free_b = 0, total_b = 0;
    CHL_CUDA(cudaMemGetInfo(&free_b, &total_b));
    unsigned long long prep_kernels = 0;
    {
        // arcs with their head's rank for this order
        const int nsides_g = g->symmetric ? 1 : 2;
        for (int s = 0; s < nsides_g; ++s) {
            const int src = g->symmetric ? 1 : s;
            const uint64_t m = g->off[src][n];
            const int grid = std::max(1, sms * 8);
            if (unit) {
                if ((rc = dalloc(&b.fhead[s], std::max<uint64_t>(m, 1)))) return rc;
                fat_heads<<<grid, 256, 0, b.st>>>(m, b.dg->head[s], b.rank, b.fhead[s]);
            } else {
                if ((rc = dalloc(&b.farc[s], std::max<uint64_t>(m, 1)))) return rc;
                fat_arcs<<<grid, 256, 0, b.st>>>(m, b.dg->arc[s], b.rank, b.dg->win[s], b.farc[s]);
            }
            CHL_CUDA(cudaGetLastError());
            ++prep_kernels;
        }
        if (nsides_g == 1) {
            b.farc[1] = b.farc[0];
            b.fhead[1] = b.fhead[0];
        }
    }
    // key, vis and three queue arrays per warp slot (the 32-bit-key size
    // sets the schedule's warp count; the slots below use the real one)
    const size_t per_slot = (size_t)n * 20;
    uint32_t want = (uint32_t)sms * 48;   // 12 blocks of 4 warps per SM at most
    if (opts.max_warps) want = std::min<uint32_t>(want, opts.max_warps);
    const size_t ws_budget = free_b / 3;
    uint32_t fit = (uint32_t)std::max<size_t>(1, ws_budget / std::max<size_t>(per_slot, 1));
    b.warps = std::max<uint32_t>(kWarpsPerBlock, std::min(want, fit));
    b.warps = (b.warps / kWarpsPerBlock) * kWarpsPerBlock;
    // Only the blocks resident from the start build trees: a block leaves
    // when no root is left for the superstep, and every refusal of a root is
    // final for it.  The grid and the workspace cover those alone (b.warps
    // still sets the first superstep's size).
    int nbo = 0;
    CHL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &nbo, unit ? batch_kernel<true, true> : batch_kernel<false, true>, kWarpsPerBlock * 32, 0));
    nbo = std::max(nbo, 1);
    b.slots = std::min(b.warps, (uint32_t)nbo * (uint32_t)sms * kWarpsPerBlock);
    {
        // weighted graphs hold 64-bit keys: 24 bytes per vertex and slot
        const size_t slot_bytes = (size_t)n * (unit ? 20 : 24);
        const uint32_t fit_slots = (uint32_t)std::max<size_t>(kWarpsPerBlock, ws_budget / std::max<size_t>(slot_bytes, 1));
        b.slots = std::max<uint32_t>(kWarpsPerBlock, (std::min(b.slots, fit_slots) / kWarpsPerBlock) * kWarpsPerBlock);
    }
    // window kernel (first superstep): one tree per block of win_tw warps
    // (auto: 8 on heavy-tailed graphs, 4 otherwise), as many trees as are
    // resident, 6 n words each
    b.win_tw = opts.window_warps ? opts.window_warps : (heavy_tail ? 8 : 4);
    if (b.win_tw != 1 && b.win_tw != 2 && b.win_tw != 4 && b.win_tw != 8) {
        set_error("window_warps must be 0, 1, 2, 4 or 8");
        return CHL_ERR_INVALID;
    }
    {
        // the occupancy query counts a block's dynamic shared memory only up
        // to the kernel's current limit (48 KB by default): raise it first
        const int wsm = (int)window_smem(b.win_tw);
        for (int p = 0; p < 2; ++p)
            CHL_CUDA(cudaFuncSetAttribute(window_kernel_for(unit, p != 0, b.win_tw),
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, wsm));
        int nbw = 0;
        CHL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbw, window_kernel_for(unit, true, b.win_tw),
                                                                 b.win_tw * 32, wsm));
        const uint64_t fit_trees = std::max<uint64_t>(1, ws_budget / std::max<uint64_t>(24ull * n, 1));
        b.win_trees = (uint32_t)std::min<uint64_t>((uint64_t)std::max(nbw, 1) * sms, fit_trees);
    }
    // one workspace for both layouts: batch_kernel's key (two words on
    // weighted graphs), vis and queue arrays per warp slot (5 or 6 n words),
    // window_kernel's 6 n words per tree
    const size_t key_words = unit ? 1 : 2;
    const size_t ws_words = std::max((size_t)b.slots * (4 + key_words) * n, (size_t)b.win_trees * 6 * n);
    if ((rc = dalloc(&b.ws_all, ws_words))) return rc;
    b.ws_key = b.ws_all;
    b.ws_vis = b.ws_all + (size_t)b.slots * key_words * n;
    b.ws_front = b.ws_vis + (size_t)b.slots * n;
    b.ws_layout = 0;   // set before each tree launch
    {
        // root hash slots: at most 2048, and within CHL_SMEM_CAP_KB of shared
        // memory per block (measured on the 1024-square grid: 2048 slots at 2
        // resident blocks per SM beat 1024 slots at 3 by 1.3x -- entries past
        // half the table are searched in global memory)
        int max_smem = 0;
        CHL_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, 0));
        const size_t smem_cap = std::min<size_t>((size_t)max_smem, CHL_SMEM_CAP_KB * 1024);
        uint32_t t = 64;
        while (2 * t <= 2048 && kWarpsPerBlock * batch_smem_per_warp(2 * t) <= smem_cap) t *= 2;
        b.hash_max = t;
    }

    // superstep loop
    // label budget per superstep (the reference's sf * N); auto: 32 on
    // heavy-tailed graphs, 1024 on road-like ones.  On road-like graphs a
    // superstep lasts as long as its largest tree, so fewer, larger
    // supersteps pay off once the near/far queue and the distance cutoff
    // keep the less-pruned trees cheap; from 1024 on the growth schedule,
    // not the budget, sets their size (measured on the 512/1024-square
    // grids: 1024 and unbounded within 1%, 128 1.27x slower; RMAT scale
    // 20: 16-64 within 3%)
    const double sf = opts.sf > 0 ? opts.sf : (heavy_tail ? 32.0 : 1024.0);
    // label_limit = sf * N counts both sides' labels (shared_memory/hhl.cpp:65);
    // a symmetric build stores one side.
    const unsigned long long budget_base =
        (unsigned long long)std::max(1.0, sf * (double)n / (b.sides == 1 ? 2.0 : 1.0));
    if (opts.label_cap == 0) {
        // Room for every new label of a superstep: the budget plus what the
        // trees still running when it is spent can add (at most sides * n
        // each), so that a superstep does not overflow and run twice.  At
        // most a quarter of the free memory (36 bytes per entry: two key and
        // two value arrays for the sort, the clean's flags and prefix);
        // beyond that an overflow re-runs the superstep's root range.
        size_t fr = 0, tot = 0;
        CHL_CUDA(cudaMemGetInfo(&fr, &tot));
        const uint64_t want = (uint64_t)budget_base + (uint64_t)std::max(b.slots, b.win_trees) * b.sides * n;
        const uint64_t fit = (uint64_t)(fr / 4 / 36);
        if ((rc = grow_new(b, std::min(want, fit)))) return rc;
    }
    bool do_plant = opts.mode != CHL_MODE_GLL;
    bool switch_open = opts.mode == CHL_MODE_HYBRID;
    uint32_t r0 = 0;
    uint64_t committed = 0;
    uint32_t supersteps = 0, plant_roots = 0;
    unsigned long long visits = 0, reads = 0, arcs = 0, launches = 0, kernels = prep_kernels;
    double tree_ms = 0, sort_ms = 0, commit_ms = 0;
    uint32_t max_list = 0;   // longest committed list
    float step_tree_ms = 0;
    uint32_t step_slots = 0;   // warp slots of the last tree launch
    // Superstep schedule: superstep k covers roots [r0, r0 + size) with
    // size = clamp(growth * r0, first, n) -- small while the top hubs are not
    // yet committed (their labels prune everything later), geometric after.
    // The label budget sf * n (the reference's label_limit) also ends a
    // superstep early.
    // label-correcting windows of the first superstep's trees: about this
    // many vertices per window (1: IN-criterion rounds instead).  Auto: on
    // heavy-tailed graphs, whose first trees are huge BFS-like searches
    // (RMAT scale 20: 1.4x faster builds with 8 warps per tree); off on
    // road-like ones (the 1024-square grid: 3.81-4.1 s with windows of
    // 256-4096 vertices against 3.83 s without)
    const uint32_t win_target = opts.window_target ? opts.window_target : (heavy_tail ? 1024u : 1u);
    // Schedule defaults from graph statistics (measured on RMAT scale 18/20
    // and 512/1024-square grids): heavy-tailed degree distributions start
    // with one root per resident window tree (RMAT scale 20: 608 roots,
    // 2.15 s against 2.28 s with 256 and 2.34 s with 1024) and double, so the
    // hubs commit before the bulk of the trees while the early supersteps
    // still fill the GPU; bounded-degree (road-like) graphs start with two
    // roots per warp of the schedule (the 1024-square grid: 1.15x faster than
    // one) and grow by half of the committed prefix.
    const uint32_t auto_first = heavy_tail ? (win_target > 1 ? std::max<uint32_t>(64u, b.win_trees) : 1024u)
                                           : std::max<uint32_t>(64u, 2 * b.warps);
    const double auto_growth = heavy_tail ? 2.0 : 0.5;
    // phase switch ratio (the reference's -ps, default 1024): auto 8 on
    // heavy-tailed graphs (RMAT scale 20: pruned GLL supersteps after the
    // first are faster than PLaNT trees there)
    const double ps = opts.ps > 0 ? opts.ps : (heavy_tail ? 8.0 : 1024.0);
    const uint32_t first = opts.first_superstep ? opts.first_superstep : auto_first;
    const double growth = opts.growth > 0 ? opts.growth : auto_growth;
    while (r0 < n && (opts.root_limit == 0 || r0 < opts.root_limit)) {
        const uint32_t r_begin = r0;
        const bool plant_now = do_plant;
        const unsigned long long budget = budget_base;
        uint64_t size = std::max<uint64_t>(first, (uint64_t)(growth * (double)r0));
        uint32_t r_end = (uint32_t)std::min<uint64_t>(n, (uint64_t)r0 + size);
        if (opts.root_limit) r_end = std::min<uint32_t>(r_end, opts.root_limit);
        BuildCtl hc;
        bool rerun = false;
        uint32_t step_reruns = 0;
        // root hash table: a power of two at least twice the longest committed
        // list, within the occupancy-preserving size (entries beyond half the
        // table are searched in the global list)
        uint32_t hash_slots = 64;
        while (hash_slots < 2 * std::max<uint32_t>(max_list, 32) && 2 * hash_slots <= b.hash_max) hash_slots *= 2;
        const size_t smem = kWarpsPerBlock * batch_smem_per_warp(hash_slots);
        while (true) {
            std::memset(&hc, 0, sizeof(hc));
            hc.next_root = r0;
            CHL_CUDA(cudaMemcpyAsync(b.ctl, &hc, sizeof(hc), cudaMemcpyHostToDevice, b.st));
            TreeArgs ta;
            ta.n = n;
            ta.sides = b.sides;
            for (int s = 0; s < 2; ++s) {
                ta.g_off[s] = b.dg->off[s];
                ta.g_farc[s] = b.farc[s];
                ta.g_fhead[s] = b.fhead[s];
            }
            ta.order = b.order;
            ta.rank = b.rank;
            ta.l_off = b.off_a;
            ta.l_ent = b.ent_a;
            ta.l_dent = b.dent_a;
            ta.r0 = r0;
            ta.r_end = r_end;
            // work-conserving extension: up to ext x the nominal size while
            // nominal trees run; none on a rerun
            uint32_t ext = opts.superstep_extend == 0 ? (heavy_tail ? 1u : 4u)
                                                      : (uint32_t)std::max(1, opts.superstep_extend);
            if (rerun) ext = 1;
            ta.r_hard = (uint32_t)std::min<uint64_t>(n, (uint64_t)r0 + (uint64_t)ext * (r_end - r0));
            if (opts.root_limit) ta.r_hard = std::min<uint32_t>(ta.r_hard, std::max(opts.root_limit, r_end));
            ta.budget = rerun ? ~0ull : budget;
            ta.hub_bits = b.hub_bits;
            ta.out_key = b.nk0;
            ta.out_val = b.nv0;
            ta.out_cap = b.new_cap;
            ta.tree_size = b.tsize;
            ta.tree_labels = b.tlab;
            ta.ws_key = b.ws_key;
            ta.ws_vis = b.ws_vis;
            ta.ws_front = b.ws_front;
            ta.ctl = b.ctl;
            ta.hash_slots = hash_slots;
            ta.hash_shift = 32;
            for (uint32_t t = hash_slots; t > 1; t >>= 1) --ta.hash_shift;
            const int blocks = (int)(b.slots / kWarpsPerBlock);
            // near/far queue.  Auto: split above 1024 queued vertices on
            // road-like graphs, whose queues are long rings of close keys
            // (1.25x faster builds of the 512/1024-square grids); off on
            // heavy-tailed ones, whose few-level queues gain nothing (RMAT
            // scale 20: 4% slower with it)
            ta.near_on = 0;
            ta.near_target = 1;
            const int qs = opts.queue_split ? opts.queue_split : (heavy_tail ? 1 : 1024);
            if (qs > 1) {
                ta.near_on = (uint32_t)qs;
                ta.near_target = std::max<uint32_t>(1, ta.near_on / 4);
            }
            void (*kern)(TreeArgs);
            size_t smem_launch = smem;
            int grid = blocks, block = kWarpsPerBlock * 32;
            const bool windowed = committed == 0 && win_target > 1;
            if (windowed) {
                // no committed labels: no tree can be pruned, so the trees
                // are searched label-correcting in windows (window_kernel)
                ta.near_target = win_target;
                ta.ws_win = b.ws_all;
                grid = (int)b.win_trees;
                block = (int)b.win_tw * 32;
                smem_launch = window_smem(b.win_tw);
                kern = window_kernel_for(unit, plant_now, b.win_tw);
            } else if (unit) {
                kern = plant_now ? batch_kernel<true, true> : batch_kernel<true, false>;
            } else {
                kern = plant_now ? batch_kernel<false, true> : batch_kernel<false, false>;
            }
            // the two layouts share the workspace: every key the next kernel
            // reads is INF (each tree resets its own keys when it ends)
            const int layout = windowed ? 2 : 1;
            if (b.ws_layout != layout) {
                const size_t words = windowed ? (size_t)b.win_trees * 6 * n : (size_t)b.slots * (4 + key_words) * n;
                CHL_CUDA(cudaMemsetAsync(b.ws_all, 0xFF, words * 4, b.st));
                b.ws_layout = layout;
            }
            CHL_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_launch));
            CHL_CUDA(cudaEventRecord(ev_a, b.st));
            kern<<<grid, block, smem_launch, b.st>>>(ta);
            step_slots = (uint32_t)grid * (uint32_t)block / 32;
            CHL_CUDA(cudaGetLastError());
            CHL_CUDA(cudaEventRecord(ev_b, b.st));
            ++launches;
            ++kernels;
            CHL_CUDA(cudaMemcpyAsync(&hc, b.ctl, sizeof(hc), cudaMemcpyDeviceToHost, b.st));
            CHL_CUDA(cudaStreamSynchronize(b.st));
            float ms = 0;
            CHL_CUDA(cudaEventElapsedTime(&ms, ev_a, ev_b));
            tree_ms += ms;
            step_tree_ms = ms;
            const unsigned long long fetched = (hc.next_root & kClosed) ? hc.close_at : hc.next_root;
            uint32_t r1 = (uint32_t)std::min<unsigned long long>(fetched, std::max(ta.r_hard, r_end));
            if (hc.err) {
                set_error(hc.err == 1 ? "a shortest-path distance reaches INT_MAX (the reference asserts dd < infty)"
                                      : "tree workspace bound exceeded");
                return CHL_ERR_INVALID;
            }
            if (hc.overflow || hc.nlab > b.new_cap) {
                ++step_reruns;
                // re-run the same root range with room for every label
                if ((rc = grow_new(b, hc.nlab + hc.nlab / 4 + 1024))) return rc;
                r_end = r1;
                rerun = true;
                continue;
            }
            r_end = r1;
            break;
        }
        const uint32_t r1 = r_end;
        visits += hc.visits;
        reads += hc.label_reads;
        arcs += hc.arcs;
        if (plant_now) plant_roots += r1 - r0;
        unsigned long long M = hc.nlab;
        // hybrid switch (distributed_memory/akiba.hpp:297-303, 362-376)
        if (plant_now && switch_open) {
            unsigned long long zero = 0;
            CHL_CUDA(cudaMemcpyAsync(&b.ctl->max_ratio_num, &zero, 8, cudaMemcpyHostToDevice, b.st));
            ratio_max<<<std::max(1, sms), 256, 0, b.st>>>(b.tsize, b.tlab, &b.ctl->next_root, r0, r1, b.ctl);
            ++kernels;
            unsigned long long bits = 0;
            CHL_CUDA(cudaMemcpyAsync(&bits, &b.ctl->max_ratio_num, 8, cudaMemcpyDeviceToHost, b.st));
            CHL_CUDA(cudaStreamSynchronize(b.st));
            double ratio;
            std::memcpy(&ratio, &bits, 8);
            if (ratio > ps) {
                do_plant = false;
                switch_open = false;
            }
        }
        // Sort, GLL clean and merge of the new labels, then the longest
        // committed list: one stream-ordered chain with no host round trip,
        // captured as a CUDA graph when opts.use_graphs is set.  The entry
        // array is sized for every new label before the chain (the clean
        // only removes labels).
        if ((rc = ensure_ent(&b.ent_b, &b.ent_cap_b, committed + M))) return rc;
        if ((rc = ensure_ent(&b.dent_b, &b.dent_cap_b, committed + M))) return rc;
        const bool clean_now = !plant_now && M > 0;
        // bits of the distance part of the (list, distance) sort key
        const int dist_bits = bits_for((uint64_t)hc.max_dist + 1);
        auto chain = [&]() -> int {
            int rc2;
            // --- sort the new labels by (list, hub)
            int parity = 0;
            if ((rc2 = radix_sort_pairs(b.nk0, b.nv0, b.nk1, b.nv1, (const uint64_t *)&b.ctl->nlab, b.new_cap,
                                        b.key_bits, b.tmp, b.tmp_bytes, b.st, &parity)))
                return rc2;
            uint64_t *sk = parity ? b.nk1 : b.nk0;
            uint32_t *sv = parity ? b.nv1 : b.nv0;
            uint64_t *ak = parity ? b.nk0 : b.nk1;
            uint32_t *av = parity ? b.nv0 : b.nv1;
            const int cgrid = sms * 8;
            const unsigned long long *d_count = &b.ctl->nlab;
            // --- GLL clean (drops labels covered through a higher-ranked hub)
            if (clean_now) {
                CHL_CUDA(cudaMemsetAsync(b.cnt, 0, ((size_t)b.nl + 1) * 4, b.st));
                count_keys<<<cgrid, 256, 0, b.st>>>(sk, d_count, b.new_cap, b.hub_bits, b.cnt);
                if ((rc2 = scan_u32_excl(b.cnt, b.pre, b.nl, nullptr, b.tmp, b.tmp_bytes, b.st))) return rc2;
                clean_mark<<<cgrid, 256, 0, b.st>>>(sk, sv, d_count, b.new_cap, b.hub_bits, r0, b.pre, b.order,
                                                    b.rank, b.sides, b.keep);
                if ((rc2 = scan_u32_excl(b.keep, b.kpre, b.new_cap, (const uint64_t *)d_count, b.tmp,
                                         b.tmp_bytes, b.st)))
                    return rc2;
                compact_kept<<<cgrid, 256, 0, b.st>>>(sk, sv, b.keep, b.kpre, d_count, b.new_cap, ak, av,
                                                      &b.ctl->n_keep);
                CHL_CUDA(cudaMemcpyAsync(&b.ctl->nlab, &b.ctl->n_keep, 8, cudaMemcpyDeviceToDevice, b.st));
                std::swap(sk, ak);
                std::swap(sv, av);
            }
            // --- commit: merge the sorted new labels into the committed CSR
            CHL_CUDA(cudaMemsetAsync(b.cnt, 0, ((size_t)b.nl + 1) * 4, b.st));
            count_keys<<<cgrid, 256, 0, b.st>>>(sk, d_count, b.new_cap, b.hub_bits, b.cnt);
            if ((rc2 = scan_u32_excl(b.cnt, b.pre, b.nl, nullptr, b.tmp, b.tmp_bytes, b.st))) return rc2;
            merge_offsets<<<cgrid, 256, 0, b.st>>>(b.off_a, b.pre, b.off_b, b.nl);
            copy_old_lists<<<cgrid, 256, 0, b.st>>>(b.off_a, b.ent_a, b.off_b, b.ent_b, b.nl);
            place_new<<<cgrid, 256, 0, b.st>>>(sk, sv, d_count, b.new_cap, b.hub_bits, r0, b.pre, b.off_a,
                                               b.off_b, b.ent_b);
            {
                // the same labels by (list, distance, hub), merged into the
                // distance-ordered copy (the sort is stable: equal distances
                // keep hub order); the key holds the distance in the bits the
                // superstep's largest distance needs
                dist_keys<<<cgrid, 256, 0, b.st>>>(sk, sv, d_count, b.new_cap, b.hub_bits, dist_bits, r0, ak, av);
                int par2 = 0;
                if ((rc2 = radix_sort_pairs(ak, av, sk, sv, (const uint64_t *)d_count, b.new_cap,
                                            b.key_bits - b.hub_bits + dist_bits, b.tmp, b.tmp_bytes, b.st, &par2)))
                    return rc2;
                merge_dist_lists<<<cgrid, 256, 0, b.st>>>(b.off_a, b.dent_a, b.off_b, b.pre, par2 ? sk : ak,
                                                          par2 ? sv : av, b.dent_b, b.nl, dist_bits);
            }
            // longest committed list, for the next superstep's root staging
            CHL_CUDA(cudaMemsetAsync(&b.ctl->max_ratio_den, 0, 8, b.st));
            max_list_len<<<cgrid, 256, 0, b.st>>>(b.off_b, b.nl, &b.ctl->max_ratio_den);
            CHL_CUDA(cudaGetLastError());
            return CHL_OK;
        };
        kernels += 3 * ((b.key_bits + 7) / 8) + (clean_now ? 9 : 0) + 8 +
                   2 + 3 * ((b.key_bits - b.hub_bits + dist_bits + 7) / 8);
        CHL_CUDA(cudaEventRecord(ev_a, b.st));
        if (opts.use_graphs) {
            CHL_CUDA(cudaStreamBeginCapture(b.st, cudaStreamCaptureModeThreadLocal));
            const int crc = chain();
            cudaGraph_t cg = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(b.st, &cg);
            if (crc) {
                if (cg) cudaGraphDestroy(cg);
                return crc;
            }
            CHL_CUDA(ce);
            // reuse the executable graph when only kernel arguments changed
            bool updated = false;
            if (b.commit_exec) {
                cudaGraphExecUpdateResultInfo info;
                updated = cudaGraphExecUpdate(b.commit_exec, cg, &info) == cudaSuccess;
                if (!updated) {
                    (void)cudaGetLastError();
                    cudaGraphExecDestroy(b.commit_exec);
                    b.commit_exec = nullptr;
                }
            }
            cudaError_t ie = cudaSuccess;
            if (!updated) ie = cudaGraphInstantiate(&b.commit_exec, cg, 0);
            cudaGraphDestroy(cg);
            CHL_CUDA(ie);
            CHL_CUDA(cudaGraphLaunch(b.commit_exec, b.st));
            ++b.graph_launches;
        } else if ((rc = chain())) {
            return rc;
        }
        CHL_CUDA(cudaEventRecord(ev_b, b.st));
        std::swap(b.off_a, b.off_b);
        std::swap(b.ent_a, b.ent_b);
        std::swap(b.ent_cap_a, b.ent_cap_b);
        std::swap(b.dent_a, b.dent_b);
        std::swap(b.dent_cap_a, b.dent_cap_b);
        CHL_CUDA(cudaMemcpyAsync(&hc, b.ctl, sizeof(hc), cudaMemcpyDeviceToHost, b.st));
        CHL_CUDA(cudaStreamSynchronize(b.st));
        M = hc.nlab;
        committed += M;
        max_list = (uint32_t)std::min<unsigned long long>(hc.max_ratio_den, 0xFFFFFFFFu);
        float ms1 = 0;
        CHL_CUDA(cudaEventElapsedTime(&ms1, ev_a, ev_b));
        commit_ms += ms1;
        ++supersteps;
        r0 = r1;
        unsigned long long tstat[2] = {0, 0};
        if (opts.verbose >= 2) {
            CHL_CUDA(cudaMemsetAsync(&b.ctl->max_ratio_num, 0, 16, b.st));
            tree_stats<<<sms, 256, 0, b.st>>>(b.tsize, r1 - r_begin, &b.ctl->max_ratio_num);
            CHL_CUDA(cudaMemcpyAsync(tstat, &b.ctl->max_ratio_num, 16, cudaMemcpyDeviceToHost, b.st));
            CHL_CUDA(cudaStreamSynchronize(b.st));
        }
        if (opts.verbose >= 2) {
            const double tot = (double)std::max<unsigned long long>(1, hc.cyc[7]);
            fprintf(stderr, "  warp cycles: scan %.1f%% flags %.1f%% prune %.1f%% emit %.1f%% relax %.1f%% "
                            "stage %.1f%% reset %.1f%% (sum of warp residencies %.3g cycles)\n",
                    100 * hc.cyc[0] / tot, 100 * hc.cyc[1] / tot, 100 * hc.cyc[2] / tot, 100 * hc.cyc[3] / tot,
                    100 * hc.cyc[4] / tot, 100 * hc.cyc[5] / tot, 100 * hc.cyc[6] / tot, tot);
            if (kPhaseTiming) {
                // warp slots busy: summed residencies over (slots x superstep time)
                int khz = 0;
                cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, 0);
                const double avail = (double)step_slots * step_tree_ms * 1e-3 * khz * 1e3;
                fprintf(stderr, "  warp slots busy %.1f%% (at the maximum SM clock)\n", 100 * tot / std::max(avail, 1.0));
            }
            fprintf(stderr, "  prune item selection %.1f%% of warp cycles, %llu passes (%.2f per visit)\n",
                    100 * hc.cyc[8] / tot, hc.cyc[9],
                    (double)hc.cyc[9] / std::max<unsigned long long>(1, hc.visits));
            fprintf(stderr, "  frontier entries scanned %llu rounds %llu settles %llu (per visit: scanned %.2f)\n",
                    hc.cnt[0], hc.cnt[1], hc.cnt[2], (double)hc.cnt[0] / std::max<unsigned long long>(1, hc.visits));
            fprintf(stderr, "  far pile entries read by refills: %llu (%.1f%% of the frontier entries scanned)\n",
                    hc.cnt[3], 100.0 * hc.cnt[3] / std::max<unsigned long long>(1, hc.cnt[0]));
        }
        if (opts.verbose >= 2)
            fprintf(stderr, "  tree size max %llu mean %.1f\n", tstat[0],
                    (double)tstat[1] / std::max<uint32_t>(1, r1 - r_begin));
        if (opts.verbose >= 2)
            fprintf(stderr,
                    "superstep %u: roots [%u,%u) %s tree_ms %.2f commit_ms %.2f labels %llu visits %llu reads %llu "
                    "arcs %llu committed %llu max_list %u label_cap %llu reruns %u\n",
                    supersteps, r_begin, r1, plant_now ? "plant" : "gll",
                    step_tree_ms, ms1, (unsigned long long)M, (unsigned long long)hc.visits,
                    (unsigned long long)hc.label_reads, (unsigned long long)hc.arcs, (unsigned long long)committed,
                    max_list, (unsigned long long)b.new_cap, step_reruns);
    }
    CHL_CUDA(cudaEventRecord(ev1, b.st));
    CHL_CUDA(cudaStreamSynchronize(b.st));
    float total_ms = 0, up_ms = 0;
    CHL_CUDA(cudaEventElapsedTime(&total_ms, ev_up, ev1));
    CHL_CUDA(cudaEventElapsedTime(&up_ms, ev0, ev_up));

    chl_labels *L = new (std::nothrow) chl_labels();
    if (!L) return CHL_ERR_OOM;
    L->n = n;
    L->sym = b.sides == 1;
    L->d_off = b.off_a;
    L->d_ent = (LabelEnt *)b.ent_a;
    L->total = committed;
    b.off_a = nullptr;
    b.ent_a = nullptr;
    chl_build_stats &S = L->stats;
    S.build_ms = total_ms;
    S.h2d_ms = up_ms;
    S.kernel_launches = kernels;
    S.tree_ms = tree_ms;
    S.sort_ms = sort_ms;
    S.commit_ms = commit_ms;
    S.labels = committed * (L->sym ? 2 : 1);
    S.visits = visits;
    S.label_reads = reads;
    S.arcs = arcs;
    S.supersteps = supersteps;
    S.plant_roots = plant_roots;
    S.tree_launches = launches;
    S.avg_label = n ? (double)S.labels / n / 2.0 : 0.0;
    (void)t_wall0;
    *out = L;
    if (opts.verbose) {
        // the reference's summary line (shared_memory/akiba.hpp:214)
        printf("Average label size after gll is %g, labeling time = %g, sorting time = %g, "
               "cleaning time = %g, total time = %g\n",
               S.avg_label, tree_ms / 1e3, sort_ms / 1e3, commit_ms / 1e3, total_ms / 1e3);
        printf("%g %g\n", S.avg_label, total_ms / 1e3);
    }
    return CHL_OK;
}

}  // namespace chl

extern "C" void chl_build_opts_default(chl_build_opts *o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->mode = CHL_MODE_HYBRID;
    o->sf = 0.0;
    o->ps = 0.0;
    o->autotune = 1;
    o->use_graphs = 1;
    o->verbose = 0;
}

extern "C" int chl_build(const chl_graph *g, const uint32_t *order, uint32_t n,
                         const chl_build_opts *opts, chl_labels **out) {
    try {
        return chl::build_labels(g, order, n, opts, out);
    } catch (...) {
        chl::set_error("host allocation failed during build");
        return CHL_ERR_OOM;
    }
}

extern "C" int chl_graph_to_device(chl_graph *g) {
    if (!g) return CHL_ERR_INVALID;
    if (g->dev) return CHL_OK;
    chl::DevGraph *d = new (std::nothrow) chl::DevGraph();
    if (!d) return CHL_ERR_OOM;
    int rc = chl::upload_graph(g, *d, 0);
    if (rc == CHL_OK) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) rc = chl::cuda_status(e, "graph upload", __FILE__, __LINE__);
    }
    if (rc != CHL_OK) {
        d->release();
        delete d;
        return rc;
    }
    g->dev = d;
    return CHL_OK;
}

extern "C" int chl_graph_release_device(chl_graph *g) {
    if (!g) return CHL_ERR_INVALID;
    chl::graph_release_device(g);
    return CHL_OK;
}

extern "C" int chl_build_get_stats(const chl_labels *l, chl_build_stats *s) {
    if (!l || !s) return CHL_ERR_INVALID;
    *s = l->stats;
    return CHL_OK;
}
