// Plain vertex orderings computed on the GPU (no reference counterpart: the
// reference reads its order from a file produced by outside tools; its own
// degree tool is distributed_memory/degree.cpp:62-67).
//
//   degree      : Graph::get_degree(v) (shared_memory/graph.hpp:324)
//                 descending; ties by a seeded permutation (tie_key).
//   betweenness : Brandes dependencies from `sources` seeded sources over
//                 forward shortest paths, descending; same tie break.
//
// Both sort with the stable radix sort: first by the tie key, then by the
// primary key, so equal primary keys keep tie-key order.
#include "chl_dev.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace chl {

namespace {

constexpr uint32_t kInfD = 0x7FFFFFFFu;

__device__ __forceinline__ uint64_t d_mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void tie_keys(uint32_t n, uint64_t seed, uint64_t *key, uint32_t *val) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        key[v] = d_mix64(seed * 0x9E3779B97F4A7C15ull + (uint64_t)v);
        val[v] = v;
    }
}

// primary key descending == ~primary ascending
__global__ void degree_keys(uint32_t n, const uint64_t *off_out, const uint64_t *off_in,
                            const uint32_t *vals, uint64_t *key) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t v = vals[i];
        const uint64_t deg = (off_out[v + 1] - off_out[v]) + (off_in[v + 1] - off_in[v]);
        key[i] = ~deg;
    }
}

__global__ void bc_keys(uint32_t n, const double *bc, const uint32_t *vals, uint64_t *key) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t bits = (uint64_t)__double_as_longlong(bc[vals[i]]);
        key[i] = ~bits;
    }
}

// One warp per source: Dijkstra (indexed binary heap in global memory, lane
// 0), then sigma in settle order, then dependencies in reverse settle order.
// Every sum runs in adjacency order with explicitly rounded operations
// (no contraction), matching the CPU restatement bit for bit.
__global__ void brandes_kernel(uint32_t n, const uint64_t *off_out, const uint2 *arc_out,
                               const uint64_t *off_in, const uint2 *arc_in, const uint32_t *src,
                               uint32_t count, uint32_t *ws_dist, uint32_t *ws_pos,
                               uint64_t *ws_heap, uint32_t *ws_seq, double *ws_sigma,
                               double *deltas) {
    const uint32_t lane = lane_id();
    const uint32_t warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    uint32_t *dist = ws_dist + (size_t)warp * n;
    uint32_t *pos = ws_pos + (size_t)warp * n;
    uint64_t *heap = ws_heap + (size_t)warp * n;
    uint32_t *seq = ws_seq + (size_t)warp * n;
    double *sigma = ws_sigma + (size_t)warp * n;
    for (uint32_t j = warp; j < count; j += nwarps) {
        double *delta = deltas + (size_t)j * n;
        for (uint32_t v = lane; v < n; v += 32) {
            dist[v] = kInfD;
            delta[v] = 0.0;
        }
        __syncwarp();
        const uint32_t s = src[j];
        uint32_t hsize = 0, ns = 0;
        if (lane == 0) {
            dist[s] = 0;
            heap[0] = (uint64_t)s;
            pos[s] = 0;
            hsize = 1;
            while (hsize) {
                const uint64_t top = heap[0];
                const uint32_t u = (uint32_t)top;
                // pop
                const uint32_t m = --hsize;
                if (m) {
                    const uint64_t e = heap[m];
                    uint32_t i = 0;
                    while (true) {
                        uint32_t c = 2 * i + 1;
                        if (c >= m) break;
                        uint64_t ce = heap[c];
                        if (c + 1 < m && heap[c + 1] < ce) ce = heap[++c];
                        if (e <= ce) break;
                        heap[i] = ce;
                        pos[(uint32_t)ce] = i;
                        i = c;
                    }
                    heap[i] = e;
                    pos[(uint32_t)e] = i;
                }
                seq[ns++] = u;
                const uint32_t du = dist[u];
                for (uint64_t a = off_out[u]; a < off_out[u + 1]; ++a) {
                    const uint2 hl = arc_out[a];
                    const uint32_t dd = du + hl.y;
                    const uint32_t w = hl.x;
                    if (dd < dist[w]) {
                        uint32_t i = dist[w] == kInfD ? hsize++ : pos[w];
                        dist[w] = dd;
                        const uint64_t e = ((uint64_t)dd << 32) | w;
                        while (i > 0) {
                            const uint32_t p = (i - 1) >> 1;
                            const uint64_t pe = heap[p];
                            if (pe <= e) break;
                            heap[i] = pe;
                            pos[(uint32_t)pe] = i;
                            i = p;
                        }
                        heap[i] = e;
                        pos[w] = i;
                    }
                }
            }
            // sigma in settle order, predecessors in in-adjacency order
            for (uint32_t k = 0; k < ns; ++k) {
                const uint32_t w = seq[k];
                if (w == s) {
                    sigma[w] = 1.0;
                    continue;
                }
                double acc = 0.0;
                for (uint64_t a = off_in[w]; a < off_in[w + 1]; ++a) {
                    const uint2 hl = arc_in[a];
                    if (dist[hl.x] != kInfD && dist[hl.x] + hl.y == dist[w]) acc = __dadd_rn(acc, sigma[hl.x]);
                }
                sigma[w] = acc;
            }
            // dependencies in reverse settle order, successors in out order
            for (uint32_t k = ns; k-- > 0;) {
                const uint32_t v = seq[k];
                double acc = 0.0;
                for (uint64_t a = off_out[v]; a < off_out[v + 1]; ++a) {
                    const uint2 hl = arc_out[a];
                    if (dist[hl.x] != kInfD && dist[v] + hl.y == dist[hl.x]) {
                        const double q = __ddiv_rn(sigma[v], sigma[hl.x]);
                        const double t = __dadd_rn(1.0, delta[hl.x]);
                        acc = __dadd_rn(acc, __dmul_rn(q, t));
                    }
                }
                delta[v] = acc;
            }
            delta[s] = 0.0;   // the source's own dependency is not counted
        }
        __syncwarp();
    }
}

// bc[v] = sum over sources j (in list order) of delta_j[v]
__global__ void bc_sum(uint32_t n, uint32_t count, const double *deltas, double *bc) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (uint32_t j = 0; j < count; ++j) acc = __dadd_rn(acc, deltas[(size_t)j * n + v]);
        bc[v] = acc;
    }
}

struct Buf {
    void *p = nullptr;
    ~Buf() { cudaFree(p); }
    template <typename T>
    T *as() const { return (T *)p; }
};

int alloc(Buf &b, size_t bytes) {
    cudaError_t e = cudaMalloc(&b.p, bytes ? bytes : 1);
    if (e != cudaSuccess) return cuda_status(e, "cudaMalloc", __FILE__, __LINE__);
    return CHL_OK;
}

// Sort vertices by (primary descending, tie ascending); `primary` fills key
// from the tie-sorted vertex list.
template <typename F>
int order_by(uint32_t n, uint64_t seed, F primary, int primary_bits, uint32_t *order_h) {
    Buf k0, k1, v0, v1, tmp, cnt;
    int rc;
    if ((rc = alloc(k0, (size_t)n * 8)) || (rc = alloc(k1, (size_t)n * 8)) || (rc = alloc(v0, (size_t)n * 4)) ||
        (rc = alloc(v1, (size_t)n * 4)) || (rc = alloc(tmp, radix_tmp_bytes())) || (rc = alloc(cnt, 8)))
        return rc;
    const uint64_t n64 = n;
    CHL_CUDA(cudaMemcpy(cnt.p, &n64, 8, cudaMemcpyHostToDevice));
    const int grid = device_sms() * 4;
    tie_keys<<<grid, 256>>>(n, seed, k0.as<uint64_t>(), v0.as<uint32_t>());
    int par = 0;
    if ((rc = radix_sort_pairs(k0.as<uint64_t>(), v0.as<uint32_t>(), k1.as<uint64_t>(), v1.as<uint32_t>(),
                               cnt.as<uint64_t>(), n, 64, tmp.p, radix_tmp_bytes(), 0, &par)))
        return rc;
    uint64_t *ka = par ? k1.as<uint64_t>() : k0.as<uint64_t>();
    uint32_t *va = par ? v1.as<uint32_t>() : v0.as<uint32_t>();
    uint64_t *kb = par ? k0.as<uint64_t>() : k1.as<uint64_t>();
    uint32_t *vb = par ? v0.as<uint32_t>() : v1.as<uint32_t>();
    primary(va, ka);
    int par2 = 0;
    if ((rc = radix_sort_pairs(ka, va, kb, vb, cnt.as<uint64_t>(), n, primary_bits, tmp.p,
                               radix_tmp_bytes(), 0, &par2)))
        return rc;
    CHL_CUDA(cudaMemcpy(order_h, par2 ? vb : va, (size_t)n * 4, cudaMemcpyDeviceToHost));
    return CHL_OK;
}

// float score descending: order-preserving map of the IEEE bits, then complemented
__global__ void score_keys(uint32_t n, const float *score, const uint32_t *vals, uint64_t *key) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t b = __float_as_uint(score[vals[i]]);
        b = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
        key[i] = (uint64_t)(~b);
    }
}

}  // namespace

int order_by_score(uint32_t n, uint64_t seed, const float *d_score, uint32_t *order_h) {
    if (n == 0) return CHL_OK;
    const int grid = device_sms() * 4;
    return order_by(
        n, seed, [&](const uint32_t *vals, uint64_t *key) { score_keys<<<grid, 256>>>(n, d_score, vals, key); }, 32,
        order_h);
}

}  // namespace chl

using namespace chl;

extern "C" int chl_order_degree(const chl_graph *g, uint64_t seed, uint32_t *order) {
    if (!g || !order) return CHL_ERR_INVALID;
    if (g->n == 0) return CHL_OK;
    Buf off_out, off_in;
    int rc;
    if ((rc = alloc(off_out, ((size_t)g->n + 1) * 8)) || (rc = alloc(off_in, ((size_t)g->n + 1) * 8))) return rc;
    CHL_CUDA(cudaMemcpy(off_out.p, g->off[1].data(), ((size_t)g->n + 1) * 8, cudaMemcpyHostToDevice));
    CHL_CUDA(cudaMemcpy(off_in.p, g->off[0].data(), ((size_t)g->n + 1) * 8, cudaMemcpyHostToDevice));
    const int grid = device_sms() * 4;
    const uint32_t n = g->n;
    return order_by(
        n, seed,
        [&](const uint32_t *vals, uint64_t *key) {
            degree_keys<<<grid, 256>>>(n, off_out.as<uint64_t>(), off_in.as<uint64_t>(), vals, key);
        },
        64, order);
}

extern "C" int chl_order_betweenness(const chl_graph *g, uint32_t sources, uint64_t seed,
                                     uint32_t *order) {
    if (!g || !order || g->min_len < 1) return CHL_ERR_INVALID;
    const uint32_t n = g->n;
    if (n == 0) return CHL_OK;
    if (sources > n) sources = n;
    if (sources == 0) sources = 1;
    // sources: mix64(seed + j) % n, skipping repeats (host; O(sources))
    std::vector<uint32_t> src;
    {
        std::vector<uint8_t> seen(n, 0);
        for (uint64_t j = 0; src.size() < sources; ++j) {
            uint32_t s = (uint32_t)(mix64(seed + j) % n);
            if (seen[s]) continue;
            seen[s] = 1;
            src.push_back(s);
        }
    }
    Buf off_out, off_in, arc_out, arc_in, dsrc, deltas, bc;
    int rc;
    const uint64_t mo = g->off[1][n], mi = g->off[0][n];
    if ((rc = alloc(off_out, ((size_t)n + 1) * 8)) || (rc = alloc(off_in, ((size_t)n + 1) * 8)) ||
        (rc = alloc(arc_out, mo * 8)) || (rc = alloc(arc_in, mi * 8)) || (rc = alloc(dsrc, (size_t)sources * 4)) ||
        (rc = alloc(deltas, (size_t)sources * n * 8)) || (rc = alloc(bc, (size_t)n * 8)))
        return rc;
    std::vector<uint2> pk(std::max(mo, mi));
    CHL_CUDA(cudaMemcpy(off_out.p, g->off[1].data(), ((size_t)n + 1) * 8, cudaMemcpyHostToDevice));
    CHL_CUDA(cudaMemcpy(off_in.p, g->off[0].data(), ((size_t)n + 1) * 8, cudaMemcpyHostToDevice));
    for (uint64_t i = 0; i < mo; ++i) pk[i] = make_uint2(g->head[1][i], (uint32_t)g->len[1][i]);
    CHL_CUDA(cudaMemcpy(arc_out.p, pk.data(), mo * 8, cudaMemcpyHostToDevice));
    for (uint64_t i = 0; i < mi; ++i) pk[i] = make_uint2(g->head[0][i], (uint32_t)g->len[0][i]);
    CHL_CUDA(cudaMemcpy(arc_in.p, pk.data(), mi * 8, cudaMemcpyHostToDevice));
    CHL_CUDA(cudaMemcpy(dsrc.p, src.data(), (size_t)sources * 4, cudaMemcpyHostToDevice));
    // one warp per source, as many concurrent sources as sources
    const uint32_t warps = sources;
    const int wpb = 4;
    const uint32_t blocks = (warps + wpb - 1) / wpb;
    const uint32_t slots = blocks * wpb;
    Buf wd, wp, wh, wsq, wsg;
    if ((rc = alloc(wd, (size_t)slots * n * 4)) || (rc = alloc(wp, (size_t)slots * n * 4)) ||
        (rc = alloc(wh, (size_t)slots * n * 8)) || (rc = alloc(wsq, (size_t)slots * n * 4)) ||
        (rc = alloc(wsg, (size_t)slots * n * 8)))
        return rc;
    brandes_kernel<<<blocks, wpb * 32>>>(n, off_out.as<uint64_t>(), arc_out.as<uint2>(), off_in.as<uint64_t>(),
                                         arc_in.as<uint2>(), dsrc.as<uint32_t>(), sources, wd.as<uint32_t>(),
                                         wp.as<uint32_t>(), wh.as<uint64_t>(), wsq.as<uint32_t>(),
                                         wsg.as<double>(), deltas.as<double>());
    CHL_CUDA(cudaGetLastError());
    bc_sum<<<device_sms() * 4, 256>>>(n, sources, deltas.as<double>(), bc.as<double>());
    CHL_CUDA(cudaGetLastError());
    const int grid = device_sms() * 4;
    return order_by(
        n, seed,
        [&](const uint32_t *vals, uint64_t *key) { bc_keys<<<grid, 256>>>(n, bc.as<double>(), vals, key); },
        64, order);
}
