// Label storage on the device, host transfers, and the batched distance
// query kernel.
//
//   Labeling::query         shared_memory/labeling.hpp:56-65
//   batchLocalQuery         distributed_memory/query_funcs.hpp:23-30
//   query mode 1 (QLSN)     distributed_memory/query.hpp:82-91
#include "chl_dev.cuh"

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace chl {

int cuda_status(cudaError_t e, const char *what, const char *file, int line) {
    std::string msg = std::string(what) + " failed: " + cudaGetErrorString(e) + " (" + file + ":" +
                      std::to_string(line) + ")";
    set_error(msg);
    if (e == cudaErrorMemoryAllocation) return CHL_ERR_OOM;
    return CHL_ERR_CUDA;
}

int device_sms() {
    static int sms = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            sms = 1;
        }
    });
    return sms;
}

// Device -> pageable host copy through two pinned staging buffers: the DMA
// of one chunk overlaps the (multi-threaded) copy of the previous one out
// of pinned memory.
int d2h_staged(void *dst, const void *src, size_t bytes) {
    constexpr size_t kChunk = 64ull << 20;
    if (bytes <= kChunk) {
        CHL_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
        return CHL_OK;
    }
    void *pin[2] = {nullptr, nullptr};
    cudaStream_t st = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int rc = CHL_OK;
    cudaError_t e = cudaHostAlloc(&pin[0], kChunk, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaHostAlloc(&pin[1], kChunk, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
    const size_t chunks = (bytes + kChunk - 1) / kChunk;
    auto issue = [&](size_t c) {
        const size_t off = c * kChunk, len = std::min(kChunk, bytes - off);
        cudaError_t e2 = cudaMemcpyAsync(pin[c & 1], (const char *)src + off, len, cudaMemcpyDeviceToHost, st);
        if (e2 == cudaSuccess) e2 = cudaEventRecord(ev[c & 1], st);
        return e2;
    };
    if (e == cudaSuccess) e = issue(0);
    for (size_t c = 0; c < chunks && e == cudaSuccess; ++c) {
        e = cudaEventSynchronize(ev[c & 1]);
        if (e != cudaSuccess) break;
        if (c + 1 < chunks) {
            e = issue(c + 1);
            if (e != cudaSuccess) break;
        }
        const size_t off = c * kChunk, len = std::min(kChunk, bytes - off);
        const char *from = (const char *)pin[c & 1];
        char *to = (char *)dst + off;
        const int64_t pieces = 16;
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < pieces; ++q) {
            const size_t a = len * (size_t)q / pieces, b = len * (size_t)(q + 1) / pieces;
            std::memcpy(to + a, from + a, b - a);
        }
        // the next issue into this buffer happens only after this copy
    }
    if (e != cudaSuccess) rc = cuda_status(e, "staged device-to-host copy", __FILE__, __LINE__);
    if (st) cudaStreamSynchronize(st);
    for (auto x : ev)
        if (x) cudaEventDestroy(x);
    if (st) cudaStreamDestroy(st);
    for (auto x : pin)
        if (x) cudaFreeHost(x);
    return rc;
}

int labels_fetch_host(const chl_labels *l) {
    if (l->host_valid) return CHL_OK;
    if (!l->d_off) return CHL_ERR_INVALID;
    const uint32_t nl = l->nl();
    l->h_off.resize((size_t)nl + 1);
    l->h_ent.resize(l->total);
    int rc = d2h_staged(l->h_off.data(), l->d_off, ((size_t)nl + 1) * 8);
    if (!rc && l->total) rc = d2h_staged(l->h_ent.data(), l->d_ent, l->total * sizeof(LabelEnt));
    if (rc) return rc;
    l->host_valid = true;
    return CHL_OK;
}

int labels_ensure_device(const chl_labels *L) {
    if (L->d_off) return CHL_OK;
    const uint32_t nl = L->nl();
    cudaError_t e = cudaMalloc(&L->d_off, ((size_t)nl + 1) * 8);
    if (e == cudaSuccess) e = cudaMalloc(&L->d_ent, std::max<uint64_t>(L->total, 1) * sizeof(LabelEnt));
    if (e == cudaSuccess)
        e = cudaMemcpy(L->d_off, L->h_off.data(), ((size_t)nl + 1) * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && L->total)
        e = cudaMemcpy(L->d_ent, L->h_ent.data(), L->total * sizeof(LabelEnt), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        int rc = cuda_status(e, "label upload", __FILE__, __LINE__);
        cudaFree(L->d_off);
        cudaFree(L->d_ent);
        L->d_off = nullptr;
        L->d_ent = nullptr;
        return rc;
    }
    return CHL_OK;
}

int labels_from_host(uint32_t n, const uint64_t *off2, const uint32_t *hub, const int32_t *dist,
                     chl_labels **out) {
    // every list must be strictly ascending by hub with non-negative distances
    for (uint64_t x = 0; x < 2ull * n; ++x) {
        if (off2[x + 1] < off2[x]) {
            set_error("label offsets are not monotone");
            return CHL_ERR_INVALID;
        }
        for (uint64_t k = off2[x]; k < off2[x + 1]; ++k) {
            if (dist[k] < 0 || (k > off2[x] && hub[k] <= hub[k - 1])) {
                set_error("label lists must be ascending by hub with non-negative distances");
                return CHL_ERR_INVALID;
            }
        }
    }
    bool sym = true;
    for (uint32_t v = 0; v < n && sym; ++v) {
        const uint64_t a = off2[2 * v], ae = off2[2 * v + 1], b = off2[2 * v + 1], be = off2[2 * v + 2];
        if (ae - a != be - b) {
            sym = false;
            break;
        }
        for (uint64_t k = 0; k < ae - a; ++k)
            if (hub[a + k] != hub[b + k] || dist[a + k] != dist[b + k]) {
                sym = false;
                break;
            }
    }
    chl_labels *L = new (std::nothrow) chl_labels();
    if (!L) return CHL_ERR_OOM;
    L->n = n;
    L->sym = sym;
    const uint32_t nl = L->nl();
    L->h_off.assign((size_t)nl + 1, 0);
    for (uint32_t x = 0; x < nl; ++x) {
        const uint64_t src = sym ? 2ull * x : x;
        L->h_off[x + 1] = L->h_off[x] + (off2[src + 1] - off2[src]);
    }
    L->total = L->h_off[nl];
    L->h_ent.resize(L->total);
    for (uint32_t x = 0; x < nl; ++x) {
        const uint64_t src = sym ? 2ull * x : x;
        for (uint64_t k = 0; k < off2[src + 1] - off2[src]; ++k)
            L->h_ent[L->h_off[x] + k] = LabelEnt{hub[off2[src] + k], (uint32_t)dist[off2[src] + k]};
    }
    L->host_valid = true;
    L->stats.labels = L->total * (sym ? 2 : 1);
    L->stats.avg_label = n ? (double)L->stats.labels / n / 2.0 : 0.0;
    *out = L;
    return CHL_OK;
}

namespace {

// One warp per pair: merge L(s, 1) with L(t, 0) 32 entries at a time.  Each
// lane binary-searches its entry of the current A chunk inside the B chunk
// held in registers (5 shuffles); the list whose chunk ends first advances.
// Pads: A uses 0xFFFFFFFF, B 0xFFFFFFFE, so pads never match.
__device__ __forceinline__ uint32_t merge_min(const uint2 *A, uint32_t na, const uint2 *B,
                                              uint32_t nb) {
    const uint32_t lane = lane_id();
    uint32_t best = 0xFFFFFFFFu;
    uint32_t ia = 0, ib = 0;
    while (ia < na && ib < nb) {
        uint2 a = ia + lane < na ? A[ia + lane] : make_uint2(0xFFFFFFFFu, 0);
        uint2 b = ib + lane < nb ? B[ib + lane] : make_uint2(0xFFFFFFFEu, 0);
        // lower_bound of a.x in the B chunk
        uint32_t lo = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const uint32_t hb = __shfl_sync(kFull, b.x, lo + step - 1);
            if (hb < a.x) lo += step;
        }
        const uint32_t hb = __shfl_sync(kFull, b.x, lo & 31);
        const uint32_t db = __shfl_sync(kFull, b.y, lo & 31);
        if (lo < 32 && hb == a.x) best = min(best, a.y + db);
        const uint32_t lastA = __shfl_sync(kFull, a.x, 31);
        const uint32_t lastB = __shfl_sync(kFull, b.x, 31);
        if (lastA <= lastB) ia += 32;
        if (lastB <= lastA) ib += 32;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(kFull, best, o));
    return best;
}

__global__ void query_kernel(const uint64_t *__restrict__ off, const uint2 *__restrict__ ent,
                             uint32_t n, int sym, const uint32_t *__restrict__ pairs, size_t k,
                             int32_t *__restrict__ out) {
    const size_t warps = (size_t)gridDim.x * (blockDim.x >> 5);
    for (size_t q = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); q < k; q += warps) {
        const uint32_t s = pairs[2 * q], t = pairs[2 * q + 1];
        uint32_t r = 0xFFFFFFFFu;
        if (s < n && t < n) {
            const uint32_t xa = sym ? s : 2 * s + 1;   // L(s, 1): forward hubs of s
            const uint32_t xb = sym ? t : 2 * t;       // L(t, 0): reverse hubs of t
            const uint64_t a0 = off[xa], a1 = off[xa + 1], b0 = off[xb], b1 = off[xb + 1];
            r = merge_min(ent + a0, (uint32_t)(a1 - a0), ent + b0, (uint32_t)(b1 - b0));
        }
        if (lane_id() == 0) out[q] = r > 2147483647u ? 2147483647 : (int32_t)r;
    }
}

__device__ __forceinline__ uint64_t qmix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Uniform random pairs generated on the device (query benchmark input).
// k seeded uniform pairs; with hot > 0, every pair is one of `hot` fixed
// seeded pairs (drawn uniformly), as a request stream with a hot set
__global__ void gen_pairs(uint32_t *pairs, size_t k, uint32_t n, uint64_t seed, uint32_t hot) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < k; q += (size_t)gridDim.x * blockDim.x) {
        size_t a = 2 * q, b = 2 * q + 1;
        if (hot) {
            const size_t j = qmix(seed ^ (q * 0x9E3779B97F4A7C15ull) ^ 0x5A5Aull) % hot;
            a = 2 * j;
            b = 2 * j + 1;
        }
        pairs[2 * q] = (uint32_t)(qmix(seed ^ (a * 0xD1B54A32D192ED03ull)) % n);
        pairs[2 * q + 1] = (uint32_t)(qmix(seed ^ (b * 0xD1B54A32D192ED03ull)) % n);
    }
}

// Algorithmic bytes of a query batch: 8 (|L(s,1)| + |L(t,0)|) + 8 + 4 per pair.
__global__ void query_bytes(const uint64_t *off, int sym, const uint32_t *pairs, size_t k,
                            unsigned long long *bytes) {
    unsigned long long acc = 0;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < k; q += (size_t)gridDim.x * blockDim.x) {
        const uint32_t s = pairs[2 * q], t = pairs[2 * q + 1];
        const uint32_t xa = sym ? s : 2 * s + 1, xb = sym ? t : 2 * t;
        acc += 8ull * ((off[xa + 1] - off[xa]) + (off[xb + 1] - off[xb])) + 12ull;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(bytes, acc);
}

// ---- label digest (no reference counterpart)
// A position-dependent 64-bit fingerprint of the content hl::Labeling::write
// emits (shared_memory/labeling.hpp:167-183): n, then for every list
// i = 2v + side its size and its (hub, dist) entries in order.  One term per
// item, added modulo 2^64 so the sum can be taken in any order:
//   M(n + C_N) + sum_i M(B_i ^ size_i) + sum_ij M(B_i ^ M(j + C_E) ^ (hub << 32 | dist)),
// B_i = M(i + C_L), M = the SplitMix64 finaliser (Steele, Lea and Flood,
// OOPSLA 2014).  A symmetric build stores one list per vertex and stands for
// both sides.
constexpr uint64_t kDigN = 0x243F6A8885A308D3ull, kDigL = 0x13198A2E03707344ull,
                   kDigE = 0xA4093822299F31D0ull;

__host__ __device__ __forceinline__ uint64_t dig_mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// One warp per vertex (both sides), grid-stride; one atomic per warp.
__global__ void label_digest(const uint64_t *__restrict__ off, const uint2 *__restrict__ ent, uint32_t n, int sym,
                             unsigned long long *acc) {
    const uint32_t lane = lane_id();
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    uint64_t sum = 0;
    for (uint32_t v = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); v < n; v += warps) {
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const uint32_t x = sym ? v : 2 * v + (uint32_t)side;
            const uint64_t b = off[x], e = off[x + 1];
            const uint64_t base = dig_mix(2ull * v + (uint64_t)side + kDigL);
            if (lane == 0) sum += dig_mix(base ^ (e - b));
            for (uint64_t k = b + lane; k < e; k += 32) {
                const uint2 q = ent[k];
                sum += dig_mix(base ^ dig_mix((k - b) + kDigE) ^ (((uint64_t)q.x << 32) | q.y));
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(kFull, sum, o);
    if (lane == 0) atomicAdd(acc, (unsigned long long)sum);
}

__global__ void hub_count(const uint2 *ent, uint64_t total, uint32_t *cnt) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[ent[i].x], 1u);
}

}  // namespace

int query_launch(const chl_labels *l, const uint32_t *d_pairs, size_t k, int32_t *d_out,
                 cudaStream_t s) {
    if (k == 0) return CHL_OK;
    int rc = labels_ensure_device(l);
    if (rc) return rc;
    const int threads = 256;
    size_t blocks = (k + (threads / 32) - 1) / (threads / 32);
    blocks = std::min<size_t>(blocks, (size_t)device_sms() * 64);
    query_kernel<<<(unsigned)blocks, threads, 0, s>>>(l->d_off, (const uint2 *)l->d_ent, l->n,
                                                      l->sym ? 1 : 0, d_pairs, k, d_out);
    CHL_CUDA(cudaGetLastError());
    return CHL_OK;
}

}  // namespace chl

using namespace chl;

extern "C" double chl_avg_label(const chl_labels *l) { return l ? l->stats.avg_label : 0.0; }
extern "C" uint32_t chl_labels_n(const chl_labels *l) { return l ? l->n : 0; }
extern "C" uint64_t chl_labels_total(const chl_labels *l) {
    return l ? l->total * (l->sym ? 2 : 1) : 0;
}

extern "C" int chl_labels_get(const chl_labels *l, uint32_t v, int side, uint32_t *hubs,
                              int32_t *dists, uint32_t cap, uint32_t *cnt) {
    if (!l || v >= l->n || side < 0 || side > 1 || !cnt) return CHL_ERR_INVALID;
    int rc = labels_fetch_host(l);
    if (rc) return rc;
    const uint32_t x = l->list(v, side);
    const uint64_t b = l->h_off[x], e = l->h_off[x + 1];
    *cnt = (uint32_t)(e - b);
    if (hubs || dists) {
        if (cap < e - b) return CHL_ERR_INVALID;
        for (uint64_t k = b; k < e; ++k) {
            if (hubs) hubs[k - b] = l->h_ent[k].hub;
            if (dists) dists[k - b] = (int32_t)l->h_ent[k].dist;
        }
    }
    return CHL_OK;
}

extern "C" int chl_labels_list_sizes(const chl_labels *l, uint32_t *sizes) {
    if (!l || !sizes) return CHL_ERR_INVALID;
    const uint32_t nl = l->nl();
    std::vector<uint64_t> off;
    const uint64_t *o;
    if (l->host_valid) {
        o = l->h_off.data();
    } else {
        off.resize((size_t)nl + 1);
        CHL_CUDA(cudaMemcpy(off.data(), l->d_off, ((size_t)nl + 1) * 8, cudaMemcpyDeviceToHost));
        o = off.data();
    }
    for (uint32_t v = 0; v < l->n; ++v)
        for (int side = 0; side < 2; ++side) {
            const uint32_t x = l->list(v, side);
            sizes[2 * (size_t)v + side] = (uint32_t)(o[x + 1] - o[x]);
        }
    return CHL_OK;
}

extern "C" int chl_labels_export(const chl_labels *l, uint64_t *off, uint32_t *hubs,
                                 int32_t *dists) {
    if (!l || !off) return CHL_ERR_INVALID;
    int rc = labels_fetch_host(l);
    if (rc) return rc;
    // offsets of the 2n lists (both sides, even when stored once), then the
    // entries, copied in parallel over vertices
    off[0] = 0;
    for (uint32_t v = 0; v < l->n; ++v)
        for (int side = 0; side < 2; ++side) {
            const uint32_t x = l->list(v, side);
            off[2 * v + side + 1] = off[2 * v + side] + (l->h_off[x + 1] - l->h_off[x]);
        }
    if (hubs || dists) {
        const int64_t n = l->n;
#pragma omp parallel for schedule(dynamic, 1024)
        for (int64_t v = 0; v < n; ++v)
            for (int side = 0; side < 2; ++side) {
                const uint32_t x = l->list((uint32_t)v, side);
                uint64_t p = off[2 * v + side];
                for (uint64_t k = l->h_off[x]; k < l->h_off[x + 1]; ++k, ++p) {
                    if (hubs) hubs[p] = l->h_ent[k].hub;
                    if (dists) dists[p] = (int32_t)l->h_ent[k].dist;
                }
            }
    }
    return CHL_OK;
}

extern "C" int chl_labels_import(uint32_t n, const uint64_t *off, const uint32_t *hubs,
                                 const int32_t *dists, chl_labels **out) {
    if (!off || !out || (off[2ull * n] && (!hubs || !dists))) return CHL_ERR_INVALID;
    return labels_from_host(n, off, hubs, dists, out);
}

extern "C" int chl_labels_hub_freq(const chl_labels *l, const uint32_t *order, uint32_t *freq) {
    if (!l || !order || !freq) return CHL_ERR_INVALID;
    int rc = labels_ensure_device(l);
    if (rc) return rc;
    uint32_t *d_cnt = nullptr;
    CHL_CUDA(cudaMalloc(&d_cnt, (size_t)std::max<uint32_t>(l->n, 1) * 4));
    cudaError_t em = cudaMemset(d_cnt, 0, (size_t)l->n * 4);
    if (em != cudaSuccess) {
        cudaFree(d_cnt);
        return cuda_status(em, "cudaMemset", __FILE__, __LINE__);
    }
    if (l->total)
        hub_count<<<device_sms() * 8, 256>>>((const uint2 *)l->d_ent, l->total, d_cnt);
    std::vector<uint32_t> cnt(l->n);
    cudaError_t e = cudaMemcpy(cnt.data(), d_cnt, (size_t)l->n * 4, cudaMemcpyDeviceToHost);
    cudaFree(d_cnt);
    if (e != cudaSuccess) return cuda_status(e, "hub_freq", __FILE__, __LINE__);
    for (uint32_t h = 0; h < l->n; ++h) freq[order[h]] = cnt[h] * (l->sym ? 2u : 1u);
    return CHL_OK;
}

extern "C" int chl_labels_digest(const chl_labels *l, uint64_t *digest) {
    if (!l || !digest) return CHL_ERR_INVALID;
    int rc = labels_ensure_device(l);
    if (rc) return rc;
    unsigned long long *d_acc = nullptr;
    CHL_CUDA(cudaMalloc(&d_acc, sizeof(unsigned long long)));
    unsigned long long acc = 0;
    cudaError_t e = cudaMemset(d_acc, 0, sizeof(acc));
    if (e == cudaSuccess && l->n) {
        label_digest<<<device_sms() * 8, 256>>>(l->d_off, (const uint2 *)l->d_ent, l->n, l->sym ? 1 : 0, d_acc);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(&acc, d_acc, sizeof(acc), cudaMemcpyDeviceToHost);
    cudaFree(d_acc);
    if (e != cudaSuccess) return cuda_status(e, "label digest", __FILE__, __LINE__);
    *digest = dig_mix((uint64_t)l->n + kDigN) + (uint64_t)acc;
    return CHL_OK;
}

extern "C" void chl_labels_free(chl_labels *l) {
    if (!l) return;
    cudaFree(l->d_off);
    cudaFree(l->d_ent);
    delete l;
}

extern "C" int chl_query_batch_device(const chl_labels *l, const uint32_t *d_pairs, size_t k,
                                      int32_t *d_out, void *stream) {
    if (!l || (k && (!d_pairs || !d_out))) return CHL_ERR_INVALID;
    return query_launch(l, d_pairs, k, d_out, (cudaStream_t)stream);
}

extern "C" int chl_query_bench(const chl_labels *l, size_t k, uint64_t seed, int iters, uint32_t hot,
                               double *ms_per_iter, uint64_t *bytes_per_iter) {
    if (!l || !ms_per_iter || k == 0 || iters < 1 || l->n == 0) return CHL_ERR_INVALID;
    int rc = labels_ensure_device(l);
    if (rc) return rc;
    uint32_t *dp = nullptr;
    int32_t *dout = nullptr;
    unsigned long long *dbytes = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMalloc(&dp, k * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dout, k * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dbytes, 8);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float ms = 0;
    unsigned long long bytes = 0;
    if (e == cudaSuccess) {
        gen_pairs<<<device_sms() * 8, 256, 0, st>>>(dp, k, l->n, seed, hot);
        cudaMemsetAsync(dbytes, 0, 8, st);
        query_bytes<<<device_sms() * 8, 256, 0, st>>>(l->d_off, l->sym ? 1 : 0, dp, k, dbytes);
        rc = query_launch(l, dp, k, dout, st);   // warm-up
        if (rc == CHL_OK) {
            cudaEventRecord(e0, st);
            for (int i = 0; i < iters && rc == CHL_OK; ++i) rc = query_launch(l, dp, k, dout, st);
            cudaEventRecord(e1, st);
        }
        e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess) e = cudaMemcpy(&bytes, dbytes, 8, cudaMemcpyDeviceToHost);
    }
    if (e != cudaSuccess && rc == CHL_OK) rc = cuda_status(e, "query bench", __FILE__, __LINE__);
    cudaFree(dp);
    cudaFree(dout);
    cudaFree(dbytes);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    if (rc) return rc;
    *ms_per_iter = ms / iters;
    if (bytes_per_iter) *bytes_per_iter = bytes;
    return CHL_OK;
}

// ------------------------------------------------- allocation-free queries
//
// chl_query_batch stages the pairs and the answers in device memory it
// allocates per call.  Some callers cannot let a library allocate device
// memory: serving processes whose HBM is already carved up by their own
// pool allocator (a cudaMalloc here would fail or fragment it), and
// latency-critical request loops where cudaMalloc/cudaFree and their
// implicit synchronisation are not acceptable.  chl_query_batch_noalloc
// answers the same queries with the same kernel, staging through one
// file-scope device array instead.
//
// The array holds CHL_NOALLOC_MAX_PAIRS pairs (8 B) plus as many answers
// (4 B): 12 MiB, resident on every GPU that loads this library until the
// process exits.  All calls share it and it keeps the last call's contents;
// nothing in it needs to start at zero (each call overwrites the pairs and
// answers it uses).  Calls whose work overlaps on the GPU race on it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[(size_t)CHL_NOALLOC_MAX_PAIRS * 12];

namespace {
std::mutex g_noalloc_mu;
std::vector<void *> g_noalloc_ptr;   // device address of the array, per device
}  // namespace

// Host code may not use g_noalloc_scratch as an address (it is a host-side
// stand-in); the device address comes from cudaGetSymbolAddress, once per
// device, with that device current.
static int noalloc_scratch(void **ptr) {
    int dev = 0;
    CHL_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if ((int)g_noalloc_ptr.size() <= dev) g_noalloc_ptr.resize(dev + 1, nullptr);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        CHL_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = p;
    }
    *ptr = g_noalloc_ptr[dev];
    return CHL_OK;
}

extern "C" int chl_query_batch_noalloc(const chl_labels *l, const uint32_t *pairs, size_t k,
                                       int32_t *out, void *stream) {
    if (!l || (k && (!pairs || !out))) return CHL_ERR_INVALID;
    if (k > CHL_NOALLOC_MAX_PAIRS) {
        set_error("chl_query_batch_noalloc: more than CHL_NOALLOC_MAX_PAIRS pairs in one call");
        return CHL_ERR_INVALID;
    }
    if (!l->d_off) {
        // uploading the labels would allocate; the caller must make them
        // resident first (any build, chl_query_batch or chl_server_create)
        set_error("chl_query_batch_noalloc: labels are not resident on the device");
        return CHL_ERR_INVALID;
    }
    for (size_t i = 0; i < 2 * k; ++i)
        if (pairs[i] >= l->n) {
            set_error("query vertex out of range");
            return CHL_ERR_INVALID;
        }
    if (k == 0) return CHL_OK;
    void *base = nullptr;
    int rc = noalloc_scratch(&base);
    if (rc) return rc;
    uint32_t *d_pairs = (uint32_t *)base;
    int32_t *d_out = (int32_t *)((unsigned char *)base + (size_t)CHL_NOALLOC_MAX_PAIRS * 8);
    cudaStream_t s = (cudaStream_t)stream;
    CHL_CUDA(cudaMemcpyAsync(d_pairs, pairs, k * 8, cudaMemcpyHostToDevice, s));
    rc = query_launch(l, d_pairs, k, d_out, s);
    if (rc) return rc;
    CHL_CUDA(cudaMemcpyAsync(out, d_out, k * 4, cudaMemcpyDeviceToHost, s));
    CHL_CUDA(cudaStreamSynchronize(s));
    return CHL_OK;
}

extern "C" int chl_query_batch(const chl_labels *l, const uint32_t *pairs, size_t k, int32_t *out,
                               void *stream) {
    if (!l || (k && (!pairs || !out))) return CHL_ERR_INVALID;
    for (size_t i = 0; i < 2 * k; ++i)
        if (pairs[i] >= l->n) {
            set_error("query vertex out of range");
            return CHL_ERR_INVALID;
        }
    if (k == 0) return CHL_OK;
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t *dp = nullptr;
    int32_t *dout = nullptr;
    CHL_CUDA(cudaMallocAsync(&dp, k * 8, s));
    cudaError_t e = cudaMallocAsync(&dout, k * 4, s);
    if (e != cudaSuccess) {
        cudaFreeAsync(dp, s);
        return cuda_status(e, "cudaMallocAsync", __FILE__, __LINE__);
    }
    int rc = CHL_OK;
    e = cudaMemcpyAsync(dp, pairs, k * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) rc = query_launch(l, dp, k, dout, s);
    if (e == cudaSuccess && rc == CHL_OK) e = cudaMemcpyAsync(out, dout, k * 4, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(dp, s);
    cudaFreeAsync(dout, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_status(e, "query copy", __FILE__, __LINE__);
    if (e2 != cudaSuccess) return cuda_status(e2, "query sync", __FILE__, __LINE__);
    return CHL_OK;
}
