// Scan and stable radix sort used by the superstep commit.  Both take their
// item count from device memory so a superstep's whole kernel chain has a
// fixed launch shape (and can be captured in a CUDA graph).
#include "chl_dev.cuh"

namespace chl {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr uint64_t kScanTile = kScanThreads * kScanItems;  // 2048

__device__ __forceinline__ uint64_t bound_n(uint64_t n, const uint64_t *d_n) {
    if (d_n) {
        uint64_t m = *d_n;
        return m < n ? m : n;
    }
    return n;
}

// Block-wide exclusive scan of one u64 per thread; returns the block total.
__device__ uint64_t block_excl_scan(uint64_t x, uint64_t *warp_tot) {
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    uint64_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint64_t y = __shfl_up_sync(kFull, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        uint64_t t = lane < (uint32_t)nw ? warp_tot[lane] : 0;
        uint64_t ti = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint64_t y = __shfl_up_sync(kFull, ti, o);
            if (lane >= (uint32_t)o) ti += y;
        }
        if (lane < (uint32_t)nw) warp_tot[lane] = ti - t;
        if (lane == 31) warp_tot[32] = ti;
    }
    __syncthreads();
    uint64_t r = warp_tot[warp] + incl - x;
    uint64_t total = warp_tot[32];
    __syncthreads();
    return r + 0 * total;
}

__global__ void scan_tile_sums(const uint32_t *in, uint64_t n, const uint64_t *d_n,
                               uint64_t *tile_sum, uint64_t ntiles) {
    __shared__ uint64_t wt[33];
    const uint64_t m = bound_n(n, d_n);
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        uint64_t base = t * kScanTile;
        uint64_t s = 0;
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) {
            uint64_t i = base + (uint64_t)j * kScanThreads + threadIdx.x;
            if (i < m) s += in[i];
        }
        // block reduce via scan
        uint64_t ex = block_excl_scan(s, wt);
        if (threadIdx.x == blockDim.x - 1) tile_sum[t] = ex + s;
        __syncthreads();
    }
}

__global__ void scan_tile_prefix(uint64_t *tile_sum, uint64_t ntiles, uint64_t *total_out) {
    __shared__ uint64_t wt[33];
    uint64_t carry = 0;
    for (uint64_t b = 0; b < ntiles; b += blockDim.x) {
        uint64_t i = b + threadIdx.x;
        uint64_t x = i < ntiles ? tile_sum[i] : 0;
        uint64_t ex = block_excl_scan(x, wt);
        if (i < ntiles) tile_sum[i] = carry + ex;
        // last thread holds chunk total
        __shared__ uint64_t chunk;
        if (threadIdx.x == blockDim.x - 1) chunk = ex + x;
        __syncthreads();
        carry += chunk;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total_out = carry;
}

__global__ void scan_tiles(const uint32_t *in, uint64_t *out, uint64_t n,
                           const uint64_t *d_n, const uint64_t *tile_pre,
                           uint64_t ntiles) {
    __shared__ uint64_t wt[33];
    __shared__ uint32_t vals[kScanTile];
    const uint64_t m = bound_n(n, d_n);
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        uint64_t base = t * kScanTile;
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) {
            uint64_t i = base + (uint64_t)j * kScanThreads + threadIdx.x;
            vals[j * kScanThreads + threadIdx.x] = i < m ? in[i] : 0u;
        }
        __syncthreads();
        // thread owns items [threadIdx.x*kScanItems, +kScanItems)
        uint64_t loc[kScanItems];
        uint64_t s = 0;
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) {
            loc[j] = s;
            s += vals[threadIdx.x * kScanItems + j];
        }
        uint64_t ex = block_excl_scan(s, wt) + tile_pre[t];
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) {
            uint64_t i = base + (uint64_t)threadIdx.x * kScanItems + j;
            if (i < n) out[i] = ex + loc[j];
        }
        __syncthreads();
    }
}

}  // namespace

size_t scan_tmp_bytes(uint64_t n) {
    uint64_t ntiles = (n + kScanTile - 1) / kScanTile + 1;
    return (size_t)(ntiles + 1) * sizeof(uint64_t);
}

int scan_u32_excl(const uint32_t *in, uint64_t *out, uint64_t n, const uint64_t *d_n,
                  void *tmp, size_t tmp_bytes, cudaStream_t s) {
    uint64_t ntiles = (n + kScanTile - 1) / kScanTile;
    if (ntiles == 0) ntiles = 1;
    if (tmp_bytes < scan_tmp_bytes(n)) return CHL_ERR_INVALID;
    uint64_t *tile = (uint64_t *)tmp;
    int grid = (int)std::min<uint64_t>(ntiles, (uint64_t)device_sms() * 8);
    scan_tile_sums<<<grid, kScanThreads, 0, s>>>(in, n, d_n, tile, ntiles);
    scan_tile_prefix<<<1, 1024, 0, s>>>(tile, ntiles, out + n);
    scan_tiles<<<grid, kScanThreads, 0, s>>>(in, out, n, d_n, tile, ntiles);
    CHL_CUDA(cudaGetLastError());
    return CHL_OK;
}

// ------------------------------------------------------------ radix sort

namespace {

constexpr int kSortThreads = 256;     // one item per thread per tile
constexpr int kRadix = 256;
constexpr int kSortWarps = kSortThreads / 32;

__device__ __forceinline__ void block_range(uint64_t n, uint64_t &b, uint64_t &e) {
    uint64_t ntiles = (n + kSortThreads - 1) / kSortThreads;
    uint64_t per = (ntiles + gridDim.x - 1) / gridDim.x;
    uint64_t tb = (uint64_t)blockIdx.x * per, te = tb + per;
    if (te > ntiles) te = ntiles;
    if (tb > te) tb = te;
    b = tb * kSortThreads;
    e = te * kSortThreads;
    if (e > n) e = n;
    if (b > e) b = e;
}

__global__ void radix_hist(const uint64_t *keys, const uint64_t *d_n, uint64_t cap,
                           int shift, uint32_t *hist) {
    __shared__ uint32_t h[kRadix];
    for (int i = threadIdx.x; i < kRadix; i += blockDim.x) h[i] = 0;
    __syncthreads();
    uint64_t n = *d_n;
    if (n > cap) n = cap;
    uint64_t b, e;
    block_range(n, b, e);
    for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x)
        atomicAdd(&h[(keys[i] >> shift) & 255], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < kRadix; i += blockDim.x)
        hist[(uint64_t)i * gridDim.x + blockIdx.x] = h[i];
}

// Scatter of one digit pass.  A block walks its range in tiles of kTile
// items: warp w holds the tile's items [w * kWarpItems, (w + 1) *
// kWarpItems) in registers, ranks them per digit (match_any per round of 32,
// a running count per warp and digit), the block places the whole tile in
// shared memory ordered by (digit, position), and each digit's run is then
// written to its global slots with consecutive threads on consecutive
// addresses.  Positions within a digit keep the input order (stable).
constexpr int kTileItems = 8;
constexpr int kTile = kSortThreads * kTileItems;   // 2048
static_assert(kSortThreads == kRadix, "the digit prefix gives each thread one digit");
constexpr int kWarpItems = 32 * kTileItems;

__global__ void __launch_bounds__(kSortThreads) radix_scatter(const uint64_t *kin, const uint32_t *vin, uint64_t *kout,
                                                              uint32_t *vout, const uint64_t *d_n, uint64_t cap,
                                                              int shift, const uint64_t *offs) {
    __shared__ uint64_t s_k[kTile];
    __shared__ uint32_t s_v[kTile];
    __shared__ uint32_t wh[kSortWarps][kRadix];   // per-warp digit counts, then their prefix over warps
    __shared__ uint32_t t_start[kRadix + 1];      // each digit's first slot in the tile
    __shared__ uint32_t w_tot[kSortWarps];
    __shared__ uint64_t run[kRadix];              // each digit's next global slot
    const uint32_t tid = threadIdx.x, lane = lane_id(), warp = tid >> 5;
    for (int i = tid; i < kRadix; i += blockDim.x) run[i] = offs[(uint64_t)i * gridDim.x + blockIdx.x];
    uint64_t n = *d_n;
    if (n > cap) n = cap;
    uint64_t b, e;
    block_range(n, b, e);
    for (uint64_t base = b; base < e; base += kTile) {
        const uint32_t cnt = (uint32_t)((e - base) < (uint64_t)kTile ? (e - base) : (uint64_t)kTile);
        for (int i = tid; i < kSortWarps * kRadix; i += blockDim.x) (&wh[0][0])[i] = 0;
        __syncthreads();
        uint64_t k[kTileItems];
        uint32_t v[kTileItems], dg[kTileItems], pos[kTileItems];
#pragma unroll
        for (int j = 0; j < kTileItems; ++j) {
            const uint32_t idx = warp * kWarpItems + j * 32 + lane;
            const bool valid = idx < cnt;
            k[j] = valid ? kin[base + idx] : 0;
            v[j] = valid ? vin[base + idx] : 0;
            dg[j] = valid ? (uint32_t)((k[j] >> shift) & (kRadix - 1)) : (uint32_t)kRadix;
        }
#pragma unroll
        for (int j = 0; j < kTileItems; ++j) {
            const uint32_t peers = __match_any_sync(kFull, dg[j]);
            const uint32_t before = dg[j] < kRadix ? wh[warp][dg[j]] : 0u;
            __syncwarp();
            if (dg[j] < kRadix && lane == (uint32_t)(__ffs(peers) - 1)) wh[warp][dg[j]] = before + __popc(peers);
            __syncwarp();
            pos[j] = before + __popc(peers & lanemask_lt());
        }
        __syncthreads();
        // per digit (one per thread): prefix over warps, then over digits
        uint32_t tot = 0;
        for (int d = tid; d < kRadix; d += blockDim.x) {
#pragma unroll
            for (int w = 0; w < kSortWarps; ++w) {
                const uint32_t t = wh[w][d];
                wh[w][d] = tot;
                tot += t;
            }
        }
        uint32_t incl = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        if (lane == 31) w_tot[warp] = incl;
        __syncthreads();
        uint32_t wbase = 0;
        for (uint32_t w = 0; w < warp; ++w) wbase += w_tot[w];
        if (tid < kRadix) t_start[tid] = wbase + incl - tot;
        if (tid == 0) t_start[kRadix] = cnt;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < kTileItems; ++j) {
            if (dg[j] < kRadix) {
                const uint32_t p = t_start[dg[j]] + wh[warp][dg[j]] + pos[j];
                s_k[p] = k[j];
                s_v[p] = v[j];
            }
        }
        __syncthreads();
        for (uint32_t i = tid; i < cnt; i += blockDim.x) {
            const uint64_t kk = s_k[i];
            const uint32_t d = (uint32_t)((kk >> shift) & (kRadix - 1));
            const uint64_t gp = run[d] + (i - t_start[d]);
            kout[gp] = kk;
            vout[gp] = s_v[i];
        }
        __syncthreads();
        if (tid < kRadix) run[tid] += t_start[tid + 1] - t_start[tid];
        __syncthreads();
    }
}

__global__ void hist_to_u32_excl(const uint32_t *hist, uint64_t *offs, int entries) {
    // single block exclusive scan over digit-major histogram
    __shared__ uint64_t wt[33];
    __shared__ uint64_t chunk;
    uint64_t carry = 0;
    for (int b = 0; b < entries; b += blockDim.x) {
        int i = b + threadIdx.x;
        uint64_t x = i < entries ? hist[i] : 0;
        uint64_t ex = block_excl_scan(x, wt);
        if (i < entries) offs[i] = carry + ex;
        if (threadIdx.x == blockDim.x - 1) chunk = ex + x;
        __syncthreads();
        carry += chunk;
        __syncthreads();
    }
}

constexpr int kSortBlocksPerSM = 2;

}  // namespace

size_t radix_tmp_bytes() {
    size_t g = (size_t)device_sms() * kSortBlocksPerSM;
    return g * kRadix * (sizeof(uint32_t) + sizeof(uint64_t));
}

int radix_sort_pairs(uint64_t *k0, uint32_t *v0, uint64_t *k1, uint32_t *v1,
                     const uint64_t *d_n, uint64_t cap, int bits, void *tmp,
                     size_t tmp_bytes, cudaStream_t s, int *parity) {
    const int grid = device_sms() * kSortBlocksPerSM;
    if (tmp_bytes < radix_tmp_bytes()) return CHL_ERR_INVALID;
    uint32_t *hist = (uint32_t *)tmp;
    uint64_t *offs = (uint64_t *)((char *)tmp + (size_t)grid * kRadix * sizeof(uint32_t));
    // keep offs 8-byte aligned
    offs = (uint64_t *)(((uintptr_t)offs + 7) & ~(uintptr_t)7);
    int p = 0;
    uint64_t *ki = k0, *ko = k1;
    uint32_t *vi = v0, *vo = v1;
    for (int shift = 0; shift < bits; shift += 8) {
        radix_hist<<<grid, kSortThreads, 0, s>>>(ki, d_n, cap, shift, hist);
        hist_to_u32_excl<<<1, 1024, 0, s>>>(hist, offs, grid * kRadix);
        radix_scatter<<<grid, kSortThreads, 0, s>>>(ki, vi, ko, vo, d_n, cap, shift, offs);
        std::swap(ki, ko);
        std::swap(vi, vo);
        p ^= 1;
    }
    CHL_CUDA(cudaGetLastError());
    *parity = p;
    return CHL_OK;
}

}  // namespace chl
