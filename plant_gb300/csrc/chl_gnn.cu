// Learned vertex ranking: a small message-passing network that proposes the
// CHL order (no reference counterpart; the reference takes its order from
// outside tools, README.md:24).
//
// Network (hidden width H = 64, L = 3 message-passing layers):
//   x_v   = standardised [log1p deg(v), log1p sum_{u in N(v)} deg(u), cc(v)]
//   h0    = relu(x W0 + b0)                          (fp32 math, K = 3)
//   m_l   = mean_{u in N(v)} h_{l-1}(u)              (0 without neighbours)
//   h_l   = relu([h_{l-1}, m_l] W_l + b_l)           (BF16 tensor-core GEMM, K = 128)
//   s_v   = h_L . w_out + b_out                      (fp32)
// h_l and m_l are stored in BF16; GEMM operands are BF16 with FP32
// accumulation (mma.sync m16n8k16); master weights and Adam state are FP32.
// Loss: mean squared error to a per-graph target (standardised log1p hub
// frequency).  deg(v) = Graph::get_degree (out + in arcs); N(v) = out-arcs;
// cc(v) = fraction of 16 seeded neighbour pairs (a, b) with b among the
// first 256 out-arcs of a.
//
// The GEMMs are [n x 128] x [128 x 64]: far below the tensor-core ridge,
// bound by reading the activations (HBM), like every other kernel here.
#include "chl_dev.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace chl {
namespace {

constexpr int H = 64;          // hidden width
constexpr int K2 = 2 * H;      // concatenated [h, m]
constexpr int NF = 3;          // input features
constexpr int kClusterSamples = 16;
constexpr int kClusterScan = 256;

__device__ __forceinline__ uint64_t gmix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// raw features: log1p deg, log1p 2-hop degree sum, sampled clustering
__global__ void feat_raw(uint32_t n, const uint64_t *off_out, const uint32_t *head_out, const uint64_t *off_in,
                         uint64_t seed, float *x) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint64_t b = off_out[v], e = off_out[v + 1];
        const double deg = (double)(e - b) + (double)(off_in[v + 1] - off_in[v]);
        double two = 0.0;
        for (uint64_t a = b; a < e; ++a) {
            const uint32_t u = head_out[a];
            two += (double)(off_out[u + 1] - off_out[u]) + (double)(off_in[u + 1] - off_in[u]);
        }
        float cc = 0.f;
        const uint64_t d = e - b;
        if (d >= 2) {
            uint32_t hit = 0;
            for (int k = 0; k < kClusterSamples; ++k) {
                const uint64_t h = gmix(seed ^ ((uint64_t)v * 0x100000001B3ull + (uint64_t)k));
                const uint64_t i = h % d;
                uint64_t j = (h >> 32) % (d - 1);
                if (j >= i) ++j;
                const uint32_t a = head_out[b + i], c = head_out[b + j];
                const uint64_t ab = off_out[a], ae = min(off_out[a + 1], ab + kClusterScan);
                for (uint64_t q = ab; q < ae; ++q)
                    if (head_out[q] == c) {
                        ++hit;
                        break;
                    }
            }
            cc = (float)hit / (float)kClusterSamples;
        }
        x[(size_t)v * NF + 0] = (float)log1p(deg);
        x[(size_t)v * NF + 1] = (float)log1p(two);
        x[(size_t)v * NF + 2] = cc;
    }
}

// h0 = relu(x W0 + b0), one thread per (vertex, channel)
__global__ void layer0_fwd(uint32_t n, const float *x, const float *W0, const float *b0, __nv_bfloat16 *h0) {
    const size_t tot = (size_t)n * H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
        const size_t v = i / H;
        const int c = (int)(i % H);
        float z = b0[c];
#pragma unroll
        for (int k = 0; k < NF; ++k) z = fmaf(x[v * NF + k], W0[k * H + c], z);
        h0[i] = __float2bfloat16_rn(fmaxf(z, 0.f));
    }
}

// m(v) = mean over out-neighbours of h(u); one warp per vertex, 2 channels per lane
__global__ void aggregate_mean(uint32_t n, const uint64_t *off, const uint32_t *head, const __nv_bfloat16 *h,
                               __nv_bfloat16 *m) {
    const uint32_t lane = lane_id();
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t v = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); v < n; v += warps) {
        const uint64_t b = off[v], e = off[v + 1];
        float s0 = 0.f, s1 = 0.f;
        for (uint64_t a = b; a < e; ++a) {
            const __nv_bfloat162 t = *(const __nv_bfloat162 *)(h + (size_t)head[a] * H + 2 * lane);
            s0 += __bfloat162float(t.x);
            s1 += __bfloat162float(t.y);
        }
        const float inv = e > b ? 1.f / (float)(e - b) : 0.f;
        __nv_bfloat162 o;
        o.x = __float2bfloat16_rn(s0 * inv);
        o.y = __float2bfloat16_rn(s1 * inv);
        *(__nv_bfloat162 *)(m + (size_t)v * H + 2 * lane) = o;
    }
}

// mma.sync m16n8k16, BF16 inputs, FP32 accumulators
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// Y[n x 64] = A[n x K] B[K x 64] (+ bias, relu) where A's columns are the
// concatenation of two [n x 64] BF16 arrays A0 | A1 (K = 128) or one (K = 64).
// Each warp computes 16 rows at a time.  B is staged in shared memory as
// BF16, transposed (column-major, rows padded to K + 8 elements: 16-byte
// aligned rows whose eight-row groups fall in distinct banks) and read with
// ldmatrix; A fragments are read straight from global memory as BF16 pairs.
// mode 0: Y = relu(AB + bias) -> BF16 out_bf;  mode 1: Y = AB -> FP32 out_f.
template <int K>
__global__ void __launch_bounds__(128) gemm_rows(uint32_t n, const __nv_bfloat16 *A0, const __nv_bfloat16 *A1,
                                                 const float *B, const float *bias, int mode,
                                                 __nv_bfloat16 *out_bf, float *out_f, int ldo) {
    constexpr int KP = K + 8;
    __shared__ __align__(16) __nv_bfloat16 sBt[H * KP];
    for (int i = threadIdx.x; i < K * H; i += blockDim.x) sBt[(i % H) * KP + i / H] = __float2bfloat16_rn(B[i]);
    __syncthreads();
    const uint32_t lane = lane_id(), gid = lane >> 2, tig = lane & 3;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    const uint32_t tiles = (n + 15) / 16;
    for (uint32_t t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < tiles; t += warps) {
        const uint32_t r0 = t * 16 + gid, r1 = r0 + 8;
        float acc[8][4];
#pragma unroll
        for (int j = 0; j < 8; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[j][q] = 0.f;
        // two BF16 at (row, col), col even: one 4-byte load (0 past the end)
        auto ld2 = [&](const __nv_bfloat16 *src, uint32_t row, int col) -> uint32_t {
            return row < n ? __ldg((const unsigned int *)(src + (size_t)row * H + col)) : 0u;
        };
        uint32_t af[K / 16][4];
#pragma unroll
        for (int ks = 0; ks < K / 16; ++ks) {
            const __nv_bfloat16 *src = (ks * 16 < H) ? A0 : A1;
            const int kc = (ks * 16) % H + 2 * (int)tig;
            af[ks][0] = ld2(src, r0, kc);
            af[ks][1] = ld2(src, r1, kc);
            af[ks][2] = ld2(src, r0, kc + 8);
            af[ks][3] = ld2(src, r1, kc + 8);
        }
#pragma unroll
        for (int ks = 0; ks < K / 16; ++ks) {
#pragma unroll
            for (int j = 0; j < 8; j += 2) {
                // one ldmatrix.x4: the B fragments of column tiles j and j + 1
                // (8x8 matrices: rows = columns of B, 8 consecutive k each;
                // lane l addresses row l % 8 of matrix l / 8)
                const uint32_t mtx = lane >> 3;
                const __nv_bfloat16 *rowp =
                    sBt + ((j + (mtx >> 1)) * 8 + (lane & 7)) * KP + ks * 16 + (mtx & 1) * 8;
                uint32_t b[4];
                asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                             : "=r"(b[0]), "=r"(b[1]), "=r"(b[2]), "=r"(b[3])
                             : "r"((uint32_t)__cvta_generic_to_shared(rowp)));
                const uint32_t b0[2] = {b[0], b[1]}, b1[2] = {b[2], b[3]};
                mma_bf16(acc[j], af[ks], b0);
                mma_bf16(acc[j + 1], af[ks], b1);
            }
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int c = j * 8 + 2 * tig;
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                const uint32_t row = half ? r1 : r0;
                if (row >= n) continue;
                float y0 = acc[j][2 * half], y1 = acc[j][2 * half + 1];
                if (mode == 0) {
                    y0 = fmaxf(y0 + bias[c], 0.f);
                    y1 = fmaxf(y1 + bias[c + 1], 0.f);
                    __nv_bfloat162 o;
                    o.x = __float2bfloat16_rn(y0);
                    o.y = __float2bfloat16_rn(y1);
                    *(__nv_bfloat162 *)(out_bf + (size_t)row * H + c) = o;
                } else {
                    *(float2 *)(out_f + (size_t)row * ldo + c) = make_float2(y0, y1);
                }
            }
        }
    }
}

// blocks of gemm_rows<K> that fill the GPU (resident blocks per SM x SMs)
template <int K>
int gemm_grid(int sms) {
    static int per_sm = 0;
    if (!per_sm) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, gemm_rows<K>, 128, 0) != cudaSuccess || b < 1) {
            (void)cudaGetLastError();
            b = 4;
        }
        per_sm = b;
    }
    return per_sm * sms;
}

// s = h w_out + b_out; loss terms; ds = 2 (s - y) / n
__global__ void head_fwd_bwd(uint32_t n, const __nv_bfloat16 *h, const float *wout, const float *bout,
                             const float *y, float *s, float *ds, double *loss_acc) {
    const uint32_t lane = lane_id();
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    double lsum = 0.0;
    for (uint32_t v = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); v < n; v += warps) {
        const __nv_bfloat162 t = *(const __nv_bfloat162 *)(h + (size_t)v * H + 2 * lane);
        float p = __bfloat162float(t.x) * wout[2 * lane] + __bfloat162float(t.y) * wout[2 * lane + 1];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(kFull, p, o);
        const float sv = p + bout[0];
        if (lane == 0) {
            s[v] = sv;
            if (y) {
                const float r = sv - y[v];
                ds[v] = 2.f * r / (float)n;
                lsum += (double)r * r;
            }
        }
    }
    if (loss_acc && lane == 0 && lsum != 0.0) atomicAdd(loss_acc, lsum / (double)n);
}

// dW[k][c] += sum_v A[v][k] dz[v][c] (A = [h | m], BF16; dz in BF16) on the
// tensor cores: warp w of a block owns rows k in [16w, 16w+16) of dW and
// walks the block's slice of vertices 16 at a time (the reduction axis);
// partial tiles are added to dW atomically.  db[c] += sum_v dz[v][c].
__global__ void grad_w_mma(uint32_t n, const __nv_bfloat16 *A0, const __nv_bfloat16 *A1,
                           const __nv_bfloat16 *dzb, const float *dz, float *dW, float *db) {
    const uint32_t lane = lane_id(), gid = lane >> 2, tig = lane & 3;
    const uint32_t warp = threadIdx.x >> 5;          // 8 warps: 128 rows of dW
    const uint32_t per = ((n + gridDim.x - 1) / gridDim.x + 15) & ~15u;
    const uint32_t v0 = blockIdx.x * per, v1 = min(n, v0 + per);
    const int krow = (int)warp * 16;
    const __nv_bfloat16 *src = krow < H ? A0 : A1;
    const int kc = krow % H;
    const __nv_bfloat16 z = __float2bfloat16_rn(0.f);
    float acc[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[j][q] = 0.f;
    for (uint32_t vb = v0; vb < v1; vb += 16) {
        auto av = [&](uint32_t v, int k) -> __nv_bfloat16 { return v < v1 ? src[(size_t)v * H + kc + k] : z; };
        auto bv = [&](uint32_t v, int c) -> __nv_bfloat16 { return v < v1 ? dzb[(size_t)v * H + c] : z; };
        // A fragment: row = k offset, col = vertex offset
        uint32_t a[4];
        a[0] = pack2(av(vb + 2 * tig, gid), av(vb + 2 * tig + 1, gid));
        a[1] = pack2(av(vb + 2 * tig, gid + 8), av(vb + 2 * tig + 1, gid + 8));
        a[2] = pack2(av(vb + 2 * tig + 8, gid), av(vb + 2 * tig + 9, gid));
        a[3] = pack2(av(vb + 2 * tig + 8, gid + 8), av(vb + 2 * tig + 9, gid + 8));
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int c = j * 8 + gid;
            uint32_t b[2];
            b[0] = pack2(bv(vb + 2 * tig, c), bv(vb + 2 * tig + 1, c));
            b[1] = pack2(bv(vb + 2 * tig + 8, c), bv(vb + 2 * tig + 9, c));
            mma_bf16(acc[j], a, b);
        }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int c = j * 8 + 2 * tig;
        atomicAdd(&dW[(size_t)(krow + gid) * H + c], acc[j][0]);
        atomicAdd(&dW[(size_t)(krow + gid) * H + c + 1], acc[j][1]);
        atomicAdd(&dW[(size_t)(krow + gid + 8) * H + c], acc[j][2]);
        atomicAdd(&dW[(size_t)(krow + gid + 8) * H + c + 1], acc[j][3]);
    }
    // bias gradient (fp32) from the same slice
    for (int c = threadIdx.x; c < H; c += blockDim.x) {
        float s = 0.f;
        for (uint32_t v = v0; v < v1; ++v) s += dz[(size_t)v * H + c];
        atomicAdd(&db[c], s);
    }
}

__global__ void to_bf16(size_t tot, const float *in, __nv_bfloat16 *out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __float2bfloat16_rn(in[i]);
}

// Wt0[c][k] = W[k][c], Wt1[c][k] = W[H + k][c]  (W is [2H x H] row-major)
__global__ void transpose_w(const float *W, float *Wt0, float *Wt1) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < H * H; i += gridDim.x * blockDim.x) {
        const int c = i / H, k = i % H;
        Wt0[i] = W[(size_t)k * H + c];
        Wt1[i] = W[(size_t)(H + k) * H + c];
    }
}

// dz = dh * [h > 0] (relu derivative from the stored activation)
__global__ void relu_bwd(size_t tot, const float *dh, const __nv_bfloat16 *h, float *dz) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x)
        dz[i] = __bfloat162float(h[i]) > 0.f ? dh[i] : 0.f;
}

// dh_L = ds * w_out; dw_out += sum ds h_L; db_out += sum ds
__global__ void head_bwd(uint32_t n, const float *ds, const __nv_bfloat16 *h, const float *wout, float *dh,
                         float *dwout, float *dbout) {
    __shared__ float acc[H + 1];
    for (int i = threadIdx.x; i <= H; i += blockDim.x) acc[i] = 0.f;
    __syncthreads();
    float a[H / 32 + 1] = {0.f, 0.f, 0.f};
    const uint32_t lane = lane_id();
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t v = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); v < n; v += warps) {
        const float d = ds[v];
        for (int c = lane; c < H; c += 32) {
            dh[(size_t)v * H + c] = d * wout[c];
            a[c / 32] += d * __bfloat162float(h[(size_t)v * H + c]);
        }
        if (lane == 0) a[H / 32] += d;
    }
    for (int c = lane, q = 0; c < H; c += 32, ++q) atomicAdd(&acc[c], a[q]);
    if (lane == 0) atomicAdd(&acc[H], a[H / 32]);
    __syncthreads();
    for (int i = threadIdx.x; i < H; i += blockDim.x) atomicAdd(&dwout[i], acc[i]);
    if (threadIdx.x == 0) atomicAdd(dbout, acc[H]);
}

// dh_prev(u) = dA[u, :64] + sum_{v: u in N(v)} dA[v, 64:] / deg(v)
// gathered over u's in-arcs (the reverse of the out-neighbour mean)
__global__ void scatter_mean_bwd(uint32_t n, const float *dA, const uint64_t *off_in, const uint32_t *head_in,
                                 const uint64_t *off_out, float *dh) {
    const uint32_t lane = lane_id();
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t u = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); u < n; u += warps) {
        float s0 = dA[(size_t)u * K2 + 2 * lane], s1 = dA[(size_t)u * K2 + 2 * lane + 1];
        for (uint64_t a = off_in[u]; a < off_in[u + 1]; ++a) {
            const uint32_t v = head_in[a];
            const float inv = 1.f / (float)(off_out[v + 1] - off_out[v]);
            s0 += dA[(size_t)v * K2 + H + 2 * lane] * inv;
            s1 += dA[(size_t)v * K2 + H + 2 * lane + 1] * inv;
        }
        dh[(size_t)u * H + 2 * lane] = s0;
        dh[(size_t)u * H + 2 * lane + 1] = s1;
    }
}

// dW0 += x^T dz0, db0 += sum dz0
__global__ void grad_w0(uint32_t n, const float *x, const float *dz, float *dW0, float *db0) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (NF + 1) * H; i += gridDim.x * blockDim.x) {
        const int k = i / H, c = i % H;
        double a = 0.0;
        for (uint32_t v = 0; v < n; ++v) a += (double)(k < NF ? x[(size_t)v * NF + k] : 1.f) * dz[(size_t)v * H + c];
        if (k < NF) dW0[k * H + c] += (float)a;
        else db0[c] += (float)a;
    }
}

__global__ void adam_step(size_t np, float *p, const float *g, float *m, float *vv, float lr, float b1, float b2,
                          float eps, float c1, float c2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < np; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        m[i] = b1 * m[i] + (1.f - b1) * gi;
        vv[i] = b2 * vv[i] + (1.f - b2) * gi * gi;
        p[i] -= lr * (m[i] / c1) / (sqrtf(vv[i] / c2) + eps);
    }
}

// parameter layout (fp32): W0[3*H] b0[H] | per layer: W[2H*H] b[H] | wout[H] bout[1]
constexpr size_t kP0 = (size_t)NF * H + H;
constexpr size_t kPL = (size_t)K2 * H + H;

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    ~DevBuf() { cudaFree(p); }
    int ensure(size_t b) {
        if (b <= bytes) return CHL_OK;
        cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, b ? b : 1);
        if (e != cudaSuccess) return cuda_status(e, "cudaMalloc", __FILE__, __LINE__);
        bytes = b;
        return CHL_OK;
    }
    template <typename T>
    T *as() const { return (T *)p; }
};

}  // namespace
}  // namespace chl

using namespace chl;

struct chl_gnn {
    uint32_t layers = 3;
    size_t np = 0;
    std::vector<float> host;       // parameter mirror
    DevBuf p, g, m, v;             // params, grads, Adam moments
    uint64_t step = 0;
    // per-graph scratch (grown on demand)
    DevBuf x, hb, mb, dz, dh, dA, s, ds, y, loss, wt;
    uint32_t cached_n = 0;
};

namespace {

size_t param_count(uint32_t layers) { return kP0 + (size_t)layers * kPL + H + 1; }

struct GraphDev {
    DevBuf off_out, head_out, off_in, head_in;
    uint32_t n = 0;
};

int upload_csr(const chl_graph *g, GraphDev &d) {
    const uint32_t n = g->n;
    d.n = n;
    const uint64_t mo = g->off[1][n], mi = g->off[0][n];
    int rc;
    if ((rc = d.off_out.ensure(((size_t)n + 1) * 8)) || (rc = d.head_out.ensure(std::max<uint64_t>(mo, 1) * 4)) ||
        (rc = d.off_in.ensure(((size_t)n + 1) * 8)) || (rc = d.head_in.ensure(std::max<uint64_t>(mi, 1) * 4)))
        return rc;
    CHL_CUDA(cudaMemcpy(d.off_out.p, g->off[1].data(), ((size_t)n + 1) * 8, cudaMemcpyHostToDevice));
    CHL_CUDA(cudaMemcpy(d.off_in.p, g->off[0].data(), ((size_t)n + 1) * 8, cudaMemcpyHostToDevice));
    if (mo) CHL_CUDA(cudaMemcpy(d.head_out.p, g->head[1].data(), mo * 4, cudaMemcpyHostToDevice));
    if (mi) CHL_CUDA(cudaMemcpy(d.head_in.p, g->head[0].data(), mi * 4, cudaMemcpyHostToDevice));
    return CHL_OK;
}

// standardise feature columns (host, deterministic order)
int standardise(chl_gnn *M, uint32_t n) {
    std::vector<float> x((size_t)n * NF);
    CHL_CUDA(cudaMemcpy(x.data(), M->x.p, x.size() * 4, cudaMemcpyDeviceToHost));
    for (int k = 0; k < NF; ++k) {
        double s = 0, s2 = 0;
        for (uint32_t v = 0; v < n; ++v) s += x[(size_t)v * NF + k];
        const double mean = n ? s / n : 0.0;
        for (uint32_t v = 0; v < n; ++v) {
            const double d = x[(size_t)v * NF + k] - mean;
            s2 += d * d;
        }
        const double sd = n > 1 ? std::sqrt(s2 / n) : 0.0;
        const double inv = sd > 1e-12 ? 1.0 / sd : 0.0;
        for (uint32_t v = 0; v < n; ++v) x[(size_t)v * NF + k] = (float)((x[(size_t)v * NF + k] - mean) * inv);
    }
    CHL_CUDA(cudaMemcpy(M->x.p, x.data(), x.size() * 4, cudaMemcpyHostToDevice));
    return CHL_OK;
}

int ensure_scratch(chl_gnn *M, uint32_t n) {
    const uint32_t L = M->layers;
    int rc;
    if ((rc = M->x.ensure((size_t)n * NF * 4)) || (rc = M->hb.ensure((size_t)(L + 1) * n * H * 2)) ||
        (rc = M->mb.ensure((size_t)(L + 1) * n * H * 2)) || (rc = M->dz.ensure((size_t)n * H * 4)) ||
        (rc = M->dh.ensure((size_t)n * H * 4)) || (rc = M->dA.ensure((size_t)n * K2 * 4)) ||
        (rc = M->s.ensure((size_t)n * 4)) || (rc = M->ds.ensure((size_t)n * 4)) || (rc = M->y.ensure((size_t)n * 4)) ||
        (rc = M->loss.ensure(8)) || (rc = M->wt.ensure((size_t)2 * H * H * 4)))
        return rc;
    return CHL_OK;
}

// forward pass; leaves h_l, m_l in scratch and the scores in M->s
int forward(chl_gnn *M, const GraphDev &G, uint64_t seed) {
    const uint32_t n = G.n;
    const int sms = device_sms();
    feat_raw<<<sms * 4, 256>>>(n, G.off_out.as<uint64_t>(), G.head_out.as<uint32_t>(), G.off_in.as<uint64_t>(),
                               seed, M->x.as<float>());
    CHL_CUDA(cudaGetLastError());
    int rc = standardise(M, n);
    if (rc) return rc;
    const float *P = M->p.as<float>();
    __nv_bfloat16 *hb = M->hb.as<__nv_bfloat16>(), *mb = M->mb.as<__nv_bfloat16>();
    layer0_fwd<<<sms * 8, 256>>>(n, M->x.as<float>(), P, P + NF * H, hb);
    for (uint32_t l = 1; l <= M->layers; ++l) {
        const float *W = P + kP0 + (size_t)(l - 1) * kPL;
        const __nv_bfloat16 *hp = hb + (size_t)(l - 1) * n * H;
        __nv_bfloat16 *ml = mb + (size_t)l * n * H;
        aggregate_mean<<<sms * 8, 256>>>(n, G.off_out.as<uint64_t>(), G.head_out.as<uint32_t>(), hp, ml);
        gemm_rows<K2><<<gemm_grid<K2>(sms), 128>>>(n, hp, ml, W, W + (size_t)K2 * H, 0, hb + (size_t)l * n * H, nullptr, 0);
    }
    const float *wout = P + kP0 + (size_t)M->layers * kPL;
    head_fwd_bwd<<<sms * 8, 256>>>(n, hb + (size_t)M->layers * n * H, wout, wout + H, nullptr, M->s.as<float>(),
                                   nullptr, nullptr);
    CHL_CUDA(cudaGetLastError());
    return CHL_OK;
}

// loss and gradients (into M->g) for target y (device)
int backward(chl_gnn *M, const GraphDev &G, double *loss) {
    const uint32_t n = G.n;
    const int sms = device_sms();
    const uint32_t L = M->layers;
    const float *P = M->p.as<float>();
    float *Gp = M->g.as<float>();
    __nv_bfloat16 *hb = M->hb.as<__nv_bfloat16>(), *mb = M->mb.as<__nv_bfloat16>();
    CHL_CUDA(cudaMemset(M->g.p, 0, M->np * 4));
    CHL_CUDA(cudaMemset(M->loss.p, 0, 8));
    const float *wout = P + kP0 + (size_t)L * kPL;
    float *gwout = Gp + kP0 + (size_t)L * kPL;
    head_fwd_bwd<<<sms * 8, 256>>>(n, hb + (size_t)L * n * H, wout, wout + H, M->y.as<float>(), M->s.as<float>(),
                                   M->ds.as<float>(), M->loss.as<double>());
    head_bwd<<<sms * 4, 256>>>(n, M->ds.as<float>(), hb + (size_t)L * n * H, wout, M->dh.as<float>(), gwout,
                               gwout + H);
    for (uint32_t l = L; l >= 1; --l) {
        const float *W = P + kP0 + (size_t)(l - 1) * kPL;
        float *gW = Gp + kP0 + (size_t)(l - 1) * kPL;
        const __nv_bfloat16 *hl = hb + (size_t)l * n * H;
        const __nv_bfloat16 *hp = hb + (size_t)(l - 1) * n * H;
        const __nv_bfloat16 *ml = mb + (size_t)l * n * H;
        relu_bwd<<<sms * 8, 256>>>((size_t)n * H, M->dh.as<float>(), hl, M->dz.as<float>());
        // dz -> BF16 in m_0's slot (unused after the forward pass)
        to_bf16<<<sms * 8, 256>>>((size_t)n * H, M->dz.as<float>(), mb);
        const uint32_t gblocks = std::max<uint32_t>(1, std::min<uint32_t>((uint32_t)sms * 2, (n + 255) / 256));
        grad_w_mma<<<gblocks, 256>>>(n, hp, ml, mb, M->dz.as<float>(), gW, gW + (size_t)K2 * H);
        // dA = dz W^T as two K = 64 GEMMs into the two column halves of dA
        transpose_w<<<16, 256>>>(W, M->wt.as<float>(), M->wt.as<float>() + H * H);
        gemm_rows<H><<<gemm_grid<H>(sms), 128>>>(n, mb, mb, M->wt.as<float>(), nullptr, 1, nullptr, M->dA.as<float>(), K2);
        gemm_rows<H><<<gemm_grid<H>(sms), 128>>>(n, mb, mb, M->wt.as<float>() + H * H, nullptr, 1, nullptr,
                                       M->dA.as<float>() + H, K2);
        scatter_mean_bwd<<<sms * 8, 256>>>(n, M->dA.as<float>(), G.off_in.as<uint64_t>(), G.head_in.as<uint32_t>(),
                                           G.off_out.as<uint64_t>(), M->dh.as<float>());
    }
    relu_bwd<<<sms * 8, 256>>>((size_t)n * H, M->dh.as<float>(), hb, M->dz.as<float>());
    grad_w0<<<((NF + 1) * H + 127) / 128, 128>>>(n, M->x.as<float>(), M->dz.as<float>(), Gp, Gp + NF * H);
    CHL_CUDA(cudaGetLastError());
    CHL_CUDA(cudaMemcpy(loss, M->loss.p, 8, cudaMemcpyDeviceToHost));
    return CHL_OK;
}

}  // namespace

extern "C" int chl_gnn_create(uint32_t layers, uint64_t seed, chl_gnn **out) {
    if (!out || layers == 0 || layers > 8) return CHL_ERR_INVALID;
    chl_gnn *M = new (std::nothrow) chl_gnn();
    if (!M) return CHL_ERR_OOM;
    M->layers = layers;
    M->np = param_count(layers);
    M->host.assign(M->np, 0.f);
    // Glorot-uniform weights from the seeded stream, zero biases
    Rng rng(seed);
    auto fill = [&](float *w, int fan_in, int fan_out, size_t cnt) {
        const double lim = std::sqrt(6.0 / (fan_in + fan_out));
        for (size_t i = 0; i < cnt; ++i) w[i] = (float)((2.0 * rng.unit() - 1.0) * lim);
    };
    float *p = M->host.data();
    fill(p, NF, H, (size_t)NF * H);
    for (uint32_t l = 0; l < layers; ++l) fill(p + kP0 + l * kPL, K2, H, (size_t)K2 * H);
    fill(p + kP0 + layers * kPL, H, 1, H);
    int rc;
    if ((rc = M->p.ensure(M->np * 4)) || (rc = M->g.ensure(M->np * 4)) || (rc = M->m.ensure(M->np * 4)) ||
        (rc = M->v.ensure(M->np * 4))) {
        delete M;
        return rc;
    }
    cudaMemcpy(M->p.p, M->host.data(), M->np * 4, cudaMemcpyHostToDevice);
    cudaMemset(M->m.p, 0, M->np * 4);
    cudaMemset(M->v.p, 0, M->np * 4);
    *out = M;
    return CHL_OK;
}

extern "C" size_t chl_gnn_param_count(const chl_gnn *m) { return m ? m->np : 0; }

extern "C" int chl_gnn_get_params(const chl_gnn *m, float *out) {
    if (!m || !out) return CHL_ERR_INVALID;
    CHL_CUDA(cudaMemcpy(out, m->p.p, m->np * 4, cudaMemcpyDeviceToHost));
    return CHL_OK;
}

extern "C" int chl_gnn_set_params(chl_gnn *m, const float *in) {
    if (!m || !in) return CHL_ERR_INVALID;
    CHL_CUDA(cudaMemcpy(m->p.p, in, m->np * 4, cudaMemcpyHostToDevice));
    return CHL_OK;
}

extern "C" int chl_gnn_features(const chl_graph *g, uint64_t seed, float *x) {
    if (!g || !x) return CHL_ERR_INVALID;
    chl_gnn tmp;
    GraphDev G;
    int rc;
    if ((rc = upload_csr(g, G)) || (rc = tmp.x.ensure((size_t)g->n * NF * 4))) return rc;
    feat_raw<<<device_sms() * 4, 256>>>(g->n, G.off_out.as<uint64_t>(), G.head_out.as<uint32_t>(),
                                        G.off_in.as<uint64_t>(), seed, tmp.x.as<float>());
    CHL_CUDA(cudaGetLastError());
    if ((rc = standardise(&tmp, g->n))) return rc;
    CHL_CUDA(cudaMemcpy(x, tmp.x.p, (size_t)g->n * NF * 4, cudaMemcpyDeviceToHost));
    return CHL_OK;
}

extern "C" int chl_gnn_predict(chl_gnn *m, const chl_graph *g, uint64_t seed, float *score) {
    if (!m || !g || !score) return CHL_ERR_INVALID;
    GraphDev G;
    int rc;
    if ((rc = upload_csr(g, G)) || (rc = ensure_scratch(m, g->n)) || (rc = forward(m, G, seed))) return rc;
    CHL_CUDA(cudaMemcpy(score, m->s.p, (size_t)g->n * 4, cudaMemcpyDeviceToHost));
    return CHL_OK;
}

extern "C" int chl_gnn_grad(chl_gnn *m, const chl_graph *g, uint64_t seed, const float *target, double *loss,
                            float *grads) {
    if (!m || !g || !target || !loss) return CHL_ERR_INVALID;
    GraphDev G;
    int rc;
    if ((rc = upload_csr(g, G)) || (rc = ensure_scratch(m, g->n)) || (rc = forward(m, G, seed))) return rc;
    CHL_CUDA(cudaMemcpy(m->y.p, target, (size_t)g->n * 4, cudaMemcpyHostToDevice));
    if ((rc = backward(m, G, loss))) return rc;
    if (grads) CHL_CUDA(cudaMemcpy(grads, m->g.p, m->np * 4, cudaMemcpyDeviceToHost));
    return CHL_OK;
}

extern "C" int chl_gnn_train_step(chl_gnn *m, const chl_graph *g, uint64_t seed, const float *target, float lr,
                                  double *loss) {
    double l = 0;
    int rc = chl_gnn_grad(m, g, seed, target, &l, nullptr);
    if (rc) return rc;
    m->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - (float)std::pow((double)b1, (double)m->step);
    const float c2 = 1.f - (float)std::pow((double)b2, (double)m->step);
    adam_step<<<64, 256>>>(m->np, m->p.as<float>(), m->g.as<float>(), m->m.as<float>(), m->v.as<float>(), lr, b1, b2,
                           1e-8f, c1, c2);
    CHL_CUDA(cudaGetLastError());
    if (loss) *loss = l;
    return CHL_OK;
}

extern "C" int chl_gnn_order(chl_gnn *m, const chl_graph *g, uint64_t seed, uint32_t *order) {
    if (!m || !g || !order) return CHL_ERR_INVALID;
    const uint32_t n = g->n;
    if (n == 0) return CHL_OK;
    GraphDev G;
    int rc;
    if ((rc = upload_csr(g, G)) || (rc = ensure_scratch(m, n)) || (rc = forward(m, G, seed))) return rc;
    return order_by_score(n, seed, m->s.as<float>(), order);
}

extern "C" void chl_gnn_free(chl_gnn *m) { delete m; }
