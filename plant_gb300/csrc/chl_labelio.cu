// Label files at scale: the reference's text layout formatted on the GPU and
// streamed to disk, and a binary CSR twin for fast cold starts.
//
// Text (hl::Labeling::write, shared_memory/labeling.hpp:167-183): `n`, then
// for every vertex v and side 0, 1 one line `size h d h d ...`.  Line y of
// the body is (v, side) = (y / 2, y % 2).  The GPU computes every line's
// byte length, prefix-sums them, and writes the decimal text of a chunk of
// lines into a device buffer (one warp per line; the entries of a line are
// placed by a warp scan of their lengths); the chunk goes to pinned host
// memory and to the file while the next chunk is formatted.
//
// Binary (no reference counterpart): "CHLLBL01", u32 n, u32 symmetric,
// u64 entries, u64 lists, u64 offsets[lists + 1], then (u32 hub, u32 dist)
// entries; little-endian.  Lists are indexed v (symmetric) or 2v + side.
#include "chl_dev.cuh"

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

namespace chl {
namespace {

constexpr size_t kChunk = 256ull << 20;   // bytes per streamed chunk
constexpr char kMagic[8] = {'C', 'H', 'L', 'L', 'B', 'L', '0', '1'};

__device__ __forceinline__ uint32_t udigits(uint32_t x) {
    uint32_t d = 1;
    while (x >= 10) {
        x /= 10;
        ++d;
    }
    return d;
}

__device__ __forceinline__ uint32_t idigits(int32_t x) {
    return x < 0 ? 1 + udigits((uint32_t)(-(int64_t)x)) : udigits((uint32_t)x);
}

__device__ __forceinline__ void put_u(char *p, uint32_t x, uint32_t nd) {
    for (int i = (int)nd - 1; i >= 0; --i) {
        p[i] = (char)('0' + x % 10);
        x /= 10;
    }
}

__device__ __forceinline__ void put_i(char *p, int32_t x, uint32_t nd) {
    if (x < 0) {
        *p = '-';
        put_u(p + 1, (uint32_t)(-(int64_t)x), nd - 1);
    } else {
        put_u(p, (uint32_t)x, nd);
    }
}

__device__ __forceinline__ uint32_t list_of(uint64_t y, int sym) { return sym ? (uint32_t)(y >> 1) : (uint32_t)y; }

// len[y] = bytes of line y including its newline
__global__ void line_len(uint64_t lines, int sym, const uint64_t *off, const LabelEnt *ent, uint32_t *len) {
    const uint32_t lane = lane_id();
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t y = blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); y < lines; y += warps) {
        const uint32_t x = list_of(y, sym);
        const uint64_t b = off[x], e = off[x + 1];
        uint32_t s = 0;
        for (uint64_t k = b + lane; k < e; k += 32) s += 2 + udigits(ent[k].hub) + idigits((int32_t)ent[k].dist);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(kFull, s, o);
        if (lane == 0) len[y] = udigits((uint32_t)(e - b)) + s + 1;
    }
}

// text of lines [y0, y1) at out[line_off[y] - base]
__global__ void line_write(uint64_t y0, uint64_t y1, int sym, const uint64_t *off, const LabelEnt *ent,
                           const uint64_t *line_off, uint64_t base, char *out) {
    const uint32_t lane = lane_id();
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t y = y0 + blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); y < y1; y += warps) {
        const uint32_t x = list_of(y, sym);
        const uint64_t b = off[x], e = off[x + 1];
        char *p = out + (line_off[y] - base);
        const uint32_t nd = udigits((uint32_t)(e - b));
        if (lane == 0) put_u(p, (uint32_t)(e - b), nd);
        uint64_t pos = nd;
        for (uint64_t k0 = b; k0 < e; k0 += 32) {
            const uint64_t k = k0 + lane;
            uint32_t hd = 0, dd = 0, my = 0;
            LabelEnt t{0, 0};
            if (k < e) {
                t = ent[k];
                hd = udigits(t.hub);
                dd = idigits((int32_t)t.dist);
                my = 2 + hd + dd;
            }
            uint32_t incl = my;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t u = __shfl_up_sync(kFull, incl, o);
                if (lane >= (uint32_t)o) incl += u;
            }
            if (k < e) {
                char *q = p + pos + (incl - my);
                q[0] = ' ';
                put_u(q + 1, t.hub, hd);
                q[1 + hd] = ' ';
                put_i(q + 2 + hd, (int32_t)t.dist, dd);
            }
            pos += __shfl_sync(kFull, incl, 31);
        }
        if (lane == 0) p[pos] = '\n';
    }
}

// entries of every list ascending by hub, hubs below n, distances >= 0
__global__ void check_lists(uint64_t nl, uint32_t n, const uint64_t *off, const LabelEnt *ent,
                            unsigned int *bad) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < nl; x += stride) {
        const uint64_t b = off[x], e = off[x + 1];
        for (uint64_t k = b; k < e; ++k) {
            const LabelEnt t = ent[k];
            if (t.hub >= n || (int32_t)t.dist < 0 || (k > b && t.hub <= ent[k - 1].hub)) {
                atomicOr(bad, 1u);
                break;
            }
        }
    }
}

struct Pinned {
    void *p = nullptr;
    ~Pinned() { cudaFreeHost(p); }
};

struct Stream {
    cudaStream_t s = nullptr;
    cudaEvent_t ev = nullptr;
    ~Stream() {
        if (ev) cudaEventDestroy(ev);
        if (s) cudaStreamDestroy(s);
    }
};

struct DevMem {
    void *p = nullptr;
    ~DevMem() { cudaFree(p); }
};

int io_error(const std::string &what) {
    set_error(what);
    return CHL_ERR_IO;
}

bool write_all(FILE *f, const void *p, size_t bytes) { return bytes == 0 || fwrite(p, 1, bytes, f) == bytes; }

// entries per streamed chunk: an eighth of the labels, within [512, kChunk/8]
uint64_t chunk_entries(uint64_t total) {
    return std::max<uint64_t>(512, std::min<uint64_t>(kChunk / sizeof(LabelEnt), total / 8 + 1));
}

}  // namespace

int write_labels_text_device(const chl_labels *l, const char *path) {
    int rc = labels_ensure_device(l);
    if (rc) return rc;
    const uint64_t lines = 2ull * l->n;
    if (lines == 0) {
        FILE *f = fopen(path, "wb");
        if (!f) return io_error(std::string("cannot open ") + path + " for writing");
        const bool ok = fputs("0\n", f) >= 0;
        return (fclose(f) == 0 && ok) ? CHL_OK : io_error(std::string("write failed: ") + path);
    }
    const int sym = l->sym ? 1 : 0;
    const int sms = device_sms();
    DevMem d_len, d_loff, d_tmp, d_buf[2];
    const size_t tmp_bytes = scan_tmp_bytes(lines);
    CHL_CUDA(cudaMalloc(&d_len.p, std::max<uint64_t>(lines, 1) * 4));
    CHL_CUDA(cudaMalloc(&d_loff.p, (lines + 1) * 8));
    CHL_CUDA(cudaMalloc(&d_tmp.p, std::max<size_t>(tmp_bytes, 16)));
    Stream st[2];
    for (auto &s : st) {
        CHL_CUDA(cudaStreamCreateWithFlags(&s.s, cudaStreamNonBlocking));
        CHL_CUDA(cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming));
    }
    line_len<<<sms * 16, 256, 0, st[0].s>>>(lines, sym, l->d_off, l->d_ent, (uint32_t *)d_len.p);
    CHL_CUDA(cudaGetLastError());
    if ((rc = scan_u32_excl((const uint32_t *)d_len.p, (uint64_t *)d_loff.p, lines, nullptr, d_tmp.p, tmp_bytes,
                            st[0].s)))
        return rc;
    std::vector<uint64_t> loff(lines + 1);
    CHL_CUDA(cudaMemcpyAsync(loff.data(), d_loff.p, (lines + 1) * 8, cudaMemcpyDeviceToHost, st[0].s));
    CHL_CUDA(cudaStreamSynchronize(st[0].s));
    // chunks of whole lines: about an eighth of the text (so that even small
    // files stream through both buffers), at most kChunk, at least the
    // longest line
    uint64_t longest = 0;
    for (uint64_t y = 0; y < lines; ++y) longest = std::max(longest, loff[y + 1] - loff[y]);
    const uint64_t cap = std::max<uint64_t>(longest, std::min<uint64_t>(kChunk, std::max<uint64_t>(loff[lines] / 8, 4096)));
    std::vector<uint64_t> cut{0};
    while (cut.back() < lines) {
        const uint64_t y0 = cut.back();
        const uint64_t lim = loff[y0] + cap;
        // last y1 with loff[y1] <= lim
        const uint64_t y1 = (uint64_t)(std::upper_bound(loff.begin() + y0 + 1, loff.end(), lim) - loff.begin()) - 1;
        cut.push_back(std::max(y1, y0 + 1));
    }
    Pinned hbuf[2];
    const uint64_t bufsz = std::min<uint64_t>(cap, std::max<uint64_t>(loff[lines], 1));
    for (int i = 0; i < 2; ++i) {
        CHL_CUDA(cudaMalloc(&d_buf[i].p, bufsz));
        CHL_CUDA(cudaHostAlloc(&hbuf[i].p, bufsz, cudaHostAllocDefault));
    }
    FILE *f = fopen(path, "wb");
    if (!f) return io_error(std::string("cannot open ") + path + " for writing");
    char head[32];
    const int hl = snprintf(head, sizeof(head), "%u\n", l->n);
    bool ok = write_all(f, head, (size_t)hl);
    const size_t chunks = cut.size() - 1;
    auto enqueue = [&](size_t c) -> int {
        const int i = (int)(c & 1);
        const uint64_t y0 = cut[c], y1 = cut[c + 1];
        const uint64_t bytes = loff[y1] - loff[y0];
        const uint64_t warps_needed = y1 - y0;
        const unsigned blocks = (unsigned)std::min<uint64_t>((warps_needed + 7) / 8, (uint64_t)sms * 16);
        line_write<<<std::max(1u, blocks), 256, 0, st[i].s>>>(y0, y1, sym, l->d_off, l->d_ent,
                                                               (const uint64_t *)d_loff.p, loff[y0],
                                                               (char *)d_buf[i].p);
        CHL_CUDA(cudaGetLastError());
        CHL_CUDA(cudaMemcpyAsync(hbuf[i].p, d_buf[i].p, bytes, cudaMemcpyDeviceToHost, st[i].s));
        CHL_CUDA(cudaEventRecord(st[i].ev, st[i].s));
        return CHL_OK;
    };
    for (size_t c = 0; c < std::min<size_t>(2, chunks) && ok; ++c)
        if ((rc = enqueue(c))) break;
    for (size_t c = 0; c < chunks && ok && !rc; ++c) {
        const int i = (int)(c & 1);
        cudaError_t e = cudaEventSynchronize(st[i].ev);
        if (e != cudaSuccess) {
            rc = cuda_status(e, "label text chunk", __FILE__, __LINE__);
            break;
        }
        ok = write_all(f, hbuf[i].p, loff[cut[c + 1]] - loff[cut[c]]);
        if (ok && c + 2 < chunks) rc = enqueue(c + 2);
    }
    cudaStreamSynchronize(st[0].s);
    cudaStreamSynchronize(st[1].s);
    if (ferror(f)) ok = false;
    if (fclose(f) != 0) ok = false;
    if (rc) return rc;
    return ok ? CHL_OK : io_error(std::string("write failed: ") + path);
}

}  // namespace chl

using namespace chl;

extern "C" int chl_labels_save(const chl_labels *l, const char *path) {
    if (!l || !path) return CHL_ERR_INVALID;
    const uint64_t nl = l->nl();
    const uint32_t n = l->n, sym = l->sym ? 1u : 0u;
    const uint64_t total = l->total;
    const bool dev = l->d_off != nullptr;
    std::vector<uint64_t> off;
    const uint64_t *offp;
    if (dev) {
        off.resize(nl + 1);
        CHL_CUDA(cudaMemcpy(off.data(), l->d_off, (nl + 1) * 8, cudaMemcpyDeviceToHost));
        offp = off.data();
    } else {
        offp = l->h_off.data();
    }
    FILE *f = fopen(path, "wb");
    if (!f) return io_error(std::string("cannot open ") + path + " for writing");
    bool ok = write_all(f, kMagic, 8) && write_all(f, &n, 4) && write_all(f, &sym, 4) && write_all(f, &total, 8) &&
              write_all(f, &nl, 8) && write_all(f, offp, (nl + 1) * 8);
    int rc = CHL_OK;
    if (ok && total) {
        if (!dev) {
            ok = write_all(f, l->h_ent.data(), total * sizeof(LabelEnt));
        } else {
            // device entries through two pinned buffers
            Pinned hb[2];
            Stream st[2];
            const uint64_t per = chunk_entries(total);
            for (int i = 0; i < 2 && !rc; ++i) {
                cudaError_t e = cudaHostAlloc(&hb[i].p, per * sizeof(LabelEnt), cudaHostAllocDefault);
                if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st[i].s, cudaStreamNonBlocking);
                if (e == cudaSuccess) e = cudaEventCreateWithFlags(&st[i].ev, cudaEventDisableTiming);
                if (e != cudaSuccess) rc = cuda_status(e, "label save buffers", __FILE__, __LINE__);
            }
            const uint64_t chunks = (total + per - 1) / per;
            auto enqueue = [&](uint64_t c) -> int {
                const int i = (int)(c & 1);
                const uint64_t a = c * per, cnt = std::min(per, total - a);
                CHL_CUDA(cudaMemcpyAsync(hb[i].p, l->d_ent + a, cnt * sizeof(LabelEnt), cudaMemcpyDeviceToHost,
                                         st[i].s));
                CHL_CUDA(cudaEventRecord(st[i].ev, st[i].s));
                return CHL_OK;
            };
            for (uint64_t c = 0; c < std::min<uint64_t>(2, chunks) && !rc; ++c) rc = enqueue(c);
            for (uint64_t c = 0; c < chunks && ok && !rc; ++c) {
                const int i = (int)(c & 1);
                cudaError_t e = cudaEventSynchronize(st[i].ev);
                if (e != cudaSuccess) {
                    rc = cuda_status(e, "label save chunk", __FILE__, __LINE__);
                    break;
                }
                const uint64_t a = c * per, cnt = std::min(per, total - a);
                ok = write_all(f, hb[i].p, cnt * sizeof(LabelEnt));
                if (ok && c + 2 < chunks) rc = enqueue(c + 2);
            }
            if (st[0].s) cudaStreamSynchronize(st[0].s);
            if (st[1].s) cudaStreamSynchronize(st[1].s);
        }
    }
    if (ferror(f)) ok = false;
    if (fclose(f) != 0) ok = false;
    if (rc) return rc;
    return ok ? CHL_OK : io_error(std::string("write failed: ") + path);
}

extern "C" int chl_labels_load(const char *path, chl_labels **out) {
    if (!path || !out) return CHL_ERR_INVALID;
    FILE *f = fopen(path, "rb");
    if (!f) return io_error(std::string("cannot open ") + path);
    struct Closer {
        FILE *f;
        ~Closer() { fclose(f); }
    } closer{f};
    char magic[8];
    uint32_t n = 0, sym = 0;
    uint64_t total = 0, nl = 0;
    if (fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kMagic, 8) != 0 || fread(&n, 4, 1, f) != 1 ||
        fread(&sym, 4, 1, f) != 1 || fread(&total, 8, 1, f) != 1 || fread(&nl, 8, 1, f) != 1) {
        set_error(std::string("not a binary label file: ") + path);
        return CHL_ERR_FORMAT;
    }
    if (sym > 1 || nl != (sym ? (uint64_t)n : 2ull * n)) {
        set_error("binary label file: inconsistent header");
        return CHL_ERR_FORMAT;
    }
    std::vector<uint64_t> off(nl + 1);
    if (fread(off.data(), 8, nl + 1, f) != nl + 1) {
        set_error("binary label file: truncated offsets");
        return CHL_ERR_FORMAT;
    }
    if (off[0] != 0 || off[nl] != total) {
        set_error("binary label file: offsets do not span the entries");
        return CHL_ERR_FORMAT;
    }
    for (uint64_t x = 0; x < nl; ++x)
        if (off[x + 1] < off[x]) {
            set_error("binary label file: offsets are not monotone");
            return CHL_ERR_FORMAT;
        }
    DevMem d_off, d_ent, d_bad;
    CHL_CUDA(cudaMalloc(&d_off.p, (nl + 1) * 8));
    CHL_CUDA(cudaMalloc(&d_ent.p, std::max<uint64_t>(total, 1) * sizeof(LabelEnt)));
    CHL_CUDA(cudaMalloc(&d_bad.p, 4));
    CHL_CUDA(cudaMemcpy(d_off.p, off.data(), (nl + 1) * 8, cudaMemcpyHostToDevice));
    if (total) {
        Pinned hb;
        const uint64_t per = chunk_entries(total);
        CHL_CUDA(cudaHostAlloc(&hb.p, per * sizeof(LabelEnt), cudaHostAllocDefault));
        for (uint64_t a = 0; a < total; a += per) {
            const uint64_t cnt = std::min(per, total - a);
            if (fread(hb.p, sizeof(LabelEnt), cnt, f) != cnt) {
                set_error("binary label file: truncated entries");
                return CHL_ERR_FORMAT;
            }
            CHL_CUDA(cudaMemcpy((LabelEnt *)d_ent.p + a, hb.p, cnt * sizeof(LabelEnt), cudaMemcpyHostToDevice));
        }
    }
    CHL_CUDA(cudaMemset(d_bad.p, 0, 4));
    check_lists<<<device_sms() * 8, 256>>>(nl, n, (const uint64_t *)d_off.p, (const LabelEnt *)d_ent.p,
                                           (unsigned int *)d_bad.p);
    CHL_CUDA(cudaGetLastError());
    unsigned int bad = 0;
    CHL_CUDA(cudaMemcpy(&bad, d_bad.p, 4, cudaMemcpyDeviceToHost));
    if (bad) {
        set_error("binary label file: lists must be ascending by hub (< n) with non-negative distances");
        return CHL_ERR_FORMAT;
    }
    chl_labels *L = new (std::nothrow) chl_labels();
    if (!L) return CHL_ERR_OOM;
    L->n = n;
    L->sym = sym != 0;
    L->total = total;
    L->d_off = (uint64_t *)d_off.p;
    L->d_ent = (LabelEnt *)d_ent.p;
    d_off.p = nullptr;
    d_ent.p = nullptr;
    const uint64_t all = total * (L->sym ? 2 : 1);
    L->stats.labels = all;
    L->stats.avg_label = n ? (double)all / n / 2.0 : 0.0;
    *out = L;
    return CHL_OK;
}
