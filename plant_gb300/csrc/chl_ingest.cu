// GPU ingestion of DIMACS, SNAP and edge-list graph files.
//
// Follows hl::Graph::read_dimacs (shared_memory/graph.hpp:168-189),
// read_snap (:262-282) or read_edgelist (:284-308) line by line and
// hl::Graph::init_arcs (:103-153) for the arc lists, on the device.
// hl::Graph::read (:327-335) tries DIMACS, METIS, SNAP and edge lists in
// turn, so the host picks the reader the reference would end up with:
//  * first non-white-space byte '#': DIMACS fails on the first line (it
//    starts with neither 'p', 'a' nor 'c') and METIS at the '#' (it accepts
//    only digits, white space and '%' comments): SNAP;
//  * first byte 'p', 'a' or 'c', or an empty file: DIMACS;
//  * otherwise DIMACS and SNAP fail on the first line (a SNAP arc before the
//    header sees n = 0), and when the host's METIS reader rejects a prefix
//    of the file (metis_rejects_prefix), edge list; else the host parsers.
//  * the file is copied to HBM; newline positions are found per 4 KB block
//    (count, exclusive scan, ordered write), so every line is known;
//  * one thread parses one line with the rules of the reference's fgets +
//    sscanf loop: a line of 511 or more characters, or the last line without
//    a newline, is accepted only as a comment ('c'); `p sp n m` at most once;
//    `a u v w` with three integers (optional sign, leading white space); any
//    other first character rejects the file as DIMACS;
//  * SNAP: '#' lines are comments, and one of them may be the
//    `# Nodes: n Edges: m` header (matched on the first 511 bytes fgets
//    returns); any other line needs fewer than 511 characters and two
//    integers `u v` (length 1); no arc may precede the header;
//  * edge list: every line needs fewer than 511 characters and three
//    integers `u v w`; n is the number of distinct ids, and the ids, cut to
//    32 bits, must be below it;
//  * every arc (u, v, w) becomes the two records of add_tmp_arc (:156-162),
//    checked against n;
//  * init_arcs: sort by (u, reverse first, forward last, head, length) and
//    keep the first of each (u, head, forward, reverse); sort by (u, head,
//    length) and OR the direction flags of equal records; sort by the first
//    key again; the forward and reverse CSRs are the records in that order.
// Sorts are LSD passes of the project's stable radix sort (length first).
// A file the line rules reject, or one this parser does not handle exactly
// (NUL bytes, numbers of more than 18 digits), is read by the host parsers
// instead, which also try METIS and edge lists and report the errors.
#include "chl_dev.cuh"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

// CHL_CUDA for functions that return a negated status
#define CHL_CUDA_NEG(call)                                                        \
    do {                                                                          \
        cudaError_t _e = (call);                                                  \
        if (_e != cudaSuccess) return -::chl::cuda_status(_e, #call, __FILE__, __LINE__); \
    } while (0)

namespace chl {
namespace {

constexpr uint32_t kBlockBytes = 4096;
constexpr int kLineMax = 511;   // fgets buffer of 512 bytes

// line formats parsed on the device
constexpr int kFmtDimacs = 0;
constexpr int kFmtSnap = 1;
constexpr int kFmtEdgelist = 2;
constexpr int kFmtMetis = 3;

// flags in the status word
constexpr unsigned kFailFormat = 1u;    // not a file of the format by the reference's rules
constexpr unsigned kUnsupported = 2u;   // defer to the host parser

struct ParseOut {
    unsigned status;
    unsigned p_count;
    unsigned long long p_line;   // index of the `p` line
    long long n, m;
    unsigned long long arcs;     // `a` lines
    unsigned long long first_a;  // smallest index of an `a` line
};

__global__ void count_newlines(const char *buf, uint64_t S, uint32_t *cnt) {
    const uint64_t b0 = (uint64_t)blockIdx.x * kBlockBytes;
    uint32_t c = 0;
    for (uint64_t i = b0 + threadIdx.x; i < min(S, b0 + kBlockBytes); i += blockDim.x) c += buf[i] == '\n';
    __shared__ uint32_t s[8];
    c = __reduce_add_sync(kFull, c);
    if (lane_id() == 0) s[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[w];
        cnt[blockIdx.x] = t;
    }
}

// newline positions in file order: block-level exclusive scan of per-thread
// counts over contiguous 16-byte pieces of the block
__global__ void write_newlines(const char *buf, uint64_t S, const uint64_t *pre, uint64_t *pos) {
    constexpr uint32_t kPer = kBlockBytes / 256;
    const uint64_t b0 = (uint64_t)blockIdx.x * kBlockBytes + (uint64_t)threadIdx.x * kPer;
    uint32_t c = 0;
    for (uint32_t k = 0; k < kPer; ++k)
        if (b0 + k < S && buf[b0 + k] == '\n') ++c;
    __shared__ uint32_t ws[8];
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, incl, o);
        if (lane_id() >= (uint32_t)o) incl += y;
    }
    if (lane_id() == 31) ws[threadIdx.x >> 5] = incl;
    __syncthreads();
    uint32_t woff = 0;
    for (uint32_t w = 0; w < (threadIdx.x >> 5); ++w) woff += ws[w];
    uint64_t at = pre[blockIdx.x] + woff + incl - c;
    for (uint32_t k = 0; k < kPer; ++k)
        if (b0 + k < S && buf[b0 + k] == '\n') pos[at++] = b0 + k;
}

__device__ __forceinline__ bool is_space(char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

// sscanf("%lld") at p (leading white space allowed); false if no digits.
// Sets *unsupported for more than 18 digits (overflow is handled by the host).
__device__ __forceinline__ bool scan_ll(const char *&p, const char *e, long long &out, bool &unsupported) {
    while (p < e && is_space(*p)) ++p;
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) {
        neg = *p == '-';
        ++p;
    }
    int digits = 0;
    long long v = 0;
    while (p < e && *p >= '0' && *p <= '9') {
        if (++digits > 18) {
            unsupported = true;
            return false;
        }
        v = v * 10 + (*p - '0');
        ++p;
    }
    if (!digits) return false;
    out = neg ? -v : v;
    return true;
}

__device__ __forceinline__ void skip_space(const char *&p, const char *e) {
    while (p < e && is_space(*p)) ++p;
}

// a literal of the sscanf format: must match the next characters exactly
__device__ __forceinline__ bool match_lit(const char *&p, const char *e, const char *lit) {
    for (; *lit; ++lit, ++p)
        if (p >= e || *p != *lit) return false;
    return true;
}

// sscanf(line, "# Nodes: %lld Edges: %lld") == 2, with p just after the '#'
// (a blank of the format matches any run of white space, none included).
// A line that converts the vertex count but not the edge count still sets
// n in the reference (sscanf stores each conversion as it succeeds), which
// changes n between arcs: such files are left to the host (*unsup).
__device__ __forceinline__ bool snap_header(const char *p, const char *e, long long &n, long long &m, bool &unsup) {
    skip_space(p, e);
    if (!match_lit(p, e, "Nodes:") || !scan_ll(p, e, n, unsup)) return false;
    skip_space(p, e);
    const bool full = match_lit(p, e, "Edges:") && scan_ll(p, e, m, unsup);
    if (!full) unsup = true;
    return full;
}

// One line per thread.  DIMACS: `p` fills the header fields; SNAP: the
// `# Nodes:` line does.  Arcs go to unordered slots (init_arcs sorts them).
__global__ void parse_lines(const char *buf, uint64_t S, const uint64_t *nl, uint64_t nnl, uint64_t lines,
                            int fmt, ParseOut *po, int64_t *au, int64_t *av, int64_t *aw) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < lines; k += stride) {
        const uint64_t start = k == 0 ? 0 : nl[k - 1] + 1;
        const bool has_nl = k < nnl;
        const uint64_t end = has_nl ? nl[k] : S;   // exclusive, without the newline
        const uint64_t len = end - start;
        const char *p = buf + start, *e = buf + end;
        // NUL bytes change what fgets/strlen see: leave such files to the host
        for (const char *q = p; q < e; ++q)
            if (*q == '\0') {
                atomicOr(&po->status, kUnsupported);
                break;
            }
        const char c0 = len ? p[0] : '\n';
        if (fmt == kFmtSnap) {
            bool unsup = false;
            if (c0 == '#') {
                // fgets hands sscanf the first 511 bytes; the rest is skipped
                long long n = 0, m = 0;
                const char *qe = p + (len < (uint64_t)kLineMax ? len : (uint64_t)kLineMax);
                if (snap_header(p + 1, qe, n, m, unsup)) {
                    atomicAdd(&po->p_count, 1u);
                    po->p_line = k;   // meaningful only when p_count == 1
                    po->n = n;
                    po->m = m;
                }
                if (unsup) atomicOr(&po->status, kUnsupported);
                continue;
            }
            // a line fgets returns in pieces is rejected (the last line may
            // lack its newline)
            if (len >= (uint64_t)kLineMax) {
                atomicOr(&po->status, kFailFormat);
                continue;
            }
            const char *q = p;
            long long u = 0, v = 0;
            const bool ok = scan_ll(q, e, u, unsup) && scan_ll(q, e, v, unsup);
            if (unsup) atomicOr(&po->status, kUnsupported);
            if (!ok) {
                atomicOr(&po->status, kFailFormat);
                continue;
            }
            const unsigned long long slot = atomicAdd(&po->arcs, 1ull);
            atomicMin(&po->first_a, (unsigned long long)k);
            au[slot] = u;
            av[slot] = v;
            aw[slot] = 1;
            continue;
        }
        if (fmt == kFmtEdgelist) {
            // a line fgets returns in pieces is rejected (the last line may
            // lack its newline); `sscanf(buf, "%lld %lld %lld") == 3`
            bool unsup = false;
            if (len >= (uint64_t)kLineMax) {
                atomicOr(&po->status, kFailFormat);
                continue;
            }
            const char *q = p;
            long long u = 0, v = 0, w = 0;
            const bool ok = scan_ll(q, e, u, unsup) && scan_ll(q, e, v, unsup) && scan_ll(q, e, w, unsup);
            if (unsup) atomicOr(&po->status, kUnsupported);
            if (!ok) {
                atomicOr(&po->status, kFailFormat);
                continue;
            }
            const unsigned long long slot = atomicAdd(&po->arcs, 1ull);
            au[slot] = u;
            av[slot] = v;
            aw[slot] = w;
            continue;
        }
        if (len >= (uint64_t)kLineMax || !has_nl) {
            // read in pieces by fgets: acceptable only as a comment
            if (c0 != 'c') atomicOr(&po->status, kFailFormat);
            continue;
        }
        if (c0 == 'c') continue;
        bool unsup = false;
        if (c0 == 'p') {
            // "p sp %lld %lld"
            const char *q = p + 1;
            long long n = 0, m = 0;
            skip_space(q, e);
            bool ok = q + 1 < e && q[0] == 's' && q[1] == 'p';
            if (ok) {
                q += 2;
                ok = scan_ll(q, e, n, unsup) && scan_ll(q, e, m, unsup);
            }
            if (unsup) atomicOr(&po->status, kUnsupported);
            if (!ok) {
                atomicOr(&po->status, kFailFormat);
                continue;
            }
            atomicAdd(&po->p_count, 1u);
            po->p_line = k;   // meaningful only when p_count == 1
            po->n = n;
            po->m = m;
            continue;
        }
        if (c0 == 'a') {
            const char *q = p + 1;
            long long u = 0, v = 0, w = 0;
            const bool ok = scan_ll(q, e, u, unsup) && scan_ll(q, e, v, unsup) && scan_ll(q, e, w, unsup);
            if (unsup) atomicOr(&po->status, kUnsupported);
            if (!ok) {
                atomicOr(&po->status, kFailFormat);
                continue;
            }
            const unsigned long long slot = atomicAdd(&po->arcs, 1ull);
            atomicMin(&po->first_a, (unsigned long long)k);
            au[slot] = u;
            av[slot] = v;
            aw[slot] = w;
            continue;
        }
        atomicOr(&po->status, kFailFormat);
    }
}

// ---- METIS (shared_memory/graph.hpp:211-256) on the device
// The reference reads METIS byte by byte: digits make numbers, white space
// ends them, a newline ends a line, and '%' swallows everything through the
// next newline, which then ends no line.  A physical line whose first
// non-blank byte is '%' is therefore no line at all; every other physical
// line is one METIS line.  A '%' after a number on a line joins that line
// with the next (and may join two numbers): such files go to the host.

// 1 for a physical line that is a METIS line, 0 for a comment line
__global__ void metis_line_flags(const char *buf, uint64_t S, const uint64_t *nl, uint64_t nnl, uint64_t lines,
                                 uint32_t *flag) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < lines; k += stride) {
        const uint64_t start = k == 0 ? 0 : nl[k - 1] + 1;
        const uint64_t end = k < nnl ? nl[k] : S;
        uint64_t q = start;
        while (q < end && is_space(buf[q])) ++q;
        flag[k] = (q < end && buf[q] == '%') ? 0u : 1u;
    }
}

// One METIS line per thread.  idx[k]: its line number (exclusive scan of the
// flags; line 0, the header, was read on the host).  Vertex idx[k] - 1 gets
// an arc per head after the first `skip` numbers, with the following number
// as its length when `weighted`.  A line that ends with a newline must hold
// all its leading numbers and no head without a length.
__global__ void metis_parse_lines(const char *buf, uint64_t S, const uint64_t *nl, uint64_t nnl, uint64_t lines,
                                  const uint32_t *flag, const uint64_t *idx, int skip, int weighted, ParseOut *po,
                                  int64_t *au, int64_t *av, int64_t *aw) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < lines; k += stride) {
        if (!flag[k] || idx[k] == 0) continue;
        const uint64_t start = k == 0 ? 0 : nl[k - 1] + 1;
        const bool has_nl = k < nnl;
        const uint64_t end = has_nl ? nl[k] : S;
        const long long line = (long long)idx[k];
        int i = 0, digits = 0;
        long long x = 0, head = 0;
        bool bad = false;
        for (uint64_t q = start; q <= end; ++q) {
            const char c = q < end ? buf[q] : ' ';
            if (c >= '0' && c <= '9') {
                if (++digits > 18) {
                    atomicOr(&po->status, kUnsupported);
                    bad = true;
                    break;
                }
                x = x * 10 + (c - '0');
                continue;
            }
            if (c == '%') {
                atomicOr(&po->status, kUnsupported);   // a comment after numbers joins lines
                bad = true;
                break;
            }
            if (!is_space(c)) {
                atomicOr(&po->status, kFailFormat);
                bad = true;
                break;
            }
            if (digits) {
                if (i >= skip) {
                    if (weighted && ((i - skip) & 1) == 0) {
                        head = x;
                    } else {
                        const unsigned long long slot = atomicAdd(&po->arcs, 1ull);
                        au[slot] = line;                 // vertex line - 1
                        av[slot] = weighted ? head : x;  // head + 1
                        aw[slot] = weighted ? x : 1;
                    }
                }
                ++i;
                digits = 0;
                x = 0;
            }
        }
        if (!bad && has_nl && (i < skip || (weighted && ((i - skip) & 1))))
            atomicOr(&po->status, kFailFormat);
    }
}

// edge-list ids as order-preserving unsigned keys (sign bit flipped)
__global__ void id_keys(uint64_t arcs, const int64_t *au, const int64_t *av, uint64_t *key, uint32_t *val) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < arcs; i += stride) {
        key[2 * i] = (uint64_t)au[i] ^ (1ull << 63);
        key[2 * i + 1] = (uint64_t)av[i] ^ (1ull << 63);
        val[2 * i] = 0;
        val[2 * i + 1] = 0;
    }
}

// number of distinct values of a sorted key array
__global__ void count_distinct(uint64_t cnt, const uint64_t *key, unsigned long long *out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t b = blockIdx.x * (uint64_t)blockDim.x; b < cnt; b += stride) {
        const uint64_t i = b + threadIdx.x;
        const bool first = i < cnt && (i == 0 || key[i] != key[i - 1]);
        const unsigned m = __ballot_sync(0xFFFFFFFFu, first);
        if ((threadIdx.x & 31) == 0 && m) atomicAdd(out, (unsigned long long)__popc(m));
    }
}

// add_tmp_arc: bounds check of the 32-bit vertex values (ids minus `base`:
// 1 for DIMACS, 0 for SNAP) against n, then the two records
// (u, v, w, fwd, und) and (v, u, w, und, rev)
__global__ void make_records(uint64_t arcs, const int64_t *au, const int64_t *av, const int64_t *aw, long long n,
                             int base, int undirected, uint32_t *ru, uint32_t *rh, int32_t *rl, uint32_t *rf,
                             unsigned *status) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < arcs; i += stride) {
        const uint32_t u = (uint32_t)(au[i] - base), v = (uint32_t)(av[i] - base);
        if ((long long)u >= n || (long long)v >= n) atomicOr(status, kFailFormat);
        const int32_t w = (int32_t)aw[i];
        // flags: bit 0 forward, bit 1 reverse
        ru[2 * i] = u;
        rh[2 * i] = v;
        rl[2 * i] = w;
        rf[2 * i] = 1u | (undirected ? 2u : 0u);
        ru[2 * i + 1] = v;
        rh[2 * i + 1] = u;
        rl[2 * i + 1] = w;
        rf[2 * i + 1] = (undirected ? 1u : 0u) | 2u;
    }
}

__device__ __forceinline__ uint64_t len_key(int32_t l) { return (uint64_t)((uint32_t)l ^ 0x80000000u); }

// key of cmp_by_direction without the length: u, reverse first, non-forward
// first, head
__device__ __forceinline__ uint64_t dir_key(uint32_t u, uint32_t h, uint32_t f) {
    const uint64_t rev_last = (f & 2u) ? 0 : 1, fwd = f & 1u;
    return ((uint64_t)u << 32) | (rev_last << 31) | (fwd << 30) | (uint64_t)h;
}

__global__ void keys_len(uint64_t cnt, const int32_t *rl, uint64_t *key, uint32_t *val) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt; i += stride) {
        key[i] = len_key(rl[i]);
        val[i] = (uint32_t)i;
    }
}

// second LSD pass: key of record val[i] (dir: cmp_by_direction, else
// cmp_by_head's (u, head))
__global__ void keys_major(uint64_t cnt, const uint32_t *val, const uint32_t *ru, const uint32_t *rh,
                           const uint32_t *rf, int dir, uint64_t *key) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt; i += stride) {
        const uint32_t r = val[i];
        key[i] = dir ? dir_key(ru[r], rh[r], rf[r]) : (((uint64_t)ru[r] << 30) | rh[r]);
    }
}

template <typename T>
__global__ void gather(uint64_t cnt, const uint32_t *idx, const T *in, T *out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt; i += stride) out[i] = in[idx[i]];
}

// mode 0: keep the first of each (u, head, fwd, rev) run (records sorted by
// the direction key);  mode 1: first of each (u, head, len) run
__global__ void run_heads(uint64_t cnt, const uint32_t *ru, const uint32_t *rh, const int32_t *rl,
                          const uint32_t *rf, int mode, uint32_t *head) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt; i += stride) {
        bool first = i == 0;
        if (!first) {
            first = ru[i] != ru[i - 1] || rh[i] != rh[i - 1];
            if (mode == 0) first = first || rf[i] != rf[i - 1];
            else first = first || rl[i] != rl[i - 1];
        }
        head[i] = first ? 1u : 0u;
    }
}

// compact the run heads (pos = exclusive scan of head); mode 1 also ORs the
// flags of every member into its run head's slot (flags_out zeroed before)
__global__ void compact_runs(uint64_t cnt, const uint32_t *head, const uint64_t *pos, const uint32_t *ru,
                             const uint32_t *rh, const int32_t *rl, const uint32_t *rf, int mode, uint32_t *ou,
                             uint32_t *oh, int32_t *ol, uint32_t *of) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt; i += stride) {
        const uint64_t run = pos[i] + head[i] - 1;   // index of this record's run
        if (head[i]) {
            ou[run] = ru[i];
            oh[run] = rh[i];
            ol[run] = rl[i];
            if (mode == 0) of[run] = rf[i];
        }
        if (mode == 1) atomicOr(&of[run], rf[i]);
    }
}

__global__ void side_flags(uint64_t cnt, const uint32_t *rf, uint32_t bit, uint32_t *out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt; i += stride)
        out[i] = (rf[i] & bit) ? 1u : 0u;
}

// per-vertex arc counts of one side
__global__ void side_counts(uint64_t cnt, const uint32_t *ru, const uint32_t *rf, uint32_t bit, uint32_t *deg) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt; i += stride)
        if (rf[i] & bit) atomicAdd(&deg[ru[i]], 1u);
}

__global__ void side_place(uint64_t cnt, const uint32_t *rf, uint32_t bit, const uint64_t *pos, const uint32_t *rh,
                           const int32_t *rl, uint32_t *head, int32_t *len) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt; i += stride)
        if (rf[i] & bit) {
            head[pos[i]] = rh[i];
            len[pos[i]] = rl[i];
        }
}

// device buffers freed on every return path
struct Pool {
    std::vector<void *> ptrs;
    ~Pool() {
        for (void *p : ptrs) cudaFree(p);
    }
    template <typename T>
    int get(T **p, uint64_t count) {
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, std::max<uint64_t>(count, 1) * sizeof(T));
        if (e != cudaSuccess) return cuda_status(e, "cudaMalloc", __FILE__, __LINE__);
        ptrs.push_back(q);
        *p = (T *)q;
        return CHL_OK;
    }
};

// (k, v) stable radix sort on `bits` key bits; result in (k0, v0)
int sort_kv(uint64_t *&k0, uint32_t *&v0, uint64_t *&k1, uint32_t *&v1, const uint64_t *d_cnt, uint64_t cnt,
            int bits, void *tmp, size_t tmp_bytes) {
    int par = 0;
    int rc = radix_sort_pairs(k0, v0, k1, v1, d_cnt, cnt, bits, tmp, tmp_bytes, 0, &par);
    if (rc) return rc;
    if (par) {
        std::swap(k0, k1);
        std::swap(v0, v1);
    }
    return CHL_OK;
}

// Records sorted by (major key, length): permutation into v, records gathered.
int sort_records(uint64_t cnt, int dir, uint32_t *&ru, uint32_t *&rh, int32_t *&rl, uint32_t *&rf, uint32_t *&tu,
                 uint32_t *&th, int32_t *&tl, uint32_t *&tf, uint64_t *k0, uint32_t *v0, uint64_t *k1, uint32_t *v1,
                 const uint64_t *d_cnt, void *tmp, size_t tmp_bytes) {
    const int grid = device_sms() * 8;
    keys_len<<<grid, 256>>>(cnt, rl, k0, v0);
    int rc = sort_kv(k0, v0, k1, v1, d_cnt, cnt, 32, tmp, tmp_bytes);
    if (rc) return rc;
    keys_major<<<grid, 256>>>(cnt, v0, ru, rh, rf, dir, k0);
    if ((rc = sort_kv(k0, v0, k1, v1, d_cnt, cnt, dir ? 62 : 60, tmp, tmp_bytes))) return rc;
    gather<uint32_t><<<grid, 256>>>(cnt, v0, ru, tu);
    gather<uint32_t><<<grid, 256>>>(cnt, v0, rh, th);
    gather<int32_t><<<grid, 256>>>(cnt, v0, rl, tl);
    gather<uint32_t><<<grid, 256>>>(cnt, v0, rf, tf);
    CHL_CUDA(cudaGetLastError());
    std::swap(ru, tu);
    std::swap(rh, th);
    std::swap(rl, tl);
    std::swap(rf, tf);
    return CHL_OK;
}

int read_file(const char *path, std::vector<char> &buf) {
    FILE *f = fopen(path, "rb");
    if (!f) {
        set_error(std::string("cannot open graph file ") + path);
        return CHL_ERR_IO;
    }
    fseek(f, 0, SEEK_END);
    const long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    if (sz < 0) {
        fclose(f);
        set_error(std::string("cannot size graph file ") + path);
        return CHL_ERR_IO;
    }
    buf.resize((size_t)sz);
    const size_t got = sz ? fread(buf.data(), 1, (size_t)sz, f) : 0;
    fclose(f);
    if (got != (size_t)sz) {
        set_error(std::string("short read of graph file ") + path);
        return CHL_ERR_IO;
    }
    return CHL_OK;
}

// The METIS header: the first physical line whose first non-blank byte is
// not '%' (comment lines before it are swallowed), read with the reference's
// rules: `n m [fmt [ncon]]`, fmt's digits each 0 or 1 and fmt <= 111, ncon
// only when fmt's tens digit is 1.  Returns 1 with n, skip and weighted set,
// 0 when the host must decide (a rejected header, a comment after a number,
// more than 18 digits).
int metis_header(const std::vector<char> &file, long long &n, int &skip, int &weighted) {
    size_t q = 0;
    const size_t S = file.size();
    auto space = [&](char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; };
    while (true) {   // skip comment lines
        size_t a = q;
        while (a < S && space(file[a]) && file[a] != '\n') ++a;
        if (a < S && file[a] == '%') {
            while (a < S && file[a] != '\n') ++a;
            q = a + 1;
            continue;
        }
        break;
    }
    long long tok[4] = {0, 0, 0, 0};
    int cnt = 0, digits = 0;
    long long x = 0;
    for (; q <= S; ++q) {
        const char c = q < S ? file[q] : ' ';
        if (c >= '0' && c <= '9') {
            if (++digits > 18) return 0;
            x = x * 10 + (c - '0');
            continue;
        }
        if (!space(c)) return 0;
        if (digits) {
            if (cnt >= 4) return 0;
            tok[cnt++] = x;
            digits = 0;
            x = 0;
        }
        if (c == '\n' || q == S) break;
    }
    if (cnt == 0) return 0;
    n = tok[0];
    long long fmt = 0;
    skip = 0;
    if (cnt >= 3) {
        fmt = tok[2];
        if (fmt % 10 > 1 || (fmt / 10) % 10 > 1 || fmt > 111) return 0;
        skip = (fmt >= 100) + (fmt % 100 >= 10);
    }
    if (cnt == 4) {
        if (fmt % 100 < 10) return 0;
        skip = (int)((fmt >= 100) + tok[3]);
    }
    weighted = fmt % 10 == 1;
    return 1;
}

// 1: the file is of format fmt by the reference's rules and the graph was
// built; 0: defer to the host parsers; < 0: -status of an error
int ingest_text(const std::vector<char> &file, int fmt, bool undirected, chl_graph *g) {
    const uint64_t S = file.size();
    Pool pool;
    int rc;
    char *d_buf;
    if ((rc = pool.get(&d_buf, S + 16))) return -rc;
    if (S) CHL_CUDA_NEG(cudaMemcpy(d_buf, file.data(), S, cudaMemcpyHostToDevice));
    const uint64_t nblk = (S + kBlockBytes - 1) / kBlockBytes;
    uint32_t *d_cnt;
    uint64_t *d_pre;
    if ((rc = pool.get(&d_cnt, nblk + 1)) || (rc = pool.get(&d_pre, nblk + 2))) return -rc;
    void *tmp;
    const size_t tmp_bytes = std::max(scan_tmp_bytes(std::max<uint64_t>(nblk, 1)), radix_tmp_bytes());
    if ((rc = pool.get((char **)&tmp, tmp_bytes))) return -rc;
    uint64_t nnl = 0;
    if (nblk) {
        count_newlines<<<(unsigned)nblk, 256>>>(d_buf, S, d_cnt);
        CHL_CUDA_NEG(cudaGetLastError());
        if ((rc = scan_u32_excl(d_cnt, d_pre, nblk, nullptr, tmp, tmp_bytes, 0))) return -rc;
        CHL_CUDA_NEG(cudaMemcpy(&nnl, d_pre + nblk, 8, cudaMemcpyDeviceToHost));
    }
    uint64_t *d_nl;
    if ((rc = pool.get(&d_nl, nnl + 1))) return -rc;
    if (nblk) write_newlines<<<(unsigned)nblk, 256>>>(d_buf, S, d_pre, d_nl);
    // lines: one per newline, plus a last one without a newline
    const bool tail = S && file[S - 1] != '\n';
    const uint64_t lines = nnl + (tail ? 1 : 0);
    ParseOut h{0, 0, 0, 0, 0, 0, ~0ull}, *d_po;
    if ((rc = pool.get(&d_po, 1))) return -rc;
    CHL_CUDA_NEG(cudaMemcpy(d_po, &h, sizeof(h), cudaMemcpyHostToDevice));
    int64_t *au, *av, *aw;
    if ((rc = pool.get(&au, lines)) || (rc = pool.get(&av, lines)) || (rc = pool.get(&aw, lines))) return -rc;
    long long metis_n = 0;
    if (fmt == kFmtMetis) {
        int skip = 0, weighted = 0;
        if (!metis_header(file, metis_n, skip, weighted)) return 0;
        uint32_t *d_flag;
        uint64_t *d_idx;
        if ((rc = pool.get(&d_flag, lines + 1)) || (rc = pool.get(&d_idx, lines + 2))) return -rc;
        void *ltmp;
        const size_t ltmp_bytes = scan_tmp_bytes(std::max<uint64_t>(lines, 1));
        if ((rc = pool.get((char **)&ltmp, ltmp_bytes))) return -rc;
        if (lines) {
            metis_line_flags<<<device_sms() * 8, 256>>>(d_buf, S, d_nl, nnl, lines, d_flag);
            CHL_CUDA_NEG(cudaGetLastError());
            if ((rc = scan_u32_excl(d_flag, d_idx, lines, nullptr, ltmp, ltmp_bytes, 0))) return -rc;
            metis_parse_lines<<<device_sms() * 8, 256>>>(d_buf, S, d_nl, nnl, lines, d_flag, d_idx, skip, weighted,
                                                         d_po, au, av, aw);
            CHL_CUDA_NEG(cudaGetLastError());
        }
    } else if (lines) {
        parse_lines<<<device_sms() * 8, 256>>>(d_buf, S, d_nl, nnl, lines, fmt, d_po, au, av, aw);
        CHL_CUDA_NEG(cudaGetLastError());
    }
    CHL_CUDA_NEG(cudaMemcpy(&h, d_po, sizeof(h), cudaMemcpyDeviceToHost));
    if (h.status & kUnsupported) return 0;
    if (h.status & kFailFormat) return 0;
    long long n = 0;
    if (fmt == kFmtEdgelist) {
        // n = the number of distinct ids
        if (h.arcs) {
            const uint64_t c2 = 2 * h.arcs;
            uint64_t *ka, *kb, *d_c2;
            uint32_t *va, *vb;
            unsigned long long *d_dist;
            if ((rc = pool.get(&ka, c2)) || (rc = pool.get(&kb, c2)) || (rc = pool.get(&va, c2)) ||
                (rc = pool.get(&vb, c2)) || (rc = pool.get(&d_c2, 1)) || (rc = pool.get(&d_dist, 1)))
                return -rc;
            CHL_CUDA_NEG(cudaMemcpy(d_c2, &c2, 8, cudaMemcpyHostToDevice));
            CHL_CUDA_NEG(cudaMemset(d_dist, 0, 8));
            id_keys<<<device_sms() * 8, 256>>>(h.arcs, au, av, ka, va);
            CHL_CUDA_NEG(cudaGetLastError());
            if ((rc = sort_kv(ka, va, kb, vb, d_c2, c2, 64, tmp, tmp_bytes))) return -rc;
            count_distinct<<<device_sms() * 8, 256>>>(c2, ka, d_dist);
            CHL_CUDA_NEG(cudaGetLastError());
            unsigned long long nd = 0;
            CHL_CUDA_NEG(cudaMemcpy(&nd, d_dist, 8, cudaMemcpyDeviceToHost));
            n = (long long)nd;
        }
    } else if (fmt == kFmtMetis) {
        n = metis_n;
    } else {
        if (h.p_count > 1) return 0;                   // a second header
        n = h.p_count ? h.n : 0;                       // arcs before the header see n = 0
        if (h.arcs && (h.p_count == 0 || h.first_a < h.p_line)) return 0;
    }
    if (n < 0) return 0;   // the host decides (every arc fails the bounds check)
    if (n >= (1ll << 30)) {
        set_error("graph has too many vertices (the arc head field is 30 bits)");
        return -CHL_ERR_INVALID;
    }
    const uint64_t arcs = h.arcs, cnt = 2 * arcs;
    uint32_t *ru, *rh, *rf, *tu, *th, *tf, *d_status;
    int32_t *rl, *tl;
    if ((rc = pool.get(&ru, cnt)) || (rc = pool.get(&rh, cnt)) || (rc = pool.get(&rl, cnt)) ||
        (rc = pool.get(&rf, cnt)) || (rc = pool.get(&tu, cnt)) || (rc = pool.get(&th, cnt)) ||
        (rc = pool.get(&tl, cnt)) || (rc = pool.get(&tf, cnt)) || (rc = pool.get(&d_status, 1)))
        return -rc;
    const int grid = device_sms() * 8;
    CHL_CUDA_NEG(cudaMemset(d_status, 0, 4));
    if (arcs)
        make_records<<<grid, 256>>>(arcs, au, av, aw, n, (fmt == kFmtDimacs || fmt == kFmtMetis) ? 1 : 0,
                                    undirected ? 1 : 0, ru, rh,
                                    rl, rf, d_status);
    unsigned st = 0;
    CHL_CUDA_NEG(cudaMemcpy(&st, d_status, 4, cudaMemcpyDeviceToHost));
    if (st) return 0;   // an arc endpoint outside [0, n): not this format (the host tries the others)
    g->n = (uint32_t)n;
    g->m = arcs * (undirected ? 2 : 1);
    // init_arcs
    uint64_t *k0, *k1, *d_n, *pos;
    uint32_t *v0, *v1, *hd;
    if ((rc = pool.get(&k0, cnt)) || (rc = pool.get(&k1, cnt)) || (rc = pool.get(&v0, cnt)) ||
        (rc = pool.get(&v1, cnt)) || (rc = pool.get(&d_n, 1)) || (rc = pool.get(&hd, cnt + 1)) ||
        (rc = pool.get(&pos, cnt + 2)))
        return -rc;
    void *stmp;
    const size_t stmp_bytes =
        std::max(scan_tmp_bytes(std::max<uint64_t>(cnt + 1, (uint64_t)n + 1)), radix_tmp_bytes());
    if ((rc = pool.get((char **)&stmp, stmp_bytes))) return -rc;
    uint64_t live = cnt;
    auto set_count = [&](uint64_t c) -> int {
        CHL_CUDA(cudaMemcpy(d_n, &c, 8, cudaMemcpyHostToDevice));
        return CHL_OK;
    };
    auto compact = [&](int mode) -> int {
        int r;
        run_heads<<<grid, 256>>>(live, ru, rh, rl, rf, mode, hd);
        if ((r = scan_u32_excl(hd, pos, live, nullptr, stmp, stmp_bytes, 0))) return r;
        uint64_t runs = 0;
        CHL_CUDA(cudaMemcpy(&runs, pos + live, 8, cudaMemcpyDeviceToHost));
        if (mode == 1) CHL_CUDA(cudaMemset(tf, 0, runs * 4));
        compact_runs<<<grid, 256>>>(live, hd, pos, ru, rh, rl, rf, mode, tu, th, tl, tf);
        CHL_CUDA(cudaGetLastError());
        std::swap(ru, tu);
        std::swap(rh, th);
        std::swap(rl, tl);
        std::swap(rf, tf);
        live = runs;
        return CHL_OK;
    };
    if (cnt) {
        if ((rc = set_count(live)) ||
            (rc = sort_records(live, 1, ru, rh, rl, rf, tu, th, tl, tf, k0, v0, k1, v1, d_n, stmp, stmp_bytes)) ||
            (rc = compact(0)) || (rc = set_count(live)) ||
            (rc = sort_records(live, 0, ru, rh, rl, rf, tu, th, tl, tf, k0, v0, k1, v1, d_n, stmp, stmp_bytes)) ||
            (rc = compact(1)) || (rc = set_count(live)) ||
            (rc = sort_records(live, 1, ru, rh, rl, rf, tu, th, tl, tf, k0, v0, k1, v1, d_n, stmp, stmp_bytes)))
            return -rc;
    }
    // the two CSRs: side 1 = forward (flag bit 0), side 0 = reverse (bit 1)
    uint32_t *deg, *ohead;
    uint64_t *doff;
    int32_t *olen;
    if ((rc = pool.get(&deg, (uint64_t)n + 1)) || (rc = pool.get(&doff, (uint64_t)n + 2)) ||
        (rc = pool.get(&ohead, live)) || (rc = pool.get(&olen, live)))
        return -rc;
    for (int s = 0; s < 2; ++s) {
        const uint32_t bit = s == 1 ? 1u : 2u;
        CHL_CUDA_NEG(cudaMemset(deg, 0, ((uint64_t)n + 1) * 4));
        if (live) side_counts<<<grid, 256>>>(live, ru, rf, bit, deg);
        if (n && (rc = scan_u32_excl(deg, doff, (uint64_t)n, nullptr, stmp, stmp_bytes, 0))) return -rc;
        if (live) {
            side_flags<<<grid, 256>>>(live, rf, bit, hd);
            if ((rc = scan_u32_excl(hd, pos, live, nullptr, stmp, stmp_bytes, 0))) return -rc;
            side_place<<<grid, 256>>>(live, rf, bit, pos, rh, rl, ohead, olen);
        }
        CHL_CUDA_NEG(cudaGetLastError());
        uint64_t m_s = 0;
        if (n) CHL_CUDA_NEG(cudaMemcpy(&m_s, doff + n, 8, cudaMemcpyDeviceToHost));
        g->off[s].assign((size_t)n + 1, 0);
        if (n) CHL_CUDA_NEG(cudaMemcpy(g->off[s].data(), doff, ((size_t)n + 1) * 8, cudaMemcpyDeviceToHost));
        g->head[s].resize(m_s);
        g->len[s].resize(m_s);
        if (m_s) {
            CHL_CUDA_NEG(cudaMemcpy(g->head[s].data(), ohead, m_s * 4, cudaMemcpyDeviceToHost));
            CHL_CUDA_NEG(cudaMemcpy(g->len[s].data(), olen, m_s * 4, cudaMemcpyDeviceToHost));
        }
    }
    graph_fill_stats(g);
    return 1;
}

}  // namespace
}  // namespace chl

using namespace chl;

extern "C" int chl_graph_load_gpu(const char *path, int undirected, chl_graph **out, int *parsed_on_gpu) {
    if (!path || !out) return CHL_ERR_INVALID;
    if (parsed_on_gpu) *parsed_on_gpu = 0;
    std::vector<char> file;
    int rc = read_file(path, file);
    if (rc) return rc;
    chl_graph *g = new (std::nothrow) chl_graph();
    if (!g) return CHL_ERR_OOM;
    // the reader the reference would end up with (see the top of this file)
    int fmt = -1;
    char first = 0;
    for (char c : file) {
        if (c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r') continue;
        first = c;
        break;
    }
    if (first == '#') fmt = kFmtSnap;
    else if (file.empty() || file[0] == 'p' || file[0] == 'a' || file[0] == 'c') fmt = kFmtDimacs;
    else if (metis_rejects_prefix(file.data(), std::min<size_t>(file.size(), (size_t)1 << 16))) fmt = kFmtEdgelist;
    else fmt = kFmtMetis;   // files METIS rejects later are left to the host
    const int r = fmt < 0 ? 0 : ingest_text(file, fmt, undirected != 0, g);
    if (r == 1) {
        if (parsed_on_gpu) *parsed_on_gpu = 1;
        *out = g;
        return CHL_OK;
    }
    delete g;
    if (r < 0) return -r;
    return chl_graph_load(path, undirected, out);
}
