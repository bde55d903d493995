// Host-side file formats and error reporting.
//   order file  : hl::Order::read/write   shared_memory/ordering.hpp:37-67
//   label file  : hl::Labeling::write/read shared_memory/labeling.hpp:167-208
//   query file  : hl::load_query          distributed_memory/query.hpp:18-32
#include "chl_internal.h"

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace chl {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

// Whole-file reader.
static int slurp(const char *path, std::vector<char> &buf) {
    FILE *f = fopen(path, "rb");
    if (!f) {
        set_error(std::string("cannot open ") + path + ": " + strerror(errno));
        return CHL_ERR_IO;
    }
    buf.clear();
    char tmp[1 << 16];
    size_t r;
    while ((r = fread(tmp, 1, sizeof(tmp), f)) > 0) buf.insert(buf.end(), tmp, tmp + r);
    bool bad = ferror(f) != 0;
    fclose(f);
    if (bad) {
        set_error(std::string("read error on ") + path);
        return CHL_ERR_IO;
    }
    buf.push_back('\0');
    return CHL_OK;
}

// Whitespace-separated integer scanner with istream-like failure rules:
// a token must be an optional sign followed by digits.
struct Scanner {
    const char *p, *e;
    bool fail = false;
    Scanner(const std::vector<char> &b) : p(b.data()), e(b.data() + b.size() - 1) {}
    void ws() {
        while (p < e && (*p == ' ' || *p == '\n' || *p == '\t' || *p == '\r' || *p == '\v' || *p == '\f')) ++p;
    }
    bool at_end() {
        ws();
        return p >= e;
    }
    bool u64(uint64_t &out, uint64_t maxv) {
        ws();
        if (p >= e || *p < '0' || *p > '9') {
            fail = true;
            return false;
        }
        uint64_t v = 0;
        while (p < e && *p >= '0' && *p <= '9') {
            v = v * 10 + (uint64_t)(*p - '0');
            if (v > maxv) {
                fail = true;
                return false;
            }
            ++p;
        }
        out = v;
        return true;
    }
    bool i64(int64_t &out, int64_t lo, int64_t hi) {
        ws();
        bool neg = false;
        if (p < e && (*p == '-' || *p == '+')) {
            neg = *p == '-';
            ++p;
        }
        uint64_t v;
        if (!u64(v, (uint64_t)hi + 1)) return false;
        int64_t s = neg ? -(int64_t)v : (int64_t)v;
        if (s < lo || s > hi) {
            fail = true;
            return false;
        }
        out = s;
        return true;
    }
};

// Fast decimal formatting into a growing buffer.
struct Writer {
    FILE *f;
    std::vector<char> buf;
    size_t pos = 0;
    bool bad = false;
    explicit Writer(FILE *file) : f(file), buf(1 << 22) {}
    void flush() {
        if (pos && fwrite(buf.data(), 1, pos, f) != pos) bad = true;
        pos = 0;
    }
    void reserve(size_t k) {
        if (pos + k > buf.size()) flush();
    }
    void ch(char c) {
        reserve(1);
        buf[pos++] = c;
    }
    void u(uint64_t v) {
        reserve(24);
        char t[24];
        int k = 0;
        do {
            t[k++] = (char)('0' + v % 10);
            v /= 10;
        } while (v);
        while (k) buf[pos++] = t[--k];
    }
    void i(int64_t v) {
        if (v < 0) {
            ch('-');
            u((uint64_t)(-v));
        } else {
            u((uint64_t)v);
        }
    }
};

int write_labels_text(const chl_labels *l, const char *path) {
    int rc = labels_fetch_host(l);
    if (rc) return rc;
    FILE *f = fopen(path, "wb");
    if (!f) {
        set_error(std::string("cannot open ") + path + " for writing");
        return CHL_ERR_IO;
    }
    Writer w(f);
    w.u(l->n);
    w.ch('\n');
    for (uint32_t v = 0; v < l->n; ++v) {
        for (int side = 0; side < 2; ++side) {
            const uint32_t x = l->list(v, side);
            const uint64_t b = l->h_off[x], e = l->h_off[x + 1];
            w.u(e - b);
            for (uint64_t k = b; k < e; ++k) {
                w.ch(' ');
                w.u(l->h_ent[k].hub);
                w.ch(' ');
                w.i((int32_t)l->h_ent[k].dist);
            }
            w.ch('\n');
        }
    }
    w.flush();
    bool bad = w.bad || ferror(f);
    if (fclose(f) != 0) bad = true;
    return bad ? CHL_ERR_IO : CHL_OK;
}

}  // namespace chl

using namespace chl;

extern "C" const char *chl_status_str(int s) {
    switch (s) {
    case CHL_OK: return "ok";
    case CHL_ERR_IO: return "i/o error";
    case CHL_ERR_FORMAT: return "unrecognised file format";
    case CHL_ERR_OOM: return "out of memory";
    case CHL_ERR_TIMEOUT: return "timed out";
    case CHL_ERR_INVALID: return "invalid argument";
    case CHL_ERR_CUDA: return "CUDA error";
    default: return "unknown status";
    }
}

extern "C" const char *chl_last_error(void) { return g_last_error.c_str(); }

// Order::read: "n" then n ids.  The reference ignores a short or malformed
// file (it keeps whatever was parsed); here it is CHL_ERR_FORMAT.
extern "C" int chl_order_load(const char *path, uint32_t **order, uint32_t *n) {
    if (!path || !order || !n) return CHL_ERR_INVALID;
    std::vector<char> buf;
    int rc = slurp(path, buf);
    if (rc) return rc;
    Scanner sc(buf);
    uint64_t s;
    if (!sc.u64(s, 0xFFFFFFFFull)) {
        set_error("order file: missing size");
        return CHL_ERR_FORMAT;
    }
    uint32_t *o = (uint32_t *)malloc((size_t)std::max<uint64_t>(s, 1) * 4);
    if (!o) return CHL_ERR_OOM;
    for (uint64_t i = 0; i < s; ++i) {
        uint64_t v;
        if (!sc.u64(v, 0xFFFFFFFFull)) {
            free(o);
            set_error("order file: fewer ids than announced");
            return CHL_ERR_FORMAT;
        }
        o[i] = (uint32_t)v;
    }
    if (!sc.at_end()) {
        free(o);
        set_error("order file: trailing data");
        return CHL_ERR_FORMAT;
    }
    *order = o;
    *n = (uint32_t)s;
    return CHL_OK;
}

extern "C" int chl_order_write(const char *path, const uint32_t *order, uint32_t n) {
    if (!path || (n && !order)) return CHL_ERR_INVALID;
    FILE *f = fopen(path, "wb");
    if (!f) return CHL_ERR_IO;
    Writer w(f);
    w.u(n);
    w.ch('\n');
    for (uint32_t i = 0; i < n; ++i) {
        w.u(order[i]);
        w.ch('\n');
    }
    w.flush();
    bool bad = w.bad || ferror(f);
    if (fclose(f) != 0) bad = true;
    return bad ? CHL_ERR_IO : CHL_OK;
}

extern "C" void chl_order_free(uint32_t *order) { free(order); }

extern "C" int chl_labels_write(const chl_labels *l, const char *path) {
    if (!l || !path) return CHL_ERR_INVALID;
    // labels in HBM are formatted there; labels that only exist in host
    // memory (read from a file, imported) are written from the host copy
    if (l->d_off) return write_labels_text_device(l, path);
    return write_labels_text(l, path);
}

// Labeling::read: n, then per vertex two lists `size h d ...`.
extern "C" int chl_labels_read(const char *path, chl_labels **out) {
    if (!path || !out) return CHL_ERR_INVALID;
    std::vector<char> buf;
    int rc = slurp(path, buf);
    if (rc) return rc;
    Scanner sc(buf);
    uint64_t n;
    if (!sc.u64(n, 0xFFFFFFFFull)) {
        set_error("label file: missing n");
        return CHL_ERR_FORMAT;
    }
    std::vector<uint64_t> off(2 * n + 1, 0);
    std::vector<uint32_t> hub;
    std::vector<int32_t> dist;
    for (uint64_t x = 0; x < 2 * n; ++x) {
        uint64_t s;
        if (!sc.u64(s, 0xFFFFFFFFull)) {
            set_error("label file: truncated");
            return CHL_ERR_FORMAT;
        }
        for (uint64_t k = 0; k < s; ++k) {
            uint64_t h;
            int64_t d;
            if (!sc.u64(h, 0xFFFFFFFFull) || !sc.i64(d, -2147483648ll, 2147483647ll)) {
                set_error("label file: bad entry");
                return CHL_ERR_FORMAT;
            }
            hub.push_back((uint32_t)h);
            dist.push_back((int32_t)d);
        }
        off[x + 1] = hub.size();
    }
    if (!sc.at_end()) {
        set_error("label file: trailing data");
        return CHL_ERR_FORMAT;
    }
    return labels_from_host((uint32_t)n, off.data(), hub.data(), dist.data(), out);
}

extern "C" int chl_query_generate(uint32_t *pairs, size_t k, uint32_t range, uint64_t seed) {
    if ((k && !pairs) || range == 0) return CHL_ERR_INVALID;
    Rng r(seed);
    for (size_t i = 0; i < 2 * k; ++i) pairs[i] = (uint32_t)r.below(range);
    return CHL_OK;
}

// load_query: one `u v` pair per line (lines over 511 characters or without
// two integers make the reference stop and report failure).
extern "C" int chl_query_load(const char *path, uint32_t **pairs, size_t *k) {
    if (!path || !pairs || !k) return CHL_ERR_INVALID;
    FILE *f = fopen(path, "r");
    if (!f) return CHL_ERR_IO;
    std::vector<uint32_t> q;
    char buf[512];
    long long u, v;
    while (fgets(buf, sizeof(buf), f)) {
        size_t L = strlen(buf);
        if ((L == 0 || buf[L - 1] != '\n') && !feof(f)) {
            fclose(f);
            return CHL_ERR_FORMAT;
        }
        if (sscanf(buf, "%lld %lld", &u, &v) != 2) {
            fclose(f);
            return CHL_ERR_FORMAT;
        }
        q.push_back((uint32_t)u);
        q.push_back((uint32_t)v);
    }
    fclose(f);
    uint32_t *p = (uint32_t *)malloc(std::max<size_t>(q.size(), 1) * 4);
    if (!p) return CHL_ERR_OOM;
    memcpy(p, q.data(), q.size() * 4);
    *pairs = p;
    *k = q.size() / 2;
    return CHL_OK;
}
