// Internal host-side structures shared by the C++ host code and the CUDA
// translation units.  Nothing here is part of the public C ABI.
#pragma once

#include <cstdint>
#include <cstddef>
#include <string>
#include <memory>
#include <utility>
#include <vector>

#include "../../include/chl.h"

namespace chl {

// Reference vertex / distance conventions (shared_memory/graph.hpp:42-47):
// Vertex is unsigned 32-bit, Distance is int, infty = INT_MAX.
constexpr int32_t kInfty = 2147483647;

void set_error(const std::string &msg);

// Seeded bijective 64-bit mixer (the splitmix64 finaliser).  Used for
// reproducible tie breaks and counter-based random streams; identical on
// every host architecture.
inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Sequential splitmix64 stream.
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    // Integer in [0, range) (range > 0); modulo reduction of a 64-bit draw.
    uint64_t below(uint64_t range) { return next() % range; }
    // Double in [0, 1) from the top 53 bits.
    double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// Tie-break key of vertex v under `seed`: a bijection of v for a fixed seed,
// so sorting by it yields a seeded random permutation.
inline uint64_t tie_key(uint64_t seed, uint32_t v) {
    return mix64(seed * 0x9E3779B97F4A7C15ull + (uint64_t)v);
}

}  // namespace chl

// Graph after the reference's init_arcs merge (shared_memory/graph.hpp:103-153):
// per vertex, the forward (out) and reverse (in) arc lists in the reference's
// arc order.  Stored as two CSRs.
struct chl_graph {
    uint32_t n = 0;
    uint64_t m = 0;                  // arcs added, counted as add_tmp_arc does
    std::vector<uint64_t> off[2];    // [0] = reverse (in) arcs, [1] = forward (out)
    std::vector<uint32_t> head[2];
    std::vector<int32_t> len[2];
    bool symmetric = false;
    bool unit = false;               // every arc length is 1
    int32_t min_len = 0, max_len = 0;
    void *dev = nullptr;             // device CSR (chl_graph_to_device), owned
};

// One label entry: hub rank and distance (8 bytes, read as uint2 on device).
struct alignas(8) LabelEnt {
    uint32_t hub;
    uint32_t dist;
};

// Allocator whose resize() leaves trivially constructible elements
// uninitialised (host mirrors of multi-GB device arrays are overwritten at
// once; zero-filling them first would double the host-side cost).
template <typename T>
struct NoInitAlloc : std::allocator<T> {
    template <typename U>
    struct rebind {
        using other = NoInitAlloc<U>;
    };
    NoInitAlloc() = default;
    template <typename U>
    NoInitAlloc(const NoInitAlloc<U> &) {}
    template <typename U>
    void construct(U *p) noexcept {
        ::new (static_cast<void *>(p)) U;
    }
    template <typename U, typename... A>
    void construct(U *p, A &&...args) {
        ::new (static_cast<void *>(p)) U(std::forward<A>(args)...);
    }
};

// Labels: CSR over label lists, entries (hub, dist) ascending by hub.  A
// symmetric build stores one list per vertex (index v, both sides equal);
// otherwise list 2v+side.  Device copy plus a lazily fetched host mirror in
// the same layout.
struct chl_labels {
    uint32_t n = 0;
    bool sym = false;
    mutable uint64_t *d_off = nullptr;   // nl+1 entries, nl = sym ? n : 2n
    mutable LabelEnt *d_ent = nullptr;   // uploaded lazily for imported labels
    uint64_t total = 0;              // entries stored (one side if sym)
    mutable std::vector<uint64_t> h_off;
    mutable std::vector<LabelEnt, NoInitAlloc<LabelEnt>> h_ent;
    mutable bool host_valid = false;
    chl_build_stats stats{};
    uint32_t nl() const { return sym ? n : 2 * n; }
    uint32_t list(uint32_t v, int side) const { return sym ? v : 2 * v + (uint32_t)side; }
};

namespace chl {
// host helpers implemented in chl_labels.cu (device <-> host)
int labels_fetch_host(const chl_labels *l);
// upload the host mirror if the device copy does not exist yet
int labels_ensure_device(const chl_labels *l);
// Build a labels handle from a host CSR in the 2n+1 layout; stores one side
// when both sides are identical.
int labels_from_host(uint32_t n, const uint64_t *off2, const uint32_t *hub,
                     const int32_t *dist, chl_labels **out);
// min/max length, unit-length and symmetry flags of a graph's host CSR
void graph_fill_stats(chl_graph *g);
// METIS reader verdict on the complete lines of a file prefix (chl_graph.cpp)
bool metis_rejects_prefix(const char *buf, size_t len);
// hl::Labeling::write's text, formatted on the device (labels in HBM)
int write_labels_text_device(const chl_labels *l, const char *path);
// free the device copy of a graph (no-op without one)
void graph_release_device(chl_graph *g);
int build_labels(const chl_graph *g, const uint32_t *order, uint32_t n,
                 const chl_build_opts *opts, chl_labels **out);
// graph class of the tuned-schedule table (chl_tune.cpp)
std::string graph_class(const chl_graph *g);
// fill the options left at 0 from the tuned-schedule table; true if found
bool apply_tuned_schedule(const chl_graph *g, chl_build_opts &opts);
// build a graph from unique undirected edges (u < v), symmetric CSR
int graph_from_undirected_unique(uint32_t n, std::vector<uint64_t> &edges_uv,
                                 std::vector<int32_t> &w, chl_graph **out);
}  // namespace chl
