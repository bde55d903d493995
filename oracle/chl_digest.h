/*
 * Label digest, version 1 (test infrastructure: shared by the C oracle and
 * the harness compiled against the reference's headers).
 *
 * A position-dependent 64-bit fingerprint of a labeling with the content of
 * the reference's label file (shared_memory/labeling.hpp:167-183): n, then
 * for every list i = 2v + side its size and its (hub rank, distance) entries
 * in stored order.  Each item contributes one well-mixed 64-bit term and the
 * terms are added modulo 2^64, so the digest can be summed in any order (on
 * a GPU with atomics) while still depending on every entry's list and
 * position:
 *
 *   digest = M(n + C_N)
 *          + sum_i  M( M(i + C_L) ^ size_i )
 *          + sum_ij M( M(i + C_L) ^ M(j + C_E) ^ (hub_ij << 32 | dist_ij) )
 *
 * M is the finaliser of SplitMix64 (G. Steele, D. Lea, C. Flood, "Fast
 * splittable pseudorandom number generators", OOPSLA 2014), with the
 * multipliers of D. Stafford's "variant 13" mixer that SplitMix64 uses.
 * The order digest is M(n + C_N) + sum_i M(M(i + C_O) ^ order_i).
 */
#ifndef CHL_DIGEST_H
#define CHL_DIGEST_H

#include <stdint.h>

#define CHD_C_N 0x243F6A8885A308D3ull
#define CHD_C_L 0x13198A2E03707344ull
#define CHD_C_E 0xA4093822299F31D0ull
#define CHD_C_O 0x082EFA98EC4E6C89ull

static inline uint64_t chd_mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline uint64_t chd_head(uint64_t n) { return chd_mix(n + CHD_C_N); }

static inline uint64_t chd_list_base(uint64_t i) { return chd_mix(i + CHD_C_L); }

static inline uint64_t chd_list_term(uint64_t base, uint64_t size) { return chd_mix(base ^ size); }

static inline uint64_t chd_entry_term(uint64_t base, uint64_t j, uint32_t hub, uint32_t dist) {
    return chd_mix(base ^ chd_mix(j + CHD_C_E) ^ (((uint64_t)hub << 32) | (uint64_t)dist));
}

static inline uint64_t chd_order_term(uint64_t i, uint32_t v) { return chd_mix(chd_mix(i + CHD_C_O) ^ v); }

#endif
