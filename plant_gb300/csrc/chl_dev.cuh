// Device-side helpers shared by the CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "chl_internal.h"

namespace chl {

constexpr uint32_t kFull = 0xFFFFFFFFu;

// Record a CUDA failure as the thread's last error and map it to a status.
int cuda_status(cudaError_t e, const char *what, const char *file, int line);

#define CHL_CUDA(call)                                                        \
    do {                                                                      \
        cudaError_t _e = (call);                                              \
        if (_e != cudaSuccess) return ::chl::cuda_status(_e, #call, __FILE__, __LINE__); \
    } while (0)

// Number of SMs of the current device (cached).
int device_sms();

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---------------------------------------------------------------- scans
// Exclusive prefix sum of n u32 values into u64 outputs; out[n] = total.
// Entries at index >= *d_n (when d_n is non-null) count as zero, so the
// launch shape depends only on the host bound n.
int scan_u32_excl(const uint32_t *in, uint64_t *out, uint64_t n,
                  const uint64_t *d_n, void *tmp, size_t tmp_bytes,
                  cudaStream_t s);
size_t scan_tmp_bytes(uint64_t n);

// ---------------------------------------------------------------- sort
// Stable LSD radix sort of (key, value) pairs on the low `bits` key bits.
// The item count is read from device memory (*d_n <= cap); the result ends
// in (k0, v0) if the returned parity is 0, else in (k1, v1).
int radix_sort_pairs(uint64_t *k0, uint32_t *v0, uint64_t *k1, uint32_t *v1,
                     const uint64_t *d_n, uint64_t cap, int bits, void *tmp,
                     size_t tmp_bytes, cudaStream_t s, int *parity);
size_t radix_tmp_bytes();

// Vertices by device score descending, ties by the seeded tie key (the same
// rule as the degree order); writes the host order array (rank -> vertex).
int order_by_score(uint32_t n, uint64_t seed, const float *d_score, uint32_t *order_h);

}  // namespace chl
