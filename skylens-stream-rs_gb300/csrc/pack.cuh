// pack.cuh — row-major FP32 descriptors -> the exact kernel's tile layout
// (tile[slot][row], slot = the k-permuted component index).
#pragma once

#include <cstdint>

#include "slm_internal.h"

namespace slm {

// Rows [tile * 128 + g * 32, +32) of src (n rows, row-major, 16-byte aligned)
// into group g of the tile at dst; rows past n are zeros. Every thread of a
// 256-thread CTA calls it alike; sm is the CTA's staging buffer. Each thread
// issues its four 16-byte loads before the first shared-memory store, so a CTA
// has the whole 16 KiB group in flight at once: when src is host memory read
// over the chip-to-chip link, the latency of a load, not its bandwidth, sets
// the time.
__device__ __forceinline__ void pack_group(const float *__restrict__ src, uint32_t n, float *__restrict__ dst,
                                           uint32_t tile, int g, float (&sm)[32][kDesc + 1]) {
    const uint32_t r0 = tile * kTile + g * 32;
    float4 v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int q = threadIdx.x + 256 * u, r = q >> 5, c = q & 31;
        v[u] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (r0 + r < n) v[u] = reinterpret_cast<const float4 *>(src + (size_t)(r0 + r) * kDesc)[c];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int q = threadIdx.x + 256 * u, r = q >> 5, c = q & 31;
        sm[r][4 * c + 0] = v[u].x;
        sm[r][4 * c + 1] = v[u].y;
        sm[r][4 * c + 2] = v[u].z;
        sm[r][4 * c + 3] = v[u].w;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < 32 * kDesc; q += 256) {
        const int slot = q >> 5, r = q & 31;
        const int k = 8 * (slot & 15) + (slot >> 4);  // inverse of perm_slot
        dst[slot * kTile + g * 32 + r] = sm[r][k];
    }
    __syncthreads();
}

}  // namespace slm
