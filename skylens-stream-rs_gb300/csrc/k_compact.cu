// k_compact.cu — turns per-pair match slots into one dense list.
//
// Each pair owns a slot range sized for its row count (a row matches at most
// once, matching.rs:204-214). After matching, the per-pair counts are scanned
// into offsets and the slots gathered into a dense array in pair order, so a
// batch comes back to the host as two copies (offsets, pairs).
#include <cuda_runtime.h>

#include <cstdint>

#include "slm.h"

namespace slm {

// Single CTA: offsets[k] = sum of counts[0..k), offsets[np] = total.
__global__ void __launch_bounds__(1024) scan_counts_kernel(const uint32_t *__restrict__ counts, uint32_t np,
                                                           uint64_t *__restrict__ offsets) {
    __shared__ uint64_t warp_sum[32];
    __shared__ uint64_t carry_sh;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) carry_sh = 0;
    __syncthreads();
    for (uint32_t base = 0; base < np; base += 1024) {
        const uint32_t k = base + tid;
        uint64_t v = k < np ? counts[k] : 0;
        uint64_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sum[wid] = x;
        __syncthreads();
        if (wid == 0) {
            uint64_t w = warp_sum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint64_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            warp_sum[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        const uint64_t carry = carry_sh;
        const uint64_t excl = carry + (wid ? warp_sum[wid - 1] : 0) + x - v;
        if (k < np) offsets[k] = excl;
        __syncthreads();
        if (tid == 1023) carry_sh = excl + v;
        __syncthreads();
    }
    if (tid == 0) offsets[np] = carry_sh;
}

// One CTA per pair: dense[offsets[k] + t] = slots[slot_off[k] + t].
__global__ void __launch_bounds__(256) gather_kernel(const uint2 *__restrict__ slots,
                                                     const uint64_t *__restrict__ slot_off,
                                                     const uint32_t *__restrict__ counts,
                                                     const uint64_t *__restrict__ offsets, uint2 *__restrict__ dense,
                                                     uint64_t cap) {
    const uint32_t k = blockIdx.x;
    const uint32_t n = counts[k];
    const uint64_t src = slot_off[k], dst = offsets[k];
    for (uint32_t t = threadIdx.x; t < n; t += blockDim.x)
        if (dst + t < cap) dense[dst + t] = slots[src + t];
}

// Single pair into a caller buffer: copies min(total, cap) pairs and writes
// the full count.
__global__ void copy_pairs_kernel(const uint2 *__restrict__ src, const uint64_t *__restrict__ total,
                                  slm_pair *__restrict__ dst, uint32_t cap, uint32_t *__restrict__ d_count) {
    const uint64_t n = *total;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n && t < cap;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 v = src[t];
        dst[t].i = v.x;
        dst[t].j = v.y;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *d_count = (uint32_t)n;
}

// match_pairs' filter (pipeline.rs:494-496: pairs with fewer than min_matches
// matches are dropped before RANSAC): such pairs report no matches, so their
// lists are neither gathered nor copied to the host.
__global__ void filter_counts_kernel(uint32_t *__restrict__ counts, uint32_t np, uint32_t min_matches) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < np; k += gridDim.x * blockDim.x)
        if (counts[k] < min_matches) counts[k] = 0;
}

__global__ void fill_u32_kernel(uint32_t *p, uint64_t n, uint32_t v) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// Rows of many views from one staging buffer into their padded store rows.
// The table travels as the kernel parameter (no upload):
// e[v] = {first staging row, first store row, rows, 0}; blockIdx.x = view,
// blockIdx.y strides over its rows.
constexpr uint32_t kScatterMax = 1024;
struct ScatterTab {
    uint4 e[kScatterMax];
};

__global__ void __launch_bounds__(256) scatter_rows_kernel(const ScatterTab tab, const float4 *__restrict__ src,
                                                           float4 *__restrict__ dst) {
    const uint4 t = tab.e[blockIdx.x];
    constexpr uint32_t kRow4 = 128 / 4;  // float4 per descriptor
    const uint64_t n4 = (uint64_t)t.z * kRow4;
    const float4 *s = src + (uint64_t)t.x * kRow4;
    float4 *d = dst + (uint64_t)t.y * kRow4;
    for (uint64_t k = blockIdx.y * (uint64_t)blockDim.x + threadIdx.x; k < n4; k += (uint64_t)gridDim.y * blockDim.x)
        d[k] = s[k];
}

void launch_scatter_rows(const uint4 *tab, uint32_t n, const float *src, float *dst, cudaStream_t s) {
    for (uint32_t b = 0; b < n; b += kScatterMax) {
        const uint32_t m = n - b < kScatterMax ? n - b : kScatterMax;
        ScatterTab t;
        for (uint32_t k = 0; k < m; ++k) t.e[k] = tab[b + k];
        scatter_rows_kernel<<<dim3(m, 8), 256, 0, s>>>(t, reinterpret_cast<const float4 *>(src),
                                                         reinterpret_cast<float4 *>(dst));
    }
}

// Rows of many views, each from its own source address (host memory the
// device can read directly, or device memory), into their padded store rows:
// e[v] = {source address low, high 32 bits, first store row, rows}.
// Each thread issues four 16-byte loads before it stores any of them, so that
// many loads are in flight: reads of host memory over the chip-to-chip link are
// bound by their latency.
__global__ void __launch_bounds__(256) gather_rows_kernel(const ScatterTab tab, float4 *__restrict__ dst) {
    const uint4 t = tab.e[blockIdx.x];
    constexpr uint32_t kRow4 = 128 / 4;
    const float4 *__restrict__ s = reinterpret_cast<const float4 *>(((uint64_t)t.y << 32) | t.x);
    const uint64_t n4 = (uint64_t)t.w * kRow4;
    float4 *d = dst + (uint64_t)t.z * kRow4;
    const uint64_t stride = (uint64_t)gridDim.y * blockDim.x;
    for (uint64_t k = blockIdx.y * (uint64_t)blockDim.x + threadIdx.x; k < n4; k += 4 * stride) {
        float4 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (k + u * stride < n4) v[u] = s[k + u * stride];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (k + u * stride < n4) d[k + u * stride] = v[u];
    }
}

void launch_gather_rows(const uint4 *tab, uint32_t n, float *dst, cudaStream_t s) {
    for (uint32_t b = 0; b < n; b += kScatterMax) {
        const uint32_t m = n - b < kScatterMax ? n - b : kScatterMax;
        ScatterTab t;
        uint32_t rows = 0;
        for (uint32_t k = 0; k < m; ++k) {
            t.e[k] = tab[b + k];
            rows = t.e[k].w > rows ? t.e[k].w : rows;
        }
        // CTAs per entry: one per 32 rows of the largest entry (a CTA's four
        // loads per thread cover 32 rows), between 16 and 64
        uint32_t per = (rows + 31) / 32;
        per = per < 16 ? 16 : (per > 64 ? 64 : per);
        gather_rows_kernel<<<dim3(m, per), 256, 0, s>>>(t, reinterpret_cast<float4 *>(dst));
    }
}

void launch_fill_u32(uint32_t *p, uint64_t n, uint32_t v, cudaStream_t s) {
    if (!n) return;
    uint64_t blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    fill_u32_kernel<<<(unsigned)blocks, 256, 0, s>>>(p, n, v);
}

void launch_filter_counts(uint32_t *counts, uint32_t np, uint32_t min_matches, cudaStream_t s) {
    if (np) filter_counts_kernel<<<(np + 255) / 256 < 1024 ? (np + 255) / 256 : 1024, 256, 0, s>>>(counts, np, min_matches);
}

void launch_scan_counts(const uint32_t *counts, uint32_t np, uint64_t *offsets, cudaStream_t s) {
    scan_counts_kernel<<<1, 1024, 0, s>>>(counts, np, offsets);
}

void launch_gather(const uint2 *slots, const uint64_t *slot_off, const uint32_t *counts, const uint64_t *offsets,
                   uint32_t np, uint2 *dense, uint64_t cap, cudaStream_t s) {
    if (np) gather_kernel<<<np, 256, 0, s>>>(slots, slot_off, counts, offsets, dense, cap);
}

void launch_copy_pairs(const uint2 *src, const uint64_t *total, slm_pair *dst, uint32_t cap, uint32_t *d_count,
                       cudaStream_t s) {
    copy_pairs_kernel<<<64, 256, 0, s>>>(src, total, dst, cap, d_count);
}

}  // namespace slm
