// k_tracks.cu — the track builder's graph work on the GPU: build_tracks with
// ConflictPolicy::Drop (crates/core/src/tracks.rs:190-259) turns verified
// matches into edges between (image, feature) nodes and takes the connected
// components, each represented by its smallest node (tracks.rs:160-186:
// "the representative is always the smallest node", so the components and
// their representatives do not depend on the order the edges are joined in).
//
// Here: one CTA per image pair checks its matches (the reference's validity
// rule) and inserts each edge (small node << 32 | large node) into an
// open-addressing hash set, which also counts the distinct edges and lists
// them; then rounds of hooking (every edge's larger root points at the
// smaller one, atomicMin) and pointer jumping until no edge joins two roots.
#include <cuda_runtime.h>

#include <cstdint>

#include "slm_internal.h"

namespace slm {

namespace {

constexpr unsigned long long kEmpty = ~0ull;

__device__ __forceinline__ uint64_t mix64(uint64_t x) {  // a 64-bit finaliser (xor-shift-multiply)
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

__global__ void track_edges_kernel(TrackArgs a) {
    const TrackPair tp = a.pairs[blockIdx.x];
    const uint32_t ia = tp.image_a, ib = tp.image_b;
    const bool pair_ok = ia != ib && ia < a.n_images && ib < a.n_images;
    uint32_t bad = 0;
    for (uint64_t k = threadIdx.x; k < tp.count; k += blockDim.x) {
        const uint2 m = a.matches[tp.first + k];
        if (!pair_ok || m.x >= a.nf[ia] || m.y >= a.nf[ib]) {
            ++bad;
            continue;
        }
        // the smaller image's node first (node = image offset + feature)
        const uint64_t u = a.off[ia] + m.x, v = a.off[ib] + m.y;
        const unsigned long long key = (u < v) ? (u << 32 | v) : (v << 32 | u);
        uint64_t slot = mix64(key) & a.table_mask;
        for (uint64_t probe = 0; probe <= a.table_mask; ++probe) {
            const unsigned long long prev = atomicCAS(&a.table[slot], kEmpty, key);
            if (prev == kEmpty) {  // a new edge
                a.edges[atomicAdd(a.n_edges, 1ull)] = key;
                break;
            }
            if (prev == key) break;  // seen before
            slot = (slot + 1) & a.table_mask;
        }
    }
    if (bad) atomicAdd(a.n_invalid, (unsigned long long)bad);
}

__device__ __forceinline__ uint32_t find_root(const uint32_t *parent, uint32_t x) {
    uint32_t p = parent[x];
    while (p != x) {
        x = p;
        p = parent[x];
    }
    return x;
}

__global__ void track_init_kernel(uint32_t *parent, uint8_t *used, uint64_t n) {
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < n; x += (uint64_t)gridDim.x * blockDim.x) {
        parent[x] = (uint32_t)x;
        used[x] = 0;
    }
}

__global__ void track_mark_kernel(const unsigned long long *edges, const unsigned long long *n_edges, uint8_t *used) {
    const uint64_t ne = *n_edges;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < ne; e += (uint64_t)gridDim.x * blockDim.x) {
        used[edges[e] >> 32] = 1;
        used[edges[e] & 0xffffffffu] = 1;
    }
}

// Every edge whose endpoints have different roots points the larger root at
// the smaller (parents only ever decrease, so no cycle forms).
__global__ void track_hook_kernel(const unsigned long long *edges, const unsigned long long *n_edges, uint32_t *parent,
                                  uint32_t *changed) {
    const uint64_t ne = *n_edges;
    bool any = false;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < ne; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t ru = find_root(parent, (uint32_t)(edges[e] >> 32));
        const uint32_t rv = find_root(parent, (uint32_t)(edges[e] & 0xffffffffu));
        if (ru != rv) {
            atomicMin(&parent[ru > rv ? ru : rv], ru < rv ? ru : rv);
            any = true;
        }
    }
    if (any) *changed = 1;
}

__global__ void track_jump_kernel(uint32_t *parent, uint64_t n) {
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < n; x += (uint64_t)gridDim.x * blockDim.x)
        parent[x] = find_root(parent, (uint32_t)x);
}

}  // namespace

void launch_track_edges(const TrackArgs &a, uint32_t n_pairs, cudaStream_t s) {
    if (n_pairs) track_edges_kernel<<<n_pairs, 256, 0, s>>>(a);
}
void launch_track_init(uint32_t *parent, uint8_t *used, uint64_t n, int grid, cudaStream_t s) {
    if (n) track_init_kernel<<<grid, 256, 0, s>>>(parent, used, n);
}
void launch_track_mark(const unsigned long long *edges, const unsigned long long *n_edges, uint8_t *used, int grid,
                       cudaStream_t s) {
    track_mark_kernel<<<grid, 256, 0, s>>>(edges, n_edges, used);
}
void launch_track_hook(const unsigned long long *edges, const unsigned long long *n_edges, uint32_t *parent,
                       uint32_t *changed, int grid, cudaStream_t s) {
    track_hook_kernel<<<grid, 256, 0, s>>>(edges, n_edges, parent, changed);
}
void launch_track_jump(uint32_t *parent, uint64_t n, int grid, cudaStream_t s) {
    if (n) track_jump_kernel<<<grid, 256, 0, s>>>(parent, n);
}

}  // namespace slm
