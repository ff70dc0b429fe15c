// k_exact.cu — the plain FP32 matcher (exact, bit-identical to the reference).
//
// Reference: crates/core/src/matching.rs:144-215 (sq_dist + ratio_match).
//
// Layout. Descriptors live in store tiles of 128 rows: tile[slot][row] with
// slot = perm_slot(k) = (k % 8) * 16 + k / 8, so walking slots 0..127 walks
// sq_dist's order: lane 0 (components 0, 8, ..., 120), then lane 1, and so
// on. One walk of 16 slots is one lane accumulator; the 8 lane sums are added
// to the distance in lane order. Every operation is an explicit _rn IEEE op
// (no FMA contraction), so each d(i, j) equals the reference's f32 value.
//
// Kernel. A persistent CTA (256 threads, one per SM) takes work items (a
// 128-row tile of a against a range of 128-column tiles of b) from a global
// counter. The a tile is bulk-copied (TMA) into shared memory once per item;
// b tiles stream through a two-slot TMA/mbarrier ring. Each thread owns an
// 8 x 8 register block of distances (rows ty*4+{0..3}, 64+ty*4+{0..3};
// columns tx*4+{0..3}, 64+tx*4+{0..3}).
//   rows:    best / second-best / argmin are carried in registers across the
//            b tiles and merged across the 16 column threads at the end of
//            the item with warp shuffles (order-independent: min, lowest j on
//            ties, second smallest of the multiset).
//   columns: (bits(d) << 32 | i) keys are min-reduced in the warp, then in
//            shared memory, then with one global atomicMin per column and
//            tile; unsigned order of the key is (d, lowest i) because d >= +0.
// The finalize kernel merges row partials, applies the ratio test
// (d1 < (r*r)*d2 in f32) and the mutual check, and compacts in ascending i.
#include <cuda_runtime.h>

#include "pack.cuh"
#include "ptx.cuh"
#include "slm_internal.h"

namespace slm {

// ------------------------------------------------------------------ pack

// Tile `tile` of the view whose rows start at store row `row0` (n rows): raw
// rows -> tile[slot][row]. Called by all 256 threads of a CTA alike.
SLM_DEV void pack_view_tile(const float *__restrict__ raw, float *__restrict__ tiled, uint32_t row0, uint32_t n,
                            uint32_t tile, float (&sm)[32][kDesc + 1]) {
    const float *src = raw + (size_t)row0 * kDesc;
    float *dst = tiled + (size_t)(row0 / kTile + tile) * kTileFloats;
    for (int g = 0; g < 4; ++g) pack_group(src, n, dst, tile, g, sm);
}

// Many views at once: one CTA per 32-row group (blockIdx.y) of each entry of
// a tile table {first store row of the view, rows of the view, tile within the
// view, view}.
__global__ void __launch_bounds__(256) pack_fp32_tiles_kernel(const uint4 *__restrict__ tab,
                                                              const float *__restrict__ raw,
                                                              float *__restrict__ tiled) {
    __shared__ float sm[32][kDesc + 1];
    const uint4 e = tab[blockIdx.x];
    pack_group(raw + (size_t)e.x * kDesc, e.y, tiled + (size_t)(e.x / kTile + e.z) * kTileFloats, e.z, blockIdx.y,
               sm);
}

// The FP32 tiles of both views of every routed pair of a low-precision batch
// (the only readers of FP32 tiles on that path), packed on the device once the
// routed pairs are known; with nothing routed every CTA returns at once. A
// view shared by several routed pairs is packed once per pair (same values).
__global__ void __launch_bounds__(256) pack_routed_kernel(const PairMeta *__restrict__ pairs,
                                                          const uint32_t *__restrict__ xlist,
                                                          const uint32_t *__restrict__ count,
                                                          const float *__restrict__ raw, float *__restrict__ tiled) {
    __shared__ float sm[32][kDesc + 1];
    const uint32_t n = *count;
    for (uint32_t k = 0; k < n; ++k) {
        const PairMeta pm = pairs[xlist[k]];
        const uint32_t ta = (pm.na + kTile - 1) / kTile, tb = (pm.nb + kTile - 1) / kTile;
        for (uint32_t t = blockIdx.x; t < ta + tb; t += gridDim.x) {
            const bool is_a = t < ta;
            pack_view_tile(raw, tiled, is_a ? pm.a_row0 : pm.b_row0, is_a ? pm.na : pm.nb, is_a ? t : t - ta, sm);
        }
    }
}

void launch_pack_routed(const PairMeta *pairs, const uint32_t *xlist, const uint32_t *count, const float *raw,
                        float *tiled, int grid, cudaStream_t s) {
    pack_routed_kernel<<<grid, 256, 0, s>>>(pairs, xlist, count, raw, tiled);
}

void launch_pack_fp32_tiles(const uint4 *tab, uint32_t ntiles, const float *raw, float *tiled, cudaStream_t s) {
    if (ntiles) pack_fp32_tiles_kernel<<<dim3(ntiles, 4), 256, 0, s>>>(tab, raw, tiled);
}

__global__ void fill_u64_kernel(unsigned long long *p, uint64_t n, unsigned long long v) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

void launch_fill_u64(unsigned long long *p, uint64_t n, unsigned long long v, cudaStream_t s) {
    if (!n) return;
    uint64_t blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    fill_u64_kernel<<<(unsigned)blocks, 256, 0, s>>>(p, n, v);
}

// ----------------------------------------------------------- exact match

constexpr int kThreads = 256;
constexpr uint32_t kTileBytes = kTileFloats * 4;

struct ExactSmem {
    float A[kTileFloats];
    float B[2][kTileFloats];
    unsigned long long colred[2][kTile];
    uint64_t barA, barB[2];
    uint32_t item;
};

typedef unsigned long long u64;

SLM_DEV u64 f2_sub(u64 a, u64 b) {
    u64 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
SLM_DEV u64 f2_mul(u64 a, u64 b) {
    u64 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
SLM_DEV u64 f2_add(u64 a, u64 b) {
    u64 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
SLM_DEV u64 f2_fma(u64 a, u64 b, u64 c) {
    u64 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
SLM_DEV u64 f2_pack(float lo, float hi) {
    u64 d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}
SLM_DEV float f2_lo(u64 v) { return __uint_as_float(static_cast<uint32_t>(v)); }
SLM_DEV float f2_hi(u64 v) { return __uint_as_float(static_cast<uint32_t>(v >> 32)); }

// 8 x 8 block of spec-order distances between the thread's rows of A and
// columns of B (both tiles in [slot][row] layout).
template <bool X2>
SLM_DEV void tile_distances(const float *__restrict__ sa, const float *__restrict__ sb, int ty, int tx,
                            u64 zero2, float (&d)[8][8]) {
    if constexpr (!X2) {
        float s[8][8];
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int c = 0; c < 8; ++c) s[r][c] = 0.0f;
#pragma unroll 1
        for (int lane = 0; lane < 8; ++lane) {
            float acc[8][8];
            const float *pa = sa + lane * 16 * kTile;
            const float *pb = sb + lane * 16 * kTile;
#pragma unroll
            for (int c16 = 0; c16 < 16; ++c16) {
                const float4 a0 = *reinterpret_cast<const float4 *>(pa + c16 * kTile + ty * 4);
                const float4 a1 = *reinterpret_cast<const float4 *>(pa + c16 * kTile + 64 + ty * 4);
                const float4 b0 = *reinterpret_cast<const float4 *>(pb + c16 * kTile + tx * 4);
                const float4 b1 = *reinterpret_cast<const float4 *>(pb + c16 * kTile + 64 + tx * 4);
                const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
                for (int r = 0; r < 8; ++r)
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        const float t = __fsub_rn(av[r], bv[c]);
                        const float tt = __fmul_rn(t, t);
                        acc[r][c] = (c16 == 0) ? tt : __fadd_rn(acc[r][c], tt);
                    }
            }
#pragma unroll
            for (int r = 0; r < 8; ++r)
#pragma unroll
                for (int c = 0; c < 8; ++c) s[r][c] = __fadd_rn(s[r][c], acc[r][c]);
        }
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int c = 0; c < 8; ++c) d[r][c] = s[r][c];
    } else {
        // Packed pairs of columns (c, c+1): {a_r, a_r} - {b_c, b_c+1}. A packed
        // multiply followed by a packed add is contracted to a packed FMA by the
        // code generator (measured: 25 % of distances off by an ulp). The square
        // is therefore a packed FMA t * t + z with z a run-time zero (a kernel
        // argument the compiler cannot fold): rounded once, it is exactly
        // RN(t * t) (t * t >= 0, + 0 changes nothing), and no contraction with
        // the following add is possible.
        u64 s[8][4];
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) s[r][c] = 0ull;
#pragma unroll 1
        for (int lane = 0; lane < 8; ++lane) {
            u64 acc[8][4];
            const float *pa = sa + lane * 16 * kTile;
            const float *pb = sb + lane * 16 * kTile;
#pragma unroll
            for (int c16 = 0; c16 < 16; ++c16) {
                const float4 a0 = *reinterpret_cast<const float4 *>(pa + c16 * kTile + ty * 4);
                const float4 a1 = *reinterpret_cast<const float4 *>(pa + c16 * kTile + 64 + ty * 4);
                const ulonglong2 b0 = *reinterpret_cast<const ulonglong2 *>(pb + c16 * kTile + tx * 4);
                const ulonglong2 b1 = *reinterpret_cast<const ulonglong2 *>(pb + c16 * kTile + 64 + tx * 4);
                const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                const u64 bv[4] = {b0.x, b0.y, b1.x, b1.y};
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    const u64 ar = f2_pack(av[r], av[r]);
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const u64 t = f2_sub(ar, bv[c]);
                        const u64 tt = f2_fma(t, t, zero2);
                        acc[r][c] = (c16 == 0) ? tt : f2_add(acc[r][c], tt);
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < 8; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) s[r][c] = f2_add(s[r][c], acc[r][c]);
        }
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                d[r][2 * c] = f2_lo(s[r][c]);
                d[r][2 * c + 1] = f2_hi(s[r][c]);
            }
    }
}

SLM_DEV int row_of(int ty, int r) { return r < 4 ? ty * 4 + r : 64 + ty * 4 + (r - 4); }
SLM_DEV int col_of(int tx, int c) { return c < 4 ? tx * 4 + c : 64 + tx * 4 + (c - 4); }

template <bool X2>
__global__ void __launch_bounds__(kThreads, 1) exact_kernel(ExactArgs g) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    ExactSmem &S = *reinterpret_cast<ExactSmem *>(smem_raw);
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int lane = tid & 31;

    if (tid == 0) {
        mbar_init(&S.barA, 1);
        mbar_init(&S.barB[0], 1);
        mbar_init(&S.barB[1], 1);
        fence_mbar_init();
    }
    for (int c = tid; c < 2 * kTile; c += kThreads) (&S.colred[0][0])[c] = ~0ull;
    __syncthreads();
    // Items planned on the device (pairs routed from the shortlist path) come
    // with their count in device memory, written by an earlier kernel.
    const uint32_t n_items = g.n_items_dev ? min(*g.n_items_dev, g.n_items) : g.n_items;
    const u64 zero2 = f2_pack(g.zero, g.zero);

    uint32_t a_phase = 0;
    uint32_t seq = 0;  // b tiles consumed by this CTA (selects ring slot and parity)
    bool ok = true;    // CTA-uniform: every barrier below reduces it with AND
    for (;;) {
        if (tid == 0) S.item = atomicAdd(g.work, 1u);
        ok = __syncthreads_and(ok);
        const uint32_t it = S.item;
        if (it >= n_items || !ok) break;
        const Item item = g.items[it];
        const PairMeta pm = g.pairs[item.pair];
        const float *atile = g.tiled + (size_t)(pm.a_row0 / kTile + item.rt) * kTileFloats;
        const float *bbase = g.tiled + (size_t)(pm.b_row0 / kTile) * kTileFloats;
        const int ntiles = (int)item.ct1 - (int)item.ct0;
        if (tid == 0) {
            mbar_arrive_expect_tx(&S.barA, kTileBytes);
            bulk_g2s(S.A, atile, kTileBytes, &S.barA);
            if (ntiles > 0) {
                const uint32_t slot = seq & 1;
                mbar_arrive_expect_tx(&S.barB[slot], kTileBytes);
                bulk_g2s(S.B[slot], bbase + (size_t)item.ct0 * kTileFloats, kTileBytes, &S.barB[slot]);
            }
        }
        uint32_t irow[8];
        bool rvalid[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            irow[r] = item.rt * kTile + row_of(ty, r);
            rvalid[r] = irow[r] < pm.na;
        }
        float d1[8], d2[8];
        uint32_t j1[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            d1[r] = __int_as_float(0x7f800000);
            d2[r] = __int_as_float(0x7f800000);
            j1[r] = 0xffffffffu;
        }
        bool mine = mbar_wait(&S.barA, a_phase, g.err);
        a_phase ^= 1;

        for (int t = 0; t < ntiles; ++t) {
            const uint32_t slot = seq & 1, parity = (seq >> 1) & 1;
            const uint32_t ct = item.ct0 + t;
            if (tid == 0 && t + 1 < ntiles) {
                mbar_arrive_expect_tx(&S.barB[slot ^ 1], kTileBytes);
                bulk_g2s(S.B[slot ^ 1], bbase + (size_t)(ct + 1) * kTileFloats, kTileBytes, &S.barB[slot ^ 1]);
            }
            mine = mine && mbar_wait(&S.barB[slot], parity, g.err);
            const uint32_t cb = seq & 1;
            if (mine) {
                float d[8][8];
                tile_distances<X2>(S.A, S.B[slot], ty, tx, zero2, d);

                uint32_t jc[8];
                bool cvalid[8];
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    jc[c] = ct * kTile + col_of(tx, c);
                    cvalid[c] = jc[c] < pm.nb;
                }
                // rows: ratio_match's update (matching.rs:182-187), columns in increasing j.
#pragma unroll
                for (int r = 0; r < 8; ++r)
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        const float v = d[r][c];
                        if (cvalid[c]) {
                            if (v < d1[r]) {
                                d2[r] = d1[r];
                                d1[r] = v;
                                j1[r] = jc[c];
                            } else if (v < d2[r]) {
                                d2[r] = v;
                            }
                        }
                    }
                // columns: (d, lowest i) (matching.rs:188-190, 196-203).
                if (g.mutual) {
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        u64 key = ~0ull;
#pragma unroll
                        for (int r = 0; r < 8; ++r) {
                            const u64 k = ((u64)__float_as_uint(d[r][c]) << 32) | irow[r];
                            if (rvalid[r] && k < key) key = k;
                        }
                        const u64 o = __shfl_xor_sync(0xffffffffu, key, 16);
                        key = o < key ? o : key;
                        if (lane < 16 && key != ~0ull) atomicMin(&S.colred[cb][col_of(tx, c)], key);
                    }
                }
            }
            ok = __syncthreads_and(mine);
            if (!ok) break;
            if (g.mutual && tid < kTile) {
                const u64 v = S.colred[cb][tid];
                const uint32_t j = ct * kTile + tid;
                if (v != ~0ull && j < pm.nb) atomicMin(&g.colbest[pm.col_base + j], v);
                S.colred[cb][tid] = ~0ull;
            }
            ++seq;
        }
        // End of item: every thread is done with S.item and the a tile before
        // thread 0 fetches the next item (also when the item had no b tiles).
        ok = __syncthreads_and(ok && mine);
        if (!ok) break;
        // Merge row states across the 16 column threads (lanes xor 1..8).
#pragma unroll
        for (int r = 0; r < 8; ++r) {
#pragma unroll
            for (int off = 1; off < 16; off <<= 1) {
                const float o1 = __shfl_xor_sync(0xffffffffu, d1[r], off);
                const float o2 = __shfl_xor_sync(0xffffffffu, d2[r], off);
                const uint32_t oj = __shfl_xor_sync(0xffffffffu, j1[r], off);
                const float nd2 = fminf(fmaxf(d1[r], o1), fminf(d2[r], o2));
                if (o1 < d1[r] || (o1 == d1[r] && oj < j1[r])) {
                    d1[r] = o1;
                    j1[r] = oj;
                }
                d2[r] = nd2;
            }
        }
        if (tx == 0) {
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                RowPart p;
                p.d1 = d1[r];
                p.d2 = d2[r];
                p.j1 = j1[r];
                p.pad = 0;
                g.parts[(size_t)item.part * kTile + row_of(ty, r)] = p;
            }
        }
    }
}

cudaError_t init_exact_kernels() {
    const int smem = (int)sizeof(ExactSmem);
    cudaError_t e = cudaFuncSetAttribute(exact_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(exact_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    return e;
}

void launch_exact(const ExactArgs &a, int grid, cudaStream_t s) {
    const size_t smem = sizeof(ExactSmem);
    if (a.x2)
        exact_kernel<true><<<grid, kThreads, smem, s>>>(a);
    else
        exact_kernel<false><<<grid, kThreads, smem, s>>>(a);
}

// -------------------------------------------------------------- finalize

// One CTA per pair: merge the row partials of every column chunk, apply
// matching.rs:204-214 and write matches in ascending i. One thread per row and
// step, partials loaded four at a time: a batch of few pairs runs 1024 threads
// per pair, since a single small pair is a chain of dependent loads, not a
// bandwidth problem; larger batches run 256 (more pairs resident per SM).
constexpr int kFinThreadsMax = 1024;

template <int kThreads>
__global__ void __launch_bounds__(kThreads) finalize_kernel(FinalizeArgs g) {
    __shared__ uint32_t warp_tot[kThreads / 32];
    constexpr uint32_t nthr = kThreads;
    constexpr int nwarps = kThreads / 32;
    const PairMeta pm = g.pairs[blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const float kInf = __int_as_float(0x7f800000);
    uint32_t base = 0;
    for (uint32_t row0 = 0; row0 < pm.na; row0 += nthr) {
        const uint32_t i = row0 + tid;
        uint32_t flag = 0, jout = 0;
        if (i < pm.na) {
            const uint32_t rt = i / kTile;
            float d1 = kInf, d2 = kInf;
            uint32_t j1 = 0xffffffffu;
            const RowPart *pr = g.parts + (size_t)(pm.part_base + rt * pm.nchunk) * kTile + (i % kTile);
            if constexpr (kThreads == 256) {  // many pairs: mostly one column range per row
                for (uint32_t c = 0; c < pm.nchunk; ++c) merge_rowpart(pr[(size_t)c * kTile], d1, d2, j1);
            } else
            for (uint32_t c0 = 0; c0 < pm.nchunk; c0 += 4) {
                RowPart q[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    // an absent chunk merges as the neutral partial (inf, inf, none)
                    q[u] = RowPart{kInf, kInf, 0xffffffffu, 0u};
                    if (c0 + u < pm.nchunk) q[u] = pr[(size_t)(c0 + u) * kTile];
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) merge_rowpart(q[u], d1, d2, j1);
            }
            const bool d2_finite = d2 < kInf;
            if (j1 != 0xffffffffu && d2_finite && !(d1 >= __fmul_rn(g.ratio2, d2))) {
                if (!g.mutual || static_cast<uint32_t>(g.colbest[pm.col_base + j1]) == i) {
                    flag = 1;
                    jout = j1;
                }
            }
        }
        // Block-wide exclusive scan of the flags.
        const uint32_t ballot = __ballot_sync(0xffffffffu, flag);
        const uint32_t wpre = __popc(ballot & ((1u << lane) - 1u));
        if (lane == 0) warp_tot[wid] = __popc(ballot);
        __syncthreads();
        uint32_t off = 0, tot = 0;
        for (int w = 0; w < nwarps; ++w) {
            const uint32_t t = warp_tot[w];
            off += (w < wid) ? t : 0;
            tot += t;
        }
        if (flag) g.slots[pm.slot_off + base + off + wpre] = make_uint2(i, jout);
        base += tot;
        __syncthreads();
    }
    if (tid == 0) g.counts[blockIdx.x] = (g.err && *g.err) ? 0xffffffffu : base;
}

void launch_finalize(const FinalizeArgs &a, cudaStream_t s) {
    if (!a.npairs) return;
    if (a.npairs <= kFewPairs)
        finalize_kernel<kFinThreadsMax><<<a.npairs, kFinThreadsMax, 0, s>>>(a);
    else
        finalize_kernel<256><<<a.npairs, 256, 0, s>>>(a);
}

// Self-test of the bounded waits: thread 0 waits on an mbarrier that expects
// one arrival nobody makes, gives up after `polls` polls and records
// DERR_TIMEOUT_BAR in *err, the path every kernel's timed-out wait takes.
__global__ void wait_selftest_kernel(uint32_t polls, uint32_t *err) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_wait(&bar, 0, err, polls);
}

void launch_wait_selftest(uint32_t polls, uint32_t *err, cudaStream_t s) {
    wait_selftest_kernel<<<1, 32, 0, s>>>(polls, err);
}

}  // namespace slm
