// k_shortlist.cu — BF16 / FP8 tcgen05 shortlist path of ratio_match.
//
// Reference: crates/core/src/matching.rs:144-215. See slm_shortlist.h for the
// passes and the certification rules. Every match decision is either proven
// by the per-pair error bound eps or settled with exact spec-order FP32
// distances (matching.rs:146-155), so results equal the reference's.
//
// Tensor-core kernel (sl_pass_kernel, one persistent CTA per SM, 18 warps):
//   warp 0      TMA producer: per item the a tiles (1 or 2 x 128 rows, K-major,
//               128B-swizzled operand images copied verbatim from the store;
//               FP8 also norms and scales); per 128-column b tile the operand
//               tile (and, in pass 2, column thresholds) through a ring of 3
//               (BF16) or 4 (FP8) slots.
//   warp 1      allocates 512 TMEM columns; one thread issues tcgen05.mma
//               (M=128, N=128, K=16 bf16 / K=32 e4m3) into a double-buffered
//               pair of 128x128 f32 accumulators per a tile. BF16 adds a ninth
//               K step over the norm extension (slm_shortlist.h), so the
//               accumulator is d~ / 2.
//   warps 2-17  epilogue: warp w reads TMEM lane quarter w % 4 of a tile
//               ((w - 2) / 4) % 2, column half (w - 2) / 8 of every b tile,
//               one thread per row, 16 columns per tcgen05.ld. Row minima use
//               a 3-input min tree per 16 columns; column minima use
//               redux.sync.min.f32 per column, merged across warps in shared
//               memory (by the epilogue warps of sub-partitions 2 and 3) and
//               across CTAs with one atomicMin per column and tile. Pass 2
//               looks for row-candidate and column-window hits in groups of 4
//               columns behind the chunk minimum. BF16 pass 1 never reads the
//               b stage: the MMA's commit alone frees it.
#include <cuda_fp8.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "ptx.cuh"
#include "slm_shortlist.h"

namespace slm {

// ------------------------------------------------------------ small helpers

// Order-preserving map of f32 to u32 (unsigned order == float order).
SLM_DEV uint32_t f2ord(float f) {
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
SLM_DEV float ord2f(uint32_t u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u); }

SLM_DEV float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

SLM_DEV float warp_min_f32(float v) {
    float r;
    asm volatile("redux.sync.min.f32 %0, %1, 0xffffffff;" : "=f"(r) : "f"(v));
    return r;
}

SLM_DEV uint64_t globaltimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Minimum of 32 values (NaN inputs are ignored by min.f32).
SLM_DEV float min32(const float (&d)[32]) {
    float m[11];
#pragma unroll
    for (int k = 0; k < 10; ++k) m[k] = min3f(d[3 * k], d[3 * k + 1], d[3 * k + 2]);
    m[10] = fminf(d[30], d[31]);
    const float x = min3f(m[0], m[1], m[2]);
    const float y = min3f(m[3], m[4], m[5]);
    const float z = min3f(m[6], m[7], m[8]);
    return fminf(min3f(x, y, z), fminf(m[9], m[10]));
}

typedef unsigned long long u64x;
SLM_DEV u64x f2_pack(float lo, float hi) {
    u64x d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}
SLM_DEV float f2_lo(u64x v) { return __uint_as_float(static_cast<uint32_t>(v)); }
SLM_DEV float f2_hi(u64x v) { return __uint_as_float(static_cast<uint32_t>(v >> 32)); }
SLM_DEV u64x f2_add(u64x a, u64x b) {
    u64x d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
SLM_DEV u64x f2_sub(u64x a, u64x b) {
    u64x d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// Approximate-path arithmetic: one rounding, covered by the error bound.
SLM_DEV u64x f2_fma(u64x a, u64x b, u64x c) {
    u64x d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// 32 lanes x 16 consecutive 32-bit TMEM columns (asynchronous until the wait).
SLM_DEV void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}
// Waits for this thread's TMEM loads; the registers are operands so no use
// of them can be scheduled before the wait.
SLM_DEV void tmem_wait_ld16(uint32_t (&r)[16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]),
                   "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]),
                   "+r"(r[14]), "+r"(r[15])
                 :
                 : "memory");
}

// Column-window counts of 4 consecutive columns (16-byte aligned): adds 1.0
// to each column whose x <= 0 (not for NaN) with one vector reduction, issued
// only when pred holds (the group has a hit), without a branch. The counts are
// f32: exact far beyond any row count (2^24).
SLM_DEV void red_add4_le0(float *p, float x0, float x1, float x2, float x3, bool pred) {
    asm volatile(
        "{\n"
        ".reg .pred q;\n"
        ".reg .f32 a, b, c, d;\n"
        "set.le.f32.f32 a, %1, 0f00000000;\n"
        "set.le.f32.f32 b, %2, 0f00000000;\n"
        "set.le.f32.f32 c, %3, 0f00000000;\n"
        "set.le.f32.f32 d, %4, 0f00000000;\n"
        "setp.ne.u32 q, %5, 0;\n"
        "@q red.relaxed.gpu.global.add.v4.f32 [%0], {a, b, c, d};\n"
        "}\n" ::"l"(p),
        "f"(x0), "f"(x1), "f"(x2), "f"(x3), "r"((uint32_t)pred)
        : "memory");
}

// st.global.v2 of (a, b) when pred holds, without a branch.
SLM_DEV void st_pair_if(uint2 *p, uint32_t a, uint32_t b, bool pred) {
    asm volatile(
        "{\n"
        ".reg .pred q;\n"
        "setp.ne.u32 q, %3, 0;\n"
        "@q st.global.v2.u32 [%0], {%1, %2};\n"
        "}\n" ::"l"(p),
        "r"(a), "r"(b), "r"((uint32_t)pred)
        : "memory");
}

// One record (4 values, first column) when pred holds, without a branch.
SLM_DEV void st_rec_if(float4 *p, uint32_t *pj, float a, float b, float c, float d, uint32_t j, bool pred) {
    asm volatile(
        "{\n"
        ".reg .pred q;\n"
        "setp.ne.u32 q, %6, 0;\n"
        "@q st.global.v4.f32 [%0], {%2, %3, %4, %5};\n"
        "@q st.global.u32 [%1], %7;\n"
        "}\n" ::"l"(p),
        "l"(pj), "f"(a), "f"(b), "f"(c), "f"(d), "r"((uint32_t)pred), "r"(j)
        : "memory");
}

// Minimum of 16 values, and with the minima of its two groups of 8.
SLM_DEV float min16(const float (&d)[16]) {
    const float a = min3f(d[0], d[1], d[2]), b = min3f(d[3], d[4], d[5]), c = min3f(d[6], d[7], d[8]);
    const float e = min3f(d[9], d[10], d[11]), f = min3f(d[12], d[13], d[14]);
    return fminf(min3f(a, b, c), min3f(e, f, d[15]));
}
// Minimum of 16 values, and with the minima of its four groups of 4: a rare
// hit below a threshold is then looked for in 4 values (measured faster than
// groups of 2 or 8 on the pass-2 tests).
SLM_DEV float min16q(const float (&d)[16], float (&g4)[4]) {
#pragma unroll
    for (int q = 0; q < 4; ++q) g4[q] = min3f(d[4 * q], d[4 * q + 1], fminf(d[4 * q + 2], d[4 * q + 3]));
    return min3f(g4[0], g4[1], fminf(g4[2], g4[3]));
}

// Exact reference distance (matching.rs:146-155): lane k = components 8c+k.
SLM_DEV float sq_dist_spec(const float *__restrict__ p, const float *__restrict__ r) {
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const float4 *p4 = reinterpret_cast<const float4 *>(p);
    const float4 *r4 = reinterpret_cast<const float4 *>(r);
#pragma unroll 4
    for (int c = 0; c < 16; ++c) {
        const float4 x0 = p4[2 * c], x1 = p4[2 * c + 1];
        const float4 y0 = r4[2 * c], y1 = r4[2 * c + 1];
        const float xs[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
        const float ys[8] = {y0.x, y0.y, y0.z, y0.w, y1.x, y1.y, y1.z, y1.w};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float t = __fsub_rn(xs[k], ys[k]);
            acc[k] = __fadd_rn(acc[k], __fmul_rn(t, t));
        }
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s = __fadd_rn(s, acc[k]);
    return s;
}

// ------------------------------------------------------------ store packing

// One CTA (128 threads) per 128-row tile of a view: low-precision operand
// image (K-major, 128B swizzle: 16-byte chunk c of row r at c ^ (r % 8)),
// f32 squared norms, and the view's error statistics.
template <bool FP8>
__global__ void __launch_bounds__(128) pack_lowp_kernel(const uint4 *__restrict__ tab, const float *__restrict__ raw,
                                                        uint8_t *__restrict__ optiles, float *__restrict__ norms,
                                                        float *__restrict__ qscale, ViewStat *__restrict__ vstats) {
    const uint4 te = tab[blockIdx.x];  // {first store row of the view, rows, tile within the view, view}
    const uint32_t row0 = te.x, n = te.y, view = te.w;
    const uint32_t r = threadIdx.x;
    const uint32_t tile = te.z;
    const uint32_t row = tile * kTile + r;  // row within the view
    const bool valid = row < n;
    const float *src = raw + (size_t)(row0 + row) * kDesc;
    constexpr uint32_t kTileBytes = FP8 ? kFp8TileBytes : kBf16TileStride;
    uint8_t *dst = optiles + (size_t)(row0 / kTile + tile) * kTileBytes;
    float x[kDesc];
#pragma unroll
    for (int q = 0; q < 32; ++q) {
        float4 v = valid ? reinterpret_cast<const float4 *>(src)[q] : make_float4(0.f, 0.f, 0.f, 0.f);
        x[4 * q] = v.x;
        x[4 * q + 1] = v.y;
        x[4 * q + 2] = v.z;
        x[4 * q + 3] = v.w;
    }
    float nrm = 0.f, res = 0.f, nq = 0.f, amax = 0.f;
    bool bad = false;
#pragma unroll
    for (int k = 0; k < kDesc; ++k) {
        nrm = __fadd_rn(nrm, __fmul_rn(x[k], x[k]));
        bad |= !isfinite(x[k]);
        amax = fmaxf(amax, fabsf(x[k]));
    }
    float scale = 1.f, inv = 1.f;
    if constexpr (FP8) {
        // per-descriptor power-of-two scale: max |a| * scale <= 448 (E4M3 max)
        if (amax > 0.f && isfinite(amax)) {
            int e;
            frexpf(448.f / amax, &e);
            scale = ldexpf(1.f, e - 1);
            inv = ldexpf(1.f, 1 - e);
        }
    }
#pragma unroll
    for (int c16 = 0; c16 < (FP8 ? 8 : 16); ++c16) {
        uint32_t w[4];
        if constexpr (FP8) {
            // 16 components -> 16 bytes
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                uint32_t word = 0;
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    const int k = c16 * 16 + h * 4 + b;
                    const __nv_fp8_storage_t q = __nv_cvt_float_to_fp8(x[k] * scale, __NV_SATFINITE, __NV_E4M3);
                    __nv_fp8_e4m3 qq;
                    qq.__x = q;
                    const float back = static_cast<float>(qq) * inv;
                    const float e = x[k] - back;
                    res = fmaf(e, e, res);
                    nq = fmaf(back, back, nq);
                    word |= (uint32_t)q << (8 * b);
                }
                w[h] = word;
            }
            const uint32_t chunk = (uint32_t)c16;  // 128 bytes per row = one swizzle span
            uint4 *d = reinterpret_cast<uint4 *>(dst + r * 128 + ((chunk ^ (r & 7)) * 16));
            *d = make_uint4(w[0], w[1], w[2], w[3]);
        } else {
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                const int k = c16 * 8 + h * 2;
                const __nv_bfloat16 lo = __float2bfloat16_rn(x[k]);
                const __nv_bfloat16 hi = __float2bfloat16_rn(x[k + 1]);
                const float blo = __bfloat162float(lo), bhi = __bfloat162float(hi);
                const float e0 = x[k] - blo, e1 = x[k + 1] - bhi;
                res = fmaf(e0, e0, fmaf(e1, e1, res));
                nq = fmaf(blo, blo, fmaf(bhi, bhi, nq));
                w[h] = (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
            }
            const uint32_t kb = (uint32_t)c16 >> 3, chunk = (uint32_t)c16 & 7;
            uint4 *d = reinterpret_cast<uint4 *>(dst + kb * 16384 + r * 128 + ((chunk ^ (r & 7)) * 16));
            *d = make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
    if constexpr (!FP8) {
        // norm extension (slm_shortlist.h): |a|^2 / 2 = hi + lo (the difference
        // of a float and its bf16 rounding is exact in f32). Padding rows get
        // hi = NaN: every product with a padding row or column is NaN, which
        // min.f32 and redux.min ignore and no threshold admits, so the pass
        // kernels need no masks for ragged tiles
        const float half = valid ? 0.5f * nrm : 0.f;
        const __nv_bfloat16 hi = __float2bfloat16_rn(half);
        const __nv_bfloat16 lo = __float2bfloat16_rn(half - __bfloat162float(hi));
        const uint32_t hl = valid ? ((uint32_t)__bfloat16_as_ushort(hi) | ((uint32_t)__bfloat16_as_ushort(lo) << 16))
                                  : 0x00007fc0u;  // padding rows: hi = NaN, lo = 0
        const uint32_t ones = 0x3f803f80u;  // two bf16 1.0
        uint8_t *ext = dst + kBf16TileBytes + (r >> 3) * 384 + (r & 7) * 16;
        *reinterpret_cast<uint4 *>(ext) = make_uint4(hl, ones, 0u, 0u);        // kc0: hi lo 1 1
        *reinterpret_cast<uint4 *>(ext + 128) = make_uint4(ones, hl, 0u, 0u);  // kc1: 1 1 hi lo
        *reinterpret_cast<uint4 *>(ext + 256) = make_uint4(0u, 0u, 0u, 0u);    // kc2
    }
    norms[row0 + row] = valid ? nrm : __int_as_float(0x7fc00000);  // FP8: NaN distances to padding rows too
    if constexpr (FP8) qscale[row0 + row] = inv;
    // statistics (non-negative floats compare as their bit patterns)
    float s_n = valid ? sqrtf(nrm) : 0.f, s_r = valid ? sqrtf(res) : 0.f, s_q = valid ? sqrtf(nq) : 0.f;
    if (!isfinite(s_n) || !isfinite(s_r) || !isfinite(s_q)) bad = bad || valid;
    uint32_t b = (valid && bad) ? 1u : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s_n = fmaxf(s_n, __shfl_xor_sync(0xffffffffu, s_n, o));
        s_r = fmaxf(s_r, __shfl_xor_sync(0xffffffffu, s_r, o));
        s_q = fmaxf(s_q, __shfl_xor_sync(0xffffffffu, s_q, o));
        b |= __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((r & 31) == 0) {
        ViewStat *vs = vstats + view;
        if (isfinite(s_n)) atomicMax(&vs->nmax, __float_as_uint(s_n));
        if (isfinite(s_r)) atomicMax(&vs->rho, __float_as_uint(s_r));
        if (isfinite(s_q)) atomicMax(&vs->nqmax, __float_as_uint(s_q));
        if (b) atomicOr(&vs->bad, 1u);
    }
}

void launch_pack_lowp(const uint4 *tab, uint32_t ntiles, const float *raw, int fp8, uint8_t *optiles, float *norms,
                      float *qscale, ViewStat *vstats, cudaStream_t s) {
    if (!ntiles) return;
    if (fp8)
        pack_lowp_kernel<true><<<ntiles, 128, 0, s>>>(tab, raw, optiles, norms, qscale, vstats);
    else
        pack_lowp_kernel<false><<<ntiles, 128, 0, s>>>(tab, raw, optiles, norms, qscale, vstats);
}

// ------------------------------------------------------------ tcgen05 pieces

// Shared-memory matrix descriptor (tcgen05): K-major, 128B swizzle, 8-row
// groups 1024 bytes apart (stride byte offset), version 1, base offset 0.
SLM_DEV uint64_t umma_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3fffu);   // start address
    d |= (uint64_t)1 << 16;                    // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset
    d |= (uint64_t)1 << 46;                    // descriptor version
    d |= (uint64_t)2 << 61;                    // SWIZZLE_128B
    return d;
}

// Shared-memory matrix descriptor: K-major without swizzle. Core matrices of
// 8 rows x 16 bytes (rows 16 bytes apart); lbo = bytes between core matrices
// along K, sbo = bytes between 8-row groups.
SLM_DEV uint64_t umma_desc_plain(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3fffu);
    d |= (uint64_t)((lbo >> 4) & 0x3fffu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3fffu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version; layout type 0 = no swizzle
    return d;
}

// Instruction descriptor: f32 accumulate, K-major A and B, M=128, N=128.
// kind::f16 with bf16 inputs (format 1) or kind::f8f6f4 with e4m3 (format 0);
// negate_b (bit 14) negates operand B.
__host__ __device__ constexpr uint32_t umma_idesc(bool fp8, bool negate_b = false) {
    return (1u << 4) | ((fp8 ? 0u : 1u) << 7) | ((fp8 ? 0u : 1u) << 10) | ((negate_b ? 1u : 0u) << 14) |
           ((128u >> 3) << 17) | ((128u >> 4) << 24);
}

template <bool FP8>
struct SlSmem {
    static constexpr uint32_t kOp = FP8 ? kFp8TileBytes : kBf16TileStride;  // bytes per operand tile
    static constexpr int kStages = FP8 ? kSlStages : 3;                      // b-tile ring depth
    uint8_t A[2][kOp];
    uint8_t B[kStages][kOp];
    float bnorm[kStages][128];  // FP8 only (BF16 carries the norms in the operands)
    float bthr[kStages][128];
    float bthr2[kStages][128];  // pass 2, items of two pairs: the second pair's column thresholds
    float bscale[kStages][128];
    float anorm[256];
    float athr[256];
    float ascale[256];
    float colpart[2][8][128];  // [tile parity][(a tile, lane quarter)][column]
    float2 rowx[256];          // pass 1: the second column half's row state
    uint32_t rownear[256];     // pass 1: the second column half's near-chunk count
    uint64_t a_full, a_empty;
    uint64_t b_full[kStages], b_empty[kStages];
    uint64_t t_full[2], t_empty[2];
    uint64_t ep_bar;  // epilogue warps: column partials of a tile are stored
    uint32_t tmem_base;
    uint32_t abort_flag;
};

template <bool FP8>
constexpr size_t sl_smem_bytes() {
    return sizeof(SlSmem<FP8>) + 1024;  // slack for 1024-byte alignment
}

// Bounded wait (about 2 s of wall time); on timeout raises the CTA abort flag
// and records an error so every role leaves its loop.
SLM_DEV bool sl_wait(uint64_t *bar, uint32_t parity, volatile uint32_t *abort_flag, uint32_t *err) {
    uint64_t t0 = 0;
    for (uint32_t it = 0;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63) == 63) {
            if (*abort_flag) return false;
            const uint64_t now = globaltimer();
            if (t0 == 0) t0 = now;
            else if (now - t0 > 2000000000ull) {
                *abort_flag = 1;
                atomicCAS(err, 0u, (uint32_t)DERR_TIMEOUT_MMA);
                return false;
            }
        }
    }
}

// Items of two pairs (odd row-tile counts sharing a b view).
SLM_DEV bool item_two_pairs(const SlItem &it) { return it.nat == 2 && it.pair[1] != it.pair[0]; }

// Whether a pass works on a pair: tier 0's pass 1 on every pair, otherwise
// the pairs of the tier (sl_pair_on).
template <int PASS>
SLM_DEV bool pass_pair_on(const SlArgs &g, const SlPair &sp) {
    return (PASS == 1 && !g.tier) || sl_pair_on(g, sp);
}
// A pass skips an item when none of its pairs is on (all roles read the same
// flags: earlier kernels wrote them).
template <int PASS>
SLM_DEV bool item_off(const SlArgs &g, const SlItem &it) {
    return !pass_pair_on<PASS>(g, g.spairs[it.pair[0]]) && (it.nat == 1 || !pass_pair_on<PASS>(g, g.spairs[it.pair[1]]));
}

// One CTA of kSlThreads per SM. Warps are spread over the SM's four
// sub-partitions, each with 16384 registers: 18 warps put 5 on two of them, so
// 5 x 32 x R <= 16384, R in steps of 8: 96 registers per thread.
constexpr int kSlWarpsPerQuarter = (kSlThreads / 32 + 3) / 4;
constexpr int kSlMaxRegs = (16384 / (32 * kSlWarpsPerQuarter)) & ~7;
static_assert(kSlMaxRegs == 96, "register budget of the 18-warp pass kernel");

template <int PASS, bool FP8, bool DUMP>
__global__ void __maxnreg__(kSlMaxRegs) sl_pass_kernel(SlArgs g) {
    extern __shared__ uint8_t sl_smem_raw[];
    const uint32_t pad = (1024u - (smem_u32(sl_smem_raw) & 1023u)) & 1023u;
    SlSmem<FP8> &S = *reinterpret_cast<SlSmem<FP8> *>(sl_smem_raw + pad);
    constexpr uint32_t kOp = SlSmem<FP8>::kOp;
    constexpr int kStg = SlSmem<FP8>::kStages;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t *err = g.ctl + 1;
    volatile uint32_t *abort_flag = &S.abort_flag;
    // the epilogue reads the b stage in pass 2 (thresholds) and for FP8 (norms, scales)
    constexpr bool kEpReadsB = PASS == 2 || FP8;

    if (threadIdx.x == 0) {
        mbar_init(&S.a_full, 1);
        mbar_init(&S.a_empty, 1 + kSlEpWarps);
        for (int s = 0; s < kStg; ++s) {
            mbar_init(&S.b_full[s], 1);
            // BF16 pass 1's epilogue reads nothing of the b stage (norms are in the
            // product): the MMA's commit alone frees it, one use earlier
            mbar_init(&S.b_empty[s], kEpReadsB ? 1 + kSlEpWarps : 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&S.t_full[b], 1);
            mbar_init(&S.t_empty[b], kSlEpWarps);
        }
        mbar_init(&S.ep_bar, kSlEpWarps);
        S.abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == 1) {
        tmem_alloc(&S.tmem_base, 512);
        tmem_relinquish();
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;

    if (warp == 0) {
        // ---------------------------------------------------------- producer
        if (lane == 0) {
            uint32_t st = 0, sph = 0, iter = 0;  // iter: items processed (routed pairs skip pass 2)
            for (uint32_t it = blockIdx.x; it < g.n_items; it += gridDim.x) {
                const SlItem item = g.items[it];
                if (item_off<PASS>(g, item)) continue;
                if (iter > 0 && !sl_wait(&S.a_empty, (iter - 1) & 1, abort_flag, err)) break;
                const bool two = item_two_pairs(item);
                const PairMeta pm = g.pairs[item.pair[0]];  // both pairs have this b view
                const uint32_t cbase0 = g.spairs[item.pair[0]].cbase;
                const uint32_t cbase1 = two ? g.spairs[item.pair[1]].cbase : 0;
                uint32_t bytes = item.nat * kOp;
                if (PASS == 2) bytes += item.nat * 512;
                if (FP8) bytes += item.nat * 1024;  // norms and scales
                mbar_arrive_expect_tx(&S.a_full, bytes);
#pragma unroll
                for (uint32_t a = 0; a < 2; ++a) {  // static indices keep the item in registers
                    if (a >= item.nat) break;
                    const uint32_t pa = item.pair[a];
                    const uint32_t arow = g.pairs[pa].a_row0 + item.rt[a] * kTile;  // store row of the tile
                    bulk_g2s(S.A[a], g.optiles + (size_t)(arow / kTile) * kOp, kOp, &S.a_full);
                    if (FP8) bulk_g2s(&S.anorm[a * 128], g.norms + arow, 512, &S.a_full);
                    if (PASS == 2)
                        bulk_g2s(&S.athr[a * 128], g.rowthr + g.spairs[pa].rbase + item.rt[a] * kTile, 512, &S.a_full);
                    if (FP8) bulk_g2s(&S.ascale[a * 128], g.qscale + arow, 512, &S.a_full);
                }
                for (uint32_t t = item.ct0; t < item.ct1; ++t) {
                    if (!sl_wait(&S.b_empty[st], sph ^ 1, abort_flag, err)) break;
                    const uint32_t brow = pm.b_row0 + t * kTile;
                    uint32_t bb = kOp + (PASS == 2 ? (two ? 1024 : 512) : 0) + (FP8 ? 1024 : 0);
                    mbar_arrive_expect_tx(&S.b_full[st], bb);
                    bulk_g2s(S.B[st], g.optiles + (size_t)(brow / kTile) * kOp, kOp, &S.b_full[st]);
                    if (FP8) bulk_g2s(S.bnorm[st], g.norms + brow, 512, &S.b_full[st]);
                    if (PASS == 2) {
                        bulk_g2s(S.bthr[st], g.colthr + cbase0 + t * kTile, 512, &S.b_full[st]);
                        if (two) bulk_g2s(S.bthr2[st], g.colthr + cbase1 + t * kTile, 512, &S.b_full[st]);
                    }
                    if (FP8) bulk_g2s(S.bscale[st], g.qscale + brow, 512, &S.b_full[st]);
                    if (++st == kStg) st = 0, sph ^= 1;
                }
                ++iter;
                if (*abort_flag) break;
            }
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------- MMA issue
        constexpr uint32_t idesc = umma_idesc(FP8);
        constexpr uint32_t idesc_neg = umma_idesc(FP8, true);
        // Every operand tile has a fixed shared-memory address for the whole
        // kernel: the descriptors are made once, and a tile, stage or K step
        // adds its byte offset / 16 to the 14-bit start-address field (all
        // shared addresses lie below 256 KiB, so the field never carries).
        constexpr uint32_t kOp16 = kOp >> 4;
        const uint64_t adesc0 = umma_desc(smem_u32(S.A[0])), bdesc0 = umma_desc(smem_u32(S.B[0]));
        const uint64_t aext0 = umma_desc_plain(smem_u32(S.A[0]) + kBf16TileBytes, 128, 384);
        const uint64_t bext0 = umma_desc_plain(smem_u32(S.B[0]) + kBf16TileBytes + 128, 128, 384);
        uint32_t st = 0, sph = 0, tb = 0, tph = 0, iter = 0;
        for (uint32_t it = blockIdx.x; it < g.n_items; it += gridDim.x) {
            const SlItem item = g.items[it];
            if (item_off<PASS>(g, item)) continue;
            if (!sl_wait(&S.a_full, iter & 1, abort_flag, err)) break;
            ++iter;
            bool ok = true;
            for (uint32_t t = item.ct0; t < item.ct1; ++t) {
                if (!sl_wait(&S.b_full[st], sph, abort_flag, err) || !sl_wait(&S.t_empty[tb], tph ^ 1, abort_flag, err)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                if (lane == 0) {
                    const uint64_t bd = bdesc0 + (uint64_t)(st * kOp16);
#pragma unroll
                    for (uint32_t a = 0; a < 2; ++a) {
                        if (a >= item.nat) break;
                        const uint32_t d_tmem = tmem + (tb * 2 + a) * 128;
                        const uint64_t ad = adesc0 + (uint64_t)(a * kOp16);
                        if constexpr (FP8) {
#pragma unroll
                            for (int k = 0; k < 4; ++k)  // K = 32 e4m3 = 32 bytes per step
                                mma_f8(d_tmem, ad + 2 * k, bd + 2 * k, idesc, k > 0);
                        } else {
#pragma unroll
                            for (int k = 0; k < 8; ++k) {  // K = 16 bf16 = 32 bytes per step; -a.b
                                const uint32_t off16 = (k >> 2) * (16384 >> 4) + (k & 3) * 2;
                                mma_f16(d_tmem, ad + off16, bd + off16, idesc_neg, k > 0);
                            }
                            // + (|a|^2 + |b|^2) / 2: A from kc0, B from kc1 of the norm extension
                            mma_f16(d_tmem, aext0 + (uint64_t)(a * kOp16), bext0 + (uint64_t)(st * kOp16), idesc, true);
                        }
                    }
                    mma_commit(&S.b_empty[st]);
                    mma_commit(&S.t_full[tb]);
                }
                __syncwarp();
                if (++st == kStg) st = 0, sph ^= 1;
                tb ^= 1;
                if (tb == 0) tph ^= 1;
            }
            if (lane == 0) mma_commit(&S.a_empty);
            __syncwarp();
            if (!ok) break;
        }
    } else {
        // ---------------------------------------------------------- epilogue
        // 16 warps. Warp w reads TMEM lane quarter q = w % 4 (the only quarter
        // it may access) of a tile `at`, columns [h*64, h*64 + 64) of every
        // 128-column b tile; one thread per row, 16 columns per tcgen05.ld,
        // the next load issued before the current chunk is reduced.
        const int ep = warp - 2;                 // 0..15
        const int q = warp & 3;
        const int at = (ep >> 2) & 1;
        const int h = ep >> 3;
        const int combo = at * 4 + q;
        const int r = at * 128 + q * 32 + lane;  // row within the item
        const uint32_t lane_addr = (uint32_t)(q * 32) << 16;
        uint32_t st = 0, sph = 0, tb = 0, tph = 0, iter = 0, eph = 0;
        const float kInf = __int_as_float(0x7f800000);
        // BF16 accumulators hold d~ / 2 (norms folded into the product): the
        // epilogue compares in that domain and scales by 2 (exact) where values
        // leave the kernel; FP8 computes d~ itself
        constexpr float kDom = FP8 ? 1.f : 2.f;
        for (uint32_t it = blockIdx.x; it < g.n_items; it += gridDim.x) {
            const SlItem item = g.items[it];
            if (item_off<PASS>(g, item)) continue;
            if (!sl_wait(&S.a_full, iter & 1, abort_flag, err)) break;
            ++iter;
            const bool two = item_two_pairs(item);
            // this warp's a tile (clamped to tile 0); selects, not indexing: the
            // item stays in registers
            const bool mine1 = at == 1 && item.nat == 2;
            const uint32_t pid = mine1 ? item.pair[1] : item.pair[0];
            const PairMeta pm = g.pairs[pid];
            const SlPair sp = g.spairs[pid];
            // pass 1 merges the column partials of each pair of the item
            const uint32_t na0 = g.pairs[item.pair[0]].na, na1 = two ? g.pairs[item.pair[1]].na : na0;
            const uint32_t cb0 = g.spairs[item.pair[0]].cbase, cb1 = two ? g.spairs[item.pair[1]].cbase : cb0;
            // warp-uniform: the warp's a tile exists and its pair is still open
            const bool active = at < (int)item.nat && pass_pair_on<PASS>(g, sp);
            // pass 1: whether each pair of the item is on (column-minimum merge)
            const bool on0 = pass_pair_on<PASS>(g, g.spairs[item.pair[0]]);
            const bool on1 = two ? pass_pair_on<PASS>(g, g.spairs[item.pair[1]]) : on0;
            const uint32_t rt = mine1 ? item.rt[1] : item.rt[0];
            const uint32_t mypart = mine1 ? item.part[1] : item.part[0];
            // warp-uniform: this lane quarter holds at least one row of the pair
            // (quarters of padding rows skip their chunks)
            const bool qvalid = active && rt * kTile + q * 32 < pm.na;
            const uint32_t i = rt * kTile + q * 32 + lane;    // row within the pair
            const bool rvalid = active && i < pm.na;
            const float na_i = (FP8 && active) ? S.anorm[r] : 0.f;
            const float thr_i = (PASS == 2 && active) ? S.athr[r] * (1.f / kDom) : -kInf;
            const float sa_i = (FP8 && active) ? S.ascale[r] : 1.f;
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.a_empty);
            float m1 = kInf, m2 = kInf;
            // pass 1: 16-column chunks whose minimum lies within 2 eps above the
            // running row minimum (new minima excluded), the estimate of the
            // row's shortlist size that pair routing uses
            const float w2 = 2.f * sp.eps;
            uint32_t near = 0;
            // pass 2: the records of this row and of the item's column range
            // (exactly one item writes them: plain stores, a running count)
            const uint32_t crow = PASS == 2 ? sl_cand_row(sp, pm.na, (mypart - sp.part_base) % sp.nchunk, i) : 0;
            const uint32_t hr = g.half_recs;
            const uint32_t rec0 = (2 * crow + h) * hr;
            uint32_t ncand = 0;
            bool ok = true;
            for (uint32_t t = item.ct0; t < item.ct1; ++t) {
                // without the epilogue's b_empty arrivals the producer may refill a
                // stage twice before this warp would wait on it (its parity would be
                // ambiguous): an epilogue that does not read the stage waits on t_full
                // only, which implies the MMA consumed the stage
                if ((kEpReadsB && !sl_wait(&S.b_full[st], sph, abort_flag, err)) ||
                    !sl_wait(&S.t_full[tb], tph, abort_flag, err)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                if (qvalid) {
                    const uint32_t tcol = tmem + lane_addr + (tb * 2 + at) * 128 + h * 64;
                    // chunks of 16 columns, two per iteration: loads double-buffered,
                    // the body kept at two copies (instruction-cache footprint)
                    auto chunk = [&](const uint32_t (&vc)[16], int c, const ulonglong2 (&tt)[4]) {
                        const uint32_t cb = h * 64 + c * 16;   // column within the tile
                        const uint32_t j0 = t * kTile + cb;    // column within the pair
                        float d[16];
                        if constexpr (FP8) {
                            const float4 *bn4 = reinterpret_cast<const float4 *>(&S.bnorm[st][cb]);
                            const float4 *bs4 = reinterpret_cast<const float4 *>(&S.bscale[st][cb]);
                            const float m2sa = -2.f * sa_i;
#pragma unroll
                            for (int k4 = 0; k4 < 4; ++k4) {
                                const float4 nb = bn4[k4], sb = bs4[k4];
                                const float nbv[4] = {nb.x, nb.y, nb.z, nb.w}, sbv[4] = {sb.x, sb.y, sb.z, sb.w};
#pragma unroll
                                for (int e = 0; e < 4; ++e)
                                    d[4 * k4 + e] = fmaf(__uint_as_float(vc[4 * k4 + e]), m2sa * sbv[e], na_i + nbv[e]);
                            }
                        } else {
#pragma unroll
                            for (int k = 0; k < 16; ++k) d[k] = __uint_as_float(vc[k]);  // d~ / 2
                        }
                        if constexpr (PASS == 1) {
                            if (DUMP && pid == 0 && rvalid) {
#pragma unroll
                                for (int k = 0; k < 16; ++k)
                                    if (j0 + k < pm.nb) g.dump[(size_t)i * pm.nb + j0 + k] = kDom * d[k];
                            }
                            const float cm = min16(d);
                            // FP8 only: the bf16 bound is too tight for rows to go wide
                            // (the overflow count after pass 2 still routes such pairs)
                            if constexpr (FP8) near += (cm >= m1 && cm <= m1 + w2) ? 1u : 0u;
                            m2 = fminf(m2, fmaxf(m1, cm));
                            m1 = fminf(m1, cm);

                            float4 *cp = reinterpret_cast<float4 *>(&S.colpart[tb][combo][cb]);
#pragma unroll
                            for (int k4 = 0; k4 < 4; ++k4) {
                                float4 o;
                                o.x = warp_min_f32(d[4 * k4 + 0]);
                                o.y = warp_min_f32(d[4 * k4 + 1]);
                                o.z = warp_min_f32(d[4 * k4 + 2]);
                                o.w = warp_min_f32(d[4 * k4 + 3]);
                                if (lane == 0) cp[k4] = o;
                            }
                        } else {
                            // both tests' group minima first (independent chains), then
                            // the rare bodies. Row candidates: d~ <= T (rows certain to
                            // have no match carry T = -inf); column window: d~ <= c1 + 2 eps,
                            // x = d - thr in the accumulator domain (the sign is exact)
                            float x[16];
#pragma unroll
                            for (int k4 = 0; k4 < 4; ++k4) {
                                u64x x0, x1;
                                if constexpr (FP8) {
                                    x0 = f2_sub(f2_pack(d[4 * k4], d[4 * k4 + 1]), tt[k4].x);
                                    x1 = f2_sub(f2_pack(d[4 * k4 + 2], d[4 * k4 + 3]), tt[k4].y);
                                } else {
                                    const u64x mhalf = f2_pack(-0.5f, -0.5f);
                                    x0 = f2_fma(tt[k4].x, mhalf, f2_pack(d[4 * k4], d[4 * k4 + 1]));
                                    x1 = f2_fma(tt[k4].y, mhalf, f2_pack(d[4 * k4 + 2], d[4 * k4 + 3]));
                                }
                                x[4 * k4 + 0] = f2_lo(x0);
                                x[4 * k4 + 1] = f2_hi(x0);
                                x[4 * k4 + 2] = f2_lo(x1);
                                x[4 * k4 + 3] = f2_hi(x1);
                            }
                            float gr[4], gc[4];
                            const float cm = min16q(d, gr);
                            const float xm = rvalid ? min16q(x, gc) : kInf;
                            if (cm <= thr_i) {
                                // a hit group: one record of its 4 values (accumulator domain)
#pragma unroll
                                for (int qq = 0; qq < 4; ++qq) {
                                    if (gr[qq] <= thr_i) {
                                        // past the capacity the store is predicated off (no access)
                                        st_rec_if(g.rowrec + (rec0 + ncand), g.rowrecj + (rec0 + ncand), d[4 * qq],
                                                  d[4 * qq + 1], d[4 * qq + 2], d[4 * qq + 3], j0 + 4 * qq,
                                                  ncand < hr);
                                        ++ncand;
                                    }
                                }
                            }
                            if (xm <= 0.f) {
                                float *cc = g.colcnt + sp.cbase + j0;
#pragma unroll
                                for (int qq = 0; qq < 4; ++qq)
                                    red_add4_le0(cc + 4 * qq, x[4 * qq], x[4 * qq + 1], x[4 * qq + 2], x[4 * qq + 3],
                                                 gc[qq] <= 0.f);
                            }
                        }
                    };
                    // one chunk of 16 columns per TMEM load, one copy of the body: the
                    // epilogue is bound by its instruction stream (measured: a second
                    // copy of the body to overlap the next load with this chunk, or
                    // four loads in flight, ran slower), and the other epilogue warps
                    // of the sub-partition cover the load's latency
                    const ulonglong2 *bt2 = reinterpret_cast<const ulonglong2 *>(
                        two && at == 1 ? &S.bthr2[st][h * 64] : &S.bthr[st][h * 64]);
                    // chunks of this tile's column half holding columns of the pair
                    // (warp-uniform; the rest are padding): a loop bound, not a test per chunk
                    const uint32_t jt = t * kTile + h * 64;
                    const int nc = jt >= pm.nb ? 0 : (int)min(4u, (pm.nb - jt + 15) / 16);
#pragma unroll 1
                    for (int c = 0; c < nc; ++c) {
                        ulonglong2 tt[4];  // pass 2: the chunk's column thresholds, read before the wait
                        if constexpr (PASS == 2) {
#pragma unroll
                            for (int k4 = 0; k4 < 4; ++k4) tt[k4] = bt2[c * 4 + k4];
                        }
                        uint32_t v[16];
                        tmem_ld16(tcol + c * 16, v);
                        tmem_wait_ld16(v);
                        chunk(v, c, tt);
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&S.t_empty[tb]);
                if constexpr (PASS == 1) {
                    // all 16 epilogue warps have stored their column partials of this tile
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&S.ep_bar);
                    if (!sl_wait(&S.ep_bar, eph, abort_flag, err)) {
                        ok = false;
                        break;
                    }
                    eph ^= 1;
                    // one thread per column and pair of the item: the minimum over
                    // the (a tile, lane quarter) partials of that pair. The 8 epilogue
                    // warps on SM sub-partitions 2 and 3 do it (e = 0..255); 0 and 1
                    // also host the producer and MMA warps
                    const int wq = warp & 3;
                    const int e = wq >= 2 ? ((((warp - 2) >> 2) * 2 + (wq - 2)) * 32 + lane) : 512;
                    const int grp = e >> 7;
                    if (e < (two ? 256 : 128)) {
                        const int col = e & 127;
                        float m = kInf;
#pragma unroll
                        for (int cmb = 0; cmb < 8; ++cmb) {
                            const int ca = cmb >> 2;  // a tile of the partial
                            const uint32_t rt_c = ca ? item.rt[1] : item.rt[0];
                            const uint32_t na_c = ca ? na1 : na0;
                            if (ca < (int)item.nat && (!two || ca == grp) &&
                                rt_c * kTile + (cmb & 3) * 32 < na_c)  // quarter has rows
                                m = fminf(m, S.colpart[tb][cmb][col]);
                        }
                        const uint32_t j = t * kTile + col;
                        if (j < pm.nb && m < kInf && (grp ? on1 : on0))
                            atomicMin(&g.colmin[(grp ? cb1 : cb0) + j], f2ord(kDom * m));
                    }
                }
                __syncwarp();
                if (kEpReadsB && lane == 0) mbar_arrive(&S.b_empty[st]);
                if (++st == kStg) st = 0, sph ^= 1;
                tb ^= 1;
                if (tb == 0) tph ^= 1;
            }
            if (!ok) break;
            if constexpr (PASS == 1) {
                // merge the two column halves of each row, then store the partial
                if (h == 1 && active) {
                    S.rowx[r] = make_float2(m1, m2);
                    S.rownear[r] = near;
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(&S.ep_bar);
                if (!sl_wait(&S.ep_bar, eph, abort_flag, err)) break;
                eph ^= 1;
                if (h == 0 && active) {
                    const float2 o = S.rowx[r];
                    m2 = fminf(fminf(m2, o.y), fmaxf(m1, o.x));
                    m1 = fminf(m1, o.x);
                    // slot = row within its 256-row group (items of one 128-row tile start mid-group)
                    const size_t slot = (size_t)mypart * 256 + (i & 255u);
                    g.rowpart[slot] = make_float2(kDom * m1, kDom * m2);
                    g.rownear[slot] = near + S.rownear[r];
                }
            } else {
                if (rvalid && thr_i > -kInf) {
                    g.rowcnt[2 * crow + h] = ncand;
                    // a wide shortlist (more than half the records): the pair's bound may be
                    // too loose for its distances (routing estimate of finalize)
                    if (ncand > hr / 2) atomicAdd(&g.pairctl[4 * (size_t)pid + kPcOver], 1u);
                }
            }
        }
    }
    // Everyone done: no MMA in flight (the epilogue consumed every commit).
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, 512);
    }
}

// ------------------------------------------------------------------ eps

// Per pair, before pass 1: the error bound eps from the two views'
// statistics. A pair with non-finite or huge inputs cannot be certified and is
// routed to the exact kernel.
// The per-pair error bound of this launch's precision (g.fp8) from the two
// views' statistics; false when the pair cannot be certified (non-finite or
// huge inputs).
SLM_DEV bool pair_eps(const SlArgs &g, const SlPair &sp, float *eps_out) {
    const ViewStat va = g.vstats[sp.view_a], vb = g.vstats[sp.view_b];
    const double A = __uint_as_float(va.nmax), B = __uint_as_float(vb.nmax);
    const double Ra = __uint_as_float(va.rho), Rb = __uint_as_float(vb.rho);
    const double Qa = __uint_as_float(va.nqmax), Qb = __uint_as_float(vb.nqmax);
    bool unsafe = va.bad || vb.bad || !(A <= 64.0) || !(B <= 64.0);
    // |d~ - d| <= 2 |a.b - q(a).q(b)| + accumulation and rounding terms, with
    // |a.b - q(a).q(b)| <= |a - q(a)| |b| + |q(a)| |b - q(b)| (Cauchy-Schwarz).
    double eps = 2.0 * (Ra * B + Qa * Rb) * (1.0 + 1e-3);
    eps += 5e-4 * Qa * Qb + 5e-5 * (A * A + B * B) + 2e-5 * (A + B) * (A + B) + 1e-6;
    // BF16: the tensor core also accumulates the folded norms (|a|^2 + |b|^2) / 2
    // and their bf16 split (relative 2^-17); the accumulation is taken as no
    // better than 2^-11 relative to that magnitude, doubled with d~
    if (!g.fp8) eps += 5e-4 * (A * A + B * B);
    if (!(eps < 1e30)) unsafe = true;
    *eps_out = unsafe ? __int_as_float(0x7f800000) : (float)(eps * (1.0 + 1e-6));
    return !unsafe;
}

__global__ void __launch_bounds__(256) sl_eps_kernel(SlArgs g) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= g.npairs) return;
    const PairMeta pm = g.pairs[p];
    SlPair &sp = g.spairs[p];
    float eps;
    const bool unsafe = !pair_eps(g, sp, &eps);
    sp.eps = eps;
    sp.unsafe = unsafe ? 1u : 0u;
    sp.routed = (unsafe && pm.na && pm.nb) ? 1u : 0u;
    sp.rescued = 0;
    if (sp.routed) atomicAdd(&g.ctl[kCtlRouteMarks], 1u);
}

// Tier 1 (the BF16 rescue of an FP8 plan), one CTA per pair and block of
// kSlRowBlock columns: for each rescued pair, the BF16 bound (block 0), its
// column minima back to +inf and its per-pair counters back to 0 (tier 0's
// pass 1 and mid wrote them; its pass 2 skipped the pair, so the records and
// window counts are still clear).
__global__ void __launch_bounds__(256) sl_rescue_prep_kernel(SlArgs g) {
    const uint32_t p = blockIdx.x, blk = blockIdx.y;
    const PairMeta pm = g.pairs[p];
    const SlPair sp = g.spairs[p];
    if (!sl_pair_on(g, sp)) return;  // block-uniform
    const uint32_t nb_pad = (pm.nb + kTile - 1) / kTile * kTile;
    const uint32_t c0 = blk * kSlRowBlock, c1 = min(c0 + kSlRowBlock, nb_pad);
    for (uint32_t j = c0 + threadIdx.x; j < c1; j += blockDim.x) g.colmin[sp.cbase + j] = 0xff800000u;  // +inf
    if (blk == 0 && threadIdx.x < 4) g.pairctl[4 * (size_t)p + threadIdx.x] = 0;
    if (blk == 0 && threadIdx.x == 0) {
        float eps;
        if (!pair_eps(g, sp, &eps)) {  // cannot happen after tier 0 (unsafe pairs are routed there)
            g.spairs[p].routed = 1;
            atomicAdd(&g.ctl[kCtlRouteMarks], 1u);
        }
        g.spairs[p].eps = eps;
        atomicAdd(&g.ctl[kCtlRescuedPairs], 1u);
        atomicAdd(&g.ctl[kCtlRescuedRows], pm.na);
    }
}

// ------------------------------------------------------- certified tests

// The decisions below are proved in f32 with directed rounding: each side of
// a comparison is rounded toward the weaker claim, so a true comparison of the
// rounded values implies it for the real numbers. The factors cover the
// reference's own rounding of (r*r)*d2 (at most 2^-24 relative).
constexpr float kUp = 1.000001f;    // > 1 + 2^-24
constexpr float kDown = 0.999999f;  // < 1 - 2^-24

// No match for the row: d1 >= m1 - eps >= r^2 (m2 + eps) kUp >= fl(r^2 d2),
// where m1 - eps bounds d1 from below and m2 + eps bounds d2 from above.
SLM_DEV bool certain_no_match(float m1, float m2, float eps, float r2) {
    return __fsub_rd(m1, eps) >= __fmul_ru(__fmul_ru(r2, __fadd_ru(m2, eps)), kUp);
}

// The ratio test passes: d1 <= a1 + eps < r^2 (a2 - eps) kDown <= fl(r^2 d2).
SLM_DEV bool certain_ratio_pass(float a1, float a2, float eps, float r2) {
    return __fadd_ru(a1, eps) < __fmul_rd(__fmul_rd(r2, __fsub_rd(a2, eps)), kDown);
}

// Window x + 2 eps, rounded up (a larger threshold only admits more); NaN
// becomes +inf (admit everything).
SLM_DEV float window_up(float x, float eps) {
    const float t = __fmul_ru(__fadd_ru(x, 2.f * eps), kUp);
    return t == t ? t : __int_as_float(0x7f800000);
}

// ------------------------------------------------------------------ mid

// Row blocks of a pair: enough for its rows and its columns.
SLM_DEV uint32_t pair_blocks(const PairMeta &pm) {
    const uint32_t n = max(pm.na, pm.nb);
    return max(1u, (n + kSlRowBlock - 1) / kSlRowBlock);
}

// One CTA per pair and block of kSlRowBlock rows and columns: row thresholds
// from the pass-1 partials, column thresholds from the column minima, and the
// near-chunk counts; the last CTA of a pair to finish makes the routing
// decision from the pair's totals.
// kThreads: 256 for batches of many pairs, 1024 for a few (see kFewPairs);
// the bound sets the register budget the compiler schedules for.
template <int kThreads>
__global__ void __launch_bounds__(kThreads) sl_mid_kernel(SlArgs g) {
    __shared__ uint32_t wide_sh, open_sh, last_sh;
    const uint32_t p = blockIdx.x, blk = blockIdx.y;
    const PairMeta pm = g.pairs[p];
    const SlPair sp = g.spairs[p];
    const uint32_t nblk = pair_blocks(pm);
    if (!sl_pair_on(g, sp) || blk >= nblk) return;  // block-uniform
    const float kInf = __int_as_float(0x7f800000);
    if (threadIdx.x == 0) wide_sh = open_sh = 0;
    __syncthreads();
    const float eps = sp.eps;
    const uint32_t na_pad = (pm.na + kTile - 1) / kTile * kTile;
    // a row is "wide" when more than half of its 16-column chunks (and more
    // than the list capacity) came within 2 eps of the running minimum: the
    // bound is then as wide as the spread of the row's distances, and its
    // shortlist overflows. (Each column range of pass 1 restarts the running
    // minimum, so a fixed count alone would misjudge rows split into many.)
    const uint32_t wide_min = max((uint32_t)kSlRowSlots, (pm.nb + 15) / 16 / 2);
    uint32_t wide = 0, open = 0;
    const uint32_t r0 = blk * kSlRowBlock, r1 = min(r0 + kSlRowBlock, na_pad);
    for (uint32_t i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        float thr = -kInf;
        if (i < pm.na && pm.nb > 0) {
            const uint32_t super = i / 256, r = i % 256;
            float m1 = kInf, m2 = kInf;
            uint32_t near = 0;
            // the column ranges' partials: one load per step in batches of many
            // pairs (mostly one range per row); four independent loads per step
            // for a few pairs split into many ranges (an absent range merges as
            // (inf, inf), near 0)
            const size_t slot0 = (size_t)(sp.part_base + super * sp.nchunk) * 256 + r;
            if constexpr (kThreads == 256) {
                for (uint32_t c = 0; c < sp.nchunk; ++c) {
                    const float2 v = g.rowpart[slot0 + (size_t)c * 256];
                    near += g.rownear[slot0 + (size_t)c * 256];
                    m2 = fminf(fminf(m2, v.y), fmaxf(m1, v.x));
                    m1 = fminf(m1, v.x);
                }
            } else
            for (uint32_t c0 = 0; c0 < sp.nchunk; c0 += 4) {
                float2 v[4];
                uint32_t nr[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    v[u] = make_float2(kInf, kInf);
                    nr[u] = 0;
                    if (c0 + u < sp.nchunk) {
                        v[u] = g.rowpart[slot0 + (size_t)(c0 + u) * 256];
                        nr[u] = g.rownear[slot0 + (size_t)(c0 + u) * 256];
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    near += nr[u];
                    m2 = fminf(fminf(m2, v[u].y), fmaxf(m1, v[u].x));
                    m1 = fminf(m1, v[u].x);
                }
            }
            // m2' bounds the second smallest d~ from above
            if (!certain_no_match(m1, m2, eps, g.ratio2)) {
                thr = window_up(m2, eps);
                ++open;
                wide += near > wide_min ? 1u : 0u;
            }
        }
        g.rowthr[sp.rbase + i] = thr;
    }
    const uint32_t nb_pad = (pm.nb + kTile - 1) / kTile * kTile;
    const uint32_t c0 = blk * kSlRowBlock, c1 = min(c0 + kSlRowBlock, nb_pad);
    for (uint32_t j = c0 + threadIdx.x; j < c1; j += blockDim.x) {
        float thr = -kInf;
        if (j < pm.nb) thr = window_up(ord2f(g.colmin[sp.cbase + j]), eps);
        g.colthr[sp.cbase + j] = thr;
    }
    if (wide) atomicAdd(&wide_sh, wide);
    if (open) atomicAdd(&open_sh, open);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t *pc = g.pairctl + 4 * (size_t)p;
        if (wide_sh) atomicAdd(&pc[kPcWide], wide_sh);
        if (open_sh) atomicAdd(&pc[kPcOpen], open_sh);
        __threadfence();
        last_sh = atomicAdd(&pc[kPcMidDone], 1u) == nblk - 1;
    }
    __syncthreads();
    if (last_sh && threadIdx.x == 0) {
        __threadfence();
        const uint32_t *pc = g.pairctl + 4 * (size_t)p;
        const uint32_t w = atomicAdd(const_cast<uint32_t *>(&pc[kPcWide]), 0u);
        const uint32_t o = atomicAdd(const_cast<uint32_t *>(&pc[kPcOpen]), 0u);
        // more than 1/8 of the undecided rows are expected to overflow their
        // shortlist: settle the whole pair with the BF16 passes (tier 0 of an
        // FP8 plan) or with the exact kernel
        if (w * 8 > o && o) {
            if (g.rescue) {
                g.spairs[p].rescued = 1;
            } else {
                g.spairs[p].routed = 1;
                atomicAdd(&g.ctl[kCtlRouteMarks], 1u);
            }
        }
    }
}

// ------------------------------------------------------------- finalize

SLM_DEV void sl_push(SlQueue *q, uint32_t *len, uint32_t cap, uint32_t *err, uint32_t pair, uint32_t kind, uint32_t i,
                     uint32_t j) {
    const uint32_t s = atomicAdd(len, 1u);
    if (s < cap) {
        SlQueue e;
        e.pair = pair;
        e.kind = kind;
        e.i = i;
        e.j = j;
        q[s] = e;
    } else {
        atomicCAS(err, 0u, (uint32_t)DERR_BAD_ITEM);
    }
}

SLM_DEV void push_scan(const SlArgs &g, uint32_t pair, uint32_t kind, uint32_t i, uint32_t j) {
    sl_push(g.queue, &g.ctl[kCtlScanLen], g.queue_cap, g.ctl + 1, pair, kind, i, j);
    atomicAdd(&g.ctl[kind == 0 ? kCtlQueueRows : kCtlQueueCols], 1u);
}

// Mutual check of a candidate (i, j) from the column window counts: a row
// whose d~ lies above the window (c1 + 2 eps) is provably not the column's
// nearest; the only row inside it provably is. Returns the decision or
// kDecPending after queueing an exact column check.
SLM_DEV uint32_t mutual_from_counts(const SlArgs &g, uint32_t p, const SlPair &sp, uint32_t i, uint32_t j, float dij) {
    const uint32_t cidx = sp.cbase + j;
    if (!(dij <= g.colthr[cidx])) return kDecNone;
    if (g.colcnt[cidx] == 1.f) return j;
    push_scan(g, p, 1, i, j);
    return kDecPending;
}

// One thread per row (CTA per pair and row block): decide from the bounds, or
// queue exact work. A pair with more than 1/8 as many wide row halves
// (counted by pass 2) as rows is routed to the exact kernel instead (exact
// rescoring of long shortlists or scans per row would cost more).
template <int kThreads>
__global__ void __launch_bounds__(kThreads, 1) sl_finalize_kernel(SlArgs g) {
    const uint32_t p = blockIdx.x, blk = blockIdx.y;
    const PairMeta pm = g.pairs[p];
    const SlPair sp = g.spairs[p];
    // block-uniform: route_finalize decides routed pairs' rows, the other tier its own pairs'
    if (!sl_pair_on(g, sp) || blk * kSlRowBlock >= pm.na) return;
    const float kInf = __int_as_float(0x7f800000);
    const float eps = sp.eps;
    // every CTA of the pair reads the same total (written by the previous kernel)
    if (g.pairctl[4 * (size_t)p + kPcOver] * 8 > pm.na) {
        if (blk == 0 && threadIdx.x == 0) {
            g.spairs[p].routed = 1;
            atomicAdd(&g.ctl[kCtlRouteMarks], 1u);
        }
        return;
    }
    const uint32_t r1 = min(blk * kSlRowBlock + kSlRowBlock, pm.na);
    for (uint32_t i = blk * kSlRowBlock + threadIdx.x; i < r1; i += blockDim.x) {
        const uint32_t ridx = sp.rbase + i;
        uint32_t dec = kDecNone;
        if (g.rowthr[ridx] > -kInf) {
            // the row's records: two column halves per column range of the pair.
            // S = the records' columns with d~ <= T (values above T, and the NaN of
            // padding columns, are not in S); a half with more hit groups than
            // records overflowed and the row is scanned exactly instead
            const float T = g.rowthr[ridx];
            const float dom = g.fp8 ? 1.f : 2.f;
            float a1 = kInf, a2 = kInf;
            uint32_t j1 = 0xffffffffu, n = 0;
            bool over = false;
            for (uint32_t l = 0; l < 2 * sp.nchunk; ++l) {
                const uint32_t cr = sl_cand_row(sp, pm.na, l >> 1, i);
                const uint32_t nl = g.rowcnt[2 * cr + (l & 1)];
                over |= nl > g.half_recs;
                const uint32_t b0 = (2 * cr + (l & 1)) * g.half_recs;
                // two records per step, loaded before they are used
                for (uint32_t r = 0; r < nl && r < g.half_recs; r += 2) {
                    const bool two = r + 1 < nl && r + 1 < g.half_recs;
                    const float4 v0 = g.rowrec[b0 + r];
                    const uint32_t jb0 = g.rowrecj[b0 + r];
                    const float4 v1 = two ? g.rowrec[b0 + r + 1] : make_float4(kInf, kInf, kInf, kInf);
                    const uint32_t jb1 = two ? g.rowrecj[b0 + r + 1] : 0u;
                    const float vs[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const float v = dom * vs[q];
                        const uint32_t j = (q < 4 ? jb0 : jb1) + (q & 3);
                        if (!(v <= T)) continue;
                        ++n;
                        if (v < a1 || (v == a1 && j < j1)) {
                            a2 = a1;
                            a1 = v;
                            j1 = j;
                        } else if (v < a2) {
                            a2 = v;
                        }
                    }
                }
            }
            if (over) {
                push_scan(g, p, 0, i, 0);
                dec = kDecPending;
            } else {
                // S holds every column with d~ <= T, T >= (second smallest d~) + 2 eps,
                // so the exact two smallest distances are among S. With fewer than
                // two finite entries the exact second best is infinite
                // (matching.rs:205: no match).
                const bool no_match = n < 2 || !(a2 < kInf) || certain_no_match(a1, a2, eps, g.ratio2);
                // and the argmin is unique: a2 - a1 > 2 eps
                const bool sure = !no_match && certain_ratio_pass(a1, a2, eps, g.ratio2) &&
                                  __fsub_rd(a2, a1) > 2.f * eps;
                if (sure) {
                    dec = g.mutual ? mutual_from_counts(g, p, sp, i, j1, a1) : j1;
                } else if (!no_match) {
                    sl_push(g.rqueue, &g.ctl[kCtlRescoreLen], g.queue_cap, g.ctl + 1, p, 2, i, 0);
                    dec = kDecPending;
                }
            }
        }
        g.rowdec[ridx] = dec;
    }
}

// ------------------------------------------------------------- exact work

// Exact distance by 8 lanes: lane k of the group accumulates components
// 8c+k for c = 0..15 (matching.rs:146-155), then the lane sums are added in
// order 0..7. p and r may differ per group; the result is valid in all 8 lanes.
SLM_DEV float dist8(const float *__restrict__ p, const float *__restrict__ r) {
    const uint32_t lane = threadIdx.x & 31, k = lane & 7, base = lane & ~7u;
    float acc = 0.f;
#pragma unroll
    for (int c = 0; c < 16; ++c) {
        const float t = __fsub_rn(p[8 * c + k], r[8 * c + k]);
        acc = __fadd_rn(acc, __fmul_rn(t, t));
    }
    float s = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) s = __fadd_rn(s, __shfl_sync(0xffffffffu, acc, base + q));
    return s;
}

// One warp per row of the rescore queue: exact distances of S (4 at a time),
// the reference's row rule (matching.rs:182-187, 204-206), then the mutual
// check from the column window counts.
__global__ void __launch_bounds__(256) sl_rescore_kernel(SlArgs g) {
    const uint32_t lane = threadIdx.x & 31, grp = lane >> 3;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t qn = min(g.ctl[kCtlRescoreLen], g.queue_cap);
    const float kInf = __int_as_float(0x7f800000);
    uint32_t w_rows = 0;  // statistics of this warp's rows, added once at the end
    float w_err = 0.f;
    for (uint32_t e = gw; e < qn; e += nw) {
        const SlQueue qe = g.rqueue[e];
        const PairMeta pm = g.pairs[qe.pair];
        const SlPair sp = g.spairs[qe.pair];
        const uint32_t ridx = sp.rbase + qe.i;
        const float *a = g.raw + (size_t)(pm.a_row0 + qe.i) * kDesc;
        const float *B = g.raw + (size_t)pm.b_row0 * kDesc;
        float e1 = kInf, e2 = kInf, ad = kInf, maxerr = 0.f;
        uint32_t ej = 0xffffffffu;
        // S = the records' columns with d~ <= T, four entries at a time: lane group
        // grp computes queued entry grp, every lane merges the results in order
        const float T = g.rowthr[ridx];
        // records of FP8 pairs hold d~, those of BF16 (and rescued) pairs d~ / 2
        const float dom = g.fp8 && !sp.rescued ? 1.f : 2.f;
        uint32_t qj = 0, nq = 0;  // this lane group's queued column (0: a valid placeholder)
        float qv = kInf;
        auto flush = [&](uint32_t cnt) {
            const float d = dist8(a, B + (size_t)qj * kDesc);
#pragma unroll
            for (uint32_t q = 0; q < 4; ++q) {
                const float dq = __shfl_sync(0xffffffffu, d, q * 8);
                const uint32_t jq = __shfl_sync(0xffffffffu, qj, q * 8);
                const float approx = __shfl_sync(0xffffffffu, qv, q * 8);
                if (q < cnt) {
                    maxerr = fmaxf(maxerr, fabsf(dq - approx));
                    if (dq < e1 || (dq == e1 && jq < ej)) {
                        e2 = e1;
                        e1 = dq;
                        ej = jq;
                        ad = approx;
                    } else if (dq < e2) {
                        e2 = dq;
                    }
                }
            }
        };
        for (uint32_t l = 0; l < 2 * sp.nchunk; ++l) {
            const uint32_t cr = sl_cand_row(sp, pm.na, l >> 1, qe.i);
            const uint32_t nl = g.rowcnt[2 * cr + (l & 1)];
            const uint32_t b0 = (2 * cr + (l & 1)) * g.half_recs;
            for (uint32_t r = 0; r < nl; ++r) {
                const float4 v4 = g.rowrec[b0 + r];
                const uint32_t jb = g.rowrecj[b0 + r];
                const float vs[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
                for (uint32_t q = 0; q < 4; ++q) {
                    const float v = dom * vs[q];
                    if (!(v <= T)) continue;  // warp-uniform: every lane reads the same record
                    if (grp == nq) {
                        qj = jb + q;
                        qv = v;
                    }
                    if (++nq == 4) {
                        flush(4);
                        nq = 0;
                    }
                }
            }
        }
        if (nq) flush(nq);
        if (lane == 0) {
            ++w_rows;
            if (maxerr == maxerr) w_err = fmaxf(w_err, maxerr);
            uint32_t dec = kDecNone;
            if (ej != 0xffffffffu && e2 < kInf && !(e1 >= __fmul_rn(g.ratio2, e2)))
                dec = g.mutual ? mutual_from_counts(g, qe.pair, sp, qe.i, ej, ad) : ej;
            g.rowdec[ridx] = dec;
        }
    }
    if (lane == 0 && w_rows) {
        atomicAdd(&g.ctl[kCtlRescored], w_rows);
        atomicMax(&g.ctl[kCtlMaxErr], __float_as_uint(w_err));  // non-negative: bits order as values
    }
}

// Block-wide (d, index) minimum with the lowest index on ties; all threads
// get the result.
SLM_DEV void block_argmin(float &d, uint32_t &idx, float *sd, uint32_t *si) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float od = __shfl_xor_sync(0xffffffffu, d, o);
        const uint32_t oi = __shfl_xor_sync(0xffffffffu, idx, o);
        if (od < d || (od == d && oi < idx)) {
            d = od;
            idx = oi;
        }
    }
    const int w = threadIdx.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        sd[w] = d;
        si[w] = idx;
    }
    __syncthreads();
    d = sd[0];
    idx = si[0];
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q)
        if (sd[q] < d || (sd[q] == d && si[q] < idx)) {
            d = sd[q];
            idx = si[q];
        }
}

// One CTA per entry of the scan queue: exact full scans, 32 distances at a
// time (8 lanes each).
__global__ void __launch_bounds__(256) sl_scan_kernel(SlArgs g) {
    __shared__ float sd[8], s2[8];
    __shared__ uint32_t si[8];
    const uint32_t lane = threadIdx.x & 31, grp = threadIdx.x >> 3;  // 32 groups of 8 lanes
    const uint32_t qn = min(g.ctl[kCtlScanLen], g.queue_cap);
    const float kInf = __int_as_float(0x7f800000);
    for (uint32_t e = blockIdx.x; e < qn; e += gridDim.x) {
        const SlQueue qe = g.queue[e];
        const PairMeta pm = g.pairs[qe.pair];
        const SlPair sp = g.spairs[qe.pair];
        const float *A = g.raw + (size_t)pm.a_row0 * kDesc;
        const float *B = g.raw + (size_t)pm.b_row0 * kDesc;
        uint32_t dec = kDecNone, col = qe.j;
        bool check_col = qe.kind == 1;
        if (qe.kind == 0) {
            float d1 = kInf, d2 = kInf;
            uint32_t j1 = 0xffffffffu;
            for (uint32_t j0 = 0; j0 < pm.nb; j0 += 32) {
                const uint32_t j = j0 + grp;
                const float d = dist8(A + (size_t)qe.i * kDesc, B + (size_t)(j < pm.nb ? j : 0) * kDesc);
                if (j < pm.nb) {
                    if (d < d1) {
                        d2 = d1;
                        d1 = d;
                        j1 = j;
                    } else if (d < d2) {
                        d2 = d;
                    }
                }
            }
            // merge (d1, j1, d2) across the 32 groups (lanes within a group agree)
            float m2 = d2;
            float b1 = d1;
            uint32_t bj = j1;
#pragma unroll
            for (int o = 8; o < 32; o <<= 1) {
                const float o1 = __shfl_xor_sync(0xffffffffu, b1, o);
                const float o2 = __shfl_xor_sync(0xffffffffu, m2, o);
                const uint32_t oj = __shfl_xor_sync(0xffffffffu, bj, o);
                const float n2 = fminf(fminf(m2, o2), fmaxf(b1, o1));
                if (o1 < b1 || (o1 == b1 && oj < bj)) {
                    b1 = o1;
                    bj = oj;
                }
                m2 = n2;
            }
            const int w = threadIdx.x >> 5;
            __syncthreads();
            if (lane == 0) {
                sd[w] = b1;
                s2[w] = m2;
                si[w] = bj;
            }
            __syncthreads();
            b1 = sd[0];
            m2 = s2[0];
            bj = si[0];
            for (int q = 1; q < 8; ++q) {
                const float n2 = fminf(fminf(m2, s2[q]), fmaxf(b1, sd[q]));
                if (sd[q] < b1 || (sd[q] == b1 && si[q] < bj)) {
                    b1 = sd[q];
                    bj = si[q];
                }
                m2 = n2;
            }
            if (bj != 0xffffffffu && m2 < kInf && !(b1 >= __fmul_rn(g.ratio2, m2))) {
                if (g.mutual) {
                    check_col = true;
                    col = bj;
                } else {
                    dec = bj;
                }
            }
        }
        if (check_col) {
            float bd = kInf;
            uint32_t bi = 0xffffffffu;
            for (uint32_t r0 = 0; r0 < pm.na; r0 += 32) {
                const uint32_t r = r0 + grp;
                const float d = dist8(A + (size_t)(r < pm.na ? r : 0) * kDesc, B + (size_t)col * kDesc);
                if (r < pm.na && (d < bd || (d == bd && r < bi))) {
                    bd = d;
                    bi = r;
                }
            }
            block_argmin(bd, bi, sd, si);
            dec = bi == qe.i ? col : kDecNone;
        }
        if (threadIdx.x == 0) g.rowdec[sp.rbase + qe.i] = dec;
        __syncthreads();
    }
}

// -------------------------------------------------------------- routing

// Exclusive scan over the 1024 threads of a block; returns this thread's
// prefix and writes the block total.
SLM_DEV uint32_t block_scan_1024(uint32_t v, uint32_t *sh, uint32_t &total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __syncthreads();
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t t = sh[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        sh[lane] = t;  // inclusive over warps
    }
    __syncthreads();
    total = sh[31];
    return (w ? sh[w - 1] : 0u) + x - v;
}

// One CTA of 1024 threads: plans the exact work of the routed pairs. Column
// chunks per row tile are chosen over all routed pairs together, as the
// FP32 batch plan does: enough items to fill the GPU, at most kXChunkMax.
// Writes each routed pair's first item and chunk count, the list of routed
// pairs and the counters.
__global__ void __launch_bounds__(1024) sl_route_plan_kernel(SlArgs g) {
    __shared__ uint32_t sh[32];
    __shared__ uint32_t carry_items, carry_list;
    if (g.ctl[kCtlRouteMarks] == 0) return;  // nothing routed: the counters stay 0
    uint32_t rt = 0, rows = 0, cols = 0, total = 0;
    for (uint32_t p = threadIdx.x; p < g.npairs; p += blockDim.x)
        if (g.spairs[p].routed) {
            const PairMeta pm = g.pairs[p];
            rt += (pm.na + kTile - 1) / kTile;
            rows += pm.na;
            cols += pm.nb;
        }
    block_scan_1024(rt, sh, total);
    const uint32_t rt_total = total;
    block_scan_1024(rows, sh, total);
    const uint32_t rows_total = total;
    block_scan_1024(cols, sh, total);
    const uint32_t cols_total = total;
    uint32_t split = 1;
    if (rt_total && rt_total < g.want_items) split = (g.want_items + rt_total - 1) / rt_total;
    split = min(split, kXChunkMax);
    if (threadIdx.x == 0) carry_items = carry_list = 0;
    __syncthreads();
    for (uint32_t base = 0; base < g.npairs; base += blockDim.x) {
        const uint32_t p = base + threadIdx.x;
        uint32_t routed = 0, n = 0, chunks = 0;
        if (p < g.npairs && g.spairs[p].routed) {
            const PairMeta pm = g.pairs[p];
            const uint32_t rt_n = (pm.na + kTile - 1) / kTile, ct_n = (pm.nb + kTile - 1) / kTile;
            routed = 1;
            chunks = max(1u, min(split, ct_n));
            n = rt_n * chunks;
        }
        uint32_t t_items = 0, t_list = 0;
        const uint32_t off = block_scan_1024(n, sh, t_items);
        const uint32_t idx = block_scan_1024(routed, sh, t_list);
        const uint32_t ci = carry_items, cl = carry_list;
        if (routed) {
            g.spairs[p].xpart = ci + off;
            g.spairs[p].xchunk = chunks;
            g.xlist[cl + idx] = p;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            carry_items = ci + t_items;
            carry_list = cl + t_list;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        uint32_t items = carry_items;
        if (items > g.xitem_cap) {  // cannot happen with the plan's capacity
            atomicCAS(g.ctl + 1, 0u, (uint32_t)DERR_BAD_ITEM);
            items = g.xitem_cap;
        }
        g.ctl[kCtlXItems] = items;
        g.ctl[kCtlRoutedPairs] = carry_list;
        g.ctl[kCtlRoutedRows] = rows_total;
        g.ctl[kCtlRoutedCols] = cols_total;
    }
}

// Writes the exact work items of the routed pairs and resets their column
// minima keys (one CTA per routed pair at a time).
__global__ void __launch_bounds__(256) sl_route_apply_kernel(SlArgs g) {
    const uint32_t n = g.ctl[kCtlRoutedPairs];
    for (uint32_t k = blockIdx.x; k < n; k += gridDim.x) {
        const uint32_t p = g.xlist[k];
        const PairMeta pm = g.pairs[p];
        const SlPair sp = g.spairs[p];
        const uint32_t rt_n = (pm.na + kTile - 1) / kTile, ct_n = (pm.nb + kTile - 1) / kTile;
        const uint32_t chunks = sp.xchunk, nit = rt_n * chunks;
        for (uint32_t t = threadIdx.x; t < nit; t += blockDim.x) {
            const uint32_t rt = t / chunks, c = t % chunks;
            Item it;
            it.pair = p;
            it.rt = rt;
            it.ct0 = (uint32_t)((uint64_t)ct_n * c / chunks);
            it.ct1 = (uint32_t)((uint64_t)ct_n * (c + 1) / chunks);
            it.part = sp.xpart + t;  // = xpart + rt * chunks + c
            it.pad[0] = it.pad[1] = it.pad[2] = 0;
            if (sp.xpart + t < g.xitem_cap) g.xitems[sp.xpart + t] = it;
        }
        if (g.mutual)
            for (uint32_t j = threadIdx.x; j < pm.nb; j += blockDim.x) g.colbest[pm.col_base + j] = ~0ull;
    }
}

// After exact_kernel: the routed pairs' row decisions, as finalize_kernel
// makes them (matching.rs:204-214), into rowdec.
__global__ void __launch_bounds__(256) sl_route_finalize_kernel(SlArgs g) {
    const uint32_t n = g.ctl[kCtlRoutedPairs];
    const float kInf = __int_as_float(0x7f800000);
    for (uint32_t k = blockIdx.x; k < n; k += gridDim.x) {
        const uint32_t p = g.xlist[k];
        const PairMeta pm = g.pairs[p];
        const SlPair sp = g.spairs[p];
        const uint32_t r1 = min(blockIdx.y * kSlRowBlock + kSlRowBlock, pm.na);  // this CTA's row block
        for (uint32_t i = blockIdx.y * kSlRowBlock + threadIdx.x; i < r1; i += blockDim.x) {
            const uint32_t rt = i / kTile;
            float d1 = kInf, d2 = kInf;
            uint32_t j1 = 0xffffffffu;
            for (uint32_t c = 0; c < sp.xchunk; ++c) {
                const uint32_t part = sp.xpart + rt * sp.xchunk + c;
                if (part < g.xitem_cap) merge_rowpart(g.xparts[(size_t)part * kTile + (i % kTile)], d1, d2, j1);
            }
            uint32_t dec = kDecNone;
            if (j1 != 0xffffffffu && d2 < kInf && !(d1 >= __fmul_rn(g.ratio2, d2)))
                if (!g.mutual || static_cast<uint32_t>(g.colbest[pm.col_base + j1]) == i) dec = j1;
            g.rowdec[sp.rbase + i] = dec;
        }
    }
}

// -------------------------------------------------------------- compact

// Matches of a pair's row block in ascending i, at the block's slot range
// (CTA per pair and row block); the block's count goes to blkcnt and the
// pair's total to counts.
__global__ void __launch_bounds__(256) sl_compact_kernel(SlArgs g) {
    __shared__ uint32_t warp_tot[8];
    const uint32_t p = blockIdx.x, blk = blockIdx.y;
    const PairMeta pm = g.pairs[p];
    const SlPair sp = g.spairs[p];
    const uint32_t r0 = blk * kSlRowBlock;
    if (r0 >= pm.na) return;  // block-uniform
    const uint32_t r1 = min(r0 + kSlRowBlock, pm.na);
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    uint32_t base = 0;
    for (uint32_t row0 = r0; row0 < r1; row0 += 256) {
        const uint32_t i = row0 + tid;
        uint32_t dec = kDecNone;
        if (i < r1) dec = g.rowdec[sp.rbase + i];
        if (dec == kDecPending) {
            atomicCAS(g.ctl + 1, 0u, (uint32_t)DERR_BAD_ITEM);
            dec = kDecNone;
        }
        const uint32_t flag = dec != kDecNone;
        const uint32_t ballot = __ballot_sync(0xffffffffu, flag);
        const uint32_t wpre = __popc(ballot & ((1u << lane) - 1u));
        if (lane == 0) warp_tot[wid] = __popc(ballot);
        __syncthreads();
        uint32_t off = 0, tot = 0;
        for (int w = 0; w < 8; ++w) {
            off += (w < wid) ? warp_tot[w] : 0;
            tot += warp_tot[w];
        }
        if (flag) g.slots[pm.slot_off + r0 + base + off + wpre] = make_uint2(i, dec);
        base += tot;
        __syncthreads();
    }
    if (tid == 0) {
        g.blkcnt[sp.blk + blk] = base;
        if (base) atomicAdd(&g.counts[p], base);
    }
}

// One CTA per pair: its row blocks' matches, in order, to the dense list.
__global__ void __launch_bounds__(256) sl_gather_kernel(SlArgs g, const uint64_t *__restrict__ slot_off,
                                                        const uint64_t *__restrict__ offsets, uint2 *__restrict__ dense,
                                                        uint64_t cap) {
    const uint32_t p = blockIdx.x;
    if (g.counts[p] == 0) return;  // no matches, or filtered out
    const uint32_t na = g.pairs[p].na, blk = g.spairs[p].blk;
    uint64_t dst = offsets[p];
    for (uint32_t b = 0; b * kSlRowBlock < na; ++b) {
        const uint32_t n = g.blkcnt[blk + b];
        const uint64_t src = slot_off[p] + (uint64_t)b * kSlRowBlock;
        for (uint32_t t = threadIdx.x; t < n; t += blockDim.x)
            if (dst + t < cap) dense[dst + t] = g.slots[src + t];
        dst += n;
    }
}

void launch_gather_blocks(const SlArgs &a, const uint64_t *slot_off, const uint64_t *offsets, uint2 *dense,
                          uint64_t cap, cudaStream_t s) {
    if (a.npairs) sl_gather_kernel<<<a.npairs, 256, 0, s>>>(a, slot_off, offsets, dense, cap);
}

// ---------------------------------------------------------------- launch

cudaError_t init_shortlist_kernels() {
    const int sb = (int)sl_smem_bytes<false>(), s8 = (int)sl_smem_bytes<true>();
    const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaFuncSetAttribute(sl_pass_kernel<1, false, false>, at, sb);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(sl_pass_kernel<1, false, true>, at, sb);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(sl_pass_kernel<2, false, false>, at, sb);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(sl_pass_kernel<1, true, false>, at, s8);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(sl_pass_kernel<1, true, true>, at, s8);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(sl_pass_kernel<2, true, false>, at, s8);
    return e;
}

int launch_shortlist_eps(const SlArgs &a, cudaStream_t s) {
    if (!a.npairs) return 0;
    sl_eps_kernel<<<(a.npairs + 255) / 256, 256, 0, s>>>(a);
    return 1;
}

int launch_shortlist_pass(const SlArgs &a, int pass, int sms, cudaStream_t s) {
    const int grid = (int)(a.n_items < (uint32_t)sms ? a.n_items : (uint32_t)sms);
    if (!grid) return 0;
    const size_t sb = sl_smem_bytes<false>(), s8 = sl_smem_bytes<true>();
    if (pass == 1) {
        if (a.fp8)
            a.dump ? sl_pass_kernel<1, true, true><<<grid, kSlThreads, s8, s>>>(a)
                   : sl_pass_kernel<1, true, false><<<grid, kSlThreads, s8, s>>>(a);
        else
            a.dump ? sl_pass_kernel<1, false, true><<<grid, kSlThreads, sb, s>>>(a)
                   : sl_pass_kernel<1, false, false><<<grid, kSlThreads, sb, s>>>(a);
    } else {
        if (a.fp8)
            sl_pass_kernel<2, true, false><<<grid, kSlThreads, s8, s>>>(a);
        else
            sl_pass_kernel<2, false, false><<<grid, kSlThreads, sb, s>>>(a);
    }
    return 1;
}

int launch_shortlist_mid(const SlArgs &a, cudaStream_t s) {
    if (!a.npairs) return 0;
    if (a.npairs <= kFewPairs)
        sl_mid_kernel<1024><<<dim3(a.npairs, a.row_blocks), 1024, 0, s>>>(a);
    else
        sl_mid_kernel<256><<<dim3(a.npairs, a.row_blocks), 256, 0, s>>>(a);
    return 1;
}

int launch_shortlist_finalize(const SlArgs &a, cudaStream_t s) {
    if (!a.npairs) return 0;
    const dim3 per_block(a.npairs, a.row_blocks);  // CTA per pair and row block
    if (a.npairs <= kFewPairs)
        sl_finalize_kernel<1024><<<per_block, 1024, 0, s>>>(a);
    else
        sl_finalize_kernel<256><<<per_block, 256, 0, s>>>(a);
    return 1;
}

int launch_shortlist_rescue_prep(const SlArgs &a, cudaStream_t s) {
    if (!a.npairs) return 0;
    sl_rescue_prep_kernel<<<dim3(a.npairs, a.row_blocks), 256, 0, s>>>(a);
    return 1;
}

int launch_shortlist_tail(const SlArgs &a, int sms, cudaStream_t s) {
    if (!a.npairs) return 0;
    const unsigned rgrid = (unsigned)(a.npairs < (uint32_t)(4 * sms) ? a.npairs : (uint32_t)(4 * sms));
    const dim3 per_block(a.npairs, a.row_blocks);  // CTA per pair and row block
    // routed pairs: plan, exact kernel over all their rows and columns, decisions
    sl_route_plan_kernel<<<1, 1024, 0, s>>>(a);
    sl_route_apply_kernel<<<rgrid, 256, 0, s>>>(a);
    ExactArgs x{};
    x.tiled = a.tiled;
    x.items = a.xitems;
    x.n_items = a.xitem_cap;
    x.n_items_dev = a.ctl + kCtlXItems;
    x.pairs = a.pairs;
    x.parts = a.xparts;
    x.colbest = a.colbest;
    x.work = a.ctl + kCtlXWork;
    x.err = a.ctl + 1;
    x.mutual = a.mutual;
    x.x2 = 1;
    // BF16 batches rarely route a pair: the FP32 tiles the exact kernel reads
    // are packed here for the routed pairs' views only (FP8 batches, which
    // route most pairs of unit descriptors, keep the store's packed tiles)
    if (!a.fp8)
        launch_pack_routed(a.pairs, a.xlist, a.ctl + kCtlRoutedPairs, a.raw, const_cast<float *>(a.tiled), 2 * sms, s);
    launch_exact(x, sms, s);
    sl_route_finalize_kernel<<<dim3(rgrid, a.row_blocks), 256, 0, s>>>(a);
    sl_rescore_kernel<<<5 * sms, 256, 0, s>>>(a);  // 40 warps per SM: latency-bound gathers
    sl_scan_kernel<<<2 * sms, 256, 0, s>>>(a);
    sl_compact_kernel<<<per_block, 256, 0, s>>>(a);
    return a.fp8 ? 7 : 8;
}

}  // namespace slm
