// k_sampson.cu — batched Sampson scoring of essential-matrix hypotheses.
//
// Reference: crates/core/src/two_view.rs:456-465 (`sampson_residual`) and
// :804-823 (`inliers_of` and `count_at_least` in ransac_essential_inner, the
// per-hypothesis work of the RANSAC stage that runs on every pair kept by
// match_pairs, pipeline.rs:505). The reference scores each 5-point hypothesis
// over the pair's matches in f64; here one warp scores one hypothesis, 32
// matches at a time, every residual in the reference's f64 operation order
// (explicit round-to-nearest operations: nothing is contracted to an FMA), so
// counts and inlier sets are the reference's bit for bit. count_at_least's
// early exit changes only when it stops, not its answer: it returns the full
// count when that reaches `need` and nothing otherwise, so the full count
// settles it.
#include <cuda_runtime.h>

#include <cstdint>

#include "slm_internal.h"

namespace slm {

namespace {

// The signed residual e p . q / |grad| of one correspondence, p = (ax, ay, 1),
// q = (bx, by, 1), e row-major. The order is the reference's linear algebra:
// row i of e p is ((e[i][0] ax + e[i][1] ay) + e[i][2] 1), the same for
// e^T q with the rows of e^T; den = sqrt(((ep0^2 + ep1^2) + etq0^2) + etq1^2);
// the residual is (bx ep0 + by ep1 + ep2) / den, or 0 when den is not > 0
// (also when it is NaN). Division and square root are IEEE round-to-nearest.
__device__ __forceinline__ double residual(const double (&e)[9], double ax, double ay, double bx, double by) {
    double ep[3], etq[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double y = __dmul_rn(e[3 * i], ax);
        y = __dadd_rn(__dmul_rn(e[3 * i + 1], ay), y);
        ep[i] = __dadd_rn(__dmul_rn(e[3 * i + 2], 1.0), y);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double y = __dmul_rn(e[i], bx);
        y = __dadd_rn(__dmul_rn(e[3 + i], by), y);
        etq[i] = __dadd_rn(__dmul_rn(e[6 + i], 1.0), y);
    }
    const double s = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(ep[0], ep[0]), __dmul_rn(ep[1], ep[1])),
                                         __dmul_rn(etq[0], etq[0])),
                               __dmul_rn(etq[1], etq[1]));
    const double den = __dsqrt_rn(s);
    if (den > 0.0) {
        const double dot = __dadd_rn(__dadd_rn(__dmul_rn(bx, ep[0]), __dmul_rn(by, ep[1])), __dmul_rn(1.0, ep[2]));
        return __ddiv_rn(dot, den);
    }
    return 0.0;
}

constexpr int kWarpsPerBlock = 8;

// One warp per hypothesis: its pair's matches 32 at a time, the inlier bits
// of each group of 32 by ballot (one mask word, written by lane 0 when the
// hypothesis asks for its mask), the count by population count.
__global__ void __launch_bounds__(32 * kWarpsPerBlock) sampson_kernel(SampsonArgs a) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t h = (uint64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (h >= a.nh) return;  // warp-uniform
    const uint32_t p = a.hyp_pair[h];
    const uint64_t m0 = a.pair_off[p], m1 = a.pair_off[p + 1];
    const double th = a.thresh[p];
    double e[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) e[k] = a.E[9 * h + k];
    uint32_t *mk = nullptr;
    if (a.masks && a.mask_off && a.mask_off[h] != ~0ull) mk = a.masks + a.mask_off[h];
    uint32_t c = 0;
    for (uint64_t i0 = m0; i0 < m1; i0 += 32) {
        const uint64_t i = i0 + lane;
        bool in = false;
        if (i < m1) {
            const double4 q = a.pts[i];
            // inliers_of / count_at_least: |r| < th, strict (two_view.rs:806, :812)
            in = fabs(residual(e, q.x, q.y, q.z, q.w)) < th;
        }
        const uint32_t bits = __ballot_sync(0xffffffffu, in);
        c += __popc(bits);
        if (mk && lane == 0) mk[(i0 - m0) >> 5] = bits;
    }
    if (lane == 0) a.counts[h] = c;
}

}  // namespace

void launch_sampson(const SampsonArgs &a, cudaStream_t s) {
    if (!a.nh) return;
    const uint64_t blocks = (a.nh + kWarpsPerBlock - 1) / kWarpsPerBlock;
    sampson_kernel<<<(unsigned)blocks, 32 * kWarpsPerBlock, 0, s>>>(a);
}

}  // namespace slm
