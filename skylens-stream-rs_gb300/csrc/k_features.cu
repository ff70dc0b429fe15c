// k_features.cu — the descriptor producer on the GPU: Gaussian pyramid, DoG
// extrema with sub-pixel refinement, orientation assignment and the 128-d
// descriptor of crates/core/src/features.rs (detect_core :650-781,
// gaussian_blur :214-250, pixel_grad :327-332, orientations_with :361-420,
// refine_extremum :431-484, describe_with :521-592), over a batch of images
// of one size.
//
// Every arithmetic expression keeps the reference's operand order; the file
// is compiled without FMA contraction and with IEEE division and square root,
// so each f32 value is the reference's. The reference's per-pixel and
// per-keypoint transcendental functions (atan2, exp, powf, cos, sin; the
// platform's float functions) are evaluated correctly rounded: atan2 and exp,
// called per pixel and per window sample, by the float-float evaluations of
// fmath_cr.h (FP32 and FMA, with a rounding test that falls back to double in
// a few calls in 10^5), powf, cos and sin, once per keypoint, in double
// rounded to float. Both equal the double function rounded to float (double
// rounding aside, probability about 2^-29 a call), which equals the
// platform's float result wherever that one is correctly rounded. Sums that
// the reference accumulates in one order (histogram bins, the descriptor's
// norm) are accumulated in that order.
#include <cuda_runtime.h>

#include <cstdint>

#include "fmath_cr.h"
#include "slm_internal.h"

namespace slm {

namespace {

constexpr float kTwoPi = 6.28318530717958647692f;  // std::f32::consts::TAU
constexpr float kSqrt2 = 1.41421356237309504880f;  // std::f32::consts::SQRT_2
constexpr int kOriBins = 36;                        // features.rs:307

__device__ __forceinline__ float exp_cr(float x) { return slm_expf_cr(x); }
__device__ __forceinline__ float atan2_cr(float y, float x) { return slm_atan2f_cr(y, x); }

// f32::rem_euclid(a, b) for b > 0: a % b (fmodf), plus b when negative. For
// |a| < 2b the remainder is a, or a - b with a's sign (exact: b <= |a| < 2b),
// and a zero remainder keeps a's sign as fmodf's does; fmodf otherwise.
__device__ __forceinline__ float rem_euclid(float a, float b) {
    float r;
    const float aa = fabsf(a);
    if (aa < b) {
        r = a;
    } else if (aa < 2.0f * b) {
        r = copysignf(aa - b, a);
    } else {
        r = fmodf(a, b);
    }
    return r < 0.0f ? r + b : r;
}

// `v as isize` (truncation; the values here are small and finite)
__device__ __forceinline__ int f2i(float v) { return v != v ? 0 : (int)v; }

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : v > hi ? hi : v; }

// ------------------------------------------------------------------ blur

constexpr int kBlurX = 256;

// Horizontal pass: tmp[y][x] = sum_j k[j] * src[y][clamp(x + j - r)], j in
// order, starting from 0.0 (features.rs:226-238).
__global__ void __launch_bounds__(kBlurX) blur_rows_kernel(const float *__restrict__ src, float *__restrict__ dst,
                                                           int w, int h, uint64_t img_stride_src,
                                                           uint64_t img_stride_dst, BlurTaps t) {
    __shared__ float row[kBlurX + 2 * kMaxBlurR];
    const int y = blockIdx.y, b = blockIdx.z;
    const int x0 = blockIdx.x * kBlurX;
    const float *s = src + b * img_stride_src + (uint64_t)y * w;
    const int n = kBlurX + 2 * t.r;
    for (int i = threadIdx.x; i < n; i += kBlurX) row[i] = s[clampi(x0 + i - t.r, 0, w - 1)];
    __syncthreads();
    const int x = x0 + threadIdx.x;
    if (x >= w) return;
    float acc = 0.0f;
    for (int j = 0; j <= 2 * t.r; ++j) acc += t.k[j] * row[threadIdx.x + j];
    dst[b * img_stride_dst + (uint64_t)y * w + x] = acc;
}

// Vertical pass: out[y][x] = sum_j k[j] * tmp[clamp(y + j - r)][x], j in
// order from 0.0 (features.rs:240-249); with `prev`, also the DoG layer
// out - prev (features.rs:674-685).
__global__ void __launch_bounds__(kBlurX) blur_cols_kernel(const float *__restrict__ tmp, float *__restrict__ out,
                                                           const float *__restrict__ prev, float *__restrict__ dog,
                                                           int w, int h, uint64_t img_stride_tmp,
                                                           uint64_t img_stride_out, uint64_t img_stride_dog,
                                                           BlurTaps t) {
    const int x = blockIdx.x * kBlurX + threadIdx.x, y = blockIdx.y, b = blockIdx.z;
    if (x >= w) return;
    const float *c = tmp + b * img_stride_tmp + x;
    float acc = 0.0f;
    for (int j = 0; j <= 2 * t.r; ++j) acc += t.k[j] * c[(uint64_t)clampi(y + j - t.r, 0, h - 1) * w];
    const uint64_t p = (uint64_t)y * w + x;
    out[b * img_stride_out + p] = acc;
    if (dog) dog[b * img_stride_dog + p] = acc - prev[b * img_stride_out + p];
}

// Both passes in one kernel for radii up to kFusedR: a 64 x 32 output tile
// with its halo of clamped input pixels in shared memory, the horizontal sums
// of the tile's rows (halo rows included) in shared memory, then the vertical
// sums; with `dog`, also dog = out - src at each pixel (src is the previous
// layer). Each sum runs over j in order from 0.0, exactly as the two-kernel
// form and the reference do.
constexpr int kFusedR = 16;
constexpr int kFX = 64, kFY = 32;
__global__ void __launch_bounds__(256) blur_fused_kernel(const float *__restrict__ src, float *__restrict__ dst,
                                                         float *__restrict__ dog, int w, int h,
                                                         uint64_t img_stride_src, uint64_t img_stride_dst,
                                                         uint64_t img_stride_dog, BlurTaps t) {
    __shared__ float in[kFY + 2 * kFusedR][kFX + 2 * kFusedR];
    __shared__ float hs[kFY + 2 * kFusedR][kFX];
    const int r = t.r, b = blockIdx.z;
    const int x0 = blockIdx.x * kFX, y0 = blockIdx.y * kFY;
    const float *S = src + b * img_stride_src;
    const int rows = kFY + 2 * r, cols = kFX + 2 * r;
    for (int e = threadIdx.x; e < rows * cols; e += 256) {
        const int ry = e / cols, rx = e % cols;
        const int yy = clampi(y0 + ry - r, 0, h - 1), xx = clampi(x0 + rx - r, 0, w - 1);
        in[ry][rx] = S[(uint64_t)yy * w + xx];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < rows * kFX; e += 256) {
        const int ry = e / kFX, cx = e % kFX;
        float acc = 0.0f;
        for (int j = 0; j <= 2 * r; ++j) acc += t.k[j] * in[ry][cx + j];
        hs[ry][cx] = acc;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kFY * kFX; e += 256) {
        const int ty = e / kFX, cx = e % kFX;
        const int x = x0 + cx, y = y0 + ty;
        if (x >= w || y >= h) continue;
        float acc = 0.0f;
        for (int j = 0; j <= 2 * r; ++j) acc += t.k[j] * hs[ty + j][cx];
        const uint64_t p = (uint64_t)y * w + x;
        dst[b * img_stride_dst + p] = acc;
        if (dog) dog[b * img_stride_dog + p] = acc - in[ty + r][cx + r];
    }
}

// base of the next octave: the even pixels of gauss[s] (GrayImage::downsample)
__global__ void downsample_kernel(const float *__restrict__ src, float *__restrict__ dst, int w, int h, int nw, int nh,
                                  uint64_t img_stride_src, uint64_t img_stride_dst) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, b = blockIdx.z;
    if (x >= nw) return;
    dst[b * img_stride_dst + (uint64_t)y * nw + x] = src[b * img_stride_src + (uint64_t)(2 * y) * w + 2 * x];
}

// GrayImage::upsample2 (features.rs:62-85): bilinear at pixel centres.
__global__ void upsample2_kernel(const float *__restrict__ src, float *__restrict__ dst, int w, int h) {
    const int W = 2 * w;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, b = blockIdx.z;
    if (x >= W) return;
    const float *s = src + (uint64_t)b * w * h;
    const float sy = ((float)y + 0.5f) / 2.0f - 0.5f;
    const float y0 = floorf(sy), fy = sy - y0;
    const int ya = clampi(f2i(y0), 0, h - 1), yb = clampi(f2i(y0) + 1, 0, h - 1);
    const float sx = ((float)x + 0.5f) / 2.0f - 0.5f;
    const float x0 = floorf(sx), fx = sx - x0;
    const int xa = clampi(f2i(x0), 0, w - 1), xb = clampi(f2i(x0) + 1, 0, w - 1);
    const float top = s[(uint64_t)ya * w + xa] * (1.0f - fx) + s[(uint64_t)ya * w + xb] * fx;
    const float bot = s[(uint64_t)yb * w + xa] * (1.0f - fx) + s[(uint64_t)yb * w + xb] * fx;
    dst[(uint64_t)b * W * (2 * h) + (uint64_t)y * W + x] = top * (1.0f - fy) + bot * fy;
}

// GrayImage::from_rgb (features.rs:165-189)
__global__ void gray_from_rgb8_kernel(const uint8_t *__restrict__ rgb, float *__restrict__ out, uint64_t n) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint8_t *c = rgb + 3 * i;
    out[i] = (0.299f * (float)c[0] + 0.587f * (float)c[1] + 0.114f * (float)c[2]) / 255.0f;
}

// ------------------------------------------------------------- gradients

// GradTable (features.rs:335-359) of s consecutive layers from l0: |g| and
// atan2(gy, gx) of central differences at interior pixels (pixel_grad,
// :327-332); grad is [img][s][h][w].
__global__ void grad_kernel(const float *__restrict__ gauss, float2 *__restrict__ grad, int w, int h, int s,
                            uint64_t layer_stride, uint64_t img_stride, int l0) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    const int b = blockIdx.z / s, l = blockIdx.z % s;
    if (x >= w) return;
    float2 g = make_float2(0.0f, 0.0f);
    if (x >= 1 && y >= 1 && x + 1 < w && y + 1 < h) {
        const float *im = gauss + (uint64_t)b * img_stride + (uint64_t)(l0 + l) * layer_stride;
        const float gx = im[(uint64_t)y * w + x + 1] - im[(uint64_t)y * w + x - 1];
        const float gy = im[(uint64_t)(y + 1) * w + x] - im[(uint64_t)(y - 1) * w + x];
        g.x = sqrtf(gx * gx + gy * gy);
        g.y = atan2_cr(gy, gx);
    }
    grad[((uint64_t)b * s + l) * layer_stride + (uint64_t)y * w + x] = g;
}

// ---------------------------------------------------------------- extrema

// nalgebra 0.33 Matrix3::try_inverse (cofactor formula), m row-major;
// false when the determinant is exactly zero.
__device__ bool inverse3(const float (&m)[9], float (&o)[9]) {
    const float m11 = m[0], m12 = m[1], m13 = m[2];
    const float m21 = m[3], m22 = m[4], m23 = m[5];
    const float m31 = m[6], m32 = m[7], m33 = m[8];
    const float minor_m12_m23 = m22 * m33 - m32 * m23;
    const float minor_m11_m23 = m21 * m33 - m31 * m23;
    const float minor_m11_m22 = m21 * m32 - m31 * m22;
    const float det = m11 * minor_m12_m23 - m12 * minor_m11_m23 + m13 * minor_m11_m22;
    if (det == 0.0f) return false;
    o[0] = minor_m12_m23 / det;
    o[1] = (m13 * m32 - m33 * m12) / det;
    o[2] = (m12 * m23 - m22 * m13) / det;
    o[3] = -minor_m11_m23 / det;
    o[4] = (m11 * m33 - m31 * m13) / det;
    o[5] = (m13 * m21 - m23 * m11) / det;
    o[6] = minor_m11_m22 / det;
    o[7] = (m12 * m31 - m32 * m11) / det;
    o[8] = (m11 * m22 - m21 * m12) / det;
    return true;
}

// One thread per interior pixel and DoG layer l in 1..s (detect_core's scan,
// features.rs:700-768): the 26-neighbour test, refine_extremum, the contrast
// and edge tests, then sig_oct = sigma0 * kstep^s; survivors are appended to
// the candidate list with their emission-order key.
__global__ void extrema_kernel(ExtremaArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    const int b = blockIdx.z / a.s, l0 = 1 + blockIdx.z % a.s;
    const int w = a.w, h = a.h;
    if (x < 1 || y < 1 || x + 1 >= w || y + 1 >= h) return;
    const float *dog = a.dog + (uint64_t)b * (a.ng - 1) * a.layer_stride;
#define D(L, X, Y) dog[(uint64_t)(L) * a.layer_stride + (uint64_t)(Y) * w + (X)]
    const float v0 = D(l0, x, y);
    if (fabsf(v0) < a.contrast) return;
    bool is_max = true, is_min = true;
#pragma unroll
    for (int k = -1; k <= 1; ++k)
#pragma unroll
        for (int yy = -1; yy <= 1; ++yy)
#pragma unroll
            for (int xx = -1; xx <= 1; ++xx) {
                if (k == 0 && xx == 0 && yy == 0) continue;
                const float u = D(l0 + k, x + xx, y + yy);
                is_max &= v0 > u;
                is_min &= v0 < u;
            }
    if (!(is_max || is_min)) return;
    // refine_extremum (features.rs:431-484)
    int cx = x, cy = y, cl = l0;
    bool ok = false;
    float d[3], g[3], v = 0.0f;
    for (int it = 0; it < 5; ++it) {
        v = D(cl, cx, cy);
        g[0] = 0.5f * (D(cl, cx + 1, cy) - D(cl, cx - 1, cy));
        g[1] = 0.5f * (D(cl, cx, cy + 1) - D(cl, cx, cy - 1));
        g[2] = 0.5f * (D(cl + 1, cx, cy) - D(cl - 1, cx, cy));
        const float hxx = D(cl, cx + 1, cy) + D(cl, cx - 1, cy) - 2.0f * v;
        const float hyy = D(cl, cx, cy + 1) + D(cl, cx, cy - 1) - 2.0f * v;
        const float hss = D(cl + 1, cx, cy) + D(cl - 1, cx, cy) - 2.0f * v;
        const float hxy = 0.25f * (D(cl, cx + 1, cy + 1) - D(cl, cx - 1, cy + 1) - D(cl, cx + 1, cy - 1) +
                                   D(cl, cx - 1, cy - 1));
        const float hxs = 0.25f * (D(cl + 1, cx + 1, cy) - D(cl + 1, cx - 1, cy) - D(cl - 1, cx + 1, cy) +
                                   D(cl - 1, cx - 1, cy));
        const float hys = 0.25f * (D(cl + 1, cx, cy + 1) - D(cl + 1, cx, cy - 1) - D(cl - 1, cx, cy + 1) +
                                   D(cl - 1, cx, cy - 1));
        const float hm[9] = {hxx, hxy, hxs, hxy, hyy, hys, hxs, hys, hss};
        float inv[9];
        if (!inverse3(hm, inv)) return;
#pragma unroll
        for (int i = 0; i < 3; ++i) {  // matrix x vector: columns added in order (gemv)
            float acc = inv[3 * i] * g[0];
            acc = acc + inv[3 * i + 1] * g[1];
            acc = acc + inv[3 * i + 2] * g[2];
            d[i] = -acc;
        }
        if (fabsf(d[0]) <= 0.5f && fabsf(d[1]) <= 0.5f && fabsf(d[2]) <= 0.5f) {
            ok = true;
            break;
        }
        if (!(isfinite(d[0]) && isfinite(d[1]) && isfinite(d[2]))) return;
        const int nx = cx + f2i(roundf(d[0])), ny = cy + f2i(roundf(d[1])), nl = cl + f2i(roundf(d[2]));
        if (nx < 1 || ny < 1 || nl < 1 || nx >= w - 1 || ny >= h - 1 || nl > a.s) return;
        cx = nx;
        cy = ny;
        cl = nl;
    }
    if (!ok) return;
    const float value = v + 0.5f * (g[0] * d[0] + g[1] * d[1] + g[2] * d[2]);
    if (fabsf(value) < a.contrast) return;
    // edge test on the refined sample (features.rs:735-746)
    const float c = D(cl, cx, cy);
    const float dxx = D(cl, cx + 1, cy) + D(cl, cx - 1, cy) - 2.0f * c;
    const float dyy = D(cl, cx, cy + 1) + D(cl, cx, cy - 1) - 2.0f * c;
    const float dxy =
        0.25f * (D(cl, cx + 1, cy + 1) - D(cl, cx - 1, cy + 1) - D(cl, cx + 1, cy - 1) + D(cl, cx - 1, cy - 1));
#undef D
    const float tr = dxx + dyy;
    const float det = dxx * dyy - dxy * dxy;
    if (det <= 0.0f || tr * tr / det >= a.edge_thr) return;
    const float rs = (float)cl + d[2];
    const float sig = a.sigma0 * (float)pow((double)a.kstep, (double)rs);
    const uint32_t slot = atomicAdd(a.count, 1u);
    if (slot >= a.cap) return;  // the host sees count > cap and runs again with room
    FeatCand fc;
    fc.x = (float)cx + d[0];
    fc.y = (float)cy + d[1];
    fc.sig = sig;
    fc.value = value;
    fc.img = (uint16_t)b;
    fc.octave = (uint8_t)a.octave;
    fc.layer = (uint8_t)cl;
    fc.key = ((uint64_t)a.octave << 48) | ((uint64_t)l0 << 32) | ((uint64_t)y << 16) | (uint64_t)x;
    a.cands[slot] = fc;
}

// --------------------------------------------------------------- orientations

// One warp per candidate (orientations_with, features.rs:361-420): samples of
// the (2r+1)^2 window in raster order, 32 at a time; each bin's sum is added
// in raster order (lane b owns bins b and b + 32); then lane 0 smooths and
// picks the peaks.
__global__ void __launch_bounds__(256) orient_kernel(OrientArgs a) {
    __shared__ float hs[8][kOriBins];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t ci = blockIdx.x * 8 + warp;
    const uint32_t n = min(*a.count, a.cap);
    if (ci >= n) return;
    const FeatCand c = a.cands[ci];
    const OctaveGeom &G = a.geom[c.octave];
    const float2 *grad = a.grads + G.grad_off + ((uint64_t)c.img * a.s + (c.layer - 1)) * G.layer_stride;
    const int w = G.w, h = G.h;
    const float sw = 1.5f * c.sig;
    const int r = f2i(roundf(3.0f * sw));
    const int xi = f2i(roundf(c.x)), yi = f2i(roundf(c.y));
    const int side = 2 * r + 1;
    const int total = side * side;
    float h0 = 0.0f, h1 = 0.0f;
    for (int base = 0; base < total; base += 32) {
        const int t = base + lane;
        int bin = -1;
        float val = 0.0f;
        if (t < total) {
            const int px = xi + (t % side) - r, py = yi + (t / side) - r;
            if (!(px < 1 || py < 1 || px >= w - 1 || py >= h - 1)) {
                const float2 gm = grad[(uint64_t)py * w + px];
                const float fx = (float)px - c.x, fy = (float)py - c.y;
                const float wgt = exp_cr(-(fx * fx + fy * fy) / (2.0f * sw * sw));
                const float ang = rem_euclid(gm.y, kTwoPi);
                const float bf = roundf(ang / kTwoPi * (float)kOriBins);
                bin = (int)((unsigned)(bf < 0.0f ? 0 : f2i(bf)) % kOriBins);
                val = wgt * gm.x;
            }
        }
        unsigned any = __ballot_sync(0xffffffffu, bin >= 0);
        while (any) {
            const int j = __ffs(any) - 1;
            any &= any - 1;
            const int bj = __shfl_sync(0xffffffffu, bin, j);
            const float vj = __shfl_sync(0xffffffffu, val, j);
            if (bj == lane) h0 += vj;
            if (bj == lane + 32) h1 += vj;
        }
    }
    // six [1,1,1]/3 smoothings, lane b computing bins b and b + 32 (each bin
    // from the previous pass's three, ((l + c) + r) / 3 as the reference)
    float *hist = hs[warp];
    const int b1 = lane + 32;
    const bool has1 = b1 < kOriBins;
    for (int it = 0; it < 6; ++it) {
        hist[lane] = h0;
        if (has1) hist[b1] = h1;
        __syncwarp();
        const float n0 = (hist[(lane + kOriBins - 1) % kOriBins] + h0 + hist[(lane + 1) % kOriBins]) / 3.0f;
        const float n1 = has1 ? (hist[(b1 + kOriBins - 1) % kOriBins] + h1 + hist[(b1 + 1) % kOriBins]) / 3.0f : 0.0f;
        __syncwarp();
        h0 = n0;
        h1 = n1;
    }
    hist[lane] = h0;
    if (has1) hist[b1] = h1;
    __syncwarp();
    // fold(0.0, f32::max): fmaxf is order-free (NaN ignored either way)
    float mx = fmaxf(h0, has1 ? h1 : 0.0f);
#pragma unroll
    for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    mx = fmaxf(0.0f, mx);
    // peaks in bin order: bins 0..31 by lane, then 32..35
    float *out = a.angles + (uint64_t)ci * kMaxAngles;
    int na = 0;
    if (mx > 0.0f) {
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int i = half ? b1 : lane;
            bool peak = false;
            float ang = 0.0f;
            if (i < kOriBins) {
                const float l = hist[(i + kOriBins - 1) % kOriBins], cc = hist[i], rr = hist[(i + 1) % kOriBins];
                if (cc >= 0.8f * mx && cc > l && cc > rr) {
                    const float off = 0.5f * (l - rr) / (l - 2.0f * cc + rr);
                    ang = rem_euclid(((float)i + off) / (float)kOriBins * kTwoPi, kTwoPi);
                    peak = true;
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, peak);
            if (peak) out[na + __popc(m & ((1u << lane) - 1u))] = ang;
            na += __popc(m);
        }
    }
    if (lane == 0) a.nang[ci] = (uint8_t)na;
}

// ----------------------------------------------------------------- describe

constexpr int kDescThreads = 128;

// One window sample's contributions: the products m * (1 - dv) and m * dv
// for its two spatial rows iv0 and iv0 + 1 (the first factor of the
// reference's ((m * wv) * wu) * wo), the column and orientation weights, and
// the lanes (iu * 8 + io) it adds to in a row: `hit`, of which `second_u`
// take du instead of 1 - du and `second_o` take dob instead of 1 - dob.
struct DescSample {
    float pv0, pv1, wu0, wu1;
    float wo0, wo1;
    int iv0;
    uint32_t hit, second_u, second_o, pad0, pad1;
};

// One CTA per feature (describe_with, features.rs:521-592). The (2r+1)^2
// window goes through in chunks of 128 samples in raster order: each thread
// computes one sample (rotated cell coordinates, the trilinear weights) and
// marks, for each bin it adds to, its bit in that bin's mask of the chunk's
// 32-sample group; then thread (warp iv, lane iu * 8 + io) owns bin (iv, iu,
// io) and adds the contributions of the samples whose bits its masks hold,
// in sample order: every bin's sum is the reference's, in its order, and a
// thread steps only through the samples that touch its own bin.
__global__ void __launch_bounds__(kDescThreads) describe_kernel(DescribeArgs a) {
    __shared__ DescSample smp[kDescThreads];
    // per chunk parity, 32-sample group, spatial row and lane: the group's samples adding to that bin
    __shared__ uint32_t bmask[2][kDescThreads / 32][4][32];
    __shared__ float hist[kDesc];
    __shared__ float norm_s;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const DescJob job = a.jobs[blockIdx.x];
    float x, y, sig, angle;
    const float2 *grad;
    int w, h;
    if (a.cands) {
        const FeatCand c = a.cands[job.cand];
        const OctaveGeom &G = a.geom[c.octave];
        grad = a.grads + G.grad_off + ((uint64_t)c.img * a.s + (c.layer - 1)) * G.layer_stride;
        w = G.w;
        h = G.h;
        x = c.x;
        y = c.y;
        sig = c.sig;
    } else {  // describe(img, x, y, sigma, angle) on one gradient table
        const slm_keypoint &k = a.kps[job.cand];
        grad = a.grads;
        w = a.geom[0].w;
        h = a.geom[0].h;
        x = k.x;
        y = k.y;
        sig = k.sigma;
    }
    angle = job.angle;
    const int NC = 4, NO = 8;
    const float cell = 3.0f * sig;
    const int r = f2i(roundf(cell * kSqrt2 * ((float)NC + 1.0f) * 0.5f));
    const float c = (float)cos((double)angle), sn = (float)sin((double)angle);
    const int xi = f2i(roundf(x)), yi = f2i(roundf(y));
    const int side = 2 * r + 1;
    const int total = side * side;
    float acc = 0.0f;  // bin (warp, lane)
    const uint32_t my_bit = 1u << lane;
    for (int e = tid; e < (kDescThreads / 32) * 4 * 32; e += kDescThreads) (&bmask[0][0][0][0])[e] = 0u;
    __syncthreads();
    int par = 0;
    for (int base = 0; base < total; base += kDescThreads, par ^= 1) {
        const int t = base + tid;
        bool valid = false;
        DescSample q{};
        if (t < total) {
            const int px = xi + (t % side) - r, py = yi + (t / side) - r;
            const float fx = (float)px - x, fy = (float)py - y;
            const float pu = c * fx + sn * fy, pv_ = -sn * fx + c * fy;
            // |numerator| above 2.6 cells puts bu or bv beyond (-1, 4) whatever
            // the division rounds to: such samples skip the divisions (NaN goes on
            // to the reference's test)
            const float lim = 2.6f * cell;
            if (!(px < 1 || py < 1 || px >= w - 1 || py >= h - 1) && !(fabsf(pu) > lim) && !(fabsf(pv_) > lim)) {
                const float u = pu / cell;
                const float v = pv_ / cell;
                const float bu = u + (float)NC / 2.0f - 0.5f, bv = v + (float)NC / 2.0f - 0.5f;
                if (!(bu <= -1.0f || bv <= -1.0f || bu >= (float)NC || bv >= (float)NC)) {
                    const float2 gm = grad[(uint64_t)py * w + px];
                    const float ori = rem_euclid(gm.y - angle, kTwoPi);
                    const float bo = ori / kTwoPi * (float)NO;
                    const float wgt = exp_cr(-(u * u + v * v) / (2.0f * 4.0f));
                    const float m = gm.x * wgt;
                    const float u0 = floorf(bu), v0 = floorf(bv), o0 = floorf(bo);
                    const float du = bu - u0, dv = bv - v0, dob = bo - o0;
                    q.pv0 = m * (1.0f - dv);
                    q.pv1 = m * dv;
                    q.wu0 = 1.0f - du;
                    q.wu1 = du;
                    q.wo0 = 1.0f - dob;
                    q.wo1 = dob;
                    q.iv0 = f2i(v0);
                    const int iu0 = f2i(u0);
                    const int io0 = o0 < 0.0f ? 0 : f2i(o0);
                    const int olo = io0 % NO, ohi = (io0 + 1) % NO;
#pragma unroll
                    for (int da = 0; da < 2; ++da) {
                        const int iu = iu0 + da;
                        if (iu < 0 || iu >= NC) continue;
                        const uint32_t blo = 1u << (iu * NO + olo), bhi = 1u << (iu * NO + ohi);
                        q.hit |= blo | bhi;
                        q.second_o |= bhi;
                        if (da) q.second_u |= blo | bhi;
                    }
                    valid = true;
                }
            }
        }
        smp[tid] = q;
        if (valid) {
#pragma unroll
            for (int dv = 0; dv < 2; ++dv) {
                const int row = q.iv0 + dv;
                if (row < 0 || row >= NC) continue;
                uint32_t hm = q.hit;
                while (hm) {
                    const int l = __ffs(hm) - 1;
                    hm &= hm - 1;
                    atomicOr(&bmask[par][warp][row][l], my_bit);
                }
            }
        }
        __syncthreads();
        // thread (warp, lane) owns bin (iv = warp, iu = lane / 8, io = lane % 8)
        auto contrib = [&](const DescSample &s) {
            const float pv = s.iv0 == warp ? s.pv0 : s.pv1;
            const float wu = (s.second_u & my_bit) ? s.wu1 : s.wu0;
            const float wo = (s.second_o & my_bit) ? s.wo1 : s.wo0;
            return pv * wu * wo;
        };
        for (int g = 0; g < kDescThreads / 32; ++g) {
            unsigned m = bmask[par][g][warp][lane];
            while (m) {
                const int j = g * 32 + __ffs(m) - 1;
                m &= m - 1;
                acc += contrib(smp[j]);
            }
        }
        // the other parity's masks, free since the last chunk's barrier, for the next chunk
        for (int e = tid; e < (kDescThreads / 32) * 4 * 32; e += kDescThreads) (&bmask[par ^ 1][0][0][0])[e] = 0u;
        __syncthreads();
    }
    hist[warp * 32 + lane] = acc;  // (iv * 4 + iu) * 8 + io
    __syncthreads();
    for (int pass = 0; pass < 2; ++pass) {
        if (tid == 0) {  // the norm's sum in index order
            float n2 = -0.0f;
            for (int i = 0; i < kDesc; ++i) n2 += hist[i] * hist[i];
            norm_s = sqrtf(n2);
        }
        __syncthreads();
        const float nrm = norm_s;
        float v = hist[tid];
        if (nrm > 0.0f) v = v / nrm;
        if (pass == 0) v = fminf(v, 0.2f);
        __syncthreads();
        hist[tid] = v;
        __syncthreads();
    }
    a.desc[(uint64_t)job.out_row * kDesc + tid] = hist[tid];
}

}  // namespace

void launch_blur(const float *src, float *tmp, float *dst, const float *prev, float *dog, int w, int h, int nimg,
                 uint64_t stride_src, uint64_t stride_dst, uint64_t stride_dog, const BlurTaps &t, cudaStream_t s) {
    if (t.r <= kFusedR && (!dog || (prev == src && stride_src == stride_dst))) {
        const dim3 g((w + kFX - 1) / kFX, (h + kFY - 1) / kFY, nimg);
        blur_fused_kernel<<<g, 256, 0, s>>>(src, dst, dog, w, h, stride_src, stride_dst, stride_dog, t);
        return;
    }
    const dim3 grid((w + kBlurX - 1) / kBlurX, h, nimg);
    blur_rows_kernel<<<grid, kBlurX, 0, s>>>(src, tmp, w, h, stride_src, (uint64_t)w * h, t);
    blur_cols_kernel<<<grid, kBlurX, 0, s>>>(tmp, dst, prev, dog, w, h, (uint64_t)w * h, stride_dst, stride_dog, t);
}

void launch_downsample(const float *src, float *dst, int w, int h, int nimg, uint64_t stride_src,
                       uint64_t stride_dst, cudaStream_t s) {
    const int nw = w / 2, nh = h / 2;
    if (!nw || !nh) return;
    downsample_kernel<<<dim3((nw + 255) / 256, nh, nimg), 256, 0, s>>>(src, dst, w, h, nw, nh, stride_src,
                                                                       stride_dst);
}

void launch_upsample2(const float *src, float *dst, int w, int h, int nimg, cudaStream_t s) {
    upsample2_kernel<<<dim3((2 * w + 255) / 256, 2 * h, nimg), 256, 0, s>>>(src, dst, w, h);
}

void launch_gray_from_rgb8(const uint8_t *rgb, float *out, uint64_t n, cudaStream_t s) {
    if (n) gray_from_rgb8_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(rgb, out, n);
}

void launch_grad(const float *gauss, float2 *grad, int w, int h, int s_, uint64_t img_stride, int l0, int nimg,
                 cudaStream_t s) {
    grad_kernel<<<dim3((w + 255) / 256, h, nimg * s_), 256, 0, s>>>(gauss, grad, w, h, s_, (uint64_t)w * h,
                                                                    img_stride, l0);
}

void launch_extrema(const ExtremaArgs &a, int nimg, cudaStream_t s) {
    extrema_kernel<<<dim3((a.w + 127) / 128, a.h, nimg * a.s), 128, 0, s>>>(a);
}

void launch_orient(const OrientArgs &a, uint32_t n, cudaStream_t s) {
    if (n) orient_kernel<<<(n + 7) / 8, 256, 0, s>>>(a);
}

void launch_describe(const DescribeArgs &a, uint32_t njobs, cudaStream_t s) {
    if (njobs) describe_kernel<<<njobs, kDescThreads, 0, s>>>(a);
}

}  // namespace slm
