/* CPU restatement of skylens-stream-rs's descriptor producer
 * (crates/core/src/features.rs): Gaussian pyramid, DoG extrema with
 * sub-pixel refinement, orientation assignment and the 128-d descriptor.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the GPU descriptor producer and
 * the timed CPU baseline, never the product path.
 *
 * Every floating-point expression keeps the reference's operand order and
 * rounding (compiled with -ffp-contract=off: no FMA, as Rust). The reference
 * calls f32 transcendental functions of the platform math library
 * (f32::exp, atan2, powf, cos, sin, hypot). `cr` selects how the per-sample
 * and per-keypoint ones are evaluated here:
 *   cr = 0: the platform's float functions, as the reference does;
 *   cr = 1: the double function rounded once to float (correctly rounded
 *           but for double-rounding cases of probability about 2^-29),
 *           which is what the GPU kernels compute.
 * Scalars computed once per image or layer (the blur taps' exp, the scale
 * step's powf, the de-duplication's hypot) are the platform's in both modes:
 * the GPU path's host code computes them with the same library calls.
 *
 * Parity of this restatement is unpinned: the reference's feature tests are
 * property tests (blob position and scale, orientation under rotation), with
 * no golden vectors, and no Rust toolchain runs here. The refinement's 3x3
 * inverse follows nalgebra 0.33's published cofactor formula, which is not
 * part of the reference tree.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    float x, y, sigma, response, angle; /* Keypoint, features.rs:296-304 */
} orc_kp;

typedef struct { /* DetectorConfig, features.rs:253-293 */
    int64_t octaves, scales;
    float sigma0, contrast, edge_ratio;
    int64_t max_features, upscale_below;
    int upscale_fill;
} orc_det_cfg;

#define TWO_PI_F 6.28318530717958647692f /* std::f32::consts::TAU */
#define SQRT2_F 1.41421356237309504880f  /* std::f32::consts::SQRT_2 */
#define ORI_BINS 36                      /* features.rs:307 */
#define DESC_LEN 128                     /* features.rs:495 */

static float f_exp(float x, int cr) { return cr ? (float)exp((double)x) : expf(x); }
static float f_atan2(float y, float x, int cr) { return cr ? (float)atan2((double)y, (double)x) : atan2f(y, x); }
static float f_pow(float b, float e, int cr) { return cr ? (float)pow((double)b, (double)e) : powf(b, e); }
static float f_cos(float a, int cr) { return cr ? (float)cos((double)a) : cosf(a); }
static float f_sin(float a, int cr) { return cr ? (float)sin((double)a) : sinf(a); }

/* f32::rem_euclid: r = a % b, plus |b| when negative */
static float rem_euclid(float a, float b) {
    float r = fmodf(a, b);
    return r < 0.0f ? r + fabsf(b) : r;
}

/* f32::powi with a run-time exponent lowers to compiler-rt's __powisf2:
 * square and multiply over the exponent's bits. */
static float powi_f(float a, int b) {
    const int recip = b < 0;
    float r = 1.0f;
    for (;;) {
        if (b & 1) r *= a;
        b /= 2;
        if (b == 0) break;
        a *= a;
    }
    return recip ? 1.0f / r : r;
}

/* `v as isize` for f32 (Rust: truncation, saturating, NaN -> 0) */
static int64_t f2i(float v) {
    if (v != v) return 0;
    if (v >= 9.2e18f) return INT64_MAX;
    if (v <= -9.2e18f) return INT64_MIN;
    return (int64_t)v;
}

static int64_t clampi(int64_t v, int64_t lo, int64_t hi) { return v < lo ? lo : v > hi ? hi : v; }

/* ---- image operations ------------------------------------------------- */

/* gaussian_blur, features.rs:214-250: taps exp(-(i*i) / (2 sigma sigma)),
 * normalised by their sum; a horizontal pass over edge-replicated rows, then
 * a vertical pass accumulating rows j = 0..2r in order. */
int64_t orc_blur_taps(float sigma, float *k /* >= 2r+1 */) {
    float rf = ceilf(3.0f * sigma);
    if (!(rf >= 1.0f)) rf = 1.0f; /* f32::max(1.0) keeps 1.0 against NaN */
    const int64_t r = f2i(rf);
    float s = -0.0f;
    for (int64_t i = -r; i <= r; ++i) {
        k[i + r] = expf((float)(-(i * i)) / (2.0f * sigma * sigma));
    }
    for (int64_t i = 0; i < 2 * r + 1; ++i) s += k[i];
    for (int64_t i = 0; i < 2 * r + 1; ++i) k[i] /= s;
    return r;
}

void orc_gaussian_blur(const float *img, int64_t w, int64_t h, float sigma, float *out) {
    float k[1024];
    const int64_t r = orc_blur_taps(sigma, k);
    float *tmp = (float *)malloc(sizeof(float) * (size_t)(w * h));
    for (int64_t y = 0; y < h; ++y) {
        const float *src = img + y * w;
        for (int64_t x = 0; x < w; ++x) {
            float acc = 0.0f;
            for (int64_t j = 0; j < 2 * r + 1; ++j) acc += k[j] * src[clampi(x + j - r, 0, w - 1)];
            tmp[y * w + x] = acc;
        }
    }
    for (int64_t y = 0; y < h; ++y) {
        float *o = out + y * w;
        for (int64_t x = 0; x < w; ++x) o[x] = 0.0f;
        for (int64_t j = 0; j < 2 * r + 1; ++j) {
            const int64_t yy = clampi(y + j - r, 0, h - 1);
            for (int64_t x = 0; x < w; ++x) o[x] += k[j] * tmp[yy * w + x];
        }
    }
    free(tmp);
}

/* GrayImage::upsample2, features.rs:62-85 (bilinear, pixel centres) */
void orc_upsample2(const float *img, int64_t w, int64_t h, float *out) {
    const int64_t W = w * 2, H = h * 2, mw = w - 1, mh = h - 1;
    for (int64_t y = 0; y < H; ++y) {
        const float sy = ((float)y + 0.5f) / 2.0f - 0.5f;
        const float y0 = floorf(sy), fy = sy - y0;
        const int64_t ya = clampi(f2i(y0), 0, mh), yb = clampi(f2i(y0) + 1, 0, mh);
        for (int64_t x = 0; x < W; ++x) {
            const float sx = ((float)x + 0.5f) / 2.0f - 0.5f;
            const float x0 = floorf(sx), fx = sx - x0;
            const int64_t xa = clampi(f2i(x0), 0, mw), xb = clampi(f2i(x0) + 1, 0, mw);
            const float top = img[ya * w + xa] * (1.0f - fx) + img[ya * w + xb] * fx;
            const float bot = img[yb * w + xa] * (1.0f - fx) + img[yb * w + xb] * fx;
            out[y * W + x] = top * (1.0f - fy) + bot * fy;
        }
    }
}

/* GrayImage::from_rgb, features.rs:165-189: (0.299 r + 0.587 g + 0.114 b) / 255 */
void orc_gray_from_rgb8(const uint8_t *rgb, int64_t n, float *out) {
    for (int64_t i = 0; i < n; ++i) {
        const uint8_t *c = rgb + 3 * i;
        out[i] = (0.299f * (float)c[0] + 0.587f * (float)c[1] + 0.114f * (float)c[2]) / 255.0f;
    }
}

/* pixel_grad, features.rs:327-332: central differences, |g| and atan2(gy, gx) */
static void pixel_grad(const float *img, int64_t w, int64_t ux, int64_t uy, int cr, float *mag, float *ang) {
    const float gx = img[uy * w + ux + 1] - img[uy * w + ux - 1];
    const float gy = img[(uy + 1) * w + ux] - img[(uy - 1) * w + ux];
    *mag = sqrtf(gx * gx + gy * gy);
    *ang = f_atan2(gy, gx, cr);
}

/* GradTable::new, features.rs:341-353: every interior pixel's gradient */
static void grad_table(const float *img, int64_t w, int64_t h, int cr, float *mag, float *ang) {
    memset(mag, 0, sizeof(float) * (size_t)(w * h));
    memset(ang, 0, sizeof(float) * (size_t)(w * h));
    for (int64_t y = 1; y + 1 < h; ++y)
        for (int64_t x = 1; x + 1 < w; ++x) pixel_grad(img, w, x, y, cr, &mag[y * w + x], &ang[y * w + x]);
}

/* ---- orientation and descriptor --------------------------------------- */

/* orientations_with, features.rs:361-420: a 36-bin histogram of gradient
 * directions weighted by exp(-(fx^2+fy^2) / (2 sw^2)), sw = 1.5 sigma, radius
 * round(3 sw); six [1,1,1]/3 smoothings; every local maximum >= 0.8 max,
 * parabola-interpolated. Returns the number of angles (<= 18). */
int64_t orc_orientations(const float *mag, const float *ang, int64_t w, int64_t h, float x, float y, float sigma,
                         int cr, float *out) {
    const float sw = 1.5f * sigma;
    const int64_t r = f2i(roundf(3.0f * sw));
    const int64_t xi = f2i(roundf(x)), yi = f2i(roundf(y));
    float hist[ORI_BINS] = {0};
    for (int64_t dy = -r; dy <= r; ++dy) {
        for (int64_t dx = -r; dx <= r; ++dx) {
            const int64_t px = xi + dx, py = yi + dy;
            if (px < 1 || py < 1 || px >= w - 1 || py >= h - 1) continue;
            const float m = mag[py * w + px], at = ang[py * w + px];
            const float fx = (float)px - x, fy = (float)py - y;
            const float wgt = f_exp(-(fx * fx + fy * fy) / (2.0f * sw * sw), cr);
            const float a = rem_euclid(at, TWO_PI_F);
            const float bf = roundf(a / TWO_PI_F * (float)ORI_BINS);
            const uint64_t bin = (uint64_t)(bf < 0.0f ? 0 : f2i(bf)) % ORI_BINS;
            hist[bin] += wgt * m;
        }
    }
    for (int it = 0; it < 6; ++it) {
        float prev[ORI_BINS];
        memcpy(prev, hist, sizeof prev);
        for (int i = 0; i < ORI_BINS; ++i)
            hist[i] = (prev[(i + ORI_BINS - 1) % ORI_BINS] + prev[i] + prev[(i + 1) % ORI_BINS]) / 3.0f;
    }
    float mx = 0.0f;
    for (int i = 0; i < ORI_BINS; ++i) mx = fmaxf(mx, hist[i]);
    if (mx <= 0.0f) return 0;
    int64_t n = 0;
    for (int i = 0; i < ORI_BINS; ++i) {
        const float l = hist[(i + ORI_BINS - 1) % ORI_BINS], c = hist[i], rr = hist[(i + 1) % ORI_BINS];
        if (c >= 0.8f * mx && c > l && c > rr) {
            const float off = 0.5f * (l - rr) / (l - 2.0f * c + rr);
            out[n++] = rem_euclid(((float)i + off) / (float)ORI_BINS * TWO_PI_F, TWO_PI_F);
        }
    }
    return n;
}

/* describe_with, features.rs:521-592: 4x4 cells of width 3 sigma rotated to
 * the keypoint's angle, 8 orientation bins each; Gaussian weight exp(-(u^2 +
 * v^2) / 8) in cell units; trilinear interpolation (two spatial axes, one
 * orientation axis); normalise, clip at 0.2, normalise. */
void orc_describe_grad(const float *mag, const float *ang, int64_t w, int64_t h, float x, float y, float sigma,
                       float angle, int cr, float *hist) {
    const int NC = 4, NO = 8;
    const float cell = 3.0f * sigma;
    const int64_t r = f2i(roundf(cell * SQRT2_F * ((float)NC + 1.0f) * 0.5f));
    const float c = f_cos(angle, cr), sn = f_sin(angle, cr);
    const int64_t xi = f2i(roundf(x)), yi = f2i(roundf(y));
    for (int i = 0; i < DESC_LEN; ++i) hist[i] = 0.0f;
    for (int64_t dy = -r; dy <= r; ++dy) {
        for (int64_t dx = -r; dx <= r; ++dx) {
            const int64_t px = xi + dx, py = yi + dy;
            if (px < 1 || py < 1 || px >= w - 1 || py >= h - 1) continue;
            const float fx = (float)px - x, fy = (float)py - y;
            const float u = (c * fx + sn * fy) / cell;
            const float v = (-sn * fx + c * fy) / cell;
            const float bu = u + (float)NC / 2.0f - 0.5f, bv = v + (float)NC / 2.0f - 0.5f;
            if (bu <= -1.0f || bv <= -1.0f || bu >= (float)NC || bv >= (float)NC) continue;
            const float m0 = mag[py * w + px], at = ang[py * w + px];
            const float ori = rem_euclid(at - angle, TWO_PI_F);
            const float bo = ori / TWO_PI_F * (float)NO;
            const float wgt = f_exp(-(u * u + v * v) / (2.0f * 4.0f), cr);
            const float m = m0 * wgt;
            const float u0 = floorf(bu), v0 = floorf(bv), o0 = floorf(bo);
            const float du = bu - u0, dv = bv - v0, dob = bo - o0;
            const int64_t iv0 = f2i(v0), iu0 = f2i(u0);
            const uint64_t io0 = (uint64_t)(o0 < 0.0f ? 0 : f2i(o0));
            for (int a = 0; a < 2; ++a) {
                const int64_t iv = iv0 + a;
                const float wv = a ? dv : 1.0f - dv;
                if (iv < 0 || iv >= NC) continue;
                for (int b = 0; b < 2; ++b) {
                    const int64_t iu = iu0 + b;
                    const float wu = b ? du : 1.0f - du;
                    if (iu < 0 || iu >= NC) continue;
                    for (int e = 0; e < 2; ++e) {
                        const uint64_t io = (io0 + (uint64_t)e) % (uint64_t)NO;
                        const float wo = e ? dob : 1.0f - dob;
                        hist[(iv * NC + iu) * NO + (int64_t)io] += m * wv * wu * wo;
                    }
                }
            }
        }
    }
    for (int pass = 0; pass < 2; ++pass) {
        float n2 = -0.0f;
        for (int i = 0; i < DESC_LEN; ++i) n2 += hist[i] * hist[i];
        const float n = sqrtf(n2);
        if (n > 0.0f)
            for (int i = 0; i < DESC_LEN; ++i) hist[i] /= n;
        if (pass == 0)
            for (int i = 0; i < DESC_LEN; ++i) hist[i] = fminf(hist[i], 0.2f);
    }
}

/* describe(img, x, y, sigma, angle), features.rs:509-519 */
void orc_describe(const float *img, int64_t w, int64_t h, float x, float y, float sigma, float angle, int cr,
                  float *out) {
    float *mag = (float *)malloc(sizeof(float) * (size_t)(w * h));
    float *ang = (float *)malloc(sizeof(float) * (size_t)(w * h));
    grad_table(img, w, h, cr, mag, ang);
    orc_describe_grad(mag, ang, w, h, x, y, sigma, angle, cr, out);
    free(mag);
    free(ang);
}

/* dominant_orientations(img, x, y, sigma), features.rs:314-323 */
int64_t orc_dominant_orientations(const float *img, int64_t w, int64_t h, float x, float y, float sigma, int cr,
                                  float *out) {
    float *mag = (float *)malloc(sizeof(float) * (size_t)(w * h));
    float *ang = (float *)malloc(sizeof(float) * (size_t)(w * h));
    grad_table(img, w, h, cr, mag, ang);
    const int64_t n = orc_orientations(mag, ang, w, h, x, y, sigma, cr, out);
    free(mag);
    free(ang);
    return n;
}

/* ---- detection ---------------------------------------------------------- */

typedef struct {
    int64_t xi, yi, layer;
    float x, y, s, value;
} refined;

/* nalgebra 0.33 Matrix3::try_inverse (cofactor formula). Returns 0 when the
 * determinant is exactly zero. m is row-major. */
static int inverse3(const float *m, float *o) {
    const float m11 = m[0], m12 = m[1], m13 = m[2];
    const float m21 = m[3], m22 = m[4], m23 = m[5];
    const float m31 = m[6], m32 = m[7], m33 = m[8];
    const float minor_m12_m23 = m22 * m33 - m32 * m23;
    const float minor_m11_m23 = m21 * m33 - m31 * m23;
    const float minor_m11_m22 = m21 * m32 - m31 * m22;
    const float det = m11 * minor_m12_m23 - m12 * minor_m11_m23 + m13 * minor_m11_m22;
    if (det == 0.0f) return 0;
    o[0] = minor_m12_m23 / det;
    o[1] = (m13 * m32 - m33 * m12) / det;
    o[2] = (m12 * m23 - m22 * m13) / det;
    o[3] = -minor_m11_m23 / det;
    o[4] = (m11 * m33 - m31 * m13) / det;
    o[5] = (m13 * m21 - m23 * m11) / det;
    o[6] = minor_m11_m22 / det;
    o[7] = (m12 * m31 - m32 * m11) / det;
    o[8] = (m11 * m22 - m21 * m12) / det;
    return 1;
}

/* refine_extremum, features.rs:431-484: delta = -H^-1 g of the 3-D quadratic
 * fit; moves to the neighbouring sample (at most 5 times) while a component
 * of delta exceeds 0.5. dog: layers of w x h. */
static int refine_extremum(const float *const *dog, int64_t w, int64_t h, int64_t x, int64_t y, int64_t l, int64_t s,
                           refined *out) {
#define AT(L, X, Y) dog[(L)][(Y) * w + (X)]
    for (int it = 0; it < 5; ++it) {
        const float v = AT(l, x, y);
        const float g[3] = {0.5f * (AT(l, x + 1, y) - AT(l, x - 1, y)), 0.5f * (AT(l, x, y + 1) - AT(l, x, y - 1)),
                            0.5f * (AT(l + 1, x, y) - AT(l - 1, x, y))};
        const float hxx = AT(l, x + 1, y) + AT(l, x - 1, y) - 2.0f * v;
        const float hyy = AT(l, x, y + 1) + AT(l, x, y - 1) - 2.0f * v;
        const float hss = AT(l + 1, x, y) + AT(l - 1, x, y) - 2.0f * v;
        const float hxy =
            0.25f * (AT(l, x + 1, y + 1) - AT(l, x - 1, y + 1) - AT(l, x + 1, y - 1) + AT(l, x - 1, y - 1));
        const float hxs = 0.25f * (AT(l + 1, x + 1, y) - AT(l + 1, x - 1, y) - AT(l - 1, x + 1, y) + AT(l - 1, x - 1, y));
        const float hys = 0.25f * (AT(l + 1, x, y + 1) - AT(l + 1, x, y - 1) - AT(l - 1, x, y + 1) + AT(l - 1, x, y - 1));
        const float hm[9] = {hxx, hxy, hxs, hxy, hyy, hys, hxs, hys, hss};
        float inv[9];
        if (!inverse3(hm, inv)) return 0;
        float d[3];
        for (int i = 0; i < 3; ++i) {
            /* matrix x vector: columns added in order (gemv) */
            float acc = inv[i * 3 + 0] * g[0];
            acc = acc + inv[i * 3 + 1] * g[1];
            acc = acc + inv[i * 3 + 2] * g[2];
            d[i] = -acc;
        }
        if (fabsf(d[0]) <= 0.5f && fabsf(d[1]) <= 0.5f && fabsf(d[2]) <= 0.5f) {
            out->xi = x;
            out->yi = y;
            out->layer = l;
            out->x = (float)x + d[0];
            out->y = (float)y + d[1];
            out->s = (float)l + d[2];
            out->value = v + 0.5f * (g[0] * d[0] + g[1] * d[1] + g[2] * d[2]);
            return 1;
        }
        if (!(isfinite(d[0]) && isfinite(d[1]) && isfinite(d[2]))) return 0;
        const int64_t nx = x + f2i(roundf(d[0])), ny = y + f2i(roundf(d[1])), nl = l + f2i(roundf(d[2]));
        if (nx < 1 || ny < 1 || nl < 1 || nx >= w - 1 || ny >= h - 1 || nl > s) return 0;
        x = nx;
        y = ny;
        l = nl;
    }
    return 0;
#undef AT
}

typedef struct {
    orc_kp kp;
    float desc[DESC_LEN];
} feat;

typedef struct {
    feat *v;
    int64_t n, cap;
} featvec;

static void fv_push(featvec *f, const feat *x) {
    if (f->n == f->cap) {
        f->cap = f->cap ? f->cap * 2 : 256;
        f->v = (feat *)realloc(f->v, sizeof(feat) * (size_t)f->cap);
    }
    f->v[f->n++] = *x;
}

typedef struct {
    float key; /* |response| */
    int64_t idx;
} sort_item;

static int cmp_desc_abs(const void *a, const void *b) {
    const sort_item *x = (const sort_item *)a, *y = (const sort_item *)b;
    if (x->key > y->key) return -1;
    if (x->key < y->key) return 1;
    return x->idx < y->idx ? -1 : x->idx > y->idx; /* stable */
}

/* detect_core, features.rs:650-781. Keypoints in input-image pixels. */
static void detect_core(const float *img, int64_t w0, int64_t h0, const orc_det_cfg *cfg, float in_sigma, int cr,
                        featvec *outv) {
    const int64_t s = cfg->scales;
    const float kstep = powf(2.0f, 1.0f / (float)s);
    float sb = cfg->sigma0 * cfg->sigma0 - in_sigma * in_sigma;
    if (!(sb >= 0.01f)) sb = 0.01f;
    int64_t w = w0, h = h0;
    float *base = (float *)malloc(sizeof(float) * (size_t)(w * h));
    orc_gaussian_blur(img, w, h, sqrtf(sb), base);
    featvec out = {0};
    const int64_t ng = s + 3;
    for (int64_t o = 0; o < cfg->octaves; ++o) {
        if (w < 16 || h < 16) break;
        const int64_t np = w * h;
        float *gauss = (float *)malloc(sizeof(float) * (size_t)(np * ng));
        float *dogb = (float *)malloc(sizeof(float) * (size_t)(np * (ng - 1)));
        memcpy(gauss, base, sizeof(float) * (size_t)np);
        for (int64_t i = 1; i < ng; ++i) {
            const float prev = cfg->sigma0 * powi_f(kstep, (int)(i - 1));
            const float cur = prev * kstep;
            orc_gaussian_blur(gauss + (i - 1) * np, w, h, sqrtf(cur * cur - prev * prev), gauss + i * np);
        }
        for (int64_t i = 0; i + 1 < ng; ++i)
            for (int64_t p = 0; p < np; ++p) dogb[i * np + p] = gauss[(i + 1) * np + p] - gauss[i * np + p];
        const float *dog[64];
        for (int64_t i = 0; i + 1 < ng; ++i) dog[i] = dogb + i * np;
        float *gmag = (float *)malloc(sizeof(float) * (size_t)(np * (s + 1)));
        float *gang = (float *)malloc(sizeof(float) * (size_t)(np * (s + 1)));
        for (int64_t l = 1; l <= s; ++l) grad_table(gauss + l * np, w, h, cr, gmag + l * np, gang + l * np);
        const float scale = (float)((uint64_t)1 << o);
        const float er1 = cfg->edge_ratio + 1.0f;
        const float edge_thr = er1 * er1 / cfg->edge_ratio;
        for (int64_t l = 1; l <= s; ++l) {
            const float *d0 = dog[l - 1], *d1 = dog[l], *d2 = dog[l + 1];
            for (int64_t y = 1; y < h - 1; ++y) {
                for (int64_t x = 1; x < w - 1; ++x) {
                    const float v = d1[y * w + x];
                    if (fabsf(v) < cfg->contrast) continue;
                    int is_max = 1, is_min = 1;
                    const float *ds[3] = {d0, d1, d2};
                    for (int k = 0; k < 3 && (is_max || is_min); ++k)
                        for (int64_t yy = y - 1; yy <= y + 1 && (is_max || is_min); ++yy)
                            for (int64_t xx = x - 1; xx <= x + 1; ++xx) {
                                if (k == 1 && xx == x && yy == y) continue;
                                const float u = ds[k][yy * w + xx];
                                is_max &= v > u;
                                is_min &= v < u;
                                if (!is_max && !is_min) break;
                            }
                    if (!(is_max || is_min)) continue;
                    refined rf;
                    if (!refine_extremum(dog, w, h, x, y, l, s, &rf)) continue;
                    if (fabsf(rf.value) < cfg->contrast) continue;
                    const float *d = dog[rf.layer];
                    const int64_t xi = rf.xi, yi = rf.yi;
                    const float c = d[yi * w + xi];
                    const float dxx = d[yi * w + xi + 1] + d[yi * w + xi - 1] - 2.0f * c;
                    const float dyy = d[(yi + 1) * w + xi] + d[(yi - 1) * w + xi] - 2.0f * c;
                    const float dxy = 0.25f * (d[(yi + 1) * w + xi + 1] - d[(yi + 1) * w + xi - 1] -
                                               d[(yi - 1) * w + xi + 1] + d[(yi - 1) * w + xi - 1]);
                    const float tr = dxx + dyy;
                    const float det = dxx * dyy - dxy * dxy;
                    if (det <= 0.0f || tr * tr / det >= edge_thr) continue;
                    const float sig_oct = cfg->sigma0 * f_pow(kstep, rf.s, cr);
                    const float *gm = gmag + rf.layer * np, *ga = gang + rf.layer * np;
                    float angles[ORI_BINS];
                    const int64_t na = orc_orientations(gm, ga, w, h, rf.x, rf.y, sig_oct, cr, angles);
                    for (int64_t a = 0; a < na; ++a) {
                        feat f;
                        f.kp.x = rf.x * scale;
                        f.kp.y = rf.y * scale;
                        f.kp.sigma = sig_oct * scale;
                        f.kp.response = rf.value;
                        f.kp.angle = angles[a];
                        orc_describe_grad(gm, ga, w, h, rf.x, rf.y, sig_oct, angles[a], cr, f.desc);
                        fv_push(&out, &f);
                    }
                }
            }
        }
        /* base = gauss[s].downsample() (even pixels) */
        const int64_t nw = w / 2, nh = h / 2;
        float *nb = (float *)malloc(sizeof(float) * (size_t)(nw * nh + 1));
        for (int64_t y = 0; y < nh; ++y)
            for (int64_t x = 0; x < nw; ++x) nb[y * nw + x] = gauss[s * np + (2 * y) * w + 2 * x];
        free(base);
        base = nb;
        w = nw;
        h = nh;
        free(gauss);
        free(dogb);
        free(gmag);
        free(gang);
    }
    free(base);
    /* stable sort by |response|, descending; truncate */
    sort_item *it = (sort_item *)malloc(sizeof(sort_item) * (size_t)(out.n + 1));
    for (int64_t i = 0; i < out.n; ++i) it[i].key = fabsf(out.v[i].kp.response), it[i].idx = i;
    qsort(it, (size_t)out.n, sizeof(sort_item), cmp_desc_abs);
    const int64_t keep = out.n < cfg->max_features ? out.n : cfg->max_features;
    for (int64_t i = 0; i < keep; ++i) fv_push(outv, &out.v[it[i].idx]);
    free(it);
    free(out.v);
}

/* detect_and_describe, features.rs:594-648: the input-size detection, and,
 * for small images that found fewer than the target, features of the 2x
 * upsampled image that are not at the place of an original one (1 px, scale
 * ratio 1.5), in response order. Returns the feature count; writes at most
 * cap keypoints (5 floats) and descriptors. */
int64_t orc_detect_and_describe(const float *img, int64_t w, int64_t h, const orc_det_cfg *cfg, int cr, float *kps,
                                float *desc, int64_t cap) {
    featvec feats = {0};
    detect_core(img, w, h, cfg, 0.5f, cr, &feats);
    const int64_t big = w > h ? w : h;
    if (!(cfg->upscale_below == 0 || big >= cfg->upscale_below || feats.n >= cfg->max_features ||
          (!cfg->upscale_fill && feats.n * 2 >= cfg->max_features))) {
        float *up = (float *)malloc(sizeof(float) * (size_t)(4 * w * h));
        orc_upsample2(img, w, h, up);
        featvec extra = {0};
        detect_core(up, 2 * w, 2 * h, cfg, 1.0f, cr, &extra);
        free(up);
        const int64_t need = cfg->max_features - feats.n;
        const float cell = 4.0f;
        const int64_t gw = f2i((float)w / cell) + 2, gh = f2i((float)h / cell) + 2;
        const int64_t n0 = feats.n;
        int64_t added = 0;
        for (int64_t e = 0; e < extra.n && added < need; ++e) {
            feat f = extra.v[e];
            f.kp.x = f.kp.x / 2.0f - 0.25f;
            f.kp.y = f.kp.y / 2.0f - 0.25f;
            f.kp.sigma /= 2.0f;
            const int64_t kx = clampi(f2i(floorf(f.kp.x / cell)), -1, gw - 1);
            const int64_t ky = clampi(f2i(floorf(f.kp.y / cell)), -1, gh - 1);
            int dup = 0;
            for (int64_t q = 0; q < n0 && !dup; ++q) {
                const orc_kp *o = &feats.v[q].kp;
                const int64_t ox = clampi(f2i(floorf(o->x / cell)), -1, gw - 1);
                const int64_t oy = clampi(f2i(floorf(o->y / cell)), -1, gh - 1);
                if (ox < kx - 1 || ox > kx + 1 || oy < ky - 1 || oy > ky + 1) continue;
                const float rr = fmaxf(o->sigma / f.kp.sigma, f.kp.sigma / o->sigma);
                if (hypotf(o->x - f.kp.x, o->y - f.kp.y) <= 1.0f && rr <= 1.5f) dup = 1;
            }
            if (!dup) {
                fv_push(&feats, &f);
                ++added;
            }
        }
        free(extra.v);
    }
    const int64_t n = feats.n;
    for (int64_t i = 0; i < n && i < cap; ++i) {
        if (kps) memcpy(kps + 5 * i, &feats.v[i].kp, sizeof(orc_kp));
        if (desc) memcpy(desc + DESC_LEN * i, feats.v[i].desc, sizeof(float) * DESC_LEN);
    }
    free(feats.v);
    return n;
}
