// fmath_cr.h — correctly rounded float exp and atan2 without FP64 in the
// common case, for the descriptor producer's per-pixel and per-sample calls.
//
// Each function evaluates its result as a float-float pair (hi + lo, about 46
// significant bits: table-driven argument reduction and short polynomials,
// every product made exact with fmaf), rounds hi + lo once to float, and
// checks that the float-float value lies far enough from the rounding
// boundary on its side of that float for the error bound to settle the
// rounding (Ziv's test). Then the float is the correctly rounded value, which
// is also what the double function rounded to float gives. Otherwise (a few
// calls in 10^5, and arguments outside the reduced ranges) the double function
// rounded to float is returned. Either way the result equals
// (float)exp((double)x) and (float)atan2((double)y, (double)x) except where
// that double result itself lies within a double ulp of a float rounding
// boundary.
//
// The same code compiles for the host (tests check it against the double
// functions over every float in exp's range and over random atan2 arguments).
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#include "fmath_tables.h"

#ifdef __CUDACC__
#define SLM_FM __host__ __device__ __forceinline__
#else
#define SLM_FM static inline
#endif

#ifdef __CUDACC__
__device__ static const float slm_fm_exp2_dev[128] = {SLM_EXP2_TABLE};
__device__ static const float slm_fm_atan_dev[34] = {SLM_ATAN_TABLE};
#endif
static const float slm_fm_exp2_host[128] = {SLM_EXP2_TABLE};
static const float slm_fm_atan_host[34] = {SLM_ATAN_TABLE};

#ifdef __CUDA_ARCH__
#define SLM_FM_EXP2 slm_fm_exp2_dev
#define SLM_FM_ATAN slm_fm_atan_dev
#else
#define SLM_FM_EXP2 slm_fm_exp2_host
#define SLM_FM_ATAN slm_fm_atan_host
#endif

// s + e = a + b exactly
SLM_FM void slm_two_sum(float a, float b, float *s, float *e) {
    const float t = a + b;
    const float bb = t - a;
    *e = (a - (t - bb)) + (b - bb);
    *s = t;
}

// p + e = a * b exactly
SLM_FM void slm_two_prod(float a, float b, float *p, float *e) {
    const float t = a * b;
    *e = fmaf(a, b, -t);
    *p = t;
}

SLM_FM uint32_t slm_fbits(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}

SLM_FM float slm_bitsf(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}

// Rounds the float-float value hi + lo (|lo| well below ulp(hi)) to float;
// *ok is set when no float rounding boundary lies within rel_err * |hi + lo|
// of it, so that the rounding is that of every value within that distance.
SLM_FM float slm_round_checked(float hi, float lo, float rel_err, bool *ok) {
    const float f = hi + lo;
    // d = (hi + lo) - f: hi - f is exact (f is hi or a neighbour of it)
    const float d = (hi - f) + lo;
    const uint32_t u = slm_fbits(f) & 0x7fffffffu;
    if (u == 0 || u >= 0x7f000000u) {  // zero, huge, inf or NaN: let the caller fall back
        *ok = false;
        return f;
    }
    // the gap to the neighbour on d's side of f (below f's magnitude the gap
    // halves at a power of two)
    const bool toward_zero = (d < 0.0f) == (f > 0.0f);
    const uint32_t un = toward_zero ? u - 1 : u + 1;
    const float gap = fabsf(slm_bitsf(u) - slm_bitsf(un));
    const float ad = fabsf(d);
    *ok = ad < 0.5f * gap - rel_err * fabsf(f) - 0x1p-24f * ad;
    return f;
}

// e^x
SLM_FM float slm_expf_cr(float x) {
    if (!(x > -87.0f && x < 88.0f)) return (float)exp((double)x);  // NaN, overflow, subnormal results
    const float nf = rintf(x * SLM_INV_LN2_64);
    const int n = (int)nf;
    // r = x - n ln2/64 as float-float (n * L1 exact, x - n * L1 exact)
    const float r1 = x - nf * SLM_LN2_64_1;
    float p2, e2;
    slm_two_prod(nf, SLM_LN2_64_2, &p2, &e2);
    float rh, t;
    slm_two_sum(r1, -p2, &rh, &t);
    float rl = (t - e2) - nf * SLM_LN2_64_3;
    slm_two_sum(rh, rl, &rh, &rl);
    // e^r - 1 = r + r^2/2 + r^3 (1/6 + r/24 + r^2/120), |r| <= ln2/128 (plus rounding of n)
    float sh, sl;
    slm_two_prod(rh, rh, &sh, &sl);
    sl = fmaf(2.0f * rh, rl, sl);
    const float c = sh * rh * fmaf(rh, fmaf(rh, 1.0f / 120.0f, 1.0f / 24.0f), 1.0f / 6.0f);
    float ah, al;
    slm_two_sum(0.5f * sh, fmaf(0.5f, sl, c), &ah, &al);
    float qh, qe;
    slm_two_sum(rh, ah, &qh, &qe);
    const float ql = qe + (rl + al);
    // 2^(j/64) (1 + q)
    const int j = n & 63;
    const float th = SLM_FM_EXP2[2 * j], tl = SLM_FM_EXP2[2 * j + 1];
    float ph, pl;
    slm_two_prod(th, qh, &ph, &pl);
    const float lo = tl + (pl + fmaf(th, ql, tl * qh));
    float vh, ve;
    slm_two_sum(th, ph, &vh, &ve);
    bool ok;
    float f = slm_round_checked(vh, ve + lo, 0x1p-41f, &ok);
    if (!ok) return (float)exp((double)x);
    return ldexpf(f, n >> 6);  // 2^(n >> 6) scaling: exact (results stay normal above e^-87)
}

// atan2(y, x)
SLM_FM float slm_atan2f_cr(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    const bool swap = ay > ax;
    const float mn = swap ? ax : ay, mx = swap ? ay : ax;
    // NaN, inf, zeros, and ratios whose float-float quotient could underflow
    if (!(mx < 0x1p100f) || !(mn > 0x1p-60f * mx) || !(mn > 0x1p-60f))
        return (float)atan2((double)y, (double)x);
    // t = mn / mx in float-float (the division's remainder is exact with fmaf)
    const float th = mn / mx;
    const float tl = fmaf(-th, mx, mn) / mx;
    // t = c + delta (1 + t c) with c = j / 16: atan(t) = atan(c) + atan(delta)
    const int j = (int)rintf(th * 16.0f);
    const float c = (float)j * 0.0625f;
    float nh, nl;
    slm_two_sum(th - c, tl, &nh, &nl);  // th - c is exact (Sterbenz, or c = 0)
    float pc, pe;
    slm_two_prod(th, c, &pc, &pe);
    float dh, de;
    slm_two_sum(1.0f, pc, &dh, &de);
    const float dl = de + fmaf(tl, c, pe);
    const float q1 = nh / dh;
    const float rem = fmaf(-q1, dh, nh) + (nl - q1 * dl);
    float eh, el;
    slm_two_sum(q1, rem / dh, &eh, &el);  // delta, |delta| <= 1/32
    // atan(delta) = delta + delta P, P = -z/3 + z^2 (1/5 - z/7 + z^2/9), z = delta^2
    float zh, zl;
    slm_two_prod(eh, eh, &zh, &zl);
    zl = fmaf(2.0f * eh, el, zl);
    const float z3 = zh / 3.0f;
    const float z3l = (fmaf(-z3, 3.0f, zh) + zl) / 3.0f;
    const float tail = zh * zh * fmaf(zh, fmaf(zh, 1.0f / 9.0f, -1.0f / 7.0f), 1.0f / 5.0f);
    float Ph, Pl;
    slm_two_sum(-z3, tail - z3l, &Ph, &Pl);
    float mh, ml;
    slm_two_prod(eh, Ph, &mh, &ml);
    ml = ml + fmaf(eh, Pl, el * Ph);
    float ah, al;
    slm_two_sum(eh, mh, &ah, &al);
    al = al + (el + ml);
    // + atan(c)
    const float Ah = SLM_FM_ATAN[2 * j], Al = SLM_FM_ATAN[2 * j + 1];
    float sh, se;
    slm_two_sum(Ah, ah, &sh, &se);
    float sl = se + (Al + al);
    // octants: pi/2 - a when |y| > |x|, pi - a when x < 0, the sign of y
    if (swap) {
        float u, ue;
        slm_two_sum(SLM_PIO2_HI, -sh, &u, &ue);
        sl = ue + (SLM_PIO2_LO - sl);
        sh = u;
    }
    if (x < 0.0f) {
        float u, ue;
        slm_two_sum(SLM_PI_HI, -sh, &u, &ue);
        sl = ue + (SLM_PI_LO - sl);
        sh = u;
    }
    if (y < 0.0f) {
        sh = -sh;
        sl = -sl;
    }
    bool ok;
    const float f = slm_round_checked(sh, sl, 0x1p-40f, &ok);
    if (!ok) return (float)atan2((double)y, (double)x);
    return f;
}
