// Host check of csrc/fmath_cr.h against the double functions rounded to
// float (built and run by tests/test_fmath.py). mode 0: every `stride`-th
// float in (-87, 88) for exp; mode 1: `count` pseudo-random atan2 arguments
// (pixel differences, uniform, arbitrary bit patterns, points on circles).
#include <cstdio>
#include <cstdlib>

#include "fmath_cr.h"

int main(int argc, char **argv) {
    const int mode = atoi(argv[1]);
    const unsigned long arg = strtoul(argv[2], nullptr, 10);
    unsigned long bad = 0, n = 0;
    if (mode == 0) {
        for (unsigned long u = 0; u < (1ul << 32); u += arg) {
            const float x = slm_bitsf((uint32_t)u);
            if (!(x > -87.0f && x < 88.0f)) continue;
            ++n;
            if (slm_fbits(slm_expf_cr(x)) != slm_fbits((float)exp((double)x))) {
                if (bad++ < 5) printf("exp(%a)\n", x);
            }
        }
    } else {
        unsigned long long s = 0x9E3779B97F4A7C15ull;
        auto nx = [&]() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; };
        for (unsigned long i = 0; i < arg; ++i) {
            float x, y;
            switch (nx() & 3) {
                case 0: x = ((int)(nx() % 511) - 255) / 255.0f; y = ((int)(nx() % 511) - 255) / 255.0f; break;
                case 1: x = (float)((double)(nx() >> 11) / 4503599627370496.0 - 1.0);
                        y = (float)((double)(nx() >> 11) / 4503599627370496.0 - 1.0); break;
                case 2: x = slm_bitsf((uint32_t)nx()); y = slm_bitsf((uint32_t)nx()); break;
                default: { const float a = (float)(nx() % 100000) * 6.2831853e-5f;
                           x = cosf(a); y = sinf(a) * ((nx() & 1) ? 1e-3f : 1.0f); }
            }
            const float got = slm_atan2f_cr(y, x), want = (float)atan2((double)y, (double)x);
            ++n;
            if (slm_fbits(got) != slm_fbits(want) && !(got != got && want != want)) {
                if (bad++ < 5) printf("atan2(%a, %a)\n", y, x);
            }
        }
    }
    printf("%lu %lu\n", bad, n);
    return bad != 0;
}
