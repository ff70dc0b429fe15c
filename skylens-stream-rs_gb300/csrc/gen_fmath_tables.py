"""Writes fmath_tables.h: the float-float constants of fmath_cr.h
(2^(j/64) for j = 0..63, atan(j/16) for j = 0..16, pi / 2, pi, and the
Cody-Waite split of ln2 / 64), each the exact value rounded to a float `hi`
plus the rounded remainder `lo`, from 60-digit decimal arithmetic."""
import math
import os
import struct
from decimal import Decimal, getcontext

getcontext().prec = 60


def f32(x: Decimal) -> float:
    v = struct.unpack("f", struct.pack("f", float(x)))[0]
    best = v
    for c in (math.nextafter(v, math.inf), math.nextafter(v, -math.inf)):
        c = struct.unpack("f", struct.pack("f", c))[0]
        if abs(Decimal(c) - x) < abs(Decimal(best) - x):
            best = c
    return best


def split(x: Decimal):
    hi = f32(x)
    return hi, f32(x - Decimal(hi))


def atan(x: Decimal) -> Decimal:
    k = 0
    while abs(x) > Decimal("0.1"):  # atan(x) = 2 atan(x / (1 + sqrt(1 + x^2)))
        x = x / (1 + (1 + x * x).sqrt())
        k += 1
    s, term, n, sign, x2 = Decimal(0), x, 1, 1, x * x
    while True:
        t = term / n
        if abs(t) < Decimal(10) ** -58:
            break
        s += sign * t
        term *= x2
        n += 2
        sign = -sign
    return s * (2 ** k)


def hx(v: float) -> str:
    return "0.0f" if v == 0 else float(v).hex() + "f"


def main():
    exp_tab = [split(Decimal(2) ** (Decimal(j) / 64)) for j in range(64)]
    atan_tab = [split(atan(Decimal(j) / 16)) for j in range(17)]
    pi = 4 * atan(Decimal(1))
    L = Decimal(2).ln() / 64
    m, e = math.frexp(float(L))
    L1 = math.floor(m * 2 ** 11) / 2 ** 11 * 2 ** e  # 11 significant bits: n * L1 is exact for |n| < 2^13
    L2 = f32(L - Decimal(L1))
    L3 = f32(L - Decimal(L1) - Decimal(L2))
    lines = ["// Generated by gen_fmath_tables.py: float-float constants of fmath_cr.h.", "#pragma once", "",
             "// 2^(j/64), j = 0..63: hi, lo",
             "#define SLM_EXP2_TABLE \\"]
    lines += [f"    {hx(h)}, {hx(l)}," + (" \\" if j < 63 else "") for j, (h, l) in enumerate(exp_tab)]
    lines += ["", "// atan(j/16), j = 0..16: hi, lo", "#define SLM_ATAN_TABLE \\"]
    lines += [f"    {hx(h)}, {hx(l)}," + (" \\" if j < 16 else "") for j, (h, l) in enumerate(atan_tab)]
    pio2, pi1 = split(pi / 2), split(pi)
    lines += ["", f"#define SLM_PIO2_HI {hx(pio2[0])}", f"#define SLM_PIO2_LO {hx(pio2[1])}",
              f"#define SLM_PI_HI {hx(pi1[0])}", f"#define SLM_PI_LO {hx(pi1[1])}",
              "// ln2 / 64 = L1 + L2 + L3 (L1: 11 significant bits), 64 / ln2",
              f"#define SLM_LN2_64_1 {hx(L1)}", f"#define SLM_LN2_64_2 {hx(L2)}", f"#define SLM_LN2_64_3 {hx(L3)}",
              f"#define SLM_INV_LN2_64 {hx(f32(Decimal(64) / Decimal(2).ln()))}", ""]
    here = os.path.dirname(os.path.abspath(__file__))
    open(os.path.join(here, "fmath_tables.h"), "w").write("\n".join(lines))


if __name__ == "__main__":
    main()
