"""Generate dftables.h: constants of the double-float (FP32 pair) arithmetic in dfloat.h.

* pi/32 split into three floats (p0 + p1 + p2, Cody-Waite reduction) and 32/pi;
* sin(m pi/32), cos(m pi/32) for m = 0..63 as float pairs (hi + lo);
* 1/(4 pi) as a float pair.

Values come from sympy at 60 digits; a pair is hi = fl32(x), lo = fl32(x - hi).
usage: python gen_dftables.py > dftables.h
"""
import numpy as np
import sympy as sp

DIGITS = 60


def f32(x):
    return float(np.float32(float(x)))


def pair(x):
    hi = f32(x)
    lo = f32(sp.N(x - sp.Float(hi, DIGITS), DIGITS))
    return hi, lo


def lit(v):
    return f"{np.float32(v).item():.9e}f"


def main():
    pi = sp.pi.evalf(DIGITS)
    q = pi / 32
    p0 = f32(q)
    p1 = f32(sp.N(q - sp.Float(p0, DIGITS), DIGITS))
    p2 = f32(sp.N(q - sp.Float(p0, DIGITS) - sp.Float(p1, DIGITS), DIGITS))
    i4 = pair(1 / (4 * pi))
    out = ["// generated by gen_dftables.py -- do not edit",
           "#pragma once",
           "// pi/32 = DF_PI32_0 + DF_PI32_1 + DF_PI32_2 (Cody-Waite split); 32/pi rounded",
           f"#define DF_PI32_0 {lit(p0)}",
           f"#define DF_PI32_1 {lit(p1)}",
           f"#define DF_PI32_2 {lit(p2)}",
           f"#define DF_32_OVER_PI {lit(f32(32 / pi))}",
           "// 1/(4 pi) as hi + lo",
           f"#define DF_I4PI_HI {lit(i4[0])}",
           f"#define DF_I4PI_LO {lit(i4[1])}",
           "// sin(m pi/32) hi, lo, cos(m pi/32) hi, lo for m = 0..63",
           "#define DF_SINCOS_TABLE_INIT { \\"]
    for m in range(64):
        a = m * pi / 32
        s, c = pair(sp.sin(a).evalf(DIGITS)), pair(sp.cos(a).evalf(DIGITS))
        sep = "," if m < 63 else ""
        out.append(f"  {{{lit(s[0])}, {lit(s[1])}, {lit(c[0])}, {lit(c[1])}}}{sep} \\")
    out.append("}")
    print("\n".join(out))


if __name__ == "__main__":
    main()
