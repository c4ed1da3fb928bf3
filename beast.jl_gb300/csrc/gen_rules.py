"""Generate rules_gen.h: the quadrature tables compiled into libbeastgpu.

* symmetric triangle rules exact to degree 1..8 and 10 (the `trgauss(n)` rules of the
  default strategies: far 2/3, near 6/7, excitation 8, far field 10).  Structure and
  starting values are those of the published symmetric (Dunavant 1985) rules; the orbit
  parameters are refined here by Gauss-Newton on the moment equations (numpy).
* Gauss-Legendre nodes/weights on [0,1] for n = 1..20 (Sauter-Schwab orders).

Points are barycentric (u, v) of x = u v1 + v v2 + (1-u-v) v3; weights sum to 1.
usage: python gen_rules.py > rules_gen.h
"""
import math
import sys

import numpy as np

SPECS = {
    1: [(0, 0, 0, 1.0)],
    2: [(1, 0.166666666666667, 0, 1 / 3)],
    3: [(0, 0, 0, -0.5625), (1, 0.2, 0, 0.520833333333333)],
    4: [(1, 0.445948490915965, 0, 0.223381589678011), (1, 0.091576213509771, 0, 0.109951743655322)],
    5: [(0, 0, 0, 0.225), (1, 0.470142064105115, 0, 0.132394152788506),
        (1, 0.101286507323456, 0, 0.125939180544827)],
    6: [(1, 0.249286745170910, 0, 0.116786275726379), (1, 0.063089014491502, 0, 0.050844906370207),
        (2, 0.053145049844817, 0.310352451033784, 0.082851075618374)],
    7: [(0, 0, 0, -0.149570044467682), (1, 0.260345966079040, 0, 0.175615257433208),
        (1, 0.065130102902216, 0, 0.053347235608838),
        (2, 0.048690315425316, 0.312865496004874, 0.077113760890257)],
    8: [(0, 0, 0, 0.144315607677787), (1, 0.459292588292723, 0, 0.095091634267285),
        (1, 0.170569307751760, 0, 0.103217370534718), (1, 0.050547228317031, 0, 0.032458497623198),
        (2, 0.008394777409958, 0.263112829634638, 0.027230314174435)],
    10: [(0, 0, 0, 0.090817990382754), (1, 0.485577633383657, 0, 0.036725957756467),
         (1, 0.109481575485037, 0, 0.045321059435528),
         (2, 0.141707219414880, 0.307939838764121, 0.072757916845420),
         (2, 0.025003534762686, 0.246672560639903, 0.028327242531057),
         (2, 0.009540815400299, 0.066803251012200, 0.009421666963733)],
}


def orbit(t, a, b):
    if t == 0:
        return [(1 / 3, 1 / 3, 1 / 3)]
    if t == 1:
        c = 1 - 2 * a
        return [(a, a, c), (a, c, a), (c, a, a)]
    c = 1 - a - b
    return [(a, b, c), (b, a, c), (a, c, b), (c, a, b), (b, c, a), (c, b, a)]


def unpack(spec, x):
    out, k = [], 0
    for (t, _, _, _) in spec:
        w = x[k]; k += 1
        a = b = 0.0
        if t >= 1:
            a = x[k]; k += 1
        if t == 2:
            b = x[k]; k += 1
        out.append((t, a, b, w))
    return out


def residual(spec, x, deg):
    orbs = unpack(spec, x)
    res = []
    for p in range(deg + 1):
        for q in range(deg + 1 - p):
            s = sum(w * sum(P[0] ** p * P[1] ** q for P in orbit(t, a, b)) for (t, a, b, w) in orbs)
            res.append(s - 2.0 * math.factorial(p) * math.factorial(q) / math.factorial(p + q + 2))
    return np.array(res)


def refine(deg):
    spec = SPECS[deg]
    x = []
    for (t, a, b, w) in spec:
        x.append(w)
        if t >= 1:
            x.append(a)
        if t == 2:
            x.append(b)
    x = np.array(x, dtype=np.float64)
    for _ in range(50):
        r = residual(spec, x, deg)
        if np.abs(r).max() < 1e-17:
            break
        J = np.zeros((len(r), len(x)))
        for j in range(len(x)):
            h = 1e-7
            xp, xm = x.copy(), x.copy()
            xp[j] += h
            xm[j] -= h
            J[:, j] = (residual(spec, xp, deg) - residual(spec, xm, deg)) / (2 * h)
        x = x - np.linalg.lstsq(J, r, rcond=None)[0]
    pts = []
    for (t, a, b, w) in unpack(spec, x):
        for P in orbit(t, a, b):
            pts.append((P[0], P[1], w))
    return pts


def main(out=sys.stdout):
    w = out.write
    w("// generated by gen_rules.py -- do not edit\n#pragma once\n")
    degs = sorted(SPECS)
    rules = {d: refine(d) for d in degs}
    maxn = max(len(r) for r in rules.values())
    w(f"#define BEAST_TRI_MAXDEG 10\n#define BEAST_TRI_MAXPTS {maxn}\n")
    # offsets by degree (index 0..10), degree 9 maps to the degree-10 rule
    off, cnt, flat = [], [], []
    for d in range(11):
        dd = d if d in rules else (10 if d == 9 else 1)
        off.append(len(flat))
        cnt.append(len(rules[dd]))
        flat += rules[dd]
    w("static const int beast_tri_off[11] = {" + ",".join(map(str, off)) + "};\n")
    w("static const int beast_tri_cnt[11] = {" + ",".join(map(str, cnt)) + "};\n")
    w(f"static const double beast_tri_pts[{len(flat)}][3] = {{\n")
    for (u, v, wt) in flat:
        w(f"  {{{float(u)!r}, {float(v)!r}, {float(wt)!r}}},\n")
    w("};\n")
    w("#define BEAST_GL_MAXN 20\n")
    goff, gflat = [0], []
    for n in range(1, 21):
        x, wt = np.polynomial.legendre.leggauss(n)
        for xi, wi in zip(x, wt):
            gflat.append(((xi + 1) / 2, wi / 2))
        goff.append(len(gflat))
    w("static const int beast_gl_off[21] = {" + ",".join(map(str, goff[:21])) + "};\n")
    w(f"static const double beast_gl_pts[{len(gflat)}][2] = {{\n")
    for (x, wt) in gflat:
        w(f"  {{{float(x)!r}, {float(wt)!r}}},\n")
    w("};\n")


if __name__ == "__main__":
    main()
