"""Double-float (FP32 pair) arithmetic of csrc/dfloat.h, built for the host with g++ (the
header's products and sums are written so that host and device round alike), checked against
float64; and a device compile of the same header for sm_103a."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "beast.jl_gb300", "csrc")

HARNESS = r"""
#include "far_df.h"
#include <stdint.h>
using namespace dfl;
static df from(double x) { float h = (float)x; return {h, (float)(x - (double)h)}; }
static double to(df a) { return (double)a.hi + (double)a.lo; }
extern "C" {
void t_two(const float* a, const float* b, int64_t n, float* s, float* p) {
  for (int64_t i = 0; i < n; ++i) {
    df x = two_sum(a[i], b[i]), y = two_prod(a[i], b[i]);
    s[2 * i] = x.hi; s[2 * i + 1] = x.lo; p[2 * i] = y.hi; p[2 * i + 1] = y.lo;
  }
}
void t_ops(const double* a, const double* b, int64_t n, double* out) {  // add, mul, sqrt|a|, 1/a
  for (int64_t i = 0; i < n; ++i) {
    df x = from(a[i]), y = from(b[i]);
    out[4 * i] = to(add(x, y)); out[4 * i + 1] = to(mul(x, y));
    out[4 * i + 2] = to(dfl::sqrt(from(a[i] < 0 ? -a[i] : a[i]))); out[4 * i + 3] = to(rcp(x));
  }
}
void t_sincos(const double* th, int64_t n, double* s, double* c) {
  for (int64_t i = 0; i < n; ++i) { df a, b; dfl::sincos(from(th[i]), &a, &b); s[i] = to(a); c[i] = to(b); }
}
void t_sincos_tab(const double* th, int64_t n, double* s, double* c) {
  for (int64_t i = 0; i < n; ++i) { df a, b; sincos_tab(from(th[i]), sincos_tab_host, &a, &b); s[i] = to(a); c[i] = to(b); }
}
// the unnormalised forms the far cores use where pair products consume the result
void t_unnorm(const double* th, const double* a, const double* b, int64_t n, double* out) {
  for (int64_t i = 0; i < n; ++i) {
    df s, c;
    sincos_tab<false>(from(th[i]), sincos_tab_host, &s, &c);
    const double aa = a[i] < 0 ? -a[i] : a[i];
    out[5 * i] = to(s); out[5 * i + 1] = to(c); out[5 * i + 2] = to(rsqrtu(from(aa)));
    out[5 * i + 3] = to(addu(from(a[i]), from(b[i]))); out[5 * i + 4] = to(subu(from(a[i]), from(b[i])));
  }
}
void t_green(const double* R, const double* k, int64_t n, double* out) {
  for (int64_t i = 0; i < n; ++i) { df re, im; green(from(R[i]), from(k[i]), &re, &im); out[2 * i] = to(re); out[2 * i + 1] = to(im); }
}
// EFIE far block of one cell pair from double geometry (staged as the kernel would: centroid
// differences and rule points relative to the centroids in double, then split into pairs)
void t_efie_pair(const double* tv, const double* bv, int no, const double* uvo, const double* wo, int ni,
                 const double* uvi, const double* wi, double k, const double* al, const double* be, double* out,
                 int fast) {
  double cp[3], cq[3];
  for (int c = 0; c < 3; ++c) { cp[c] = (tv[c] + tv[3 + c] + tv[6 + c]) / 3; cq[c] = (bv[c] + bv[3 + c] + bv[6 + c]) / 3; }
  df d[3], tau[3][3], sig[3][3], xi[16][3], eta[16][3], w1[16], w2[16];
  for (int c = 0; c < 3; ++c) d[c] = from(cp[c] - cq[c]);
  for (int i = 0; i < 3; ++i)
    for (int c = 0; c < 3; ++c) { tau[i][c] = from(tv[3 * i + c] - cp[c]); sig[i][c] = from(bv[3 * i + c] - cq[c]); }
  for (int a = 0; a < no; ++a) {
    const double u = uvo[2 * a], v = uvo[2 * a + 1], w = 1 - u - v;
    for (int c = 0; c < 3; ++c) xi[a][c] = from(u * (tv[c] - cp[c]) + v * (tv[3 + c] - cp[c]) + w * (tv[6 + c] - cp[c]));
    w1[a] = from(wo[a]);
  }
  for (int b = 0; b < ni; ++b) {
    const double u = uvi[2 * b], v = uvi[2 * b + 1], w = 1 - u - v;
    for (int c = 0; c < 3; ++c) eta[b][c] = from(u * (bv[c] - cq[c]) + v * (bv[3 + c] - cq[c]) + w * (bv[6 + c] - cq[c]));
    w2[b] = from(wi[b]);
  }
  cdf z[9];
  if (fast && no == 3 && ni == 4) {
    df e2[4], wab[3][4];
    for (int b = 0; b < 4; ++b) e2[b] = dot3s(eta[b], eta[b]);
    efie_far_weights<3, 4>(w1, w2, wab);
    if (fast == 2)
      efie_far_pair_beta<3, 4>(d, tau, sig, xi, wab, eta, e2, from(k), cdf{from(al[0]), from(al[1])},
                               cdf{from(be[0]), from(be[1])}, sincos_tab_host, z);
    else
      efie_far_pair_fast<3, 4>(d, tau, sig, xi, wab, eta, e2, from(k), cdf{from(al[0]), from(al[1])},
                               cdf{from(be[0]), from(be[1])}, sincos_tab_host, z);
  } else {
    efie_far_pair(d, tau, sig, no, xi, w1, ni, eta, w2, from(k), cdf{from(al[0]), from(al[1])},
                  cdf{from(be[0]), from(be[1])}, z);
  }
  for (int e = 0; e < 9; ++e) { out[2 * e] = to(z[e].re); out[2 * e + 1] = to(z[e].im); }
}
}
"""


def _pair(x):
    hi = np.asarray(x, np.float64).astype(np.float32).astype(np.float64)
    return hi + (np.asarray(x, np.float64) - hi).astype(np.float32).astype(np.float64)


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("dfloat")
    src = d / "h.cpp"
    src.write_text(HARNESS)
    so = d / "h.so"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I", CSRC, str(src), "-o", str(so)],
                   check=True)
    L = C.CDLL(str(so))
    for f in ("t_two", "t_ops", "t_sincos", "t_sincos_tab", "t_unnorm", "t_green", "t_efie_pair"):
        getattr(L, f).restype = None
    return L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def test_error_free_transforms(lib):
    rng = np.random.default_rng(0)
    a = (rng.normal(size=100000) * 10.0 ** rng.integers(-8, 8, 100000)).astype(np.float32)
    b = (rng.normal(size=100000) * 10.0 ** rng.integers(-8, 8, 100000)).astype(np.float32)
    s = np.zeros(2 * a.size, np.float32)
    p = np.zeros(2 * a.size, np.float32)
    lib.t_two(_p(a), _p(b), C.c_int64(a.size), _p(s), _p(p))
    a64, b64 = a.astype(np.float64), b.astype(np.float64)
    # float32 sums and products are exact in float64
    assert np.array_equal(s[0::2].astype(np.float64) + s[1::2], a64 + b64)
    assert np.array_equal(p[0::2].astype(np.float64) + p[1::2], a64 * b64)


def test_pair_operations(lib):
    rng = np.random.default_rng(1)
    a = rng.uniform(0.1, 10, 50000) * rng.choice([-1, 1], 50000)
    b = rng.uniform(0.1, 10, 50000)
    out = np.zeros(4 * a.size)
    lib.t_ops(_p(a), _p(b), C.c_int64(a.size), _p(out))
    x, y = _pair(a), _pair(b)
    for got, ref in ((out[0::4], x + y), (out[1::4], x * y), (out[2::4], np.sqrt(np.abs(x))), (out[3::4], 1 / x)):
        assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)) < 2e-14


def test_sincos(lib):
    rng = np.random.default_rng(2)
    th = np.concatenate([np.linspace(-7, 7, 20001), rng.uniform(-1e3, 1e3, 50000)])
    s, c = np.zeros_like(th), np.zeros_like(th)
    lib.t_sincos(_p(th), C.c_int64(th.size), _p(s), _p(c))
    x = _pair(th)
    assert np.abs(s - np.sin(x)).max() < 1e-11
    assert np.abs(c - np.cos(x)).max() < 1e-11


def test_sincos_with_the_table(lib):
    """the kernels' sine / cosine (table passed in, fewer FP32 additions): same error class as
    sincos over the range of k R on the assembly path, and at the reduction's edges"""
    rng = np.random.default_rng(5)
    edges = (np.arange(-64, 65) * np.pi / 32)[:, None] + np.array([-1e-9, -1e-12, 0.0, 1e-12, 1e-9])[None, :]
    th = np.concatenate([np.linspace(-7, 7, 20001), rng.uniform(-1e3, 1e3, 50000), edges.ravel(),
                         rng.uniform(0, 1e-6, 1000)])
    s, c = np.zeros_like(th), np.zeros_like(th)
    lib.t_sincos_tab(_p(th), C.c_int64(th.size), _p(s), _p(c))
    x = _pair(th)
    assert np.abs(s - np.sin(x)).max() < 1e-11
    assert np.abs(c - np.cos(x)).max() < 1e-11


def test_unnormalised_forms(lib):
    """the unnormalised sine / cosine, reciprocal square root and pair sums of the far cores
    (their low parts a few ulp of the high part instead of half an ulp): the values hi + lo keep
    the pair accuracy of the normalised forms"""
    rng = np.random.default_rng(11)
    n = 40000
    th = np.concatenate([np.linspace(-7, 7, n // 2), rng.uniform(-1e3, 1e3, n // 2)])
    a = 10 ** rng.uniform(-4, 4, n) * rng.choice([-1.0, 1.0], n)
    b = a * (1 + rng.uniform(-1e-3, 1e-3, n)) * rng.choice([-1.0, 1.0], n)  # includes near cancellation
    out = np.zeros(5 * n)
    lib.t_unnorm(_p(th), _p(a), _p(b), C.c_int64(n), _p(out))
    out = out.reshape(n, 5)
    x, pa, pb = _pair(th), _pair(np.abs(a)), _pair(a)
    pbb = _pair(b)
    assert np.abs(out[:, 0] - np.sin(x)).max() < 1e-11
    assert np.abs(out[:, 1] - np.cos(x)).max() < 1e-11
    assert np.abs(out[:, 2] * np.sqrt(pa) - 1).max() < 2e-13
    scale = np.maximum(np.abs(pb), np.abs(pbb))
    assert (np.abs(out[:, 3] - (pb + pbb)) / scale).max() < 1e-13
    assert (np.abs(out[:, 4] - (pb - pbb)) / scale).max() < 1e-13


def test_green_function(lib):
    """exp(-i k R) / (4 pi R) to 1e-10 relative: 2000 x better than FP32, which limits the mixed
    far-pair matrix entries"""
    rng = np.random.default_rng(3)
    R = 10 ** rng.uniform(-3, 1, 50000)
    k = rng.uniform(0.1, 50, 50000)
    out = np.zeros(2 * R.size)
    lib.t_green(_p(R), _p(k), C.c_int64(R.size), _p(out))
    Rx, kx = _pair(R), _pair(k)
    ref = np.exp(-1j * kx * Rx) / (4 * np.pi * Rx)
    got = out[0::2] + 1j * out[1::2]
    assert np.max(np.abs(got - ref) / np.abs(ref)) < 1e-10


def test_device_compile(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "k.cu"
    src.write_text('#include "far_df.h"\n'
                   "__global__ void k(const float* r, float* o) {\n"
                   "  using namespace dfl;\n"
                   "  df re, im;\n"
                   "  green(df{r[threadIdx.x], 0.f}, df{10.f, 0.f}, &re, &im);\n"
                   "  df d[3] = {re, im, re}, t[3][3] = {}, x[3][3] = {}, w[3] = {re, re, re};\n"
                   "  cdf z[9];\n"
                   "  efie_far_pair(d, t, t, 3, x, w, 3, x, w, re, cdf{re, im}, cdf{im, re}, z);\n"
                   "  o[threadIdx.x] = z[4].re.hi + z[8].im.lo;\n}\n")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-c", "-I", CSRC, str(src), "-o",
                    str(tmp_path / "k.o")], check=True)


# (core, alpha on): 0 the general core, 1 the one for the default rule sizes (3 x 4 points)
# that the mixed-accurate kernel runs, 2 the balanced core (alpha terms in FP32: about 1e-7 of a
# block's largest entry, 3e-8 measured); with alpha = 0 the balanced block is its beta term
# alone, which stays double-float
@pytest.mark.parametrize("fast,alpha_on,tol", [(0, 1, 1e-10), (1, 1, 1e-10), (2, 1, 3e-7), (2, 0, 1e-10)])
def test_efie_far_pair_matches_the_fp64_oracle(lib, fast, alpha_on, tol):
    """the double-float EFIE far block against the oracle's FP64 double quadrature (the
    reference's DoubleQuadRule), on far pairs of a level-3 icosphere at k = 10"""
    import beastgpu as bg
    import oracle as O
    m = bg.icosphere(3)
    T = np.asarray(m.vertices)[np.asarray(m.cells)]
    k = 10.0
    g = 1j * k
    al, be = -g * alpha_on, -1 / g
    op = O.make_op(O.MW_SL, g, al, be)
    qs = O.make_qs(O.QS_WILTON_SAUTER, 2, 3, 6, 7, 5, 5, 4, 3)
    uvo, wo = O.trirule(2)
    uvi, wi = O.trirule(3)
    rng = np.random.default_rng(4)
    worst, tested = 0.0, 0
    for p, q in rng.integers(0, T.shape[0], size=(400, 2)):
        if O.classify(op, qs, T[p], T[q]) != 0:
            continue
        ref = O.cellpair(op, O.RT, O.RT, T[p], T[q], O.RULE_DQ, 2, 3)
        out = np.zeros(18)
        args = [np.ascontiguousarray(a, np.float64) for a in (T[p].ravel(), T[q].ravel(), uvo.ravel(), wo,
                                                              uvi.ravel(), wi, [al.real, al.imag],
                                                              [be.real, be.imag])]
        lib.t_efie_pair(_p(args[0]), _p(args[1]), C.c_int(len(wo)), _p(args[2]), _p(args[3]), C.c_int(len(wi)),
                        _p(args[4]), _p(args[5]), C.c_double(k), _p(args[6]), _p(args[7]), _p(out),
                        C.c_int(fast))
        z = (out[0::2] + 1j * out[1::2]).reshape(3, 3)
        worst = max(worst, np.abs(z - ref).max() / np.abs(ref).max())
        tested += 1
    assert tested > 300
    assert worst < tol, worst
