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
#include "dfloat.h"
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
void t_green(const double* R, const double* k, int64_t n, double* out) {
  for (int64_t i = 0; i < n; ++i) { df re, im; green(from(R[i]), from(k[i]), &re, &im); out[2 * i] = to(re); out[2 * i + 1] = to(im); }
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
    for f in ("t_two", "t_ops", "t_sincos", "t_green"):
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
    src.write_text('#include "dfloat.h"\n'
                   "__global__ void k(const float* r, float* o) {\n"
                   "  dfl::df re, im;\n"
                   "  dfl::green(dfl::df{r[threadIdx.x], 0.f}, dfl::df{10.f, 0.f}, &re, &im);\n"
                   "  o[threadIdx.x] = re.hi + im.lo;\n}\n")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-c", "-I", CSRC, str(src), "-o",
                    str(tmp_path / "k.o")], check=True)
