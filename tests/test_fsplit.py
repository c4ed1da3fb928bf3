"""The integer split of an FP64 value into two floats (csrc/fsplit.h) that the c128 refinement
matvec uses on the FP32 pipes: built for the host with g++ (host and device builds give the
same bits) and checked against float64 over the exponent range of the matrix entries and at
the edges of its special cases."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "beast.jl_gb300", "csrc")

HARNESS = r"""
#include "fsplit.h"
extern "C" void t_split(const double* a, long n, float* hi, float* lo) {
  for (long i = 0; i < n; ++i) fsplit::split_f64(a[i], hi + i, lo + i);
}
"""


@pytest.fixture(scope="module")
def split(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("fsplit")
    src, so = d / "h.cpp", d / "h.so"
    src.write_text(HARNESS)
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-I", CSRC, str(src), "-o", str(so)])
    L = C.CDLL(str(so))
    L.t_split.argtypes = [C.c_void_p, C.c_long, C.c_void_p, C.c_void_p]

    def run(a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        hi = np.zeros(a.size, np.float32)
        lo = np.zeros(a.size, np.float32)
        L.t_split(a.ctypes.data, a.size, hi.ctypes.data, lo.ctypes.data)
        return hi, lo
    return run


def test_split_is_accurate_over_the_entry_range(split):
    rng = np.random.default_rng(0)
    a = rng.uniform(0.5, 1.0, 200000) * 2.0 ** rng.integers(-70, 100, 200000)
    a *= rng.choice([-1.0, 1.0], a.size)
    hi, lo = split(a)
    err = np.abs(a - (hi.astype(np.float64) + lo.astype(np.float64))) / np.abs(a)
    assert err.max() < 2.0 ** -46
    # hi is the truncation of a to 24 significant bits: same sign, |lo| < ulp(hi)
    assert np.all(np.sign(hi) == np.sign(a))
    assert np.all(np.abs(lo) < np.spacing(np.abs(hi)))


def test_split_special_ranges(split):
    a = np.array([0.0, -0.0, 1e-300, -3e-30, 2.0 ** -80, 2.0 ** 200, -2.0 ** 130, 1.0, -1.0,
                  np.inf, -np.inf, np.nan])
    hi, lo = split(a)
    s = hi.astype(np.float64) + lo.astype(np.float64)
    assert s[0] == 0.0 and s[1] == 0.0 and s[2] == 0.0 and s[3] == 0.0   # below 2^-97: zero
    assert abs(s[4] - a[4]) <= 2.0 ** -80 * 2.0 ** -23                    # low part dropped
    assert s[5] == np.inf and s[6] == -np.inf                             # overflow to +-inf
    assert s[7] == 1.0 and s[8] == -1.0 and lo[7] == 0.0
    assert s[9] == np.inf and s[10] == -np.inf and np.isnan(s[11])       # classes kept


def test_float_to_double_by_integer_ops(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = tmp_path / "f.cpp"
    src.write_text('#include "fsplit.h"\n'
                   'extern "C" void t_f2d(const float* f, long n, double* d) {\n'
                   '  for (long i = 0; i < n; ++i) d[i] = fsplit::f2d(f[i]);\n}\n')
    so = tmp_path / "f.so"
    subprocess.check_call(["g++", "-O2", "-shared", "-fPIC", "-I", CSRC, str(src), "-o", str(so)])
    L = C.CDLL(str(so))
    L.t_f2d.argtypes = [C.c_void_p, C.c_long, C.c_void_p]
    rng = np.random.default_rng(1)
    f = (rng.uniform(1, 2, 100000) * 2.0 ** rng.integers(-126, 128, 100000)).astype(np.float32)
    f *= rng.choice([-1, 1], f.size).astype(np.float32)
    f = np.concatenate([f, np.array([0.0, -0.0, np.inf, -np.inf, 1.0, -2.5], np.float32)])
    d = np.zeros(f.size)
    L.t_f2d(f.ctypes.data, f.size, d.ctypes.data)
    assert np.array_equal(d, f.astype(np.float64))
    assert np.array_equal(np.signbit(d), np.signbit(f))
    nan = np.array([np.nan], np.float32)
    L.t_f2d(nan.ctypes.data, 1, d.ctypes.data)
    assert np.isnan(d[0])
    sub = np.array([1e-40, -3e-45], np.float32)  # subnormal floats become zero
    L.t_f2d(sub.ctypes.data, 2, d.ctypes.data)
    assert d[0] == 0.0 and d[1] == 0.0


def test_round_to_float_by_integer_ops(tmp_path):
    """fsplit::to_float_rn gives the conversion's bits (round to nearest, ties to even) over the
    normal float range, including the ties, overflow to infinity and NaN"""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = tmp_path / "r.cpp"
    src.write_text('#include "fsplit.h"\n'
                   'extern "C" void t_rn(const double* a, long n, float* f) {\n'
                   '  for (long i = 0; i < n; ++i) f[i] = fsplit::to_float_rn(a[i]);\n}\n')
    so = tmp_path / "r.so"
    subprocess.check_call(["g++", "-O2", "-shared", "-fPIC", "-I", CSRC, str(src), "-o", str(so)])
    L = C.CDLL(str(so))
    L.t_rn.argtypes = [C.c_void_p, C.c_long, C.c_void_p]
    rng = np.random.default_rng(2)
    a = rng.uniform(1, 2, 200000) * 2.0 ** rng.integers(-125, 127, 200000)
    a *= rng.choice([-1.0, 1.0], a.size)
    # exact ties: a float plus half its ulp, both parities of the last mantissa bit
    f0 = rng.uniform(1, 2, 1000).astype(np.float32)
    ties = f0.astype(np.float64) + np.spacing(f0).astype(np.float64) / 2
    big = np.array([3.4028235677973366e38, 3.4028235e38 * 1.0000001, 1e300, -1e300, np.inf, -np.inf, np.nan, 0.0, -0.0])
    a = np.concatenate([a, ties, -ties, big])
    f = np.zeros(a.size, np.float32)
    L.t_rn(a.ctypes.data, a.size, f.ctypes.data)
    with np.errstate(over="ignore"):
        ref = a.astype(np.float32)
    ok = (f.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(f) & np.isnan(ref))
    assert ok.all(), a[~ok][:5]
