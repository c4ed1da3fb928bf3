"""The product's singular-extraction code (csrc/se_core.h: the Wilton integrals and the
singular part that the near-pair kernel runs on the device) built for the host with g++ and
compared with the oracle's singular part (its extraction block minus its regular-part block,
over the same outer rule points), for the Maxwell single / double layer on RT and the Helmholtz
single, double and transposed double layers on every P0 / P1 combination."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
from conftest import ROOT

HARNESS = r"""
#include "se_core.h"
extern "C" int t_sing(int kind, int tk, int bk, const double* op6, const double* tv, const double* bv,
                      int npts, const double* uvw, double* out) {
  OpParams op;
  op.kind = kind; op.gr = op6[0]; op.gi = op6[1]; op.ar = op6[2]; op.ai = op6[3]; op.br = op6[4]; op.bi = op6[5];
  auto geo = [](const double* v) {  // the per-cell record k_geometry writes
    double g[16];
    for (int i = 0; i < 9; ++i) g[i] = v[i];
    const double e1[3] = {v[0] - v[6], v[1] - v[7], v[2] - v[8]}, e2[3] = {v[3] - v[6], v[4] - v[7], v[5] - v[8]};
    const double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const double j = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int k = 0; k < 3; ++k) { g[9 + k] = (v[k] + v[3 + k] + v[6 + k]) / 3; g[12 + k] = n[k] / j; }
    g[15] = 0.5 * j;
    return load_geo(g);
  };
  const Geo t = geo(tv), s = geo(bv);
  C2<double> acc[9];
  for (auto& a : acc) a = C2<double>{0, 0};
  for (int a = 0; a < npts; ++a) {
    const double bx[3] = {uvw[3 * a], uvw[3 * a + 1], 1 - uvw[3 * a] - uvw[3 * a + 1]};
    const V3<double> x = bx[0] * t.v[0] + bx[1] * t.v[1] + bx[2] * t.v[2];
    if (!se_singular(op, tk, bk, t, s, x, bx, uvw[3 * a + 2] * t.area, acc)) return 1;
  }
  for (int e = 0; e < 9; ++e) { out[2 * e] = acc[e].re; out[2 * e + 1] = acc[e].im; }
  return 0;
}
"""

REG = {O.MW_SL: O.MW_SL_REG, O.MW_DL: O.MW_DL_REG, O.HH_SL: O.HH_SL_REG, O.HH_DL: O.HH_DL_REG,
       O.HH_DLT: O.HH_DLT_REG}


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    cuda_inc = "/usr/local/cuda/include"
    if not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("CUDA headers not available")
    d = tmp_path_factory.mktemp("secore")
    (d / "h.cpp").write_text(HARNESS)
    subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-I", os.path.join(ROOT, "beast.jl_gb300", "csrc"), "-I",
                    os.path.join(ROOT, "include"), "-I", cuda_inc, str(d / "h.cpp"), "-o", str(d / "h.so")],
                   check=True)
    L = C.CDLL(str(d / "h.so"))
    L.t_sing.restype = C.c_int
    return L


CASES = [(O.MW_SL, O.RT, O.RT), (O.MW_DL, O.RT, O.RT)] + \
    [(k, a, b) for k in (O.HH_SL, O.HH_DL, O.HH_DLT) for a in (O.P0, O.P1) for b in (O.P0, O.P1)]


@pytest.mark.parametrize("kind,tk,bk", CASES)
def test_singular_part_matches_the_oracle(lib, kind, tk, bk):
    P = lambda a: np.ascontiguousarray(a, np.float64).ctypes.data_as(C.c_void_p)
    rng = np.random.default_rng(7)
    tv = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0.]])
    uvo, wo = O.trirule(6)
    uvw = np.c_[uvo, wo]
    nt, nb = (1 if tk == O.P0 else 3), (1 if bk == O.P0 else 3)
    for trial in range(4):
        bv = tv + np.array([0.3 * rng.uniform(), 0.3 * rng.uniform(), 0.1 + 0.1 * trial]) + \
            0.08 * rng.normal(size=(3, 3))
        g = complex(0.4 * rng.uniform(), 1 + rng.uniform())
        al, be = complex(*rng.normal(size=2)), complex(*rng.normal(size=2))
        ref = O.cellpair(O.make_op(kind, g, al, be), tk, bk, tv, bv, O.RULE_SE, 6, 7) - \
            O.cellpair(O.make_op(REG[kind], g, al, be), tk, bk, tv, bv, O.RULE_DQ, 6, 7)
        out = np.zeros(18)
        op6 = [g.real, g.imag, al.real, al.imag, be.real, be.imag]
        assert lib.t_sing(kind, tk, bk, P(op6), P(tv.ravel()), P(bv.ravel()), len(wo), P(uvw),
                          out.ctypes.data_as(C.c_void_p)) == 0
        z = (out[0::2] + 1j * out[1::2])[:nt * nb].reshape(nt, nb)
        assert np.abs(z - ref).max() < 1e-12 * np.abs(ref).max()
