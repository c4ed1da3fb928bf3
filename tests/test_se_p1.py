"""Singularity extraction with P1 shapes for the Helmholtz single layer
(src/helmholtz3d/wiltonints.jl:19-135; the reference takes the P1 moments from the external
WiltonInts84.higherorder).  The product's moment formula (csrc/se_p1.h, built for the host)
against brute-force quadrature, and the oracle's SE blocks against double quadrature on
subdivided triangles (converged) plus the partition-of-unity identities."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
from conftest import ROOT

CSRC = os.path.join(ROOT, "beast.jl_gb300", "csrc")


@pytest.fixture(scope="module")
def moments(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("sep1")
    (d / "h.cpp").write_text('#include "se_p1.h"\n'
                             'extern "C" void t(const double* v, const double* n, const double* rho, double S1, '
                             'double S3, const double* V1, const double* V3, double* o1, double* o3) {\n'
                             '  se_p1_moments((const double (*)[3])v, n, rho, S1, S3, V1, V3, o1, o3);\n}\n'
                             'extern "C" void t_dl(const double* v, const double* n, const double* rho, double d, '
                             'double S0, double S1, const double* V0, const double* V1, double* oa, double* ob) {\n'
                             '  se_p1_dl_moments((const double (*)[3])v, n, rho, d, S0, S1, V0, V1, oa, ob);\n}\n'
                             'extern "C" void t_dlt(const double* v, const double* n, const double* rho, double d, '
                             'double S0, double S1, double S3, const double* V0, const double* V1, const double* nx, '
                             'double* oa, double* ob) {\n'
                             '  se_p1_dlt_moments((const double (*)[3])v, n, rho, d, S0, S1, S3, V0, V1, nx, oa, ob);\n}\n')
    subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-I", CSRC, str(d / "h.cpp"), "-o", str(d / "h.so")],
                   check=True)
    L = C.CDLL(str(d / "h.so"))
    L.t.restype = None
    L.t_dl.restype = None
    L.t_dlt.restype = None
    return L


def _brute(v, x, levels=6, powers=(-1, 1)):
    """int lambda_j R^p over the triangle for p in powers: degree-8 rule on 4^levels pieces"""
    uv, w = O.trirule(8)
    N = 2 ** levels
    pts, wts = [], []
    for i in range(N):
        for j in range(N - i):
            tris = [((i, j), (i + 1, j), (i, j + 1))]
            if i + j + 1 < N:
                tris.append(((i + 1, j), (i, j + 1), (i + 1, j + 1)))
            for corners in tris:
                cb = np.array(corners, float) / N
                p = uv[:, :1] * cb[0] + uv[:, 1:] * cb[1] + (1 - uv.sum(1, keepdims=True)) * cb[2]
                pts.append(p)
                wts.append(w / (N * N))
    p = np.concatenate(pts)
    wt = np.concatenate(wts) * np.linalg.norm(np.cross(v[1] - v[0], v[2] - v[0])) / 2
    lam = np.c_[p, 1 - p.sum(1)]
    y = lam @ v
    R = np.linalg.norm(x - y, axis=1)
    return tuple((wt * R ** p) @ lam for p in powers)


def _brute_grad(v, x, nx, levels=6):
    """nx . int lambda_j grad_y(1/R) and nx . int lambda_j grad_y R (same pieces as _brute)"""
    uv, w = O.trirule(8)
    N = 2 ** levels
    pts, wts = [], []
    for i in range(N):
        for j in range(N - i):
            tris = [((i, j), (i + 1, j), (i, j + 1))]
            if i + j + 1 < N:
                tris.append(((i + 1, j), (i, j + 1), (i + 1, j + 1)))
            for corners in tris:
                cb = np.array(corners, float) / N
                pts.append(uv[:, :1] * cb[0] + uv[:, 1:] * cb[1] + (1 - uv.sum(1, keepdims=True)) * cb[2])
                wts.append(w / (N * N))
    p = np.concatenate(pts)
    wt = np.concatenate(wts) * np.linalg.norm(np.cross(v[1] - v[0], v[2] - v[0])) / 2
    lam = np.c_[p, 1 - p.sum(1)]
    r = x - lam @ v
    R = np.linalg.norm(r, axis=1)
    return (wt * (r @ nx) / R ** 3) @ lam, (wt * -(r @ nx) / R) @ lam


def test_p1_moments_against_quadrature(moments):
    rng = np.random.default_rng(0)
    P = lambda a: np.ascontiguousarray(a, np.float64).ctypes.data_as(C.c_void_p)
    for trial in range(6):
        v = rng.normal(size=(3, 3))
        n = np.cross(v[1] - v[0], v[2] - v[0])
        n /= np.linalg.norm(n)
        h = np.linalg.norm(v[1] - v[0])
        x = v.mean(0) + 0.5 * h * rng.normal(size=3) + (0.2 + 0.1 * trial) * h * n
        s, vec, _ = O.wiltonints(v[0], v[1], v[2], x)
        rho = x - np.dot(x - v[0], n) * n
        o1, o3 = np.zeros(3), np.zeros(3)
        moments.t(P(v), P(n), P(rho), C.c_double(s[1]), C.c_double(s[3]), P(vec[1]), P(vec[3]),
                  o1.ctypes.data_as(C.c_void_p), o3.ctypes.data_as(C.c_void_p))
        b1, b3, bm3 = _brute(v, x, powers=(-1, 1, -3))
        assert np.abs(o1 - b1).max() < 1e-8 * np.abs(b1).max()
        assert np.abs(o3 - b3).max() < 1e-8 * np.abs(b3).max()
        # double layer: int lambda_j d / R^3 and int lambda_j d / R
        dd = float(np.dot(x - v[0], n))
        oa, ob = np.zeros(3), np.zeros(3)
        moments.t_dl(P(v), P(n), P(rho), C.c_double(dd), C.c_double(s[0]), C.c_double(s[1]), P(vec[0]),
                     P(vec[1]), oa.ctypes.data_as(C.c_void_p), ob.ctypes.data_as(C.c_void_p))
        assert np.abs(oa - dd * bm3).max() < 1e-8 * np.abs(dd * bm3).max()
        assert np.abs(ob - dd * b1).max() < 1e-8 * np.abs(dd * b1).max()
        # transposed double layer: nx . int lambda_j grad_y(1/R), nx . int lambda_j grad_y R
        nx = rng.normal(size=3)
        nx /= np.linalg.norm(nx)
        ta, tb = np.zeros(3), np.zeros(3)
        moments.t_dlt(P(v), P(n), P(rho), C.c_double(dd), C.c_double(s[0]), C.c_double(s[1]), C.c_double(s[3]),
                      P(vec[0]), P(vec[1]), P(nx), ta.ctypes.data_as(C.c_void_p), tb.ctypes.data_as(C.c_void_p))
        ga, gb = _brute_grad(v, x, nx)
        assert np.abs(ta - ga).max() < 1e-8 * np.abs(ga).max()
        assert np.abs(tb - gb).max() < 1e-8 * np.abs(gb).max()


def _children(v):
    a, b, c = v
    P = {"a": a, "b": b, "c": c, "ab": (a + b) / 2, "bc": (b + c) / 2, "ca": (c + a) / 2}
    B = {"a": [1, 0, 0], "b": [0, 1, 0], "c": [0, 0, 1], "ab": [.5, .5, 0], "bc": [0, .5, .5], "ca": [.5, 0, .5]}
    return [(np.array([P[k] for k in t]), np.array([B[k] for k in t], float))
            for t in (("a", "ab", "ca"), ("ab", "b", "bc"), ("ca", "bc", "c"), ("ab", "bc", "ca"))]


def _pieces(v, levels):
    items = [(np.array(v), np.eye(3))]
    for _ in range(levels):
        items = [(cv, cb @ M) for tv, M in items for cv, cb in _children(tv)]
    return items


def _dq_subdivided(op, tk, bk, tv, bv, levels=2, deg=10):
    one = np.ones((1, 1))
    Z = 0
    for sv, Ms in _pieces(tv, levels):
        for bv2, Mb in _pieces(bv, levels):
            z = O.cellpair(op, tk, bk, sv, bv2, O.RULE_DQ, deg, deg)
            Z = Z + (Ms if tk == O.P1 else one).T @ z @ (Mb if bk == O.P1 else one)
    return Z


def test_oracle_p1_singularity_extraction():
    rng = np.random.default_rng(2)
    op = O.make_op(O.HH_SL, 2j, 1.0)
    tv = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0.]])
    for trial in range(2):
        bv = tv + np.array([0.3 * rng.uniform(), 0.3 * rng.uniform(), 0.12 + 0.1 * trial]) + \
            0.05 * rng.normal(size=(3, 3))
        se = {}
        for tk, bk in ((O.P0, O.P0), (O.P1, O.P0), (O.P0, O.P1), (O.P1, O.P1)):
            se[tk, bk] = O.cellpair(op, tk, bk, tv, bv, O.RULE_SE, 8, 8)
            ref = _dq_subdivided(op, tk, bk, tv, bv)
            # the P0 x P0 extraction (pinned elsewhere) is ~1e-5 from the converged reference here;
            # a wrong P1 moment would be off by orders of magnitude more
            assert np.abs(se[tk, bk] - ref).max() < 2e-4 * np.abs(ref).max()
        # partition of unity: the P1 shapes sum to the P0 shape on either side
        z00 = se[O.P0, O.P0][0, 0]
        assert abs(se[O.P0, O.P1].sum() - z00) < 1e-12 * abs(z00)
        assert abs(se[O.P1, O.P0].sum() - z00) < 1e-12 * abs(z00)
        assert np.abs(se[O.P1, O.P1].sum(1) - se[O.P1, O.P0][:, 0]).max() < 1e-12 * abs(z00)


@pytest.mark.parametrize("kind", [O.HH_DL, O.HH_DLT])
def test_oracle_p1_double_layer_singularity_extraction(kind):
    """double layer (n.grad' of the kernel is d/R^3, -d/R on the flat trial triangle) and
    transposed double layer (plus the in-plane second moments) with P1 on either side: exact
    partition of unity, and the same accuracy class as the pinned P0 x P0 extraction against
    converged subdivided quadrature"""
    rng = np.random.default_rng(5)
    op = O.make_op(kind, 2j, 1.0)
    tv = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0.]])
    combos = [(O.P0, O.P0), (O.P1, O.P0), (O.P0, O.P1), (O.P1, O.P1)]
    for trial in range(2):
        bv = tv + np.array([0.3 * rng.uniform(), 0.3 * rng.uniform(), 0.12 + 0.1 * trial]) + \
            0.05 * rng.normal(size=(3, 3))
        se, err = {}, {}
        for tk, bk in combos:
            se[tk, bk] = O.cellpair(op, tk, bk, tv, bv, O.RULE_SE, 10, 10)
            ref = _dq_subdivided(op, tk, bk, tv, bv)
            err[tk, bk] = np.abs(se[tk, bk] - ref).max() / np.abs(ref).max()
        for c in combos[1:]:
            assert err[c] < max(5 * err[O.P0, O.P0], 1e-4), (c, err)
        z00 = se[O.P0, O.P0][0, 0]
        assert abs(se[O.P1, O.P0].sum() - z00) < 1e-12 * abs(z00)
        assert abs(se[O.P0, O.P1].sum() - z00) < 1e-12 * abs(z00)
        assert np.abs(se[O.P1, O.P1].sum(1) - se[O.P1, O.P0][:, 0]).max() < 1e-12 * abs(z00)
