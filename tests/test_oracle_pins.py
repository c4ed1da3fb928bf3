"""Pins the CPU oracle to the reference's own tests and golden values (no GPU).

Reference tests restated here:
  test/test_wiltonints.jl:291-322   Wilton integrals vs quadrature
  test/test_sauterschwabints.jl     Sauter-Schwab vs singularity extraction, GL12 vs GL18
  test/test_hh3dints.jl:619-671     Helmholtz SL on separated triangles vs hcubature value
  test/test_rt.jl:60-85             RT shape values (x - v_i) / 2A
  test/test_itsolver.jl:9-37        direct residual and GMRES accuracy contract
  test/test_coloring.jl:118         threading invariance (1e-12)
  test/test_assemblerow.jl          row-subset assembly equals the full matrix rows
The triangle rules of degree 12/13 that the reference's SE checks use are not available
in-tree (CompScienceMeshes); the SE legs below use higher-degree rules, for which the
singularity-extraction result converges to the Sauter-Schwab one.
"""
import math

import numpy as np
import pytest

import oracle as O
from conftest import mesh_path


def test_triangle_rules_exact():
    for deg in [1, 2, 3, 4, 5, 6, 7, 8, 10, 12, 13]:
        uv, w = O.trirule(deg)
        for p in range(deg + 1):
            for q in range(deg + 1 - p):
                ex = 2.0 * math.factorial(p) * math.factorial(q) / math.factorial(p + q + 2)
                assert abs((w * uv[:, 0] ** p * uv[:, 1] ** q).sum() - ex) < 1e-14
    # point counts of the symmetric rules used by the default strategies
    assert [len(O.trirule(d)[1]) for d in (2, 3, 6, 7, 8, 10)] == [3, 4, 12, 13, 16, 25]


def test_gauss_legendre():
    for n in (3, 4, 5, 8, 12):
        x, w = O.gausslegendre(n)
        for k in range(2 * n):
            assert abs((w * x ** k).sum() - 1.0 / (k + 1)) < 1e-14


def _refined_quad(tr, r, lev=6):
    uvr, wr = O.trirule(10)
    T = [tuple(tr)]
    for _ in range(lev):
        N = []
        for a, b, c in T:
            ab, bc, ca = (a + b) / 2, (b + c) / 2, (c + a) / 2
            N += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        T = N
    n = np.cross(tr[0] - tr[2], tr[1] - tr[2])
    n /= np.linalg.norm(n)
    d = (r - tr[0]) @ n
    rho = r - d * n
    s = np.zeros(6)
    v = np.zeros((5, 3))
    for st in T:
        st = np.array(st)
        A = np.linalg.norm(np.cross(st[0] - st[2], st[1] - st[2])) / 2
        Y = uvr[:, :1] * st[0] + uvr[:, 1:2] * st[1] + (1 - uvr[:, :1] - uvr[:, 1:2]) * st[2]
        R = np.linalg.norm(Y - r, axis=1)
        dq = wr * A
        s += np.array([(d / R ** 3) @ dq, (1 / R) @ dq, dq.sum(), R @ dq, (R ** 2) @ dq,
                       (R ** 3) @ dq])
        for k, pw in enumerate([-3, -1, 0, 1, 2]):
            v[k] += ((Y - rho) * (R ** pw * dq)[:, None]).sum(0)
    g = np.array([-(v[0] - s[0] * n), v[1] - d * s[1] * n, 2 * (v[2] - d * s[2] * n),
                  3 * (v[3] - d * s[3] * n)])
    return s, v, g


def test_wiltonints_vs_quadrature():
    tr = np.array([[0, 0, 0], [2, 0, 0], [0, 3, 0.]])
    pts = [tr[0] + 2 * tr[1] - tr[2], (tr[0] + tr[1]) / 2 + [0, 0, .3], [3, 0, 0.],
           tr.mean(0) + [0, 0, .3], tr[1] + [0, 0, .3], tr.mean(0) + [0, 0, 100.]]
    for p in pts:
        p = np.array(p, dtype=float)
        s1, v1, g1 = O.wiltonints(tr[0], tr[1], tr[2], p)
        s2, v2, g2 = _refined_quad(tr, p)
        # the reference's tolerance is 1e-5 absolute against a 13th-degree rule
        assert np.all(np.abs(s1 - s2) <= 1e-5 + 1e-12 * np.abs(s2))
        assert np.all(np.abs(v1[:5] - v2) <= 1e-5 + 1e-12 * np.abs(v2))
        assert np.all(np.abs(g1 - g2) <= 1e-5 + 1e-12 * np.abs(g2))


def _tri(x):
    return np.array(x, dtype=np.float64)


def test_sauterschwab_vs_singularity_extraction(golden):
    tri = golden["ss_triangles"]
    t1, t2v = _tri(tri["face_t1"]), _tri(tri["vertex_t2"])
    e1, e2 = _tri(tri["edge_t1"]), _tri(tri["edge_t2"])
    op1 = O.make_op(O.MW_SL, 1.0, 250.0, 1.0)   # MWSingleLayer3D(1, 250, 1)
    op2 = O.make_op(O.MW_SL, 1.0, -1.0, -1.0)   # MWSingleLayer3D(1)
    op3 = O.make_op(O.MW_DL, 0.0, 1.0)          # MWDoubleLayer3D(0)
    RT = O.RT
    for op in (op1, op2):  # common face, tol 1e-4 (test_sauterschwabints.jl:42-58)
        se = O.cellpair(op, RT, RT, t1, t1, O.RULE_SE, 40, 41)
        ss = O.cellpair(op, RT, RT, t1, t1, O.RULE_SS_FACE, gl=8)
        assert np.linalg.norm(se - ss) < 1e-4
    for op in (op1, op2, op3):  # common vertex, tol 1e-7 (:60-92)
        se = O.cellpair(op, RT, RT, t1, t2v, O.RULE_SE, 40, 41)
        ss = O.cellpair(op, RT, RT, t1, t2v, O.RULE_SS_VERT, gl=12)
        assert np.linalg.norm(se - ss) < 1e-7 * max(1.0, 10 * np.abs(ss).max())
    for op in (op1, op2, op3):  # common edge, tol 1e-5 (:94-137)
        se = O.cellpair(op, RT, RT, e1, e2, O.RULE_SE, 40, 41)
        ss = O.cellpair(op, RT, RT, e1, e2, O.RULE_SS_EDGE, gl=12)
        assert np.linalg.norm(se - ss) < 1e-5
    # GL12 vs GL18 on the edge case (:139-143)
    a = O.cellpair(op3, RT, RT, e1, e2, O.RULE_SS_EDGE, gl=12)
    b = O.cellpair(op3, RT, RT, e1, e2, O.RULE_SS_EDGE, gl=18)
    assert np.linalg.norm(a - b) < 1e-14


def test_sauterschwab_convergence():
    # the regularised integrands are smooth: the tensor Gauss rules converge fast
    t = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0.]])
    s_edge = np.array([[0, 0, 0], [1, 0, 0], [0, -1, 0.]])
    s_vert = np.array([[0, 0, 0], [-1, 0, 0], [0, -1, 0.]])
    op = O.make_op(O.HH_SL, 0.0, 1.0)
    for tb, rule in [(t, O.RULE_SS_FACE), (s_edge, O.RULE_SS_EDGE), (s_vert, O.RULE_SS_VERT)]:
        z12 = O.cellpair(op, O.P0, O.P0, t, tb, rule, gl=12)[0, 0]
        z16 = O.cellpair(op, O.P0, O.P0, t, tb, rule, gl=16)[0, 0]
        assert abs(z12 - z16) < 1e-9 * abs(z16)


def test_helmholtz_separated_golden(golden):
    t1, t2 = _tri(golden["hh3d_separated_t1"]), _tri(golden["hh3d_separated_t2"])
    ref = complex(*golden["hh3d_separated_refval"])
    op1 = O.make_op(O.HH_SL, complex(*golden["hh3d_gamma"]), 1.0)
    se = O.cellpair(op1, O.P0, O.P0, t1, t2, O.RULE_SE, 60, 61)[0, 0]
    dq = O.cellpair(op1, O.P0, O.P0, t1, t2, O.RULE_DQ, 80, 81)[0, 0]
    assert abs(se - ref) < 1e-7 * abs(ref)
    assert abs(dq - ref) < 1e-6 * abs(ref)


def test_rt_shapes_via_identity():
    # the Gram matrix of RT functions on one triangle equals the analytic one for
    # f_i = (x - v_i) / 2A  (test/test_rt.jl:60-85)
    from beastgpu import mesh as M, spaces as S
    v = np.array([[0, 0, 0], [2, 0, 0], [0, 3, 0], [2, 3, 0.]])
    m = M.Mesh(v, np.array([[0, 1, 2], [3, 2, 1]]))
    X = S.raviartthomas(m)
    assert X.numfunctions() == 1
    G = O.assemble_local(0, X, X, degree=6)
    # direct quadrature of f.f over both cells with exact shapes
    A = 3.0
    uv, w = O.trirule(6)
    tot = 0.0
    for cell, sgn, e in [(0, 1, None), (1, -1, None)]:
        c = m.cells[cell]
        fn = X.fns[0]
        (cid, r, co) = fn[0] if fn[0][0] == cell else fn[1]
        P = v[c]
        for (u, vv), ww in zip(uv, w):
            x = u * P[0] + vv * P[1] + (1 - u - vv) * P[2]
            f = co * (x - P[r]) / (2 * A)
            tot += ww * A * f @ f
    assert abs(G[0, 0] - tot) < 1e-14


def _efie_setup(name="sphere45.in", kappa=1.0):
    from beastgpu import mesh as M, spaces as S
    m = M.readmesh(mesh_path(name))
    X = S.raviartthomas(m)
    g = 1j * kappa
    op = O.make_op(O.MW_SL, g, -g, -1 / g)
    qs = O.make_qs(O.QS_WILTON_SAUTER, 2, 3, 6, 7, 5, 5, 4, 3)
    return m, X, op, qs, g


def test_solver_contract():
    # test/test_itsolver.jl:9-37 (sphere45 instead of sphere2 to keep the CPU suite short)
    m, X, op, qs, g = _efie_setup("sphere45.in", 1.0)
    A = O.assemble(op, qs, X, X)
    b = O.rhs_planewave(0, X, [0, 0, 1], [1, 0, 0], g)
    u = O.lu_solve(A, b)
    assert np.linalg.norm(A @ u - b) / np.linalg.norm(b) < 100 * np.finfo(float).eps * 10
    for rtol in [1e-6, 1e-8, 1e-10]:
        x, it, res = O.gmres(A, b, reltol=rtol, restart=0, maxiter=2000)
        assert it > 0
        assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < rtol
        assert np.linalg.norm(x - u) / np.linalg.norm(x) < 100 * rtol


def test_threading_and_row_invariance():
    m, X, op, qs, g = _efie_setup("sphere45.in", 3.0)
    A1 = O.assemble(op, qs, X, X, nthreads=1)
    A4 = O.assemble(op, qs, X, X, nthreads=4)
    assert np.abs(A1 - A4).max() <= 1e-12 * np.abs(A1).max()
    n = X.numfunctions()
    R = O.assemble(op, qs, X, X, row_lo=n // 3, row_hi=n // 3 + 17)
    assert np.abs(R - A1[n // 3:n // 3 + 17]).max() <= 1e-12 * np.abs(A1).max()


def _farfield_golden(golden):
    """the reference's golden current on sphere824 in this package's dof order, with the
    7 directions and magnitudes of test/test_farfield.jl:17-40"""
    from beastgpu import mesh as M, spaces as S
    ffg = golden["farfield_sphere824"]
    m = M.readmesh(mesh_path("sphere824.in"))
    X = S.raviartthomas(m)
    u_ref = np.array(ffg["u_re"]) + 1j * np.array(ffg["u_im"])
    u = np.zeros_like(u_ref)
    u[np.array(ffg["dof_map"])] = np.array(ffg["sign"]) * u_ref
    th = np.linspace(0.0, np.pi, 7)
    dirs = np.stack([np.sin(th), np.zeros_like(th), np.cos(th)], axis=1)
    return X, u, dirs, np.array(ffg["a"])


def test_farfield_golden_vector(golden):
    """test/test_farfield.jl: |potential(MWFarField3D(1im), points, u, X)| * omega / (4 pi c)
    at 7 angles within 1e4 eps.  The golden magnitudes are those of the 4-point degree-3
    triangle rule: with it they are reproduced to about 1e-15, while rules of degree 4 and
    above converge to values 1.5e-7 away -- so this pins the dof map, the far-field kernel and
    that rule's points and weights against the reference."""
    X, u, dirs, a = _farfield_golden(golden)
    tol = 1e4 * np.finfo(float).eps
    ff = O.farfield(X, u, dirs, 1j, degree=3) / (4 * np.pi)
    assert np.abs(np.linalg.norm(ff, axis=1) - a).max() < tol
    ff10 = O.farfield(X, u, dirs, 1j, degree=10) / (4 * np.pi)
    assert 1e-8 < np.abs(np.linalg.norm(ff10, axis=1) - a).max() < 1e-6
