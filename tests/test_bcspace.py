"""Buffa-Christiansen functions on the barycentric refinement (beastgpu.refine), against what
the reference's test/test_bcspace.jl checks (divergence conformity: every flux leaving a fine
cell enters its neighbour) and a physics check through the oracle: the BC-tested MFIE
(K + N/2)[BC, RT] of examples/mfie.jl and the EFIE give the same far field on a sphere, with a
well-conditioned MFIE matrix (the point of BC testing)."""
import numpy as np
import pytest

import beastgpu as bg


@pytest.fixture(scope="module", params=[1, 2])
def setup(request):
    m = bg.icosphere(request.param)
    X = bg.raviartthomas(m)
    R = bg.barycentric_refinement(m)
    Y, _ = bg.buffachristiansen(m, R, X)
    return m, X, R, Y, bg.refined(X, R)


def _edge_fluxes(fn, cells):
    tot = {}
    for t, r, w in fn:
        a, b = int(cells[t][(r + 1) % 3]), int(cells[t][(r + 2) % 3])
        key = (min(a, b), max(a, b))
        tot[key] = tot.get(key, 0.0) + w
    return tot


def test_barycentric_refinement(setup):
    m, X, R, Y, Xf = setup
    nc, nv = m.numcells(), m.numvertices()
    assert R.fine.numcells() == 6 * nc
    assert R.fine.numvertices() == nv + 3 * nc // 2 + nc
    assert np.all(np.einsum("ij,ij->i", R.fine.normals(), m.normals()[R.parent]) > 0.99)
    assert np.allclose(R.fine.areas().reshape(nc, 6).sum(1), m.areas())


def test_bc_functions_are_divergence_conforming(setup):
    m, X, R, Y, Xf = setup
    assert Y.numfunctions() == X.numfunctions() and Y.mesh is R.fine
    for fn in Y.fns:
        assert len(fn) > 2
        assert max(abs(v) for v in _edge_fluxes(fn, R.fine.cells).values()) < 1e-14


def test_refined_rt_reproduces_the_coarse_fields(setup):
    m, X, R, Y, Xf = setup
    rng = np.random.default_rng(0)
    Vc, Cc, Ac = m.vertices, m.cells, m.areas()
    Vf, Cf = R.fine.vertices, R.fine.cells
    for i in rng.integers(0, X.numfunctions(), 25):
        assert max(abs(v) for v in _edge_fluxes(Xf.fns[i], Cf).values()) < 1e-14
        for c, r, w in X.fns[i]:
            for t in R.children(c):
                u, v = rng.uniform(size=2)
                if u + v > 1:
                    u, v = 1 - u, 1 - v
                tri = Vf[Cf[t]]
                x = u * tri[0] + v * tri[1] + (1 - u - v) * tri[2]
                At = 0.5 * np.linalg.norm(np.cross(tri[1] - tri[0], tri[2] - tri[0]))
                fine = sum(wk * (x - Vf[Cf[tt][k]]) / (2 * At) for tt, k, wk in Xf.fns[i] if tt == t)
                assert np.linalg.norm(w * (x - Vc[Cc[c, r]]) / (2 * Ac[c]) - fine) < 1e-13


def test_bc_mfie_matches_the_efie(setup):
    import oracle as O
    m, X, R, Y, Xf = setup
    k = 1.0
    g = 1j * k
    d, p = np.array([0, 0, 1.0]), np.array([1.0, 0, 0])
    qs = O.make_qs(O.QS_WILTON_SAUTER, 2, 3, 6, 7, 5, 5, 4, 3)
    # MFIE, examples/mfie.jl: (K + N/2)[m, j] == ((n x H) x n)[m], H = d x p for this wave
    A = O.assemble(O.make_op(O.MW_DL, g), qs, Y, Xf) + 0.5 * O.assemble_local(1, Y, Xf)
    u_m = np.linalg.solve(A, O.rhs_planewave(0, Y, d, np.cross(d, p), g))
    T = O.assemble(O.make_op(O.MW_SL, g, -g, -1 / g), qs, X, X)
    u_e = np.linalg.solve(T, O.rhs_planewave(0, X, d, p, g))
    th = np.linspace(0, np.pi, 91)
    dirs = np.stack([np.sin(th), 0 * th, np.cos(th)], 1)
    ff_m, ff_e = O.farfield(X, u_m, dirs, g), O.farfield(X, u_e, dirs, g)
    rel = np.linalg.norm(ff_m - ff_e) / np.linalg.norm(ff_e)
    assert rel < (1e-2 if X.numfunctions() <= 120 else 2e-3), rel
    assert np.linalg.cond(A) < 10
