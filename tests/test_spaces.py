"""Host-side spaces (beastgpu.spaces) against the properties the reference's own tests check:
RT functions are divergence-conforming (the flux of a function through its edge leaves one cell
and enters the other, test/test_bcspace.jl `isdivconforming`), one RT function per edge of a
closed surface (src/bases/rtspace.jl:35-105), one P1 function per vertex with its cells' local
shapes at that vertex (src/bases/lagrange.jl:340-360), and assembly data that inverts the
function lists (src/bases/basis.jl:235-294)."""
import numpy as np
import pytest

import beastgpu as bg


@pytest.fixture(scope="module", params=[1, 2, 3])
def mesh(request):
    return bg.icosphere(request.param)


def _edges(cells):
    e = np.sort(np.concatenate([cells[:, [1, 2]], cells[:, [2, 0]], cells[:, [0, 1]]]), axis=1)
    return {tuple(x) for x in e}


def test_rt_one_function_per_edge_and_divergence_conforming(mesh):
    X = bg.raviartthomas(mesh)
    cells = np.asarray(mesh.cells)
    edges = _edges(cells)
    assert X.numfunctions() == len(edges) == 3 * cells.shape[0] // 2
    seen = set()
    for fn in X.fns:
        assert len(fn) == 2
        (c1, r1, w1), (c2, r2, w2) = fn
        assert c1 != c2 and w1 == -w2 and abs(w1) == 1
        # local shape r lives on the edge opposite local vertex r: both halves name one edge
        e1 = tuple(sorted(np.delete(cells[c1], r1)))
        e2 = tuple(sorted(np.delete(cells[c2], r2)))
        assert e1 == e2
        seen.add(e1)
    assert seen == edges


def test_p1_one_function_per_vertex(mesh):
    X = bg.lagrangec0d1(mesh)
    cells = np.asarray(mesh.cells)
    nv = np.asarray(mesh.vertices).shape[0]
    assert X.numfunctions() == nv
    star = [set() for _ in range(nv)]
    for c, tri in enumerate(cells):
        for v in tri:
            star[v].add(c)
    for fn in X.fns:
        vs = {int(cells[c][r]) for (c, r, w) in fn}
        assert len(vs) == 1 and all(w == 1 for (_, _, w) in fn)
        v = vs.pop()
        assert {c for (c, _, _) in fn} == star[v]


def test_assemblydata_inverts_the_function_lists(mesh):
    for X in (bg.raviartthomas(mesh), bg.lagrangecxd0(mesh), bg.lagrangec0d1(mesh)):
        ad = X.assemblydata()
        back = {}
        for a, c in enumerate(ad.cells):
            for r in range(ad.nshapes):
                for k in range(ad.maxfn):
                    d = ad.dof[a, r, k]
                    if d >= 0:
                        back.setdefault(int(d), set()).add((int(c), r, float(ad.coeff[a, r, k])))
        assert len(back) == X.numfunctions()
        for i, fn in enumerate(X.fns):
            assert back[i] == {(int(c), int(r), float(w)) for (c, r, w) in fn}
