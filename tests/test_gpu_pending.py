"""GPU parity tests of parts built after the last GPU run (Helmholtz P1 singularity extraction,
the BC-tested MFIE on the barycentric refinement, the double-float EFIE far kernel) and of the
Maxwell singularity extraction, which no mesh of the `gpu` tests exercises.  Staged
under their own marker: `pytest -m gpu_pending` on a GB300; each moves to the `gpu` marker
once it has passed there.  Without a GPU they skip."""
import numpy as np
import pytest

import beastgpu as bg
import oracle as O

torch = pytest.importorskip("torch")
pytestmark = [pytest.mark.gpu_pending,
              pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")]


@pytest.fixture(scope="module")
def ctx():
    return bg.get_context(0)


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _check(op, X, Y, ctx, qs=None, tol=1e-10):
    qs = qs or bg.defaultquadstrat(op, X, Y)
    Z = bg.assemble(op, X, Y, quadstrat=qs, precision=bg.FP64, ctx=ctx)
    Zo = O.assemble(O.make_op(op.kind, op.gamma, op.alpha, op.beta), O.OrcQs(*qs.orders()), X, Y)
    assert _rel(Z, Zo) < tol


@pytest.mark.parametrize("which", ["singlelayer", "doublelayer", "doublelayer_transposed"])
@pytest.mark.parametrize("spaces", ["p1p1", "p0p1", "p1p0"])
def test_helmholtz_p1_singularity_extraction(ctx, which, spaces):
    # a strongly perturbed ellipsoid at small |gamma|: seven Wilton singularity-extraction pairs
    m = bg.ellipsoid(2, (1.0, 0.7, 1.3), perturb=0.3, rng=3)
    sp = {"p1": bg.lagrangec0d1(m), "p0": bg.lagrangecxd0(m)}
    op = getattr(bg.Helmholtz3D, which)(gamma=0.3j)
    _check(op, sp[spaces[:2]], sp[spaces[2:]], ctx)


def test_bc_mfie_on_the_refinement(ctx):
    m = bg.icosphere(1)
    X = bg.raviartthomas(m)
    R = bg.barycentric_refinement(m)
    Y, _ = bg.buffachristiansen(m, R, X)
    Xf = bg.refined(X, R)
    _check(bg.Maxwell3D.doublelayer(wavenumber=1.0), Y, Xf, ctx)
    N = bg.assemble(bg.NCross(), Y, Xf, ctx=ctx)
    assert _rel(N, O.assemble_local(1, Y, Xf)) < 1e-12


def test_double_float_efie_far_kernel(ctx, monkeypatch):
    monkeypatch.setenv("BEAST_FAR_DF", "1")
    X = bg.raviartthomas(bg.icosphere(2))
    _check(bg.Maxwell3D.singlelayer(wavenumber=2.0), X, X, ctx)


@pytest.mark.parametrize("which", ["singlelayer", "doublelayer"])
def test_maxwell_singularity_extraction(ctx, which):
    # the perturbed ellipsoid at k = 0.3 has seven Wilton pairs for the Maxwell strategy
    X = bg.raviartthomas(bg.ellipsoid(2, (1.0, 0.7, 1.3), perturb=0.3, rng=3))
    _check(getattr(bg.Maxwell3D, which)(wavenumber=0.3), X, X, ctx)
