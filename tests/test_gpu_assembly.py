"""GPU parity: libbeastgpu (through the C ABI) against the CPU oracle.

Tolerances: FP64 path 1e-10 relative to the largest matrix entry, per entry; mixed path
(FP32 far pairs, c64 storage) 2e-5 relative to the largest entry.
"""
import numpy as np
import pytest

import beastgpu as bg
import oracle as O
from conftest import mesh_path

pytestmark = pytest.mark.gpu

WS = (2, 3, 6, 7, 5, 5, 4, 3)


@pytest.fixture(scope="module")
def ctx():
    return bg.get_context(0)


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _orc_op(op):
    return O.make_op(op.kind, op.gamma, op.alpha, op.beta)


def _orc_qs(qs):
    o = qs.orders()
    return O.OrcQs(*o)


def _check(op, X, Y, ctx, tol=1e-10, precision=bg.FP64, qs=None):
    qs = qs or bg.defaultquadstrat(op, X, Y)
    Z = bg.assemble(op, X, Y, quadstrat=qs, precision=precision, ctx=ctx)
    Zo = O.assemble(_orc_op(op), _orc_qs(qs), X, Y)
    e = rel(Z, Zo)
    assert e < tol, e
    return Z, Zo


def test_efie_icosphere(ctx):
    X = bg.raviartthomas(bg.icosphere(2))
    _check(bg.Maxwell3D.singlelayer(wavenumber=2.0), X, X, ctx)


def test_efie_reference_mesh_with_near_pairs(ctx):
    # sphere45: an irregular reference mesh (Sauter-Schwab pairs of all three kinds; at k = 3 its
    # non-touching pairs are all far -- the singularity-extraction pairs are covered in
    # test_gpu_pending.py on a strongly perturbed ellipsoid)
    X = bg.raviartthomas(bg.readmesh(mesh_path("sphere45.in")))
    op = bg.Maxwell3D.singlelayer(wavenumber=3.0)
    _check(op, X, X, ctx)


def test_efie_static_alpha_beta(ctx):
    X = bg.raviartthomas(bg.icosphere(1))
    op = bg.operators.IntegralOperator(bg.operators.MW_SL, 1.0, 250.0, 1.0)
    _check(op, X, X, ctx)


def test_mfie_double_layer(ctx):
    X = bg.raviartthomas(bg.icosphere(2))
    _check(bg.Maxwell3D.doublelayer(wavenumber=2.0), X, X, ctx)


def test_nxk(ctx):
    X = bg.raviartthomas(bg.icosphere(1))
    _check(bg.nxdoublelayer(wavenumber=2.0), X, X, ctx, tol=1e-9)


@pytest.mark.parametrize("which", ["sl", "dl", "dlt"])
def test_helmholtz_p0(ctx, which):
    m = bg.ellipsoid(2, (1.0, 0.7, 1.3), perturb=0.01, rng=3)
    X = bg.lagrangecxd0(m)
    op = getattr(bg.Helmholtz3D, {"sl": "singlelayer", "dl": "doublelayer",
                                  "dlt": "doublelayer_transposed"}[which])(gamma=1.0 + 1.0j)
    _check(op, X, X, ctx)


def test_helmholtz_p1_sauter(ctx):
    m = bg.icosphere(1)
    X = bg.lagrangec0d1(m)
    op = bg.Helmholtz3D.singlelayer(wavenumber=1.5)
    _check(op, X, X, ctx, qs=bg.DoubleNumSauterQstrat(2, 3, 4, 4, 4, 4))


def test_mixed_precision_assembly(ctx):
    X = bg.raviartthomas(bg.icosphere(2))
    op = bg.Maxwell3D.singlelayer(wavenumber=2.0)
    Z = bg.assemble(op, X, X, precision=bg.MIXED, ctx=ctx)
    assert Z.dtype == np.complex64
    Zo = O.assemble(_orc_op(op), _orc_qs(bg.defaultquadstrat(op, X, X)), X, X)
    assert rel(Z.astype(np.complex128), Zo) < 2e-5


def test_chunked_assembly_identical(ctx):
    X = bg.raviartthomas(bg.icosphere(2))
    op = bg.Maxwell3D.singlelayer(wavenumber=2.0)
    Z1 = bg.assemble(op, X, X, ctx=ctx)
    c2 = bg.Context(0)
    c2.set_workspace_limit(4 << 20)  # forces many trial chunks
    Z2 = bg.assemble(op, X, X, ctx=c2)
    c2.close()
    assert np.array_equal(Z1, Z2)


def test_linear_combination_mfie(ctx):
    # (n x K - 1/2 Id), examples/nxmfie.jl
    X = bg.raviartthomas(bg.icosphere(1))
    nxk = bg.nxdoublelayer(wavenumber=1.0)
    Z = bg.assemble(nxk - 0.5 * bg.Identity(), X, X, ctx=ctx)
    Zo = O.assemble(_orc_op(nxk), _orc_qs(bg.defaultquadstrat(nxk, X, X)), X, X)
    Zo = Zo - 0.5 * O.assemble_local(0, X, X, degree=6)
    assert rel(Z, Zo) < 1e-9


def test_rhs_and_farfield(ctx):
    X = bg.raviartthomas(bg.icosphere(2))
    k = 2.0
    E = bg.Maxwell3D.planewave(direction=(1, 0, 0), polarization=(0, 0, 1), wavenumber=k)
    b = bg.assemble_rhs(bg.tangential_trace(E), X)
    bo = O.rhs_planewave(0, X, (1, 0, 0), (0, 0, 1), 1j * k)
    assert np.abs(b - bo).max() <= 1e-12 * np.abs(bo).max()
    bh = bg.assemble_rhs(bg.cross_trace_H(E), X)
    bho = O.rhs_planewave(1, X, (1, 0, 0), (0, 0, 1), 1j * k)
    assert np.abs(bh - bho).max() <= 1e-12 * np.abs(bho).max()
    u = np.random.default_rng(0).normal(size=X.numfunctions()) * (1 + 0.5j)
    th = np.linspace(0, np.pi, 7)
    dirs = np.stack([np.sin(th), np.zeros_like(th), np.cos(th)], axis=1)
    ff = bg.farfield(X, u, dirs, 1j * k)
    ffo = O.farfield(X, u, dirs, 1j * k)
    assert np.abs(ff - ffo).max() <= 1e-12 * np.abs(ffo).max()


def test_blockassembler_full_block_equals_assemble(ctx):
    """test_blockassembler.jl: the block over all functions equals the full matrix
    (double layer on the sphere5 mesh) to one ulp of the largest entry"""
    X = bg.raviartthomas(bg.readmesh(mesh_path("sphere5.in")))
    op = bg.Maxwell3D.doublelayer(wavenumber=2 * np.pi / 20.0)
    A = bg.assemble(op, X, X, ctx=ctx)
    blk = bg.blockassembler(op, X, X, ctx=ctx)
    n = X.numfunctions()
    B = blk(np.arange(n), np.arange(n))
    assert np.abs(A - B).max() <= np.finfo(np.float64).eps * np.abs(A).max()


@pytest.mark.parametrize("precision", [bg.FP64, bg.MIXED])
def test_assemblerow_subset_blocks(ctx, precision):
    """test_assemblerow.jl: rows of subset(X, I) against the full matrix, plus columns and
    scattered blocks with repeated ids (Maxwell single layer on sphere35; Helmholtz P0)"""
    X = bg.raviartthomas(bg.readmesh(mesh_path("sphere35.in")))
    op = bg.Maxwell3D.singlelayer(wavenumber=1.0)
    A = bg.assemble(op, X, X, precision=precision, ctx=ctx)
    scale = np.abs(A).max()
    tol = 1e-14 if precision == bg.FP64 else 1e-6
    r = bg.assemblerow(op, X, X, 0, precision=precision, ctx=ctx)
    assert np.abs(r[0] - A[0]).max() <= tol * scale
    c = bg.assemblecol(op, X, X, 5, precision=precision, ctx=ctx)
    assert np.abs(c[:, 0] - A[:, 5]).max() <= tol * scale
    I, J = [3, 2, 7], [11, 0, 11, 40]
    B = bg.blockassembler(op, X, X, precision=precision, ctx=ctx)(I, J)
    assert np.abs(B - A[np.ix_(I, J)]).max() <= tol * scale
    Y = bg.lagrangecxd0(bg.icosphere(2))
    hh = bg.Helmholtz3D.singlelayer(wavenumber=1.5)
    H = bg.assemble(hh, Y, Y, precision=precision, ctx=ctx)
    rng = np.random.default_rng(2)
    I = rng.integers(0, Y.numfunctions(), 17)
    J = rng.integers(0, Y.numfunctions(), 9)
    Hb = bg.blockassembler(hh, Y, Y, precision=precision, ctx=ctx)(I, J)
    assert np.abs(Hb - H[np.ix_(I, J)]).max() <= tol * np.abs(H).max()
