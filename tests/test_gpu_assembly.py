"""GPU parity: libbeastgpu (through the C ABI) against the CPU oracle.

Tolerances:
  FP64 path: 1e-10 relative PER ENTRY with an absolute floor at FP64 rounding level,
      |Z_ij - Zo_ij| <= 1e-10 |Zo_ij| + 1e-13 max|Zo|: relative for every entry above 1e-3 of
      the largest.  Smaller entries are sums of cell-pair terms of about that size that cancel
      (exactly zero on symmetric meshes, or the (h/R)^2 cancellation of RT divergence terms),
      so two FP64 evaluations in different order agree there to a few ulps of those terms, not
      of the entry: 1e-13 of the largest entry is 1e-10 relative to them;
  mixed-accurate path (double-float far pairs, FP64 near pairs, c128 storage): 1e-11 relative
      in the Frobenius norm and 1e-8 per entry with the same floor;
  mixed path (FP32 far pairs, c64 storage): 1e-6 relative in the Frobenius norm (the north
      star's matrix error measure; per entry the FP32 cancellation error is not bounded).
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


def rel_entry(a, b, floor=1e-3):
    """largest per-entry relative difference, with an absolute floor of floor * max|b|"""
    return float((np.abs(a - b) / (np.abs(b) + floor * np.abs(b).max())).max())


def err_profile(a, b):
    """for failure messages: relative to the largest entry, and per entry above 1e-3 of it"""
    big = np.abs(b) > 1e-3 * np.abs(b).max()
    per = np.abs(a - b)[big] / np.abs(b)[big]
    return {"max_rel": rel(a, b), "entry_q50": float(np.median(per)), "entry_max": float(per.max()),
            "floor": rel_entry(a, b)}


def rel_fro(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _orc_op(op):
    return O.make_op(op.kind, op.gamma, op.alpha, op.beta)


def _orc_qs(qs):
    o = qs.orders()
    return O.OrcQs(*o)


def _check(op, X, Y, ctx, tol=1e-10, precision=bg.FP64, qs=None):
    qs = qs or bg.defaultquadstrat(op, X, Y)
    Z = bg.assemble(op, X, Y, quadstrat=qs, precision=precision, ctx=ctx)
    Zo = O.assemble(_orc_op(op), _orc_qs(qs), X, Y)
    e = rel_entry(Z, Zo)
    assert e < tol, err_profile(Z, Zo)
    return Z, Zo


def test_efie_icosphere(ctx):
    X = bg.raviartthomas(bg.icosphere(2))
    _check(bg.Maxwell3D.singlelayer(wavenumber=2.0), X, X, ctx)


def test_efie_reference_mesh_with_near_pairs(ctx):
    # sphere45: an irregular reference mesh (Sauter-Schwab pairs of all three kinds; at k = 3 its
    # non-touching pairs are all far -- the singularity-extraction pairs are covered below on a
    # strongly perturbed ellipsoid)
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
    _check(bg.nxdoublelayer(wavenumber=2.0), X, X, ctx)


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
    assert rel_fro(Z.astype(np.complex128), Zo) < 1e-6


def test_mixed_accurate_assembly(ctx):
    """the mixed-accurate EFIE assembly: far pairs and Sauter-Schwab pairs in double-float
    arithmetic on the FP32 pipes, c128 storage"""
    X = bg.raviartthomas(bg.icosphere(2))
    op = bg.Maxwell3D.singlelayer(wavenumber=2.0)
    Z = bg.assemble(op, X, X, precision=bg.MIXED_ACCURATE, ctx=ctx)
    assert Z.dtype == np.complex128
    Zo = O.assemble(_orc_op(op), _orc_qs(bg.defaultquadstrat(op, X, X)), X, X)
    assert rel_fro(Z, Zo) < 1e-11, rel_fro(Z, Zo)
    assert rel_entry(Z, Zo) < 1e-8, err_profile(Z, Zo)


def test_mixed_accurate_assembly_into_c64(ctx):
    """double-float assembly rounded once into a c64 matrix (the large-problem mode): every
    entry is the correctly rounded float of the c128 mixed-accurate entry"""
    X = bg.raviartthomas(bg.icosphere(2))
    op = bg.Maxwell3D.singlelayer(wavenumber=3.0)
    Z64 = bg.assemble(op, X, X, precision=bg.MIXED_ACCURATE, dtype=bg.C64, ctx=ctx)
    Z128 = bg.assemble(op, X, X, precision=bg.MIXED_ACCURATE, ctx=ctx)
    assert Z64.dtype == np.complex64 and Z128.dtype == np.complex128
    assert np.array_equal(Z64, Z128.astype(np.complex64))


def test_mixed_balanced_assembly(ctx):
    """the balanced EFIE assembly: the far pairs' vector-potential (alpha) terms in FP32, about
    1e-7 of a far block's largest entry, everything else as mixed-accurate; with alpha = 0 the
    far blocks are their double-float divergence (beta) terms alone and the matrix is the
    mixed-accurate one to double-float accuracy"""
    X = bg.raviartthomas(bg.icosphere(2))
    op = bg.Maxwell3D.singlelayer(wavenumber=3.0)
    Z = bg.assemble(op, X, X, precision=bg.MIXED_BALANCED, ctx=ctx)
    assert Z.dtype == np.complex128
    Zo = O.assemble(_orc_op(op), _orc_qs(bg.defaultquadstrat(op, X, X)), X, X)
    assert rel_fro(Z, Zo) < 1e-6, rel_fro(Z, Zo)
    Za = bg.assemble(op, X, X, precision=bg.MIXED_ACCURATE, ctx=ctx)
    assert 1e-12 < rel_fro(Z, Za) < 1e-6  # the balanced core ran, and stays in its error class
    g = 3.0j
    opb = bg.Maxwell3D.singlelayer(gamma=g, alpha=0.0, beta=-1.0 / g)
    Zb = bg.assemble(opb, X, X, precision=bg.MIXED_BALANCED, ctx=ctx)
    Zab = bg.assemble(opb, X, X, precision=bg.MIXED_ACCURATE, ctx=ctx)
    assert rel_fro(Zb, Zab) < 1e-11, rel_fro(Zb, Zab)


@pytest.mark.parametrize("which", ["singlelayer", "doublelayer"])
def test_mixed_accurate_near_pairs(ctx, which):
    """the double-float Sauter-Schwab pairs (face, edge and vertex classes) of the RT Maxwell
    operators on a perturbed ellipsoid: every entry against the oracle's FP64"""
    X = bg.raviartthomas(bg.ellipsoid(2, (1.0, 0.7, 1.3), perturb=0.1, rng=5))
    op = getattr(bg.Maxwell3D, which)(wavenumber=4.0)
    Z = bg.assemble(op, X, X, precision=bg.MIXED_ACCURATE, ctx=ctx)
    Zo = O.assemble(_orc_op(op), _orc_qs(bg.defaultquadstrat(op, X, X)), X, X)
    assert rel_fro(Z, Zo) < 1e-11, rel_fro(Z, Zo)
    assert rel_entry(Z, Zo) < 1e-8, err_profile(Z, Zo)
    Z64 = bg.assemble(op, X, X, precision=bg.FP64, ctx=ctx)
    assert rel_entry(Z, Z64) < 1e-8, err_profile(Z, Z64)


def test_c1_efie_assembly(ctx):
    """the full C1 matrix: EFIE k = 2 on the 1280-triangle icosphere (1920 RT unknowns),
    default strategy, FP64, every entry against the oracle"""
    X = bg.raviartthomas(bg.icosphere(3))
    _check(bg.Maxwell3D.singlelayer(wavenumber=2.0), X, X, ctx)


def test_c2_efie_row_sample(ctx):
    """C2 (EFIE k = 10 on the 20480-triangle icosphere, 30720 RT unknowns): 256 rows in four
    blocks of 64 spread over the mesh, every column, FP64, through assemblerow-style block
    assembly, against the oracle's rows"""
    X = bg.raviartthomas(bg.icosphere(5))
    op = bg.Maxwell3D.singlelayer(wavenumber=10.0)
    qs = bg.defaultquadstrat(op, X, X)
    n = X.numfunctions()
    blk = bg.blockassembler(op, X, X, ctx=ctx)
    cols = np.arange(n)
    for lo in (0, n // 4 + 17, n // 2 + 5, n - 64):
        Zo = O.assemble(_orc_op(op), _orc_qs(qs), X, X, row_lo=lo, row_hi=lo + 64)
        Z = blk(np.arange(lo, lo + 64), cols)
        e = rel_entry(Z, Zo)
        assert e < 1e-10, (lo, err_profile(Z, Zo))


@pytest.mark.parametrize("which", ["singlelayer", "doublelayer", "doublelayer_transposed"])
@pytest.mark.parametrize("spaces", ["p1p1", "p0p1", "p1p0", "p0p0"])
def test_helmholtz_singularity_extraction(ctx, which, spaces):
    """Wilton singularity extraction for the Helmholtz operators on every P0 / P1 pairing: a
    strongly perturbed ellipsoid at small |gamma| has seven extraction pairs (the icospheres
    and the reference meshes have none for these operators)"""
    m = bg.ellipsoid(2, (1.0, 0.7, 1.3), perturb=0.3, rng=3)
    sp = {"p1": bg.lagrangec0d1(m), "p0": bg.lagrangecxd0(m)}
    op = getattr(bg.Helmholtz3D, which)(gamma=0.3j)
    _check(op, sp[spaces[:2]], sp[spaces[2:]], ctx)


@pytest.mark.parametrize("spaces", ["p0p0", "p1p1", "p0p1", "p1p0"])
def test_helmholtz_single_layer_double_float_near(ctx, spaces):
    """the Helmholtz single layer's Sauter-Schwab pairs in double-float arithmetic (the
    mixed-accurate and mixed paths, real wavenumber), with the extraction pairs of the
    perturbed ellipsoid beside them in FP64: every entry against the oracle"""
    m = bg.ellipsoid(2, (1.0, 0.7, 1.3), perturb=0.3, rng=3)
    sp = {"p1": bg.lagrangec0d1(m), "p0": bg.lagrangecxd0(m)}
    op = bg.Helmholtz3D.singlelayer(wavenumber=2.0)
    _check(op, sp[spaces[:2]], sp[spaces[2:]], ctx, tol=1e-8, precision=bg.MIXED_ACCURATE)


@pytest.mark.parametrize("which", ["singlelayer", "doublelayer"])
def test_maxwell_singularity_extraction(ctx, which):
    """the Maxwell strategy's Wilton pairs: seven on the perturbed ellipsoid at k = 0.3"""
    X = bg.raviartthomas(bg.ellipsoid(2, (1.0, 0.7, 1.3), perturb=0.3, rng=3))
    _check(getattr(bg.Maxwell3D, which)(wavenumber=0.3), X, X, ctx)


def test_bc_mfie_on_the_refinement(ctx):
    """Buffa-Christiansen testing of the MFIE on the barycentric refinement: the double layer
    through the gather's general path (functions with more than eight cell entries) and NCross
    rows that meet 19 trial functions"""
    m = bg.icosphere(1)
    X = bg.raviartthomas(m)
    R = bg.barycentric_refinement(m)
    Y, _ = bg.buffachristiansen(m, R, X)
    Xf = bg.refined(X, R)
    _check(bg.Maxwell3D.doublelayer(wavenumber=1.0), Y, Xf, ctx)
    N = bg.assemble(bg.NCross(), Y, Xf, ctx=ctx)
    assert rel_entry(N, O.assemble_local(1, Y, Xf)) < 1e-12


@pytest.mark.parametrize("which,precision,tol", [("doublelayer", bg.FP64, 1e-10), ("singlelayer", bg.FP64, 1e-10),
                                                  ("singlelayer", bg.MIXED_ACCURATE, 1e-8)])
def test_refines_strategies(ctx, which, precision, tol):
    """BC test functions on the refinement against RT trial functions on the coarse mesh: the
    library picks TestRefinesTrialQStrat (and TrialRefinesTestQStrat with the roles swapped)
    from the meshes, as src/operator.jl:256-262 does, and matches the oracle's restatement"""
    m = bg.icosphere(1)
    X = bg.raviartthomas(m)
    R = bg.barycentric_refinement(m)
    Y, _ = bg.buffachristiansen(m, R, X)
    op = getattr(bg.Maxwell3D, which)(wavenumber=1.0)
    qs = _orc_qs(bg.defaultquadstrat(op, Y, X))
    cv = R.child_vertices()
    Z = bg.assemble(op, Y, X, precision=precision, ctx=ctx)
    Zo = O.assemble_refines(_orc_op(op), qs, Y, X, cv)
    assert rel_entry(Z, Zo) < tol, err_profile(Z, Zo)
    Zt = bg.assemble(op, X, Y, precision=precision, ctx=ctx)
    Zto = O.assemble_refines(_orc_op(op), qs, X, Y, cv, split_test=True)
    assert rel_entry(Zt, Zto) < tol, err_profile(Zt, Zto)


def test_bc_mfie_across_the_refinement(ctx):
    """(K + N/2)[BC, RT] of examples/mfie.jl with the RT space on the coarse mesh: the double
    layer through TestRefinesTrialQStrat, NCross through the refined trial space (exact, as
    assemble_local_refines!); its far field agrees with the EFIE's"""
    m = bg.icosphere(2)
    X = bg.raviartthomas(m)
    R = bg.barycentric_refinement(m)
    Y, _ = bg.buffachristiansen(m, R, X)
    k = 1.0
    K = bg.Maxwell3D.doublelayer(wavenumber=k)
    A = bg.assemble(K + 0.5 * bg.NCross(), Y, X, ctx=ctx)
    N = O.assemble_local(1, Y, bg.refined(X, R))
    Ko = O.assemble_refines(_orc_op(K), _orc_qs(bg.defaultquadstrat(K, Y, X)), Y, X, R.child_vertices())
    assert rel_entry(A, Ko + 0.5 * N) < 1e-10
    # MFIE right-hand side ((n x H) x n)[BC] with H = d x p for this wave, EFIE ((n x E) x n)[RT]
    d, p = np.array([0, 0, 1.0]), np.array([1.0, 0, 0])
    H = bg.Maxwell3D.planewave(direction=d, polarization=np.cross(d, p), wavenumber=k)
    E = bg.Maxwell3D.planewave(direction=d, polarization=p, wavenumber=k)
    u_m = np.linalg.solve(A, bg.assemble_rhs(bg.tangential_trace(H), Y, ctx=ctx))
    T = bg.assemble(bg.Maxwell3D.singlelayer(wavenumber=k), X, X, ctx=ctx)
    u_e = np.linalg.solve(T, bg.assemble_rhs(bg.tangential_trace(E), X, ctx=ctx))
    th = np.linspace(0, np.pi, 91)
    dirs = np.stack([np.sin(th), 0 * th, np.cos(th)], 1)
    ff_m, ff_e = bg.farfield(X, u_m, dirs, 1j * k, ctx=ctx), bg.farfield(X, u_e, dirs, 1j * k, ctx=ctx)
    assert np.linalg.norm(ff_m - ff_e) / np.linalg.norm(ff_e) < 2e-3  # 3.1e-4 from the oracle
    assert np.linalg.cond(A) < 10


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
    assert rel_entry(Z, Zo) < 1e-10, err_profile(Z, Zo)


def test_mfie_mixed_is_near_fp32_rounding(ctx):
    """the MFIE (n x K - Id/2) assembled on the mixed path: far pairs in FP32, the pairs whose
    rule points come close in FP64 -- within 1e-6 of the FP64 matrix (Frobenius)"""
    X = bg.raviartthomas(bg.icosphere(2))
    nxk = bg.nxdoublelayer(wavenumber=3.0)
    op = nxk - 0.5 * bg.Identity()
    Zm = bg.assemble(op, X, X, precision=bg.MIXED, ctx=ctx)
    Z = bg.assemble(op, X, X, ctx=ctx)
    assert rel_fro(Zm.astype(np.complex128), Z) < 1e-6, rel_fro(Zm.astype(np.complex128), Z)


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


def test_farfield_golden_vector(ctx, golden):
    """test/test_farfield.jl on the GPU: beast_farfield of the reference's golden current
    (test/efie_solution.txt, mapped to this package's dof order) reproduces the golden
    magnitudes within the reference's 1e4 eps, with the 4-point rule they were made with"""
    from test_oracle_pins import _farfield_golden
    X, u, dirs, a = _farfield_golden(golden)
    ff = bg.farfield(X, u, dirs, 1j, degree=3, ctx=ctx) / (4 * np.pi)
    assert np.abs(np.linalg.norm(ff, axis=1) - a).max() < 1e4 * np.finfo(float).eps


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


@pytest.mark.parametrize("precision", [bg.FP64, bg.MIXED, bg.MIXED_ACCURATE])
def test_zcell_layouts_agree(ctx, monkeypatch, precision):
    """the cell-pair blocks laid out by function entries (the default for RT / P0 / P1) and by
    cells give the same matrix: the same sums in the same order"""
    X = bg.raviartthomas(bg.icosphere(2))
    op = bg.Maxwell3D.singlelayer(wavenumber=3.0)
    Ze = bg.assemble(op, X, X, precision=precision, ctx=ctx)
    monkeypatch.setenv("BEAST_ZCELL_LAYOUT", "cell")
    Zc = bg.assemble(op, X, X, precision=precision, ctx=ctx)
    assert np.array_equal(Ze, Zc)
