"""GPU: the batched assembly of many P0 meshes in one persistent launch (beast_batch_*) gives
each job the matrix its own assembly gives (to a few ulps), on the first (graph-capturing) call and on a
replay."""
import numpy as np
import pytest

import beastgpu as bg
import oracle as O

pytestmark = pytest.mark.gpu


def _jobs():
    rng = np.random.default_rng(3)
    spaces, ops = [], []
    for lv in (1, 2, 3, 2):
        m = bg.ellipsoid(lv, tuple(rng.uniform(0.5, 2.0, 3)), perturb=0.01, rng=int(rng.integers(1 << 30)))
        spaces.append(bg.lagrangecxd0(m))
        ops.append(bg.Helmholtz3D.singlelayer(wavenumber=float(rng.uniform(0.5, 8.0))))
    return ops, spaces


@pytest.mark.parametrize("precision,order", [(bg.MIXED, "largest_first"), (bg.FP64, "interleaved"),
                                             (bg.MIXED, "job")])
def test_batch_matches_per_job_assembly(precision, order):
    ops, spaces = _jobs()
    b = bg.Batch(ops, spaces, precision=precision, tile_m=64, tile_q=8, order=order)
    try:
        for call in range(2):  # capture, then replay
            Zs = [Z.cpu().numpy() for Z in b.assemble()]
            for op, X, Z in zip(ops, spaces, Zs):
                ref = bg.assemble(op, X, X, precision=precision)
                # the batched and per-mesh far kernels sum a pair's points in the same order but
                # may contract the FP64 moment updates differently: allow a few ulps of the block
                err = float(np.abs(Z - ref).max())
                assert err <= 1e-14 * float(np.abs(ref).max()), (call, err)
    finally:
        b.close()


def test_batch_fp64_matches_the_oracle():
    ops, spaces = _jobs()
    b = bg.Batch(ops[:2], spaces[:2], precision=bg.FP64)
    try:
        Zs = [Z.cpu().numpy() for Z in b.assemble()]
    finally:
        b.close()
    for op, X, Z in zip(ops[:2], spaces[:2], Zs):
        qs = bg.defaultquadstrat(op, X, X)
        Zo = O.assemble(O.make_op(op.kind, op.gamma, op.alpha, op.beta), O.OrcQs(*qs.orders()), X, X)
        err = np.abs(Z - Zo) / (np.abs(Zo) + 1e-3 * np.abs(Zo).max())
        assert err.max() < 1e-10
