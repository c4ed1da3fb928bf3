"""beast_lu_solve_noalloc: the triangular solves without any device allocation.

Callers that cannot allocate at solve time (a host runtime that owns the device memory
pool, a serving loop that reserved all memory up front) get the same answer as
beast_lu_solve from a fixed scratch array inside the library.  Compared here, through the
C ABI, with beast_lu_solve on the same factors, for two calls in a row (the second one
sees the scratch the first left behind).  Collected last so that a failure here cannot
hide another test.
"""
import ctypes as C

import numpy as np
import pytest

import beastgpu as bg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,dtype", [(700, bg.C128), (1100, bg.C64)])
def test_noalloc_matches_lu_solve(n, dtype):
    import torch
    ctx = bg.get_context(0)
    rng = np.random.default_rng(5)
    npdt = np.complex64 if dtype == bg.C64 else np.complex128
    A = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)) + 4 * n ** 0.5 * np.eye(n)).astype(npdt)
    At = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    h = C.c_void_p()
    ctx.check(ctx.lib.beast_lu_factor(ctx.handle, n, At.data_ptr(), n, dtype, C.byref(h)))
    tol = 1e-5 if dtype == bg.C64 else 1e-12
    try:
        for call in range(2):
            b = (rng.normal(size=(2, n)) + 1j * rng.normal(size=(2, n))).astype(npdt)
            B1 = torch.from_numpy(b.copy()).cuda()   # row-major (2, n) = column-major n x 2
            B2 = torch.from_numpy(b.copy()).cuda()
            ctx.check(ctx.lib.beast_lu_solve(ctx.handle, h, 2, B1.data_ptr(), n))
            ctx.check(ctx.lib.beast_lu_solve_noalloc(ctx.handle, h, 2, B2.data_ptr(), n))
            x1, x2 = B1.cpu().numpy(), B2.cpu().numpy()
            assert np.abs(x1 - x2).max() <= tol * np.abs(x1).max(), call
            # and the answer solves the system
            res = np.abs(A.astype(np.complex128) @ x2[0].astype(np.complex128) - b[0]).max()
            assert res <= 1e3 * tol * np.abs(b[0]).max()
    finally:
        ctx.lib.beast_lu_free(h)


def test_noalloc_rejects_bad_leading_dimension():
    ctx = bg.get_context(0)
    # a leading dimension below n is refused before any work is queued
    import torch
    A = torch.eye(4, dtype=torch.complex128, device="cuda")
    h = C.c_void_p()
    ctx.check(ctx.lib.beast_lu_factor(ctx.handle, 4, A.data_ptr(), 4, bg.C128, C.byref(h)))
    B = torch.ones(4, dtype=torch.complex128, device="cuda")
    rc = ctx.lib.beast_lu_solve_noalloc(ctx.handle, h, 1, B.data_ptr(), 2)  # ldb < n
    assert rc == bg.lib.ERR_ARG
    ctx.lib.beast_lu_free(h)
