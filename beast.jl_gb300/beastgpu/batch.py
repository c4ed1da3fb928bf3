"""Batched assembly of many meshes in one persistent launch (beast_batch_*).

    b = Batch(ops, spaces, precision=MIXED)    # Helmholtz SL / DL^T on P0 spaces
    b.assemble()                                # first call captures a CUDA graph, then replays it
    Z = b.matrices[j]                           # torch CUDA tensor, column-major view of job j
    b.close()

Every job's matrix is a device tensor the batch owns; `assemble()` overwrites all of them in one
graph launch (far pairs of all jobs in one persistent kernel over a tile list, then their near
pairs in a second).  The tile shape (test cells x trial cells per CTA step) and the tile order
are parameters; `beastgpu.tune.autotune_batch` picks them by timing on the device.  This is
the batched form of one `assemble(op, X, X)` per mesh (src/operator.jl:100-116).
"""
import ctypes as C

import numpy as np

from . import lib as L
from .api import _op_desc, _qs_desc, get_context
from .operators import defaultquadstrat

ORDERS = {"job": 0, "largest_first": 1, "interleaved": 2}


class Batch:
    def __init__(self, ops, spaces, precision=L.MIXED, quadstrat=None, tile_m=128, tile_q=16,
                 order="largest_first", ctx=None):
        import torch
        if len(ops) != len(spaces) or not spaces:
            raise ValueError("one operator per space, at least one job")
        self.ctx = ctx or get_context()
        self.precision = precision
        self.spaces = list(spaces)
        qs = quadstrat or defaultquadstrat(ops[0], spaces[0], spaces[0])
        self._qd = _qs_desc(qs)
        dt = torch.complex64 if precision == L.MIXED else torch.complex128
        dev = f"cuda:{self.ctx.device}"
        # column-major n x n: a row-major (n, n) tensor holds Z^T, so Z = its transpose
        self._store = [torch.empty((s.numfunctions(), s.numfunctions()), dtype=dt, device=dev) for s in spaces]
        self.matrices = [t.T for t in self._store]
        n = len(spaces)
        sh = (C.c_void_p * n)(*[self.ctx.space_handle(s).value for s in spaces])
        od = (L.OpDesc * n)(*[_op_desc(o) for o in ops])
        zp = (C.c_void_p * n)(*[t.data_ptr() for t in self._store])
        self._keep = (sh, od, zp)
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.beast_batch_create(self.ctx.handle, C.byref(self._qd), n, sh, od, zp, precision,
                                                       tile_m, tile_q, ORDERS[order], C.byref(h)))
        self.handle = h

    def assemble(self):
        self.ctx.check(self.ctx.lib.beast_batch_assemble(self.ctx.handle, self.handle))
        return self.matrices

    def close(self):
        if self.handle:
            self.ctx.lib.beast_batch_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
