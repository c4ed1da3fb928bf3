"""Host mirror of BEAST's assembly / solve API on top of the C ABI.

    Z = assemble(op, X, Y; quadstrat, precision)     src/operator.jl:100-116
    b = assemble(excitation, X)                       src/excitation.jl:17-25
    u = solve(Z, b) / gmres(Z, b)                     src/solvers/lusolver.jl, itsolver.jl
    ff = potential(MWFarField3D(gamma), dirs, u, X)    src/postproc.jl:138-147

Matrices come back as numpy complex arrays (host) or stay on the device as torch CUDA
tensors (`out=` a preallocated tensor); the compute always runs in libbeastgpu.
"""
import ctypes as C

import numpy as np

from . import lib as L
from . import mesh as M
from . import operators as O
from . import spaces as S

_CTX = {}


class Context:
    def __init__(self, device=0):
        self.lib = L.load()
        h = C.c_void_p()
        rc = self.lib.beast_ctx_create(device, C.byref(h))
        if rc != 0:
            raise L.BeastError(rc, f"cannot create a context on device {device}")
        self.handle = h
        self.device = device
        self._meshes = {}
        self._spaces = {}

    def check(self, rc):
        L.check(rc, self.handle)

    def close(self):
        if self.handle:
            for hs in self._spaces.values():
                self.lib.beast_space_free(hs[0])
            for hm in self._meshes.values():
                self.lib.beast_mesh_free(hm[0])
            self._spaces.clear()
            self._meshes.clear()
            self.lib.beast_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def prof_enable(self, on=True, kinds=None):
        """start (or stop) recording; kinds: names of L.PROF_KINDS to record (default all)"""
        if on and kinds is not None:
            mask = sum(1 << L.PROF_KINDS.index(k) for k in kinds)
            self.check(self.lib.beast_prof_enable_kinds(self.handle, mask))
        else:
            self.check(self.lib.beast_prof_enable(self.handle, 1 if on else 0))

    def prof_read(self):
        """{kind: (ms, launches, work)} for the records since prof_enable"""
        out = {}
        for k, name in enumerate(L.PROF_KINDS):
            ms, nl, w = C.c_double(), C.c_int64(), C.c_double()
            self.check(self.lib.beast_prof_read(self.handle, k, C.byref(ms), C.byref(nl),
                                                C.byref(w)))
            if nl.value:
                out[name] = (ms.value, nl.value, w.value)
        return out

    def launches(self):
        n = C.c_int64()
        self.check(self.lib.beast_prof_launches(self.handle, C.byref(n)))
        return n.value

    def last_factor_mode(self):
        """factorisation of the last dense solve: 0 pivoted LU, 1 unpivoted LU, 2 symmetric"""
        m = C.c_int(-1)
        self.check(self.lib.beast_last_factor_mode(self.handle, C.byref(m)))
        return m.value

    def set_workspace_limit(self, nbytes):
        self.check(self.lib.beast_ctx_set_workspace_limit(self.handle, int(nbytes)))

    def synchronize(self):
        self.check(self.lib.beast_ctx_synchronize(self.handle))

    # ---- resident geometry / spaces (uploaded once per object)
    def mesh_handle(self, mesh):
        key = id(mesh)
        ent = self._meshes.get(key)
        if ent is None or ent[1] is not mesh:
            h = C.c_void_p()
            v = np.ascontiguousarray(mesh.vertices, dtype=np.float64)
            c = np.ascontiguousarray(mesh.cells, dtype=np.int32)
            self.check(self.lib.beast_mesh_upload(self.handle, v.ctypes.data, v.shape[0],
                                                  c.ctypes.data, c.shape[0], 0, C.byref(h)))
            ent = (h, mesh)
            self._meshes[key] = ent
        return ent[0]

    def register_children(self, coarse, refinement):
        """the children of every cell of `coarse` (refinement.coarse) on the device, once"""
        h = self.mesh_handle(coarse)
        done = self.__dict__.setdefault("_children", {})
        if done.get(id(coarse)) is not refinement:
            cv = refinement.child_vertices()
            self.check(self.lib.beast_mesh_set_children(self.handle, h, cv.shape[1], cv.ctypes.data))
            done[id(coarse)] = refinement

    def space_handle(self, space):
        key = id(space)
        ent = self._spaces.get(key)
        if ent is None or ent[1] is not space:
            ad = space.assemblydata()
            mh = self.mesh_handle(space.mesh)
            h = C.c_void_p()
            self.check(self.lib.beast_space_upload(
                self.handle, mh, ad.kind, ad.cells.shape[0], ad.cells.ctypes.data, ad.maxfn,
                ad.nshapes, ad.dof.ctypes.data, ad.coeff.ctypes.data, space.numfunctions(), 0,
                C.byref(h)))
            ent = (h, space)
            self._spaces[key] = ent
        return ent[0]


def get_context(device=0):
    ctx = _CTX.get(device)
    if ctx is None or ctx.handle is None:
        ctx = Context(device)
        _CTX[device] = ctx
    return ctx


def _quadstrat(ctx, op, X, Y, quadstrat):
    """the strategy of an integral operator on X x Y: the given one or the default, wrapped in
    TestRefinesTrialQStrat / TrialRefinesTestQStrat when one space lives on the refinement of
    the other's mesh (src/operator.jl:256-262); the coarse mesh's children go to the device"""
    qs = quadstrat if quadstrat is not None else O.defaultquadstrat(op, X, Y)
    if M.refines(X.mesh, Y.mesh):
        ctx.register_children(Y.mesh, X.mesh.refinement)
        return qs if isinstance(qs, O.TestRefinesTrialQStrat) else O.TestRefinesTrialQStrat(qs)
    if M.refines(Y.mesh, X.mesh):
        ctx.register_children(X.mesh, Y.mesh.refinement)
        return qs if isinstance(qs, O.TrialRefinesTestQStrat) else O.TrialRefinesTestQStrat(qs)
    return qs


def _local_spaces(X, Y):
    """a local operator across a refinement: the coarse space written in the fine cells'
    shapes, exactly (assemble_local_refines!, src/localop.jl:155-216)"""
    if M.refines(X.mesh, Y.mesh):
        return X, X.mesh.refinement.refined_space(Y)
    if M.refines(Y.mesh, X.mesh):
        return Y.mesh.refinement.refined_space(X), Y
    return X, Y


def _op_desc(op):
    return L.OpDesc(op.kind, op.gamma.real, op.gamma.imag, op.alpha.real, op.alpha.imag,
                    op.beta.real, op.beta.imag)


def _qs_desc(qs):
    return L.QsDesc(*qs.orders())


def _target(out, nrows, ncols, dtype):
    """returns (pointer, ld, location, keepalive, result) for a Z argument"""
    if out is None:
        Z = np.zeros((ncols, nrows), dtype=np.complex128 if dtype == L.C128 else np.complex64)
        return Z.ctypes.data, nrows, L.HOST, Z, Z.T
    try:
        import torch
        if isinstance(out, torch.Tensor):
            assert out.is_cuda and out.dim() == 2
            # column-major (nrows x ncols): a row-major (ncols x ld) tensor, transposed view
            ld = out.stride(1) if out.stride(0) == 1 else None
            assert ld is not None, "out must be column-major (use tensor.T of a row-major buffer)"
            return out.data_ptr(), ld, L.DEVICE, out, out
    except ImportError:
        pass
    assert isinstance(out, np.ndarray) and out.flags.f_contiguous
    return out.ctypes.data, out.shape[0], L.HOST, out, out


def assemble(op, X, Y=None, quadstrat=None, precision=L.FP64, out=None, dtype=None, ctx=None,
             row_off=0, col_off=0, coeff=1.0, accumulate=False):
    """dense Galerkin matrix of `op` (integral, local or a linear combination) on X x Y"""
    ctx = ctx or get_context()
    Y = X if Y is None else Y
    if dtype is None:
        dtype = L.C64 if precision == L.MIXED else L.C128
    ptr, ld, loc, keep, result = _target(out, X.numfunctions(), Y.numfunctions(), dtype)
    terms = op.terms if isinstance(op, O.LinearCombination) else [(1.0, op)]
    acc = accumulate
    for (c, term) in terms:
        c = complex(c) * complex(coeff)
        if isinstance(term, O.LocalOperator):
            tX, tY = _local_spaces(X, Y)
            th, bh = ctx.space_handle(tX), ctx.space_handle(tY)
            if not acc:
                # the local store adds; start from zero when it is the first term
                _zero_block(result, loc, row_off, col_off, X.numfunctions(), Y.numfunctions())
            ctx.check(ctx.lib.beast_assemble_local(ctx.handle, term.which, th, bh, 6, ptr, ld, dtype,
                                                   loc, row_off, col_off, c.real, c.imag))
        else:
            qs = _quadstrat(ctx, term, X, Y, quadstrat)
            th, bh = ctx.space_handle(X), ctx.space_handle(Y)
            od, qd = _op_desc(term), _qs_desc(qs)
            ctx.check(ctx.lib.beast_assemble(ctx.handle, C.byref(od), C.byref(qd), th, bh, precision,
                                             ptr, ld, dtype, loc, row_off, col_off, c.real, c.imag,
                                             1 if acc else 0))
        acc = True
    return result


def blockassembler(op, X, Y=None, quadstrat=None, precision=L.FP64, ctx=None):
    """BEAST.blockassembler (src/integralop.jl:228-320) for an integral operator: returns
    f(test_ids, trial_ids) -> the block a(test_ids[i], trial_ids[j]) as a host array, with
    0-based function indices; every entry equals the full assembly's"""
    ctx = ctx or get_context()
    Y = X if Y is None else Y
    if isinstance(op, (O.LinearCombination, O.LocalOperator)):
        raise ValueError("blockassembler: integral operators only")
    qs = _quadstrat(ctx, op, X, Y, quadstrat)
    od, qd = _op_desc(op), _qs_desc(qs)
    dtype = L.C64 if precision == L.MIXED else L.C128

    def block(test_ids, trial_ids):
        I = np.ascontiguousarray(np.atleast_1d(test_ids), dtype=np.int64)
        J = np.ascontiguousarray(np.atleast_1d(trial_ids), dtype=np.int64)
        Z = np.zeros((len(I), len(J)), dtype=np.complex64 if dtype == L.C64 else np.complex128, order="F")
        ctx.check(ctx.lib.beast_assemble_block(ctx.handle, C.byref(od), C.byref(qd), ctx.space_handle(X),
                                               ctx.space_handle(Y), I.ctypes.data, len(I), J.ctypes.data,
                                               len(J), 0, precision, Z.ctypes.data, len(I), dtype, L.HOST,
                                               1.0, 0.0, 0))
        return Z
    return block


def assemblerow(op, X, Y, m, **kw):
    """row m of the matrix (BEAST.assemblerow on the one-function test space subset(X, m))"""
    Y = X if Y is None else Y
    return blockassembler(op, X, Y, **kw)([m], np.arange(Y.numfunctions()))


def assemblecol(op, X, Y, n, **kw):
    """column n of the matrix (BEAST.assemblecol)"""
    Y = X if Y is None else Y
    return blockassembler(op, X, Y, **kw)(np.arange(X.numfunctions()), [n])


def _zero_block(result, loc, r0, c0, nr, nc):
    if loc == L.HOST:
        result[r0:r0 + nr, c0:c0 + nc] = 0
    else:
        result[r0:r0 + nr, c0:c0 + nc].zero_()


def assemble_rhs(exc, X, ctx=None, degree=8):
    """excitation vector (complex128, host) of a plane-wave trace tested with X"""
    ctx = ctx or get_context()
    w = exc.wave
    d = np.ascontiguousarray(w.direction, dtype=np.float64)
    p = np.ascontiguousarray(getattr(w, "polarization", (0.0, 0.0, 0.0)), dtype=np.float64)
    b = np.zeros(X.numfunctions(), dtype=np.complex128)
    g, a = complex(w.gamma), complex(w.amplitude)
    ctx.check(ctx.lib.beast_rhs_planewave(ctx.handle, exc.kind, ctx.space_handle(X), d.ctypes.data,
                                          p.ctypes.data, g.real, g.imag, a.real, a.imag, degree,
                                          b.ctypes.data, L.HOST))
    return b


def solve(Z, b, precision=L.FP64, tol=1e-12, maxiter=30, ctx=None):
    """x = Z \\ b.  Z: torch CUDA tensor (column-major, c128/c64) or numpy (copied to the device)"""
    ctx = ctx or get_context()
    import torch
    if isinstance(Z, np.ndarray):
        Zt = torch.from_numpy(np.ascontiguousarray(Z.T)).cuda().T
    else:
        Zt = Z
    n = Zt.shape[0]
    dt = L.C64 if Zt.dtype == torch.complex64 else L.C128
    ld = Zt.stride(1)
    bb = np.ascontiguousarray(np.asarray(b, dtype=np.complex128).reshape(n, -1).T)
    x = np.zeros_like(bb)
    it, res = C.c_int(0), C.c_double(0.0)
    rc = ctx.lib.beast_solve_dense(ctx.handle, n, Zt.data_ptr(), ld, dt, precision, bb.ctypes.data,
                                   x.ctypes.data, bb.shape[0], L.HOST, tol, maxiter, C.byref(it),
                                   C.byref(res))
    ctx.check(rc)
    x = x.T
    return (x[:, 0] if np.ndim(b) == 1 else x), it.value, res.value


def gmres(Z, b, reltol=1e-8, restart=0, maxiter=0, ctx=None):
    ctx = ctx or get_context()
    import torch
    if isinstance(Z, np.ndarray):
        Zt = torch.from_numpy(np.ascontiguousarray(Z.T)).cuda().T
    else:
        Zt = Z
    n = Zt.shape[0]
    dt = L.C64 if Zt.dtype == torch.complex64 else L.C128
    bb = np.ascontiguousarray(b, dtype=np.complex128)
    x = np.zeros(n, dtype=np.complex128)
    it, res = C.c_int(0), C.c_double(0.0)
    rc = ctx.lib.beast_gmres(ctx.handle, n, Zt.data_ptr(), Zt.stride(1), dt, bb.ctypes.data,
                             x.ctypes.data, L.HOST, reltol, restart, maxiter, C.byref(it),
                             C.byref(res))
    ctx.check(rc)
    return x, it.value, res.value


def farfield(X, u, directions, gamma, degree=10, ctx=None):
    """potential(MWFarField3D(gamma), directions, u, X): [npts, 3] complex"""
    ctx = ctx or get_context()
    uu = np.ascontiguousarray(u, dtype=np.complex128)
    pts = np.ascontiguousarray(directions, dtype=np.float64)
    ff = np.zeros((pts.shape[0], 3), dtype=np.complex128)
    g = complex(gamma)
    ctx.check(ctx.lib.beast_farfield(ctx.handle, ctx.space_handle(X), uu.ctypes.data, pts.ctypes.data,
                                     pts.shape[0], g.real, g.imag, degree, ff.ctypes.data, L.HOST))
    return ff


def solve_job(op, X, exc, precision=L.MIXED, tol=1e-10, quadstrat=None, ctx=None):
    """assemble + excitation + dense solve in one call (matrix stays on the device)"""
    ctx = ctx or get_context()
    qs = quadstrat if quadstrat is not None else O.defaultquadstrat(op, X, X)
    od, qd = _op_desc(op), _qs_desc(qs)
    w = exc.wave
    d = np.ascontiguousarray(w.direction, dtype=np.float64)
    p = np.ascontiguousarray(getattr(w, "polarization", (0.0, 0.0, 0.0)), dtype=np.float64)
    x = np.zeros(X.numfunctions(), dtype=np.complex128)
    it, res = C.c_int(0), C.c_double(0.0)
    g = complex(w.gamma)
    rc = ctx.lib.beast_solve_job(ctx.handle, C.byref(od), C.byref(qd), ctx.space_handle(X), exc.kind,
                                 d.ctypes.data, p.ctypes.data, g.real, g.imag, precision, tol,
                                 x.ctypes.data, L.HOST, C.byref(it), C.byref(res))
    ctx.check(rc)
    return x, it.value, res.value
