"""Serving form of `solve(eq)` (src/solvers/lusolver.jl:9-39): a request loop that runs
assemble + excitation + dense-solve jobs of different sizes concurrently on one GPU.

    srv = Server(slots=2)                   # two worker contexts, one CUDA stream each
    fut = srv.submit(job)                   # job: see run_job
    x, iters, resid = fut.result()
    srv.latency_ms()                        # p50 / p99 / max of submit -> completion
    srv.close()

Admission.  A job is admitted when a worker slot is free and its device footprint fits in
what the admitted jobs leave of the HBM budget (`job_footprint`: the N^2 complex entries of
the matrix and of its factor copy dominate, plus the context's assembly workspace).  Jobs are
considered in arrival order; a job that does not fit waits, and with `allow_pass` a later job
that fits may be admitted before it.  A job larger than the whole budget fails at submit.
Admitted jobs run at the same time on their own contexts (streams), so a request that
arrives while others are on the GPU starts as soon as a slot and memory free up.  A job's
result does not depend on what runs beside it: each context has its own stream and buffers,
and the library's sums run in a fixed order (the near-pair list is filled through an atomic
counter, but every pair's block has a fixed place in the matrix).
"""
import collections
import concurrent.futures as cf
import ctypes as C
import threading
import time

import numpy as np

from . import lib as L


def job_footprint(n, nrhs=1, precision=L.MIXED, workspace=0):
    """device bytes a job holds at its peak: the matrix, the factor copy, the tensor-core
    operands of the largest trailing update (K <= 1024), the right-hand sides / solutions /
    refinement vectors, the context's assembly workspace, and 64 MiB of small buffers"""
    zel = 8 if precision == L.MIXED else 16
    fel = 16 if precision == L.FP64 else 8
    tc = 12 * 1024 * n if precision != L.FP64 and n > 1024 else 0
    return int(zel * n * n + fel * n * n + tc + 16 * n * (2 * nrhs + 4) + workspace + (64 << 20))


def _upload(ctx, m, X):
    """mesh + space handles of (m, X) on ctx"""
    lib = ctx.lib
    ad = X.assemblydata()
    verts = np.ascontiguousarray(m.vertices)
    cells = np.ascontiguousarray(m.cells, dtype=np.int32)
    mh, sh = C.c_void_p(), C.c_void_p()
    ctx.check(lib.beast_mesh_upload(ctx.handle, verts.ctypes.data, verts.shape[0], cells.ctypes.data,
                                    cells.shape[0], 0, C.byref(mh)))
    rc = lib.beast_space_upload(ctx.handle, mh, ad.kind, ad.cells.shape[0], ad.cells.ctypes.data, ad.maxfn,
                                ad.nshapes, ad.dof.ctypes.data, ad.coeff.ctypes.data, X.numfunctions(), 0,
                                C.byref(sh))
    if rc != 0:
        lib.beast_mesh_free(mh)
        ctx.check(rc)
    return mh, sh


class ResidentSpaces:
    """the last `capacity` (mesh, space) pairs a context served, kept on the device (least
    recently used first out), so that requests on a mesh already seen skip the upload"""

    def __init__(self, ctx, capacity):
        self.ctx = ctx
        self.capacity = int(capacity)
        self.entries = collections.OrderedDict()  # id(space) -> (space, mesh handle, space handle)
        self.uploads = 0

    def handles(self, m, X):
        e = self.entries.get(id(X))
        if e is not None and e[0] is X:
            self.entries.move_to_end(id(X))
            return e[1], e[2]
        if e is not None:  # a dead object's id was reused
            self._free(self.entries.pop(id(X)))
        mh, sh = _upload(self.ctx, m, X)
        self.uploads += 1
        self.entries[id(X)] = (X, mh, sh)
        while len(self.entries) > self.capacity:
            self._free(self.entries.popitem(last=False)[1])
        return mh, sh

    def _free(self, e):
        self.ctx.lib.beast_space_free(e[2])
        self.ctx.lib.beast_mesh_free(e[1])

    def close(self):
        while self.entries:
            self._free(self.entries.popitem(last=False)[1])


def run_job(ctx, job):
    """one job through the C ABI on ctx's stream: mesh + space upload (or the handles kept by
    ctx.resident, a ResidentSpaces), assembly on the device (plus an optional local operator:
    `local` = (which, coefficient), e.g. (0, -0.5) for the MFIE's -Id/2), one excitation per
    plane wave, dense solve with all right-hand sides, solution back to the host.  job: mesh,
    space, op, waves, exc_kind, and optionally local, precision (default MIXED), tol (default
    1e-10).  Returns (x [nrhs, n], iters, resid)."""
    import torch
    from . import api
    from .operators import defaultquadstrat
    m, X, op, waves, exc_kind = job["mesh"], job["space"], job["op"], job["waves"], job["exc_kind"]
    prec = job.get("precision", L.MIXED)
    tol = job.get("tol", 1e-10)
    lib = ctx.lib
    resident = getattr(ctx, "resident", None)
    if resident is not None:
        mh, sh = resident.handles(m, X)
    else:
        mh, sh = _upload(ctx, m, X)
    try:
        try:
            n = X.numfunctions()
            nr = len(waves)
            qs = defaultquadstrat(op, X, X)
            od, qd = api._op_desc(op), api._qs_desc(qs)
            dev = f"cuda:{ctx.device}"
            zdt = L.C64 if prec == L.MIXED else L.C128
            Z = torch.empty((n, n), dtype=torch.complex64 if zdt == L.C64 else torch.complex128, device=dev)
            B = torch.empty((nr, n), dtype=torch.complex128, device=dev)
            Xs = torch.empty((nr, n), dtype=torch.complex128, device=dev)
            ctx.check(lib.beast_assemble(ctx.handle, C.byref(od), C.byref(qd), sh, sh, prec, Z.data_ptr(), n,
                                         zdt, L.DEVICE, 0, 0, 1.0, 0.0, 0))
            if job.get("local"):
                which, c = job["local"]
                ctx.check(lib.beast_assemble_local(ctx.handle, which, sh, sh, 6, Z.data_ptr(), n, zdt, L.DEVICE,
                                                   0, 0, c, 0.0))
            for r, w in enumerate(waves):
                d = np.ascontiguousarray(w.direction, dtype=np.float64)
                pol = np.ascontiguousarray(getattr(w, "polarization", (0.0, 0.0, 0.0)), dtype=np.float64)
                g, a = complex(w.gamma), complex(w.amplitude)
                ctx.check(lib.beast_rhs_planewave(ctx.handle, exc_kind, sh, d.ctypes.data, pol.ctypes.data, g.real,
                                                  g.imag, a.real, a.imag, 8, B[r].data_ptr(), L.DEVICE))
            it, res = C.c_int(0), C.c_double(0)
            ctx.check(lib.beast_solve_dense(ctx.handle, n, Z.data_ptr(), n, zdt, prec, B.data_ptr(), Xs.data_ptr(),
                                            nr, L.DEVICE, tol, 30, C.byref(it), C.byref(res)))
            x = Xs.cpu().numpy()
        finally:
            if resident is None:
                lib.beast_space_free(sh)
    finally:
        if resident is None:
            lib.beast_mesh_free(mh)
    return x, it.value, res.value


class Server:
    """worker slots (one context and host thread each) behind an admission queue bounded by an
    HBM budget.  resident > 0 keeps that many (mesh, space) pairs on each slot's device context
    (ResidentSpaces).  make_context / runner are replaceable (tests drive the admission logic on
    the CPU with stand-ins); footprint(job) defaults to job_footprint of the job's space."""

    def __init__(self, slots=2, hbm_budget=None, device=0, allow_pass=False, workspace=None,
                 make_context=None, runner=None, footprint=None, resident=0):
        if slots < 1:
            raise ValueError("slots must be >= 1")
        if hbm_budget is None:
            import torch
            free, _ = torch.cuda.mem_get_info(device)
            hbm_budget = int(0.9 * free)
        self.budget = int(hbm_budget)
        # assembly workspace per context: a share of the budget, so that the slots' workspaces
        # together stay within a quarter of it
        self.workspace = int(workspace if workspace is not None else
                             max(256 << 20, min(8 << 30, self.budget // (4 * slots))))
        self.allow_pass = allow_pass
        self._runner = runner or run_job
        self._footprint = footprint or self._default_footprint
        if make_context is None:
            from .api import Context

            def make_context():
                c = Context(device)
                c.set_workspace_limit(self.workspace)
                if resident > 0:  # meshes / spaces kept on the device per slot
                    c.resident = ResidentSpaces(c, resident)
                return c
        self._cv = threading.Condition()
        self._pending = collections.deque()
        self._free = []
        self._used = 0
        self._peak = 0
        self._running = 0
        self._closed = False
        self._lat = []
        self._ctxs = [make_context() for _ in range(slots)]
        self._queues = [collections.deque() for _ in range(slots)]
        self._threads = []
        for s in range(slots):
            self._free.append(s)
            t = threading.Thread(target=self._worker, args=(s,), daemon=True)
            self._threads.append(t)
            t.start()

    def _default_footprint(self, job):
        return job_footprint(job["space"].numfunctions(), len(job.get("waves", ())) or 1,
                             job.get("precision", L.MIXED), self.workspace)

    # ---- admission
    def submit(self, job):
        fut = cf.Future()
        fp = int(self._footprint(job))
        if fp > self.budget:
            fut.set_exception(ValueError(f"job footprint {fp} B exceeds the HBM budget {self.budget} B"))
            return fut
        with self._cv:
            if self._closed:
                raise RuntimeError("server closed")
            self._pending.append((job, fut, time.perf_counter(), fp))
            self._dispatch()
        return fut

    def _dispatch(self):  # caller holds _cv
        while self._free and self._pending:
            pick = None
            for i, item in enumerate(self._pending):
                if self._used + item[3] <= self.budget:
                    pick = i
                    break
                if not self.allow_pass:
                    break
            if pick is None:
                return
            item = self._pending[pick]
            del self._pending[pick]
            self._used += item[3]
            self._peak = max(self._peak, self._used)
            self._running += 1
            s = self._free.pop()
            self._queues[s].append(item)
            self._cv.notify_all()

    def _worker(self, s):
        ctx = self._ctxs[s]
        while True:
            with self._cv:
                while not self._queues[s] and not self._closed:
                    self._cv.wait()
                if not self._queues[s]:
                    return
                job, fut, t0, fp = self._queues[s].popleft()
            try:
                if fut.set_running_or_notify_cancel():
                    out = self._runner(ctx, job)
                    fut.set_result(out)
            except BaseException as e:  # the job fails, the server keeps serving
                fut.set_exception(e)
            finally:
                with self._cv:
                    self._lat.append(time.perf_counter() - t0)
                    self._used -= fp
                    self._running -= 1
                    self._free.append(s)
                    self._dispatch()
                    self._cv.notify_all()

    # ---- state
    def drain(self):
        """wait until every submitted job has completed"""
        with self._cv:
            while self._pending or self._running:
                self._cv.wait()

    def close(self):
        self.drain()
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()
        for c in self._ctxs:
            if getattr(c, "resident", None) is not None:
                c.resident.close()
            if hasattr(c, "close"):
                c.close()

    def latency_ms(self):
        """p50 / p99 / max of submit -> completion over the completed jobs (queueing included)"""
        with self._cv:
            ms = np.array(self._lat) * 1e3
        if ms.size == 0:
            return {"p50": None, "p99": None, "max": None, "jobs": 0}
        return {"p50": float(np.percentile(ms, 50)), "p99": float(np.percentile(ms, 99)),
                "max": float(ms.max()), "jobs": int(ms.size)}

    @property
    def peak_bytes(self):
        """largest sum of admitted footprints seen (never above the budget)"""
        return self._peak

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
