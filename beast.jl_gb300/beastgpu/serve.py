"""Serving form of `solve(eq)` (src/solvers/lusolver.jl:9-39): a request loop that runs
assemble + excitation + dense-solve jobs of different sizes concurrently on one GPU.

    srv = Server(slots=2)                   # two worker contexts, one CUDA stream each
    fut = srv.submit(job)                   # job: see run_job
    x, iters, resid = fut.result()
    srv.latency_ms()                        # p50 / p99 / max of submit -> completion
    srv.close()

Residency.  Each slot keeps the meshes / spaces it served (`resident`, least recently used
out) and, with `resident_systems`, whole factored systems (`beast_system_*`: the matrix and
its factors) keyed by (space, operator, strategy, local term, precision): a request on a
resident system only builds its excitations and solves against the kept factors.  A job is
routed to the slot that holds its system when that slot is free.

Memory.  All of a job's device memory comes from the CUDA stream-ordered pool the library
allocates from (matrix, factors, vectors), so the admitted footprints, plus the bytes of the
resident systems, bound what the pool holds.

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


def system_key(job):
    """what identifies a job's system: the space (by identity), the operator, the strategy,
    the local term and the precision"""
    from .operators import defaultquadstrat
    op = job["op"]
    qs = job.get("quadstrat") or defaultquadstrat(op, job["space"], job["space"])
    return (id(job["space"]), op.kind, complex(op.gamma), complex(op.alpha), complex(op.beta), tuple(qs.orders()),
            tuple(job.get("local") or ()), job.get("precision", L.MIXED))


class ResidentSystems:
    """factored systems kept on a slot's device (least recently used first out, at most
    `capacity` of them), each with its own mesh and space handles; `bytes` is what the
    systems hold"""

    def __init__(self, ctx, capacity):
        self.ctx = ctx
        self.capacity = int(capacity)
        self.entries = collections.OrderedDict()  # key -> (space, system, bytes, mesh h, space h)
        self.created = 0

    @property
    def bytes(self):
        return sum(e[2] for e in self.entries.values())

    def __contains__(self, key):
        return key in self.entries

    def get(self, key, m, space, make):
        """the system of key (make(space handle) creates it on a miss)"""
        e = self.entries.get(key)
        if e is not None and e[0] is space:
            self.entries.move_to_end(key)
            return e[1]
        if e is not None:  # a dead space's id was reused
            self._free(self.entries.pop(key))
        mh, sh = _upload(self.ctx, m, space)
        try:
            h = make(sh)
        except BaseException:
            self.ctx.lib.beast_space_free(sh)
            self.ctx.lib.beast_mesh_free(mh)
            raise
        nb = C.c_size_t(0)
        self.ctx.check(self.ctx.lib.beast_system_bytes(h, C.byref(nb)))
        self.entries[key] = (space, h, int(nb.value), mh, sh)
        self.created += 1
        while len(self.entries) > self.capacity:
            self._free(self.entries.popitem(last=False)[1])
        return h

    def evict_oldest(self):
        """frees the least recently used system; False when there is none"""
        if not self.entries:
            return False
        self._free(self.entries.popitem(last=False)[1])
        return True

    def _free(self, e):
        self.ctx.lib.beast_system_free(e[1])
        self.ctx.lib.beast_space_free(e[4])
        self.ctx.lib.beast_mesh_free(e[3])

    def close(self):
        while self.entries:
            self._free(self.entries.popitem(last=False)[1])


def run_job(ctx, job):
    """one job through the C ABI on ctx's stream: mesh + space upload (or the handles kept by
    ctx.resident, a ResidentSpaces), the factored system (beast_system_create: assembly on the
    device, plus an optional local operator `local` = (which, coefficient), e.g. (0, -0.5) for
    the MFIE's -Id/2, and the factorisation -- or the one kept by ctx.systems, a
    ResidentSystems), one excitation per plane wave and the solve of all of them against the
    factors, solution back to the host.  job: mesh, space, op, waves, exc_kind, and optionally
    local, precision (default MIXED), tol (default 1e-10), quadstrat.  Returns
    (x [nrhs, n], iters, resid)."""
    from . import api
    from .operators import defaultquadstrat
    m, X, op, waves, exc_kind = job["mesh"], job["space"], job["op"], job["waves"], job["exc_kind"]
    prec = job.get("precision", L.MIXED)
    tol = job.get("tol", 1e-10)
    if len({complex(w.gamma) for w in waves}) != 1:
        raise ValueError("the plane waves of one job share their wavenumber")
    lib = ctx.lib
    resident = getattr(ctx, "resident", None)
    systems = getattr(ctx, "systems", None)
    n = X.numfunctions()
    nr = len(waves)
    qs = job.get("quadstrat") or defaultquadstrat(op, X, X)
    od, qd = api._op_desc(op), api._qs_desc(qs)
    which, lc = job.get("local") or (-1, 0.0)
    lc = complex(lc)

    def make(sh):
        h = C.c_void_p()
        ctx.check(lib.beast_system_create(ctx.handle, C.byref(od), C.byref(qd), sh, which, lc.real, lc.imag,
                                          prec, C.byref(h)))
        return h

    mh = sh = None
    if systems is None:
        if resident is not None:
            mh, sh = resident.handles(m, X)
        else:
            mh, sh = _upload(ctx, m, X)
    try:
        sysh = systems.get(system_key(job), m, X, make) if systems is not None else make(sh)
        try:
            dirs = np.ascontiguousarray([w.direction for w in waves], dtype=np.float64)
            pols = np.ascontiguousarray([getattr(w, "polarization", (0.0, 0.0, 0.0)) for w in waves],
                                        dtype=np.float64)
            g = complex(waves[0].gamma)
            amps = [complex(w.amplitude) for w in waves]
            x = np.zeros((nr, n), dtype=np.complex128)
            it, res = C.c_int(0), C.c_double(0)
            ctx.check(lib.beast_system_solve(ctx.handle, sysh, exc_kind, nr, dirs.ctypes.data, pols.ctypes.data,
                                             g.real, g.imag, tol, x.ctypes.data, L.HOST, C.byref(it), C.byref(res)))
            x *= np.asarray(amps)[:, None]  # the solve is linear in the wave's amplitude
        finally:
            if systems is None:
                lib.beast_system_free(sysh)
    finally:
        if systems is None and resident is None:
            lib.beast_space_free(sh)
            lib.beast_mesh_free(mh)
    return x, it.value, res.value


class Server:
    """worker slots (one context and host thread each) behind an admission queue bounded by an
    HBM budget.  resident > 0 keeps that many (mesh, space) pairs on each slot's device context
    (ResidentSpaces).  make_context / runner are replaceable (tests drive the admission logic on
    the CPU with stand-ins); footprint(job) defaults to job_footprint of the job's space."""

    def __init__(self, slots=2, hbm_budget=None, device=0, allow_pass=False, workspace=None,
                 make_context=None, runner=None, footprint=None, resident=0, resident_systems=0,
                 key=None):
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
                if resident_systems > 0:  # factored systems kept on the device per slot
                    c.systems = ResidentSystems(c, resident_systems)
                return c
        self._key = key or (system_key if resident_systems > 0 else None)
        self._cv = threading.Condition()
        self._pending = collections.deque()
        self._free = []
        self._used = 0
        self._peak = 0
        self._running = 0
        self._closed = False
        self._lat = []
        self._ctxs = [make_context() for _ in range(slots)]
        self._held = [0] * slots  # bytes of the resident systems of each slot
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

    def _slot_for(self, job):  # caller holds _cv: a free slot, the one holding the job's system first
        if self._key is not None:
            k = self._key(job)
            for s in self._free:
                systems = getattr(self._ctxs[s], "systems", None)
                if systems is not None and k in systems:
                    return s, True
        return self._free[-1], False

    def _make_room(self, need, keep):  # caller holds _cv: evict resident systems of idle slots
        for s in list(self._free):
            systems = getattr(self._ctxs[s], "systems", None)
            while systems is not None and self._used + sum(self._held) + need > self.budget:
                if s == keep and len(systems.entries) <= 1 or not systems.evict_oldest():
                    break
                self._held[s] = systems.bytes
        return self._used + sum(self._held) + need <= self.budget

    def _dispatch(self):  # caller holds _cv
        while self._free and self._pending:
            pick = None
            for i, item in enumerate(self._pending):
                s, hit = self._slot_for(item[0])
                need = self._resident_footprint(item[0]) if hit else item[3]
                if self._used + sum(self._held) + need <= self.budget or (
                        need <= self.budget and self._make_room(need, s if hit else -1)):
                    pick = i
                    break
                if not self.allow_pass:
                    break
            if pick is None:
                return
            job, fut, t0, _ = self._pending[pick]
            del self._pending[pick]
            self._used += need
            self._peak = max(self._peak, self._used + sum(self._held))
            self._running += 1
            self._free.remove(s)
            self._queues[s].append((job, fut, t0, need))
            self._cv.notify_all()

    def _resident_footprint(self, job):
        """a job on a resident system: the excitations, solutions and refinement vectors"""
        n = job["space"].numfunctions()
        return int(16 * n * (2 * (len(job.get("waves", ())) or 1) + 4) + (16 << 20))

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
                    systems = getattr(ctx, "systems", None)
                    self._held[s] = systems.bytes if systems is not None else 0
                    self._peak = max(self._peak, self._used + sum(self._held))
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
            if getattr(c, "systems", None) is not None:
                c.systems.close()
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
        """largest sum of admitted footprints and resident systems seen (never above the budget)"""
        return self._peak

    def pool_stats(self):
        """the device pool's reserved and used bytes now and at their highest"""
        c = self._ctxs[0]
        if not hasattr(c, "lib"):
            return None
        v = [C.c_size_t(0) for _ in range(4)]
        c.check(c.lib.beast_pool_stats(c.handle, *[C.byref(x) for x in v]))
        return dict(zip(("reserved", "reserved_high", "used", "used_high"), [x.value for x in v]))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
