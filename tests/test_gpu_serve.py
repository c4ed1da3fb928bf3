"""GPU: the request loop runs jobs side by side, and each job's solution is the one it gets
when it runs alone."""
import numpy as np
import pytest

import beastgpu as bg

pytestmark = pytest.mark.gpu


def _jobs():
    rng = np.random.default_rng(5)
    out = []
    for kind, lv, k, nr in (("efie", 2, 3.0, 2), ("efie", 3, 5.0, 1), ("hh", 2, 2.0, 3), ("mfie", 2, 4.0, 2),
                            ("hh", 3, 6.0, 1), ("efie", 2, 7.0, 3)):
        m = bg.icosphere(lv)
        dirs = rng.normal(size=(nr, 3))
        dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
        if kind == "hh":
            waves = [bg.Helmholtz3D.planewave(tuple(d), wavenumber=k) for d in dirs]
            out.append({"mesh": m, "space": bg.lagrangecxd0(m), "op": bg.Helmholtz3D.singlelayer(wavenumber=k),
                        "waves": waves, "exc_kind": bg.dirichlet_trace(waves[0]).kind})
        else:
            pols = [np.cross(d, rng.normal(size=3)) for d in dirs]
            waves = [bg.Maxwell3D.planewave(tuple(d), tuple(p / np.linalg.norm(p)), k) for d, p in zip(dirs, pols)]
            op = bg.Maxwell3D.singlelayer(wavenumber=k) if kind == "efie" else bg.nxdoublelayer(wavenumber=k)
            exc = bg.tangential_trace(waves[0]) if kind == "efie" else bg.cross_trace_H(waves[0])
            out.append({"mesh": m, "space": bg.raviartthomas(m), "op": op, "waves": waves, "exc_kind": exc.kind,
                        "local": None if kind == "efie" else (0, -0.5)})
    return out


@pytest.mark.parametrize("precision", [None, bg.MIXED_BALANCED])
def test_each_result_is_the_same_alone_and_in_the_mix(precision):
    """the default (mixed) requests, and the same requests in the balanced mode (double-float
    Green's function values and divergence terms, c128 matrices in the footprint)"""
    jobs = _jobs()
    if precision is not None:
        for j in jobs:
            j["precision"] = precision
    with bg.Server(slots=1, hbm_budget=16 << 30) as s:
        alone = [s.submit(j).result(timeout=600) for j in jobs]
    with bg.Server(slots=3, hbm_budget=16 << 30) as s:
        futs = [s.submit(j) for j in jobs]
        mixed = [f.result(timeout=600) for f in futs]
        lat = s.latency_ms()
        assert s.peak_bytes <= s.budget
    assert lat["jobs"] == len(jobs)
    for j, (xa, _, ra), (xm, _, rm) in zip(jobs, alone, mixed):
        assert xa.shape == (len(j["waves"]), j["space"].numfunctions())
        assert ra <= 1e-10 and rm <= 1e-10
        assert np.linalg.norm(xm - xa) / np.linalg.norm(xa) <= 1e-12


def test_resident_system_solves_like_a_fresh_job():
    """beast_system_*: assemble + factor once, solve twice with different plane waves; each
    solve equals the one-shot job (beast_solve_job) on the same wave"""
    import ctypes as C
    ctx = bg.Context(0)
    m = bg.icosphere(2)
    X = bg.raviartthomas(m)
    op = bg.Maxwell3D.singlelayer(wavenumber=3.0)
    od, qd = bg.api._op_desc(op), bg.api._qs_desc(bg.defaultquadstrat(op, X, X))
    sh = ctx.space_handle(X)
    h = C.c_void_p()
    ctx.check(ctx.lib.beast_system_create(ctx.handle, C.byref(od), C.byref(qd), sh, -1, 0.0, 0.0, bg.MIXED,
                                          C.byref(h)))
    nb = C.c_size_t(0)
    ctx.check(ctx.lib.beast_system_bytes(h, C.byref(nb)))
    n = X.numfunctions()
    assert nb.value >= n * n * 16
    rng = np.random.default_rng(8)
    try:
        for _ in range(2):
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            p = np.cross(d, rng.normal(size=3))
            p /= np.linalg.norm(p)
            dirs, pols = np.ascontiguousarray([d]), np.ascontiguousarray([p])
            x = np.zeros(n, np.complex128)
            it, res = C.c_int(0), C.c_double(0)
            ctx.check(ctx.lib.beast_system_solve(ctx.handle, h, 0, 1, dirs.ctypes.data, pols.ctypes.data, 0.0, 3.0,
                                                 1e-10, x.ctypes.data, bg.lib.HOST, C.byref(it), C.byref(res)))
            E = bg.Maxwell3D.planewave(tuple(d), tuple(p), 3.0)
            xo, _, _ = bg.solve_job(op, X, bg.tangential_trace(E), precision=bg.MIXED, tol=1e-10, ctx=ctx)
            assert res.value <= 1e-10
            assert np.linalg.norm(x - xo) / np.linalg.norm(xo) <= 1e-12
    finally:
        ctx.lib.beast_system_free(h)
        ctx.close()


def test_server_keeps_systems_resident():
    """a second request on the same system (new right-hand sides) reuses the factored system
    kept by the slot; its answer equals the one without residency, and the admitted
    footprints plus the resident systems stay within the budget"""
    jobs = _jobs()[:3]
    rng = np.random.default_rng(9)
    again = []
    for j in jobs:  # the same systems, other plane waves of the same wavenumber
        k = abs(complex(j["waves"][0].gamma))
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        if j.get("local") is None and j["space"].refspace_nshapes() == 1:
            w = [bg.Helmholtz3D.planewave(tuple(d), wavenumber=k)]
        else:
            p = np.cross(d, rng.normal(size=3))
            w = [bg.Maxwell3D.planewave(tuple(d), tuple(p / np.linalg.norm(p)), k)]
        again.append(dict(j, waves=w))
    with bg.Server(slots=1, hbm_budget=16 << 30) as s:
        ref = [s.submit(j).result(timeout=600) for j in again]
    with bg.Server(slots=2, hbm_budget=16 << 30, resident_systems=4) as s:
        for f in [s.submit(j) for j in jobs]:
            f.result(timeout=600)
        created = sum(c.systems.created for c in s._ctxs)
        got = [s.submit(j).result(timeout=600) for j in again]
        assert sum(c.systems.created for c in s._ctxs) == created  # no new system
        assert s.peak_bytes <= s.budget
        pool = s.pool_stats()
        assert pool["reserved_high"] <= s.budget + (2 << 30)
    for (x, _, _), (xr, _, _) in zip(got, ref):
        assert np.linalg.norm(x - xr) / np.linalg.norm(xr) <= 1e-12
