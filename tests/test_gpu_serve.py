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


def test_each_result_is_the_same_alone_and_in_the_mix():
    jobs = _jobs()
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
