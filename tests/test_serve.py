"""Admission logic of the request loop (beastgpu.serve.Server) on the CPU: stand-in contexts
and a stand-in job runner that records when each job runs."""
import threading
import time

import pytest

from beastgpu.serve import Server, job_footprint
from beastgpu import lib as L


class Recorder:
    def __init__(self, hold=0.05):
        self.hold = hold
        self.lock = threading.Lock()
        self.events = []  # (t, "start"/"end", name)

    def __call__(self, ctx, job):
        with self.lock:
            self.events.append((time.perf_counter(), "start", job["name"]))
        if job.get("fail"):
            raise RuntimeError("job failed")
        time.sleep(job.get("hold", self.hold))
        with self.lock:
            self.events.append((time.perf_counter(), "end", job["name"]))
        return job["name"]

    def order(self, kind):
        return [n for _, k, n in sorted(self.events) if k == kind]

    def concurrent(self, a, b):
        ev = {(k, n): t for t, k, n in self.events}
        return ev[("start", a)] < ev[("end", b)] and ev[("start", b)] < ev[("end", a)]


def server(rec, slots, budget, allow_pass=False):
    return Server(slots=slots, hbm_budget=budget, allow_pass=allow_pass, make_context=object,
                  runner=rec, footprint=lambda job: job["fp"])


def test_budget_holds_and_arrival_order_is_kept():
    rec = Recorder()
    jobs = [{"name": "a", "fp": 60}, {"name": "b", "fp": 60}, {"name": "c", "fp": 30}, {"name": "d", "fp": 30}]
    with server(rec, slots=4, budget=100) as s:
        futs = [s.submit(j) for j in jobs]
        assert [f.result(timeout=10) for f in futs] == ["a", "b", "c", "d"]
        assert s.peak_bytes <= 100
    # b does not fit beside a, and c waits behind b; then b and c run together
    assert rec.order("start") == ["a", "b", "c", "d"]
    assert not rec.concurrent("a", "b") and not rec.concurrent("a", "c")
    assert rec.concurrent("b", "c")


def test_allow_pass_admits_a_later_job_that_fits():
    rec = Recorder()
    jobs = [{"name": "a", "fp": 60}, {"name": "b", "fp": 60}, {"name": "c", "fp": 30}]
    with server(rec, slots=4, budget=100, allow_pass=True) as s:
        for f in [s.submit(j) for j in jobs]:
            f.result(timeout=10)
        assert s.peak_bytes <= 100
    assert rec.concurrent("a", "c")
    assert not rec.concurrent("a", "b")


def test_slots_bound_the_concurrency():
    rec = Recorder()
    jobs = [{"name": str(i), "fp": 1} for i in range(6)]
    with server(rec, slots=2, budget=100) as s:
        for f in [s.submit(j) for j in jobs]:
            f.result(timeout=10)
    running, peak = 0, 0
    for _, k, _ in sorted(rec.events):
        running += 1 if k == "start" else -1
        peak = max(peak, running)
    assert peak == 2


def test_oversized_job_fails_at_submit_and_a_failing_job_does_not_stop_the_loop():
    rec = Recorder()
    with server(rec, slots=1, budget=100) as s:
        big = s.submit({"name": "big", "fp": 101})
        with pytest.raises(ValueError):
            big.result(timeout=1)
        bad = s.submit({"name": "bad", "fp": 10, "fail": True})
        good = s.submit({"name": "good", "fp": 10})
        with pytest.raises(RuntimeError):
            bad.result(timeout=10)
        assert good.result(timeout=10) == "good"
        lat = s.latency_ms()
    assert lat["jobs"] == 2 and lat["p50"] > 0 and lat["p99"] >= lat["p50"]


def test_job_footprint_counts_the_matrix_and_its_factor_copy():
    n = 30720
    mixed = job_footprint(n, 1, L.MIXED)
    acc = job_footprint(n, 1, L.MIXED_ACCURATE)
    fp64 = job_footprint(n, 1, L.FP64)
    assert 16 * n * n < mixed < 16 * n * n + (1 << 30)
    assert 24 * n * n < acc < 24 * n * n + (1 << 30)
    assert 32 * n * n < fp64 < 32 * n * n + (1 << 30)


def test_a_cancelled_pending_job_never_runs():
    rec = Recorder(hold=0.1)
    with server(rec, slots=1, budget=100) as s:
        first = s.submit({"name": "first", "fp": 10})
        waiting = s.submit({"name": "waiting", "fp": 10})
        assert waiting.cancel()
        last = s.submit({"name": "last", "fp": 10})
        assert first.result(timeout=10) == "first" and last.result(timeout=10) == "last"
        assert waiting.cancelled()
    assert "waiting" not in rec.order("start")


class _FakeLib:
    """stand-in for the C library's mesh / space upload and free calls"""

    def __init__(self):
        self.next = 1
        self.live = set()
        self.uploads = 0

    def _new(self, ref):
        ref._obj.value = self.next
        self.live.add(self.next)
        self.next += 1
        return 0

    def beast_mesh_upload(self, ctx, verts, nv, cells, nc, base, ref):
        self.uploads += 1
        return self._new(ref)

    def beast_space_upload(self, ctx, mh, kind, ncells, cells, maxfn, nshapes, dof, coeff, nf, base, ref):
        return self._new(ref)

    def beast_space_free(self, h):
        self.live.remove(h.value)

    def beast_mesh_free(self, h):
        self.live.remove(h.value)


class _FakeCtx:
    def __init__(self):
        self.lib = _FakeLib()
        self.handle = None

    def check(self, rc):
        assert rc == 0


def test_resident_spaces_keep_the_last_used_meshes():
    from beastgpu.serve import ResidentSpaces
    import beastgpu as bg
    ctx = _FakeCtx()
    meshes = [bg.icosphere(1) for _ in range(3)]
    spaces = [bg.raviartthomas(m) for m in meshes]
    res = ResidentSpaces(ctx, capacity=2)
    h0 = res.handles(meshes[0], spaces[0])
    assert res.handles(meshes[0], spaces[0]) == h0 and ctx.lib.uploads == 1   # hit: no upload
    res.handles(meshes[1], spaces[1])
    res.handles(meshes[0], spaces[0])                                         # 0 most recent
    res.handles(meshes[2], spaces[2])                                         # evicts 1
    assert ctx.lib.uploads == 3 and len(ctx.lib.live) == 4                    # 2 pairs of handles
    res.handles(meshes[1], spaces[1])                                         # upload again
    assert ctx.lib.uploads == 4 and len(res.entries) == 2
    res.close()
    assert not ctx.lib.live


class Held:
    """stand-in for a slot's ResidentSystems: keys with their bytes"""

    def __init__(self):
        self.entries = {}

    def __contains__(self, k):
        return k in self.entries

    @property
    def bytes(self):
        return sum(self.entries.values())

    def evict_oldest(self):
        if not self.entries:
            return False
        self.entries.pop(next(iter(self.entries)))
        return True

    def close(self):
        self.entries.clear()


class HeldCtx:
    def __init__(self):
        self.systems = Held()


def test_resident_systems_count_in_admission_and_are_evicted_for_room():
    """a slot's resident systems count against the budget; a job that only fits without them
    evicts them from idle slots; a job on a resident system is routed to its slot and admitted
    with the small footprint of a solve"""
    runs = []

    def runner(ctx, job):
        runs.append((job["name"], id(ctx)))
        ctx.systems.entries[job["key"]] = job["keep"]  # the job leaves its system resident
        return job["name"]

    s = Server(slots=2, hbm_budget=100, make_context=HeldCtx, runner=runner, footprint=lambda j: j["fp"],
               key=lambda j: j["key"])
    s._resident_footprint = lambda j: 1
    try:
        assert s.submit({"name": "a", "fp": 50, "key": "A", "keep": 40}).result(timeout=10) == "a"
        assert sum(s._held) == 40
        # on A's system again: its slot, small footprint
        assert s.submit({"name": "a2", "fp": 50, "key": "A", "keep": 40}).result(timeout=10) == "a2"
        assert runs[1][1] == runs[0][1]
        # 70 does not fit beside the 40 held: the idle slot's system is evicted
        assert s.submit({"name": "b", "fp": 70, "key": "B", "keep": 10}).result(timeout=10) == "b"
        assert "A" not in [k for c in s._ctxs for k in c.systems.entries]
        assert s.peak_bytes <= 100
    finally:
        s.close()
