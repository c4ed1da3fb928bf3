"""The autotuner's search, cache and apply steps on the CPU (a stand-in timer; the device
timer is the mixed solve itself)."""
import json

import beastgpu as bg


def _timer(times):
    calls = []

    def t(params):
        calls.append(dict(params))
        return times[(params["BEAST_LU_NB"], params["BEAST_LU_NB2"], params["BEAST_LU_LOOKAHEAD"])]
    return t, calls


def test_picks_the_fastest_and_applies_it(tmp_path, monkeypatch):
    for k in ("BEAST_LU_NB", "BEAST_LU_NB2", "BEAST_LU_LOOKAHEAD"):
        monkeypatch.delenv(k, raising=False)
    times = {(c["BEAST_LU_NB"], c["BEAST_LU_NB2"], c["BEAST_LU_LOOKAHEAD"]): 1.0 for c in bg.tune.CANDIDATES}
    times[("2048", "512", "0")] = 0.5
    timer, calls = _timer(times)
    import os
    e = bg.tune.autotune(30720, timer=timer, cache_path=str(tmp_path / "t.json"), key="gpu|c30")
    assert e["params"] == {"BEAST_LU_NB": "2048", "BEAST_LU_NB2": "512", "BEAST_LU_LOOKAHEAD": "0"}
    assert len(calls) == len(bg.tune.CANDIDATES)
    assert os.environ["BEAST_LU_NB"] == "2048" and os.environ["BEAST_LU_NB2"] == "512"
    saved = json.load(open(tmp_path / "t.json"))
    assert saved["gpu|c30"]["params"] == e["params"] and saved["gpu|c30"]["n"] == 30720


def test_cache_is_reused_and_force_retimes(tmp_path, monkeypatch):
    for k in ("BEAST_LU_NB", "BEAST_LU_NB2", "BEAST_LU_LOOKAHEAD"):
        monkeypatch.delenv(k, raising=False)
    path = str(tmp_path / "t.json")
    times = {(c["BEAST_LU_NB"], c["BEAST_LU_NB2"], c["BEAST_LU_LOOKAHEAD"]): 2.0 for c in bg.tune.CANDIDATES}
    times[("1024", "128", "0")] = 1.0
    timer, calls = _timer(times)
    first = bg.tune.autotune(5000, timer=timer, cache_path=path, key="gpu|c25", apply=False)

    def failing(params):
        raise AssertionError("the cached setting must be used")
    again = bg.tune.autotune(5000, timer=failing, cache_path=path, key="gpu|c25", apply=False)
    assert again == first
    times[("1024", "256", "1")] = 0.1
    forced = bg.tune.autotune(5000, timer=timer, cache_path=path, key="gpu|c25", force=True, apply=False)
    assert forced["params"]["BEAST_LU_LOOKAHEAD"] == "1"


def test_size_classes():
    assert bg.tune.size_class(30720) == bg.tune.size_class(30000)
    assert bg.tune.size_class(30720) != bg.tune.size_class(15360)


def test_batch_autotuner_search_and_cache(tmp_path):
    """the batch schedule search picks the fastest candidate, caches it by signature and
    reads it back without timing again (a stand-in timer on the CPU)"""
    from beastgpu import tune
    from beastgpu.spaces import lagrangecxd0
    from beastgpu.mesh import icosphere
    from beastgpu.operators import Helmholtz3D
    spaces = [lagrangecxd0(icosphere(1)), lagrangecxd0(icosphere(2))]
    ops = [Helmholtz3D.singlelayer(wavenumber=1.0)] * 2
    calls = []

    def timer(c):
        calls.append(c)
        return 1.0 + abs(c[0] - 128) / 64 + abs(c[1] - 32) / 16 + (0 if c[2] == "interleaved" else 0.5)

    path = str(tmp_path / "t.json")
    e = tune.autotune_batch(ops, spaces, 1, timer=timer, cache_path=path, key="k")
    assert (e["tile_m"], e["tile_q"], e["order"]) == (128, 32, "interleaved")
    n = len(calls)
    assert n == len(tune.BATCH_CANDIDATES)
    e2 = tune.autotune_batch(ops, spaces, 1, timer=timer, cache_path=path, key="k")
    assert len(calls) == n and e2["tile_q"] == 32
    assert tune.batch_signature(ops, spaces, 1).startswith("k4|p1|n2|")
