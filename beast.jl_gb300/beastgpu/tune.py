"""Home-grown autotuner for the dense solve's tuning switches.

The factorisation reads its block widths and lookahead from the environment at every call
(`BEAST_LU_NB`, `BEAST_LU_NB2`, `BEAST_LU_LOOKAHEAD`).  `autotune(n)` times
the mixed solve of an n x n complex-symmetric matrix on the device under each candidate
setting, keeps the fastest, applies it to this process's environment and caches it per GPU
model and size class in a JSON file, so a later process (or a serving loop) starts from the
tuned setting without timing again.

    import beastgpu as bg
    best = bg.tune.autotune(30720)        # {'BEAST_LU_NB': '1024', 'BEAST_LU_NB2': '256', ...}

The timer is replaceable: the tests drive the search, the cache and the apply step on the CPU.
"""
import json
import math
import os
import time

# candidate settings (block widths in columns: multiples of the 64-column panel, the mid width
# dividing the outer one, the outer one at most 2048)
CANDIDATES = [
    {"BEAST_LU_NB": "1024", "BEAST_LU_NB2": "256", "BEAST_LU_LOOKAHEAD": "0"},
    {"BEAST_LU_NB": "1024", "BEAST_LU_NB2": "512", "BEAST_LU_LOOKAHEAD": "0"},
    {"BEAST_LU_NB": "1024", "BEAST_LU_NB2": "128", "BEAST_LU_LOOKAHEAD": "0"},
    {"BEAST_LU_NB": "2048", "BEAST_LU_NB2": "256", "BEAST_LU_LOOKAHEAD": "0"},
    {"BEAST_LU_NB": "2048", "BEAST_LU_NB2": "512", "BEAST_LU_LOOKAHEAD": "0"},
    {"BEAST_LU_NB": "1024", "BEAST_LU_NB2": "256", "BEAST_LU_LOOKAHEAD": "1"},
]


def default_cache_path():
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "beastgpu", "tune.json")


def size_class(n):
    """sizes within a factor sqrt(2) share a tuned setting"""
    return int(round(2 * math.log2(max(int(n), 1))))


def device_key(device=0):
    import torch
    p = torch.cuda.get_device_properties(device)
    return f"{p.name}|sm{p.major}{p.minor}|{p.multi_processor_count}"


def solve_timer(n, device=0, repeats=2, seed=0):
    """params -> seconds of the fastest of `repeats` mixed solves (after one warm-up) of a
    complex-symmetric, diagonally dominant c64 matrix (the symmetric factorisation's case)"""
    import numpy as np
    import torch
    from . import lib as L
    from .api import Context
    rng = np.random.default_rng(seed)
    gen = torch.Generator(device=f"cuda:{device}").manual_seed(seed)
    A = torch.randn(n, n, dtype=torch.complex64, device=f"cuda:{device}", generator=gen)
    A = (A + A.T) / 2 + 4 * math.sqrt(n) * torch.eye(n, dtype=torch.complex64, device=A.device)
    b = torch.from_numpy(rng.normal(size=n) + 1j * rng.normal(size=n)).to(A.device)
    x = torch.empty_like(b)
    ctx = Context(device)
    import ctypes as C
    it, res = C.c_int(0), C.c_double(0)

    def solve():
        ctx.check(ctx.lib.beast_solve_dense(ctx.handle, n, A.data_ptr(), n, L.C64, L.MIXED, b.data_ptr(),
                                            x.data_ptr(), 1, L.DEVICE, 1e-10, 30, C.byref(it), C.byref(res)))

    def timer(params):
        saved = {k: os.environ.get(k) for k in params}
        os.environ.update(params)
        try:
            solve()
            best = float("inf")
            for _ in range(repeats):
                torch.cuda.synchronize(device)
                t0 = time.perf_counter()
                solve()
                torch.cuda.synchronize(device)
                best = min(best, time.perf_counter() - t0)
            return best
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
    return timer


def _load(path):
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def autotune(n, timer=None, candidates=None, cache_path=None, device=0, key=None, force=False, apply=True):
    """the fastest candidate setting for size n (from the cache when present), applied to this
    process's environment when `apply`; returns {"params": ..., "times": ...}"""
    candidates = candidates or CANDIDATES
    cache_path = cache_path or default_cache_path()
    key = key or f"{device_key(device)}|c{size_class(n)}"
    cache = _load(cache_path)
    entry = cache.get(key)
    if entry is None or force:
        timer = timer or solve_timer(n, device)
        times = [float(timer(dict(c))) for c in candidates]
        best = min(range(len(candidates)), key=lambda i: times[i])
        entry = {"params": dict(candidates[best]), "times": times, "n": int(n)}
        cache[key] = entry
        os.makedirs(os.path.dirname(os.path.abspath(cache_path)), exist_ok=True)
        tmp = cache_path + ".tmp"
        with open(tmp, "w") as fh:
            json.dump(cache, fh, indent=1, sort_keys=True)
        os.replace(tmp, cache_path)
    if apply:
        os.environ.update(entry["params"])
    return entry
