"""Home-grown autotuners: the dense solve's tuning switches, and the batched assembly's tile
shape and tile order.

The factorisation reads its block widths and lookahead from the environment at every call
(`BEAST_LU_NB`, `BEAST_LU_NB2`, `BEAST_LU_LOOKAHEAD`).  `autotune(n)` times
the mixed solve of an n x n complex-symmetric matrix on the device under each candidate
setting, keeps the fastest, applies it to this process's environment and caches it per GPU
model and size class in a JSON file, so a later process (or a serving loop) starts from the
tuned setting without timing again.

    import beastgpu as bg
    best = bg.tune.autotune(30720)        # {'BEAST_LU_NB': '1024', 'BEAST_LU_NB2': '256', ...}

`autotune_batch(ops, spaces, precision)` times the batched assembly (beastgpu.batch) of the
given jobs under each candidate tile shape (test cells x trial cells per CTA step) and tile
order ("pair bucketing": job by job, largest jobs first, jobs interleaved) and caches the
fastest per GPU model and batch signature (operator kind, precision, job count, size classes).

The timers are replaceable: the tests drive the searches, the caches and the apply step on
the CPU.
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


# candidate batched-assembly schedules: (test cells per CTA, trial cells staged per CTA, order)
BATCH_CANDIDATES = [(tm, tq, order) for tm in (64, 128, 256) for tq in (8, 16, 32)
                    for order in ("largest_first", "interleaved", "job")]


def batch_signature(ops, spaces, precision):
    """what a tuned batch schedule is keyed by: operator kind, precision, job count and the
    histogram of size classes"""
    classes = {}
    for s in spaces:
        c = size_class(s.numfunctions())
        classes[c] = classes.get(c, 0) + 1
    return f"k{ops[0].kind}|p{precision}|n{len(spaces)}|" + ",".join(f"{c}:{k}" for c, k in sorted(classes.items()))


def batch_timer(ops, spaces, precision, device=0, repeats=3):
    """(tile_m, tile_q, order) -> seconds of the fastest of `repeats` graph replays of the
    batched assembly (after the capturing call)"""
    import torch
    from .batch import Batch

    def timer(cand):
        tm, tq, order = cand
        b = Batch(ops, spaces, precision=precision, tile_m=tm, tile_q=tq, order=order)
        try:
            b.assemble()
            best = float("inf")
            for _ in range(repeats):
                torch.cuda.synchronize(device)
                t0 = time.perf_counter()
                b.assemble()
                torch.cuda.synchronize(device)
                best = min(best, time.perf_counter() - t0)
            return best
        finally:
            b.close()
    return timer


def autotune_batch(ops, spaces, precision, timer=None, candidates=None, cache_path=None, device=0, key=None,
                   force=False):
    """the fastest batched-assembly schedule for these jobs (from the cache when present):
    {"tile_m", "tile_q", "order", "times"}"""
    candidates = candidates or BATCH_CANDIDATES
    cache_path = cache_path or default_cache_path()
    key = key or f"{device_key(device)}|batch|{batch_signature(ops, spaces, precision)}"
    cache = _load(cache_path)
    entry = cache.get(key)
    if entry is None or force:
        timer = timer or batch_timer(ops, spaces, precision, device)
        times = [float(timer(tuple(c))) for c in candidates]
        best = min(range(len(candidates)), key=lambda i: times[i])
        tm, tq, order = candidates[best]
        entry = {"tile_m": int(tm), "tile_q": int(tq), "order": order,
                 "times": {f"{c[0]}x{c[1]}:{c[2]}": t for c, t in zip(candidates, times)}}
        cache[key] = entry
        os.makedirs(os.path.dirname(os.path.abspath(cache_path)), exist_ok=True)
        tmp = cache_path + ".tmp"
        with open(tmp, "w") as fh:
            json.dump(cache, fh, indent=1, sort_keys=True)
        os.replace(tmp, cache_path)
    return entry
