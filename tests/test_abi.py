"""The C ABI library loads and exports every function include/beastgpu.h declares (no GPU)."""
import ctypes
import os
import re

from conftest import ROOT


def test_exports_match_header():
    from beastgpu import lib
    L = lib.load()
    hdr = open(os.path.join(ROOT, "include", "beastgpu.h")).read()
    names = set(re.findall(r"^\s*(?:int|const char\*)\s+(beast_\w+)\(", hdr, re.M))
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(L, n), n
        assert isinstance(getattr(L, n), ctypes._CFuncPtr)
    assert set(lib.EXPORTS) == names
    assert L.beast_version().startswith(b"beastgpu")


def test_no_device_is_an_error_not_a_fallback():
    # without a GPU the context cannot be created: the call fails loudly
    import torch
    if torch.cuda.is_available():
        return
    from beastgpu import lib
    h = ctypes.c_void_p()
    assert lib.load().beast_ctx_create(0, ctypes.byref(h)) != 0


def test_precision_constants_match_header():
    """the precision enum of the C header, the Python constants and the Julia shim agree"""
    import beastgpu as bg
    hdr = open(os.path.join(ROOT, "include", "beastgpu.h")).read()
    enum = {m.group(1): int(m.group(2)) for m in re.finditer(r"BEAST_(FP64|MIXED|MIXED_ACCURATE)\s*=\s*(\d+)", hdr)}
    assert enum == {"FP64": 0, "MIXED": 1, "MIXED_ACCURATE": 2}
    assert (bg.FP64, bg.MIXED, bg.MIXED_ACCURATE) == (0, 1, 2)
    jl = open(os.path.join(ROOT, "beast.jl_gb300", "julia", "BEASTGPU.jl")).read()
    assert "const FP64, MIXED, MIXED_ACCURATE = 0, 1, 2" in jl
