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
