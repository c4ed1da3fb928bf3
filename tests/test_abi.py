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
    enum = {m.group(1): int(m.group(2))
            for m in re.finditer(r"BEAST_(FP64|MIXED|MIXED_ACCURATE|MIXED_BALANCED)\s*=\s*(\d+)", hdr)}
    assert enum == {"FP64": 0, "MIXED": 1, "MIXED_ACCURATE": 2, "MIXED_BALANCED": 3}
    assert (bg.FP64, bg.MIXED, bg.MIXED_ACCURATE, bg.MIXED_BALANCED) == (0, 1, 2, 3)
    jl = open(os.path.join(ROOT, "beast.jl_gb300", "julia", "BEASTGPU.jl")).read()
    assert "const FP64, MIXED, MIXED_ACCURATE, MIXED_BALANCED = 0, 1, 2, 3" in jl


def _split_top(s):
    """split s at commas that are not inside brackets"""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _paren_body(s, i):
    """text inside the bracket pair that opens at s[i]"""
    depth = 0
    for j in range(i, len(s)):
        depth += s[j] == "("
        depth -= s[j] == ")"
        if depth == 0:
            return s[i + 1:j]
    raise ValueError("unbalanced")


def test_julia_shim_bindings_match_header():
    """Julia is not installed here, so the shim is checked as text: every ccall into
    libbeastgpu names a function of include/beastgpu.h with as many argument types as the C
    prototype has parameters"""
    hdr = open(os.path.join(ROOT, "include", "beastgpu.h")).read()
    protos = {}
    for m in re.finditer(r"^\s*(?:int|const char\*)\s+(beast_\w+)\(", hdr, re.M):
        body = _paren_body(hdr, m.end() - 1)
        protos[m.group(1)] = 0 if body.strip() == "void" else len(_split_top(body))
    jl = open(os.path.join(ROOT, "beast.jl_gb300", "julia", "BEASTGPU.jl")).read()
    calls = list(re.finditer(r"ccall\(\(:(beast_\w+), libbeastgpu\), Cint,\s*", jl))
    assert len(calls) >= 8
    for c in calls:
        name = c.group(1)
        assert name in protos, name
        types = _paren_body(jl, c.end())
        assert len(_split_top(types)) == protos[name], name


def test_julia_shim_dispatch_is_positional():
    """the shim must not change the reference's behaviour for calls that do not ask for the
    device: it defines no `BEAST.assemble` method (whose keyword arguments Julia does not
    dispatch on), and every `BEAST.assemble!` method it adds takes the device store
    positionally; the device is asked for through `allocatestorage`'s storage trait"""
    jl = open(os.path.join(ROOT, "beast.jl_gb300", "julia", "BEASTGPU.jl")).read()
    assert not re.search(r"function\s+BEAST\.assemble\(", jl)
    defs = list(re.finditer(r"function\s+BEAST\.assemble!\(", jl))
    assert len(defs) >= 6
    for d in defs:
        sig = _paren_body(jl, d.end() - 1)
        assert "store::DenseStore" in sig, sig[:120]
    assert re.search(r"function\s+BEAST\.allocatestorage\([^)]*policy::GPUPolicy", jl)
    assert "(s::DenseStore)(v, m, n)" in jl  # callable like the reference's store closure
