"""ctypes binding of libbeastgpu.so (include/beastgpu.h).

This is the same boundary a Julia `ccall` shim binds (see julia/BEASTGPU.jl): plain
pointers, sizes and int status codes.  A missing or unloadable library is an error --
there is no CPU fallback behind this module.
"""
import ctypes as C
import os

from . import build as _build

_LIB = None

OK, ERR_ARG, ERR_OOM, ERR_CUDA, ERR_TIMEOUT, ERR_NOCONV, ERR_SINGULAR, ERR_UNSUPPORTED = range(8)
FP64, MIXED, MIXED_ACCURATE, MIXED_BALANCED = 0, 1, 2, 3
C128, C64 = 0, 1
HOST, DEVICE = 0, 1
EXC_TANGTRACE_E, EXC_CROSSTRACE_H, EXC_HH_DIRICHLET = 0, 1, 2
PROF_KINDS = ["geometry", "far", "near", "gather", "local", "rhs", "farfield", "lu_panel",
              "lu_laswp", "lu_trsm", "lu_gemm", "trsv", "gemv", "vec", "convert", "lu_tc_gemm"]


class BeastError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"beastgpu error {code}: {msg}")
        self.code = code


class OpDesc(C.Structure):
    _fields_ = [("kind", C.c_int), ("gamma_re", C.c_double), ("gamma_im", C.c_double),
                ("alpha_re", C.c_double), ("alpha_im", C.c_double),
                ("beta_re", C.c_double), ("beta_im", C.c_double)]


class QsDesc(C.Structure):
    _fields_ = [("kind", C.c_int), ("outer_far", C.c_int), ("inner_far", C.c_int),
                ("outer_near", C.c_int), ("inner_near", C.c_int), ("ss_tetr", C.c_int),
                ("ss_face", C.c_int), ("ss_edge", C.c_int), ("ss_vert", C.c_int)]


EXPORTS = [
    "beast_ctx_create", "beast_ctx_destroy", "beast_last_error", "beast_ctx_set_stream",
    "beast_ctx_set_workspace_limit", "beast_ctx_synchronize", "beast_ctx_set_wait_limit", "beast_mesh_upload",
    "beast_mesh_free", "beast_mesh_set_children", "beast_space_upload", "beast_space_free", "beast_assemble",
    "beast_assemble_block", "beast_assemble_local", "beast_rhs_planewave", "beast_lu_factor", "beast_lu_solve",
    "beast_lu_free", "beast_lu_solve_noalloc", "beast_solve_dense", "beast_gmres", "beast_farfield", "beast_solve_job",
    "beast_system_create", "beast_system_solve", "beast_system_bytes", "beast_system_free", "beast_pool_stats",
    "beast_batch_create", "beast_batch_assemble", "beast_batch_free",
    "beast_prof_enable", "beast_prof_enable_kinds", "beast_prof_read", "beast_prof_launches", "beast_last_factor_mode", "beast_version",
]


def lib_path():
    return _build.LIB


def load(build_if_needed=True):
    """load the shared library (building it from source if it is missing or stale)"""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.build() if build_if_needed else _build.LIB
    if not os.path.exists(path):
        raise ImportError(f"libbeastgpu.so not found at {path}")
    L = C.CDLL(path)
    vp, i64, d, i = C.c_void_p, C.c_int64, C.c_double, C.c_int
    pp = C.POINTER(C.c_void_p)
    L.beast_ctx_create.argtypes = [i, pp]
    L.beast_ctx_destroy.argtypes = [vp]
    L.beast_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    L.beast_ctx_set_stream.argtypes = [vp, vp]
    L.beast_ctx_set_workspace_limit.argtypes = [vp, C.c_size_t]
    L.beast_ctx_synchronize.argtypes = [vp]
    L.beast_ctx_set_wait_limit.argtypes = [vp, i64]
    L.beast_mesh_upload.argtypes = [vp, vp, i64, vp, i64, i, pp]
    L.beast_mesh_free.argtypes = [vp]
    L.beast_mesh_set_children.argtypes = [vp, vp, i, vp]
    L.beast_space_upload.argtypes = [vp, vp, i, i64, vp, i, i, vp, vp, i64, i, pp]
    L.beast_space_free.argtypes = [vp]
    L.beast_assemble.argtypes = [vp, C.POINTER(OpDesc), C.POINTER(QsDesc), vp, vp, i, vp, i64, i, i,
                                 i64, i64, d, d, i]
    L.beast_assemble_block.argtypes = [vp, C.POINTER(OpDesc), C.POINTER(QsDesc), vp, vp, vp, i64, vp, i64,
                                       i, i, vp, i64, i, i, d, d, i]
    L.beast_assemble_local.argtypes = [vp, i, vp, vp, i, vp, i64, i, i, i64, i64, d, d]
    L.beast_rhs_planewave.argtypes = [vp, i, vp, vp, vp, d, d, d, d, i, vp, i]
    L.beast_lu_factor.argtypes = [vp, i64, vp, i64, i, pp]
    L.beast_lu_solve.argtypes = [vp, vp, i64, vp, i64]
    L.beast_lu_free.argtypes = [vp]
    L.beast_lu_solve_noalloc.argtypes = [vp, vp, i64, vp, i64]
    L.beast_solve_dense.argtypes = [vp, i64, vp, i64, i, i, vp, vp, i64, i, d, i,
                                    C.POINTER(C.c_int), C.POINTER(C.c_double)]
    L.beast_gmres.argtypes = [vp, i64, vp, i64, i, vp, vp, i, d, i, i, C.POINTER(C.c_int),
                              C.POINTER(C.c_double)]
    L.beast_farfield.argtypes = [vp, vp, vp, vp, i64, d, d, i, vp, i]
    L.beast_solve_job.argtypes = [vp, C.POINTER(OpDesc), C.POINTER(QsDesc), vp, i, vp, vp, d, d, i,
                                  d, vp, i, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    L.beast_system_create.argtypes = [vp, C.POINTER(OpDesc), C.POINTER(QsDesc), vp, i, d, d, i, pp]
    L.beast_system_solve.argtypes = [vp, vp, i, i64, vp, vp, d, d, d, vp, i, C.POINTER(C.c_int),
                                     C.POINTER(C.c_double)]
    L.beast_system_bytes.argtypes = [vp, C.POINTER(C.c_size_t)]
    L.beast_system_free.argtypes = [vp]
    L.beast_pool_stats.argtypes = [vp] + [C.POINTER(C.c_size_t)] * 4
    L.beast_batch_create.argtypes = [vp, C.POINTER(QsDesc), i64, vp, vp, vp, i, i, i, i, pp]
    L.beast_batch_assemble.argtypes = [vp, vp]
    L.beast_batch_free.argtypes = [vp]
    L.beast_prof_enable.argtypes = [vp, i]
    L.beast_prof_read.argtypes = [vp, i, C.POINTER(C.c_double), C.POINTER(C.c_int64),
                                  C.POINTER(C.c_double)]
    L.beast_prof_launches.argtypes = [vp, C.POINTER(C.c_int64)]
    L.beast_last_factor_mode.argtypes = [vp, C.POINTER(C.c_int)]
    L.beast_prof_enable_kinds.argtypes = [vp, C.c_uint]
    L.beast_version.restype = C.c_char_p
    for name in EXPORTS:
        if name != "beast_version":
            getattr(L, name).restype = C.c_int
    _LIB = L
    return L


def check(rc, ctx_handle=None):
    if rc == OK:
        return
    buf = C.create_string_buffer(1024)
    load().beast_last_error(ctx_handle, buf, 1024)
    raise BeastError(rc, buf.value.decode(errors="replace"))
