"""ctypes front end of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline / --impl reference legs as the checker.  The product package never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

MW_SL, MW_DL, MW_NXDL, HH_SL, HH_DL, HH_DLT = 1, 2, 3, 4, 5, 6
MW_SL_REG, MW_DL_REG, HH_SL_REG, HH_DL_REG, HH_DLT_REG = 11, 12, 14, 15, 16
P0, P1, RT = 0, 1, 2
QS_WILTON_SAUTER, QS_SAUTER, QS_DOUBLENUM = 1, 2, 3
RULE_DQ, RULE_SE, RULE_SS_FACE, RULE_SS_EDGE, RULE_SS_VERT = 0, 1, 2, 3, 4


class OrcOp(C.Structure):
    _fields_ = [("kind", C.c_int), ("gamma_re", C.c_double), ("gamma_im", C.c_double),
                ("alpha_re", C.c_double), ("alpha_im", C.c_double),
                ("beta_re", C.c_double), ("beta_im", C.c_double)]


class OrcQs(C.Structure):
    _fields_ = [("kind", C.c_int), ("outer_far", C.c_int), ("inner_far", C.c_int),
                ("outer_near", C.c_int), ("inner_near", C.c_int), ("ss_tetr", C.c_int),
                ("ss_face", C.c_int), ("ss_edge", C.c_int), ("ss_vert", C.c_int)]


class OrcSpace(C.Structure):
    _fields_ = [("kind", C.c_int), ("ncells", C.c_int64), ("cells", C.c_void_p),
                ("maxfn", C.c_int), ("nshapes", C.c_int), ("ad_dof", C.c_void_p),
                ("ad_coeff", C.c_void_p), ("nfuncs", C.c_int64)]


class OrcMesh(C.Structure):
    _fields_ = [("verts", C.c_void_p), ("nv", C.c_int64), ("cells", C.c_void_p),
                ("nc", C.c_int64)]


def build(force=False):
    so = os.path.join(_HERE, "liboracle.so")
    src = os.path.join(_HERE, "oracle.cpp")
    if force or not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE, "-B", "liboracle.so"])
    return so


def lib():
    global _LIB
    if _LIB is None:
        _LIB = C.CDLL(build())
        d = C.POINTER(C.c_double)
        _LIB.orc_trirule.argtypes = [C.c_int, d, d, C.c_int]
        _LIB.orc_gausslegendre.argtypes = [C.c_int, d, d]
        _LIB.orc_wiltonints.argtypes = [d, d, d, d, d, d, d]
        vp = C.c_void_p
        _LIB.orc_assemble_refines.argtypes = [vp, vp, vp, vp, vp, vp, d, C.c_int, C.c_int, d, C.c_int64,
                                              C.c_int]
        _LIB.orc_wiltonints.restype = None
        _LIB.orc_cellpair.argtypes = [C.POINTER(OrcOp), C.c_int, C.c_int, d, d, C.c_int,
                                      C.c_int, C.c_int, C.c_int, d]
        _LIB.orc_classify.argtypes = [C.POINTER(OrcOp), C.POINTER(OrcQs), d, d]
        _LIB.orc_assemble.argtypes = [C.POINTER(OrcOp), C.POINTER(OrcQs), C.POINTER(OrcMesh),
                                      C.POINTER(OrcSpace), C.POINTER(OrcSpace), d, C.c_int64,
                                      C.c_int64, C.c_int64, C.c_int]
        _LIB.orc_assemble_local.argtypes = [C.c_int, C.POINTER(OrcMesh), C.POINTER(OrcSpace),
                                            C.POINTER(OrcSpace), C.c_int, C.c_double,
                                            C.c_double, d, C.c_int64]
        _LIB.orc_rhs_planewave.argtypes = [C.c_int, C.POINTER(OrcMesh), C.POINTER(OrcSpace), d, d,
                                           C.c_double, C.c_double, C.c_double, C.c_double,
                                           C.c_int, d]
        i64p = C.POINTER(C.c_int64)
        _LIB.orc_lu_factor.argtypes = [C.c_int64, d, C.c_int64, i64p, C.c_int]
        _LIB.orc_lu_solve.argtypes = [C.c_int64, d, C.c_int64, i64p, C.c_int64, d, C.c_int64]
        _LIB.orc_gmres.argtypes = [C.c_int64, d, C.c_int64, d, d, C.c_double, C.c_int, C.c_int,
                                   C.c_int, d]
        _LIB.orc_farfield.argtypes = [C.POINTER(OrcMesh), C.POINTER(OrcSpace), d, d, C.c_int64,
                                      C.c_double, C.c_double, C.c_int, d]
    return _LIB


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def trirule(degree):
    uv = np.zeros((512, 2))
    w = np.zeros(512)
    n = lib().orc_trirule(degree, _dp(uv), _dp(w), 512)
    assert n > 0
    return uv[:n].copy(), w[:n].copy()


def gausslegendre(n):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().orc_gausslegendre(n, _dp(x), _dp(w))
    return x, w


def wiltonints(p1, p2, p3, x):
    p = [np.ascontiguousarray(v, dtype=np.float64) for v in (p1, p2, p3, x)]
    s = np.zeros(6)
    v = np.zeros((6, 3))
    g = np.zeros((4, 3))
    lib().orc_wiltonints(_dp(p[0]), _dp(p[1]), _dp(p[2]), _dp(p[3]), _dp(s), _dp(v), _dp(g))
    return s, v, g


def make_op(kind, gamma=0j, alpha=1.0, beta=0.0):
    gamma, alpha, beta = complex(gamma), complex(alpha), complex(beta)
    return OrcOp(kind, gamma.real, gamma.imag, alpha.real, alpha.imag, beta.real, beta.imag)


def make_qs(kind, *orders):
    o = list(orders) + [0] * (8 - len(orders))
    if kind == QS_SAUTER:  # (outer, inner, tetr, face, edge, vert)
        o = [orders[0], orders[1], 0, 0, orders[2], orders[3], orders[4], orders[5]]
    if kind == QS_DOUBLENUM:
        o = [orders[0], orders[1], 0, 0, 0, 0, 0, 0]
    return OrcQs(kind, *o)


def cellpair(op, tkind, bkind, tv, bv, rule, deg_o=0, deg_i=0, gl=0):
    tv = np.ascontiguousarray(tv, dtype=np.float64).reshape(9)
    bv = np.ascontiguousarray(bv, dtype=np.float64).reshape(9)
    nt = 1 if tkind == P0 else 3
    nb = 1 if bkind == P0 else 3
    out = np.zeros(2 * nt * nb)
    rc = lib().orc_cellpair(C.byref(op), tkind, bkind, _dp(tv), _dp(bv), rule, deg_o, deg_i, gl,
                            _dp(out))
    assert rc == 0, "rule not available for this operator/space pairing"
    return out.view(np.complex128).reshape(nt, nb)


def classify(op, qs, tv, bv):
    tv = np.ascontiguousarray(tv, dtype=np.float64).reshape(9)
    bv = np.ascontiguousarray(bv, dtype=np.float64).reshape(9)
    return lib().orc_classify(C.byref(op), C.byref(qs), _dp(tv), _dp(bv))


class _Keep:
    """holds numpy arrays alive while ctypes structs point into them"""

    def __init__(self):
        self.refs = []

    def arr(self, a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        self.refs.append(a)
        return a.ctypes.data


def _mesh_struct(mesh, keep):
    return OrcMesh(keep.arr(mesh.vertices, np.float64), mesh.vertices.shape[0],
                   keep.arr(mesh.cells, np.int32), mesh.cells.shape[0])


def _space_struct(space, keep):
    ad = space.assemblydata()
    return OrcSpace(ad.kind, ad.cells.shape[0], keep.arr(ad.cells, np.int64), ad.maxfn, ad.nshapes,
                    keep.arr(ad.dof, np.int64), keep.arr(ad.coeff, np.float64), space.numfunctions())


def assemble(op, qs, tspace, bspace, row_lo=0, row_hi=-1, nthreads=None):
    """dense matrix of rows [row_lo,row_hi) (complex128, shape rows x ncols)"""
    keep = _Keep()
    mesh = tspace.mesh
    m = _mesh_struct(mesh, keep)
    ts = _space_struct(tspace, keep)
    bs = _space_struct(bspace, keep)
    if row_hi < 0:
        row_hi = tspace.numfunctions()
    nrows = row_hi - row_lo
    Z = np.zeros((bspace.numfunctions(), nrows), dtype=np.complex128)  # Z.T in C order
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    lib().orc_assemble(C.byref(op), C.byref(qs), C.byref(m), C.byref(ts), C.byref(bs),
                       _dp(Z.view(np.float64)), nrows, row_lo, row_hi, nthreads)
    return Z.T  # rows x cols view of column-major storage


def assemble_refines(op, qs, tspace, bspace, children, split_test=False, nthreads=None):
    """RT x RT matrix across a barycentric refinement (TestRefinesTrialQStrat, or with
    split_test TrialRefinesTestQStrat): children [coarse cells][nchild][3][3]"""
    keep = _Keep()
    tm, bm = _mesh_struct(tspace.mesh, keep), _mesh_struct(bspace.mesh, keep)
    ts, bs = _space_struct(tspace, keep), _space_struct(bspace, keep)
    ch = np.ascontiguousarray(children, dtype=np.float64)
    n = tspace.numfunctions()
    Z = np.zeros((bspace.numfunctions(), n), dtype=np.complex128)
    rc = lib().orc_assemble_refines(C.byref(op), C.byref(qs), C.byref(tm), C.byref(bm), C.byref(ts),
                                    C.byref(bs), _dp(ch), ch.shape[1], 1 if split_test else 0,
                                    _dp(Z.view(np.float64)), n, nthreads or os.cpu_count() or 1)
    assert rc == 0, "RT spaces and a DoubleNumWiltonSauterQStrat are required"
    return Z.T


def assemble_local(which, tspace, bspace, degree=6, coeff=1.0):
    keep = _Keep()
    m = _mesh_struct(tspace.mesh, keep)
    ts = _space_struct(tspace, keep)
    bs = _space_struct(bspace, keep)
    n = tspace.numfunctions()
    Z = np.zeros((bspace.numfunctions(), n), dtype=np.complex128)
    coeff = complex(coeff)
    lib().orc_assemble_local(which, C.byref(m), C.byref(ts), C.byref(bs), degree, coeff.real,
                             coeff.imag, _dp(Z.view(np.float64)), n)
    return Z.T


def rhs_planewave(kind, tspace, direction, polarization, gamma, amplitude=1.0, degree=8):
    keep = _Keep()
    m = _mesh_struct(tspace.mesh, keep)
    ts = _space_struct(tspace, keep)
    d = np.ascontiguousarray(direction, dtype=np.float64)
    p = np.ascontiguousarray(polarization if polarization is not None else [0, 0, 0],
                             dtype=np.float64)
    b = np.zeros(tspace.numfunctions(), dtype=np.complex128)
    gamma, amplitude = complex(gamma), complex(amplitude)
    lib().orc_rhs_planewave(kind, C.byref(m), C.byref(ts), _dp(d), _dp(p), gamma.real, gamma.imag,
                            amplitude.real, amplitude.imag, degree, _dp(b.view(np.float64)))
    return b


def lu_solve(A, b, nthreads=None):
    """x = A \\ b with the oracle's partial-pivoting LU (A, b complex128)"""
    n = A.shape[0]
    F = np.asfortranarray(A.astype(np.complex128))
    ipiv = np.zeros(n, dtype=np.int64)
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    info = lib().orc_lu_factor(n, F.ctypes.data_as(C.POINTER(C.c_double)), n,
                               ipiv.ctypes.data_as(C.POINTER(C.c_int64)), nthreads)
    assert info == 0, f"singular matrix (info={info})"
    B = np.asfortranarray(np.array(b, dtype=np.complex128).reshape(n, -1))
    lib().orc_lu_solve(n, F.ctypes.data_as(C.POINTER(C.c_double)), n,
                       ipiv.ctypes.data_as(C.POINTER(C.c_int64)), B.shape[1],
                       B.ctypes.data_as(C.POINTER(C.c_double)), n)
    return B.reshape(np.shape(b)) if np.ndim(b) == 1 else B


def gmres(A, b, reltol=1e-8, restart=0, maxiter=1000, nthreads=None):
    n = A.shape[0]
    F = np.asfortranarray(A.astype(np.complex128))
    bb = np.ascontiguousarray(b, dtype=np.complex128)
    x = np.zeros(n, dtype=np.complex128)
    res = np.zeros(1)
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    it = lib().orc_gmres(n, F.ctypes.data_as(C.POINTER(C.c_double)), n, _dp(bb.view(np.float64)),
                         _dp(x.view(np.float64)), reltol, restart, maxiter, nthreads, _dp(res))
    return x, it, float(res[0])


def farfield(space, u, directions, gamma, degree=10):
    keep = _Keep()
    m = _mesh_struct(space.mesh, keep)
    ts = _space_struct(space, keep)
    uu = np.ascontiguousarray(u, dtype=np.complex128)
    pts = np.ascontiguousarray(directions, dtype=np.float64)
    ff = np.zeros((pts.shape[0], 3), dtype=np.complex128)
    gamma = complex(gamma)
    lib().orc_farfield(C.byref(m), C.byref(ts), _dp(uu.view(np.float64)), _dp(pts), pts.shape[0],
                       gamma.real, gamma.imag, degree, _dp(ff.view(np.float64)))
    return ff
