"""Triangle surface meshes.

Mirrors the parts of CompScienceMeshes that BEAST's assembly path consumes: a vertex
array and a cell (triangle) array, read from the reference's `.in` format
(`readmesh`, format of test/assets/sphere45.in:1-8: line 1 = `1`, line 2 = `nverts nfaces`,
then vertex coordinates, then 1-based vertex indices) or generated as subdivided
icospheres / perturbed ellipsoids for the benchmark workloads.

Vertices are float64 [nv, 3]; cells are int32 [nc, 3], 0-based, counter-clockwise seen
from outside (normal = (v1 - v3) x (v2 - v3), the chart convention of CompScienceMeshes).
"""
import numpy as np


class Mesh:
    def __init__(self, vertices, cells):
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float64)
        self.cells = np.ascontiguousarray(cells, dtype=np.int32)
        assert self.vertices.ndim == 2 and self.vertices.shape[1] == 3
        assert self.cells.ndim == 2 and self.cells.shape[1] == 3
        # the Refinement this mesh is the fine side of (CompScienceMeshes.parent), if any
        self.refinement = None

    def numcells(self):
        return self.cells.shape[0]

    def numvertices(self):
        return self.vertices.shape[0]

    def areas(self):
        v = self.vertices[self.cells]
        return 0.5 * np.linalg.norm(np.cross(v[:, 0] - v[:, 2], v[:, 1] - v[:, 2]), axis=1)

    def normals(self):
        v = self.vertices[self.cells]
        n = np.cross(v[:, 0] - v[:, 2], v[:, 1] - v[:, 2])
        return n / np.linalg.norm(n, axis=1, keepdims=True)

    def centroids(self):
        return self.vertices[self.cells].mean(axis=1)

    def meshsize(self):
        v = self.vertices[self.cells]
        e = np.concatenate([v[:, 1] - v[:, 0], v[:, 2] - v[:, 1], v[:, 0] - v[:, 2]])
        return float(np.linalg.norm(e, axis=1).mean())


def refines(fine, coarse):
    """CompScienceMeshes.refines: `fine` is a refinement of `coarse` made here"""
    R = getattr(fine, "refinement", None)
    return R is not None and R.coarse is coarse


def readmesh(path):
    """read the reference's `.in` mesh format"""
    with open(path) as fh:
        toks = fh.read().split()
    assert int(toks[0]) == 1, "unsupported .in header"
    nv, nf = int(toks[1]), int(toks[2])
    p = 3
    verts = np.array(toks[p:p + 3 * nv], dtype=np.float64).reshape(nv, 3)
    p += 3 * nv
    cells = np.array(toks[p:p + 3 * nf], dtype=np.int64).reshape(nf, 3) - 1
    return Mesh(verts, cells)


def _icosahedron():
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]],
                 dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9],
                  [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2],
                  [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
                  [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v, f


def _orient_outward(v, f):
    c = v[f].mean(axis=1)
    n = np.cross(v[f[:, 0]] - v[f[:, 2]], v[f[:, 1]] - v[f[:, 2]])
    flip = (n * c).sum(axis=1) < 0
    f = f.copy()
    f[flip] = f[flip][:, [1, 0, 2]]
    return f


def icosphere(level, radius=1.0):
    """icosahedron subdivided `level` times (4**level * 20 triangles), projected to the sphere"""
    v, f = _icosahedron()
    for _ in range(level):
        verts = list(v)
        mid = {}

        def midpoint(a, b):
            key = (a, b) if a < b else (b, a)
            idx = mid.get(key)
            if idx is None:
                m = 0.5 * (verts[a] + verts[b])
                m = m / np.linalg.norm(m)
                idx = len(verts)
                verts.append(m)
                mid[key] = idx
            return idx

        nf = []
        for a, b, c in f:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        v = np.array(verts)
        f = np.array(nf, dtype=np.int64)
    f = _orient_outward(v, f)
    return Mesh(radius * v, f)


def ellipsoid(level, semiaxes=(1.0, 1.0, 1.0), perturb=0.0, rng=None):
    """icosphere scaled to an ellipsoid; each vertex moved radially by N(0, perturb * h)"""
    m = icosphere(level, 1.0)
    v = m.vertices * np.asarray(semiaxes, dtype=np.float64)[None, :]
    out = Mesh(v, m.cells)
    if perturb > 0:
        rng = np.random.default_rng(rng)
        h = out.meshsize()
        r = np.linalg.norm(v, axis=1, keepdims=True)
        dr = rng.normal(0.0, perturb * h, size=(v.shape[0], 1))
        v = v * (1.0 + dr / r)
        out = Mesh(v, m.cells)
    return out
