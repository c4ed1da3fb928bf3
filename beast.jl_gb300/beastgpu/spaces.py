"""Function spaces and their assembly data.

Host-side mirror of BEAST's global spaces:
  * `raviartthomas(mesh)`  -- src/bases/rtspace.jl:35-105: one dof per interior edge,
    `Shape(c+, e+, +1)`, `Shape(c-, e-, -1)` with e the local index of the vertex opposite
    the edge (local RT shape i is (x - v_i)/(2A), src/bases/local/rtlocal.jl:8-27).
  * `lagrangecxd0(mesh)`   -- src/bases/lagrange.jl:32-49: one dof per cell.
  * `lagrangec0d1(mesh)`   -- src/bases/lagrange.jl:340-360: one dof per vertex (closed
    surface: all vertices), local shape i = barycentric coordinate of cell vertex i.
and of `assemblydata` (src/bases/basis.jl:235-294): for every active cell c and local shape
r, the list of (dof, coefficient) pairs, stored here as dense arrays
`dof[c, r, k]` (int64, -1 = empty slot) and `coeff[c, r, k]` (float64), k < maxfn.

Edge (dof) order: the reference sorts edges along a space-filling curve
(`skeleton(mesh, 1; sort=:spacefillingcurve)`, CompScienceMeshes, un-vendored).  Here edges
are sorted by the Morton (Z-order) key of their midpoints, the same kind of locality order.
The assembly kernels accept any order; only the mirror constructors choose one.
"""
import numpy as np

P0, P1, RT = 0, 1, 2


class AssemblyData:
    def __init__(self, kind, cells, dof, coeff):
        self.kind = kind
        self.cells = np.ascontiguousarray(cells, dtype=np.int64)  # active -> mesh cell
        self.dof = np.ascontiguousarray(dof, dtype=np.int64)        # [ncells, nshapes, maxfn]
        self.coeff = np.ascontiguousarray(coeff, dtype=np.float64)
        self.nshapes = self.dof.shape[1]
        self.maxfn = self.dof.shape[2]


class Space:
    """a global space: list of basis functions, each a list of (cell, refid, coeff)"""

    def __init__(self, kind, mesh, fns, pos=None):
        self.kind = kind
        self.mesh = mesh
        self.fns = fns
        self.pos = pos
        self._ad = None

    def numfunctions(self):
        return len(self.fns)

    def refspace_nshapes(self):
        return 1 if self.kind == P0 else 3

    def assemblydata(self):
        """src/bases/basis.jl:235-294 (onlyactives=true)"""
        if self._ad is not None:
            return self._ad
        nc = self.mesh.numcells()
        nr = self.refspace_nshapes()
        count = np.zeros((nc, nr), dtype=np.int64)
        for fn in self.fns:
            for (c, r, w) in fn:
                count[c, r] += 1
        active = np.nonzero(count.sum(axis=1) > 0)[0]
        index_among_actives = -np.ones(nc, dtype=np.int64)
        index_among_actives[active] = np.arange(len(active))
        maxfn = max(1, int(count.max()))
        dof = -np.ones((len(active), nr, maxfn), dtype=np.int64)
        coeff = np.zeros((len(active), nr, maxfn), dtype=np.float64)
        fill = np.zeros((nc, nr), dtype=np.int64)
        for b, fn in enumerate(self.fns):
            for (c, r, w) in fn:
                k = fill[c, r]
                fill[c, r] += 1
                l = index_among_actives[c]
                dof[l, r, k] = b
                coeff[l, r, k] = w
        self._ad = AssemblyData(self.kind, active, dof, coeff)
        return self._ad

    def subset(self, idx):
        idx = np.asarray(idx)
        return Space(self.kind, self.mesh, [self.fns[i] for i in idx],
                     None if self.pos is None else self.pos[idx])


def _morton_order(points):
    lo = points.min(axis=0)
    span = np.maximum(points.max(axis=0) - lo, 1e-300)
    q = np.clip(((points - lo) / span * 1023.0).astype(np.int64), 0, 1023)

    def spread(x):
        x = x & 0x3FF
        x = (x | (x << 16)) & 0x30000FF
        x = (x | (x << 8)) & 0x300F00F
        x = (x | (x << 4)) & 0x30C30C3
        x = (x | (x << 2)) & 0x9249249
        return x

    key = spread(q[:, 0]) | (spread(q[:, 1]) << 1) | (spread(q[:, 2]) << 2)
    return np.argsort(key, kind="stable")


def raviartthomas(mesh, sort="spacefillingcurve"):
    cells = mesh.cells
    edges = {}
    for c in range(cells.shape[0]):
        for i in range(3):
            a, b = int(cells[c, (i + 1) % 3]), int(cells[c, (i + 2) % 3])
            key = (a, b) if a < b else (b, a)
            edges.setdefault(key, []).append((c, i, a < b))
    keys, pairs = [], []
    for key, lst in edges.items():
        if len(lst) != 2:
            continue  # boundary or junction edge: no dof (dropjunctionpair)
        (c1, e1, o1), (c2, e2, o2) = lst
        if not o1:  # the cell that runs along the edge from low to high index is '+'
            (c1, e1), (c2, e2) = (c2, e2), (c1, e1)
        keys.append(key)
        pairs.append((c1, e1, c2, e2))
    keys = np.array(keys, dtype=np.int64).reshape(-1, 2)
    mids = 0.5 * (mesh.vertices[keys[:, 0]] + mesh.vertices[keys[:, 1]])
    order = _morton_order(mids) if sort == "spacefillingcurve" else np.arange(len(keys))
    cent = mesh.centroids()
    fns, pos = [], []
    for k in order:
        c1, e1, c2, e2 = pairs[k]
        fns.append([(c1, e1, 1.0), (c2, e2, -1.0)])
        pos.append(0.5 * (cent[c1] + cent[c2]))
    return Space(RT, mesh, fns, np.array(pos))


def lagrangecxd0(mesh):
    cent = mesh.centroids()
    fns = [[(c, 0, 1.0)] for c in range(mesh.numcells())]
    return Space(P0, mesh, fns, cent)


def lagrangec0d1(mesh):
    nv = mesh.numvertices()
    fns = [[] for _ in range(nv)]
    for c in range(mesh.numcells()):
        for r in range(3):
            fns[int(mesh.cells[c, r])].append((c, r, 1.0))
    used = [i for i in range(nv) if fns[i]]
    return Space(P1, mesh, [fns[i] for i in used], mesh.vertices[used])
