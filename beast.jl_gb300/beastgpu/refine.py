"""Barycentric refinement and Buffa-Christiansen functions (closed surfaces).

  * `barycentric_refinement(mesh)` -- the refinement CompScienceMeshes builds for
    `buffachristiansen` (un-vendored there): every triangle split into six by its centroid and
    edge midpoints, each child oriented like its parent.  Fine vertices: the coarse vertices,
    then one per coarse edge (its midpoint), then one per coarse cell (its centroid).
  * `buffachristiansen(mesh)` -- src/bases/bcspace.jl:90-190 with `buildhalfbc`
    (bcspace.jl:194-405) on a closed surface: for each coarse edge (v1, v2) with midpoint p, a
    half function around v1 and the negated half around v2.  A half function lives on the n
    fine cells around its vertex v, sorted into a ring: flux 1/2 leaves through each of the two
    outer edges at p (the ports); the charge is 1/n in every cell; the fluxes across the spokes
    between neighbouring cells follow by walking the ring from one port to the other.  Functions
    come in the order of `raviartthomas(mesh)`'s edges, so the BC function i and the RT function i
    share an edge (the pairing of the BC-tested MFIE).
  * `refined(X, fine)` -- the coarse RT space written exactly in the fine cells' RT shapes, so
    that BC-tested operators with RT trial functions run on one mesh (the fine one) through the
    ordinary assembly (the reference integrates fine test cells against coarse trial cells,
    `TestRefinesTrialQStrat`; on the fine mesh the trial cells are the coarse cells' children,
    so entries agree with it to quadrature accuracy rather than rounding).

RT local shape r of a cell is (x - v_r) / (2 A) (src/bases/local/rtlocal.jl:8-27): its
coefficient is the flux leaving the cell through the edge opposite vertex r.
"""
import numpy as np

from .mesh import Mesh
from .spaces import RT, Space


class Refinement:
    """fine mesh + parent cell of every fine cell, fine vertex of every coarse edge midpoint
    ((a, b) with a < b) and of every coarse centroid"""

    def __init__(self, coarse, fine, parent, midpoint, centroid):
        self.coarse = coarse
        self.fine = fine
        self.parent = parent
        self.midpoint = midpoint
        self.centroid = centroid

    def children(self, c):
        return range(6 * c, 6 * c + 6)

    def child_vertices(self):
        """[coarse cells][6][3][3]: the vertices of every coarse cell's children, in the
        children's own orientation (that of the parent)"""
        nc = self.coarse.numcells()
        return np.ascontiguousarray(self.fine.vertices[self.fine.cells[:6 * nc]].reshape(nc, 6, 3, 3))

    def refined_space(self, X):
        """refined(X, self), built once per coarse space"""
        cache = self.__dict__.setdefault("_refined", {})
        ent = cache.get(id(X))
        if ent is None or ent[0] is not X:
            ent = (X, refined(X, self))
            cache[id(X)] = ent
        return ent[1]


def barycentric_refinement(mesh):
    V = mesh.vertices
    C = mesh.cells
    nv, nc = V.shape[0], C.shape[0]
    midpoint = {}
    mids = []
    for c in range(nc):
        for i in range(3):
            a, b = int(C[c, i]), int(C[c, (i + 1) % 3])
            key = (a, b) if a < b else (b, a)
            if key not in midpoint:
                midpoint[key] = nv + len(mids)
                mids.append(0.5 * (V[a] + V[b]))
    centroid = np.arange(nc) + nv + len(mids)
    verts = np.concatenate([V, np.array(mids).reshape(-1, 3), V[C].mean(axis=1)])

    def m(a, b):
        return midpoint[(a, b) if a < b else (b, a)]

    cells = np.empty((6 * nc, 3), dtype=np.int32)
    for c in range(nc):
        a, b, d = (int(x) for x in C[c])
        g = int(centroid[c])
        cells[6 * c:6 * c + 6] = [(a, m(a, b), g), (m(a, b), b, g), (b, m(b, d), g),
                                  (m(b, d), d, g), (d, m(d, a), g), (m(d, a), a, g)]
    fine = Mesh(verts, cells)
    R = Refinement(mesh, fine, np.repeat(np.arange(nc), 6), midpoint, centroid)
    fine.refinement = R
    return R


def _vertex_to_cells(cells, nv):
    vtof = [[] for _ in range(nv)]
    for f, tri in enumerate(cells):
        for v in tri:
            vtof[int(v)].append(f)
    return vtof


def _ring(faces, cells):
    """faces around a vertex in ring order (neighbours share an edge)"""
    sets = {f: set(int(x) for x in cells[f]) for f in faces}
    order = [faces[0]]
    left = set(faces[1:])
    while left:
        last = sets[order[-1]]
        nxt = next(f for f in sorted(left) if len(sets[f] & last) == 2)
        order.append(nxt)
        left.discard(nxt)
    return order


def _half_bc(cells, vtof, v, p):
    """buildhalfbc (src/bases/bcspace.jl:194-405) for an interior vertex of a closed surface"""
    S = _ring(vtof[v], cells)
    n = len(S)
    assert n >= 2 and n % 2 == 0
    ports = [i for i, f in enumerate(S) if p in cells[f]]
    assert len(ports) == 2
    if ports[0] != (ports[1] + 1) % n:
        ports.reverse()
    assert ports[0] == (ports[1] + 1) % n
    charges = np.full(n, 1.0 / n)
    bf = []
    for i in ports:  # flux 1/2 out through the port cell's edge opposite v
        e = list(cells[S[i]]).index(v)
        bf.append((S[i], e, 0.5))
        charges[i] -= 0.5
    start = ports[0]
    for i in range(1, n):
        j0 = (start + i - 1) % n
        j1 = (j0 + 1) % n
        f0, f1 = S[j0], S[j1]
        t0, t1 = [int(x) for x in cells[f0]], [int(x) for x in cells[f1]]
        e0 = next(k for k in range(3) if t0[k] not in t1)  # the common edge is opposite e0 in f0
        e1 = next(k for k in range(3) if t1[k] not in t0)
        bf.append((f0, e0, charges[j0]))
        bf.append((f1, e1, -charges[j0]))
        charges[j1] += charges[j0]
    return bf


def _merge(fn):
    acc = {}
    for c, r, w in fn:
        acc[(c, r)] = acc.get((c, r), 0.0) + w
    return [(c, r, w) for (c, r), w in sorted(acc.items()) if abs(w) > 1e-14]


def buffachristiansen(mesh, refinement=None, rt=None):
    """BC functions on the barycentric refinement, one per edge of `raviartthomas(mesh)` (in its
    order); returns (Space on the fine mesh, Refinement)"""
    from .spaces import raviartthomas
    R = refinement or barycentric_refinement(mesh)
    X = rt or raviartthomas(mesh)
    cells = R.fine.cells
    vtof = _vertex_to_cells(cells, R.fine.numvertices())
    fns, pos = [], []
    for fn in X.fns:
        c, r, _ = fn[0]
        v1, v2 = int(mesh.cells[c, (r + 1) % 3]), int(mesh.cells[c, (r + 2) % 3])
        p = R.midpoint[(v1, v2) if v1 < v2 else (v2, v1)]
        half1 = _half_bc(cells, vtof, v1, p)
        half2 = _half_bc(cells, vtof, v2, p)
        fns.append(_merge(half1 + [(f, e, -w) for (f, e, w) in half2]))
        pos.append(R.fine.vertices[p])
    return Space(RT, R.fine, fns, np.array(pos)), R


def refined(X, R):
    """the RT space X of R.coarse written in the RT shapes of R.fine's cells: on a child t of
    coarse cell c the coarse shape (x - v_r) / (2 A_c) leaves t through its edge (a, b) with
    flux |ab| ((a - v_r) . m) / (2 A_c), m the outward unit normal of that edge"""
    assert X.kind == RT and X.mesh is R.coarse
    Vf, Cf = R.fine.vertices, R.fine.cells
    Vc, Cc = R.coarse.vertices, R.coarse.cells
    areas = R.coarse.areas()
    fns = []
    for fn in X.fns:
        out = []
        for c, r, w in fn:
            vr = Vc[Cc[c, r]]
            for t in R.children(c):
                tri = Vf[Cf[t]]
                nt = np.cross(tri[1] - tri[0], tri[2] - tri[0])
                for k in range(3):
                    a, b = tri[(k + 1) % 3], tri[(k + 2) % 3]
                    mvec = np.cross(b - a, nt)
                    mvec /= np.linalg.norm(mvec)
                    if np.dot(tri[k] - a, mvec) > 0:
                        mvec = -mvec
                    flux = np.linalg.norm(b - a) * np.dot(a - vr, mvec) / (2 * areas[c])
                    out.append((t, k, w * flux))
        fns.append(_merge(out))
    return Space(RT, R.fine, fns, X.pos)
