"""Regenerate the golden fixtures from the reference checkout (run in the authoring
container, where the reference is mounted; the GPU host only reads the committed output).

  meshes/*.in      -- copied verbatim from the reference's test/assets (mesh data files)
  golden.json      -- numeric golden values parsed out of the reference's test files:
      * hh3d_separated_refval : hcubature value of the Helmholtz single layer P0 x P0
        interaction of two separated triangles (test/test_hh3dints.jl:619-671)
      * hh3d_separated_t1/t2  : those triangles
      * ss_triangles          : the triangles of test/test_sauterschwabints.jl:8-15,94-103
      * farfield_sphere824    : the far-field test of test/test_farfield.jl: the magnitudes
        |E| at 7 angles (lines 34-40) of the golden current test/efie_solution.txt (1236 RT
        coefficients on test/assets/sphere824.in), with the map from the reference's dof order
        to this package's (see dof_map below)

The reference orders and orients its RT functions with CompScienceMeshes (not vendored), so
the golden current's dof order is recovered here: the current is the EFIE solution for the
plane wave (direction z, polarisation x, k = 1) on that mesh (its far field matches the
golden magnitudes to 4e-4 at quadrature accuracy), so the oracle's own solution of that
system in this package's dof order matches every coefficient up to sign, and a minimum-cost
assignment (scipy) on min(|x_j - u_i|, |x_j + u_i|) pairs them.  The map is checked, not
assumed: with it the golden magnitudes are reproduced to 1e-15 (tests/test_oracle_pins.py).

usage: python tests/golden/make_fixtures.py /path/to/reference
"""
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

MESHES = ["sphere45.in", "sphere5.in", "sphere35.in", "sphere2.in", "sphere824.in"]


def vecs(text):
    return [[float(x) for x in m.split(",")] for m in re.findall(r"@SVector \[([^\]]+)\]", text)]


def farfield_dof_map(u, mesh_file):
    """(perm, sign): the reference's coefficient i belongs to this package's RT function
    perm[i] with orientation sign[i]"""
    import numpy as np
    from scipy.optimize import linear_sum_assignment
    for p in (os.path.join(ROOT, "beast.jl_gb300"), os.path.join(ROOT, "oracle")):
        sys.path.insert(0, p)
    import beastgpu as bg
    import oracle as O
    X = bg.raviartthomas(bg.readmesh(mesh_file))
    g = 1j
    Z = O.assemble(O.make_op(O.MW_SL, g, -g, -1 / g), O.make_qs(O.QS_WILTON_SAUTER, 2, 3, 6, 7, 5, 5, 4, 3), X, X)
    x = np.linalg.solve(Z, O.rhs_planewave(0, X, (0, 0, 1), (1, 0, 0), g))
    cp = np.abs(x[None, :] - u[:, None])
    cm = np.abs(x[None, :] + u[:, None])
    r, c = linear_sum_assignment(np.minimum(cp, cm))
    perm = np.empty(len(u), dtype=int)
    sign = np.empty(len(u), dtype=int)
    perm[r] = c
    sign[r] = np.where(cp[r, c] <= cm[r, c], 1, -1)
    return perm, sign


def main():
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    REF = sys.argv[1]
    os.makedirs(os.path.join(HERE, "meshes"), exist_ok=True)
    for m in MESHES:
        shutil.copyfile(os.path.join(REF, "test", "assets", m), os.path.join(HERE, "meshes", m))
    golden = {}
    hh = open(os.path.join(REF, "test", "test_hh3dints.jl")).read()
    sep = hh[hh.index('@testset "Seperated triangles"'):]
    v = vecs(sep)
    golden["hh3d_separated_t1"] = v[0:3]
    golden["hh3d_separated_t2"] = v[3:6]
    m = re.search(r"refval = ([-0-9.e]+) ([+-]) ([0-9.e-]+)im", sep)
    re_, sgn, im_ = float(m.group(1)), m.group(2), float(m.group(3))
    golden["hh3d_separated_refval"] = [re_, im_ if sgn == "+" else -im_]
    golden["hh3d_gamma"] = [1.0, 1.0]
    ss = open(os.path.join(REF, "test", "test_sauterschwabints.jl")).read()
    v = vecs(ss)
    golden["ss_triangles"] = {"face_t1": v[0:3], "vertex_t2": v[3:6],
                              "edge_t1": v[6:9], "edge_t2": v[9:12]}
    ff = open(os.path.join(REF, "test", "test_farfield.jl")).read()
    import numpy as np
    u = np.array([complex(x.strip().replace(" ", "").replace("im", "j"))
                  for x in open(os.path.join(REF, "test", "efie_solution.txt")) if x.strip()])
    perm, sign = farfield_dof_map(u, os.path.join(HERE, "meshes", "sphere824.in"))
    golden["farfield_sphere824"] = {
        "a": [float(x) for x in re.findall(r"@test a\[\d\] ≈ ([0-9.e-]+)", ff)],
        "u_re": u.real.tolist(), "u_im": u.imag.tolist(),
        "dof_map": perm.tolist(), "sign": sign.tolist()}
    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump(golden, fh, indent=1)


if __name__ == "__main__":
    main()
