"""Regenerate the golden fixtures from the reference checkout (run in the authoring
container, where the reference is mounted; the GPU host only reads the committed output).

  meshes/*.in      -- copied verbatim from the reference's test/assets (mesh data files)
  golden.json      -- numeric golden values parsed out of the reference's test files:
      * hh3d_separated_refval : hcubature value of the Helmholtz single layer P0 x P0
        interaction of two separated triangles (test/test_hh3dints.jl:619-671)
      * hh3d_separated_t1/t2  : those triangles
      * ss_triangles          : the triangles of test/test_sauterschwabints.jl:8-15,94-103
      * farfield_sphere824    : far-field magnitudes |E| at 7 angles of the golden current
        (test/test_farfield.jl:34-40)

usage: python tests/golden/make_fixtures.py [/path/to/reference]
"""
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"

MESHES = ["sphere45.in", "sphere5.in", "sphere35.in", "sphere2.in", "sphere824.in"]


def vecs(text):
    return [[float(x) for x in m.split(",")] for m in re.findall(r"@SVector \[([^\]]+)\]", text)]


def main():
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
    golden["farfield_sphere824"] = [float(x) for x in
                                    re.findall(r"@test a\[\d\] ≈ ([0-9.e-]+)", ff)]
    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump(golden, fh, indent=1)


if __name__ == "__main__":
    main()
