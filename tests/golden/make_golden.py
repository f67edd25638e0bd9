"""Regenerate the golden fixtures in tests/golden/ from the FeeLLGood source tree.

Usage: ``python tests/golden/make_golden.py <path of the FeeLLGood source tree>`` (the path
is required). Nothing at test time reads the reference tree; the tests read only the files
this script writes:

* ``ellipsoid.msh``          the mesh of the reference's functional test (examples/ellipsoid.msh),
                             copied byte for byte.
* ``bad_cuboid_{1..4}.msh``  the four malformed meshes of unit-tests/meshes/, copied.
* ``golden.json``            the known answers read (as text) from the reference's tests:
                             ci-tests/full_test.py (settings, seed and final <m>, E_tot for the
                             5-point and 1-point Gauss builds), unit-tests/ut_readMesh.cpp (ellipsoid
                             counts and the four controlTriangles error messages).
* ``cuboid_3x2x2.msh``       produced by importing python-modules/meshMaker.py and calling
                             ``Cuboid((0,0,0),(7.5,5,5),3,2,2).make(...)``; the structured-mesh
                             generator of this package must reproduce it.
* ``cuboid_20.json``         node/tet/tri counts and sha256 of the file the same call writes for the
                             50 nm cube on a 2.5 nm grid (20^3 cells x 6 tets).
"""
import hashlib
import json
import os
import re
import shutil
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    shutil.copyfile(os.path.join(ref, "examples", "ellipsoid.msh"), os.path.join(HERE, "ellipsoid.msh"))
    for k in range(1, 5):
        shutil.copyfile(os.path.join(ref, "unit-tests", "meshes", f"bad_cuboid_{k}.msh"),
                        os.path.join(HERE, f"bad_cuboid_{k}.msh"))
    gold = {}
    ft = open(os.path.join(ref, "ci-tests", "full_test.py")).read()
    m1 = re.search(r'ONE_GAUSS_POINT=ON.*?expected = \{ "m": \[([^\]]*)\], "E_tot": ([-0-9.e]+)', ft, re.S)
    m5 = re.search(r'else:\s*expected = \{ "m": \[([^\]]*)\], "E_tot": ([-0-9.e]+)', ft, re.S)
    thr = re.search(r"threshold = ([0-9.e-]+)", ft)
    seed = re.search(r'"--seed", "([0-9]+)"', ft)
    gold["full_test"] = {
        "mesh": "ellipsoid.msh",
        "length_unit": float(re.search(r'"length_unit": ([0-9.e-]+)', ft).group(1)),
        "volume_region": re.search(r'"volume_regions": \{\s*"([a-z_]+)"', ft).group(1),
        "K": float(re.search(r'"K": ([0-9.e]+)', ft).group(1)),
        "uk": [float(x) for x in re.search(r'"uk": \[([^\]]*)\]', ft).group(1).split(",")],
        "initial_magnetization": [float(x) for x in
                                  re.search(r'"initial_magnetization": \[([^\]]*)\]', ft).group(1).split(",")],
        "Bext": [float(x) for x in re.search(r'"Bext": \[([^\]]*)\]', ft).group(1).split(",")],
        "evol_time_step": float(re.search(r'"evol_time_step": ([0-9.e-]+)', ft).group(1)),
        "final_time": float(re.search(r'"final_time": ([0-9.e-]+)', ft).group(1)),
        "min_dt": float(re.search(r'"min\(dt\)": ([0-9.e-]+)', ft).group(1)),
        "max_dt": float(re.search(r'"max\(dt\)": ([0-9.e-]+)', ft).group(1)),
        "max_du": float(re.search(r'"max\(du\)": ([0-9.e-]+)', ft).group(1)),
        "seed": int(seed.group(1)),
        "threshold": float(thr.group(1)),
        "expected_5pt": {"m": [float(x) for x in m5.group(1).split(",")], "E_tot": float(m5.group(2))},
        "expected_1pt": {"m": [float(x) for x in m1.group(1).split(",")], "E_tot": float(m1.group(2))},
    }
    ut = open(os.path.join(ref, "unit-tests", "ut_readMesh.cpp")).read()
    nodes = int(re.search(r"nodeT\.size\(\) == ([0-9]+)\)", ut).group(1))
    elems = [int(x) for x in re.findall(r"elemTags\.size\(\) == ([0-9]+)\)", ut)]
    gold["ellipsoid_counts"] = {"nodes": nodes, "tets": elems[0], "tris": elems[1]}
    msgs = re.findall(r'logOutput\.str\(\) == ((?:"[^"]*"\s*)+)\)', ut)
    gold["bad_cuboid_errors"] = ["".join(re.findall(r'"([^"]*)"', m)).replace("\\n", "") for m in msgs]
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(gold, f, indent=1)

    sys.path.insert(0, os.path.join(ref, "python-modules"))
    import meshMaker
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "c.msh")
        meshMaker.Cuboid((0, 0, 0), (7.5, 5, 5), 3, 2, 2).make(p, "volume", "surface")
        shutil.copyfile(p, os.path.join(HERE, "cuboid_3x2x2.msh"))
        c = meshMaker.Cuboid((0, 0, 0), (50, 50, 50), 20, 20, 20)
        c.make(p, "volume", "surface")
        data = open(p, "rb").read()
        info = {"args": [[0, 0, 0], [50, 50, 50], 20, 20, 20], "nodes": len(c.pts), "tets": len(c.Tet),
                "tris": len(c.Tri), "sha256": hashlib.sha256(data).hexdigest()}
    with open(os.path.join(HERE, "cuboid_20.json"), "w") as f:
        json.dump(info, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2 or not os.path.isdir(sys.argv[1]):
        sys.exit("usage: make_golden.py <path of the FeeLLGood source tree>")
    main(sys.argv[1])
