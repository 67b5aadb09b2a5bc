"""Generates the golden fixtures in tests/golden/ from the PANSFEM2 reference.

Runs oracle/_ref/ref_driver (the reference headers compiled by
oracle/build_ref.sh) on small SIMP problems and the reference's own test mains
(src/LinearAlgebra/Solvers/test_CG.cpp, src/Optimize/Solver/test_MMA*.cpp), CONLIN on
the optimiser test problems, the general assembly path on explicit meshes, and
stores their outputs as compressed .npz / .txt fixtures.  Needs the reference
source tree, so it runs only where that tree exists; the fixtures it writes
are committed and used everywhere else.

    python tests/golden/make_golden.py [path-to-PANSFEM2]
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import build as obuild  # noqa: E402
from oracle.pyoracle import read_dump  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")

# name -> (ref_driver args, iterations, fields to keep (None = all))
CASES = {
    "cantilever_12x6_oc": (["kind=0", "nx=12", "ny=6", "bc=cantilever", "solvers=1"], 5, None),
    "cantilever_60x30_oc": (["kind=0", "nx=60", "ny=30", "bc=cantilever", "move=0.2"], 10,
                            ["f", "g", "rho", "s_after", "n2g", "indptr", "indices", "data", "F0",
                             "result0", "Ke0", "nb_ptr", "nb_idx", "nb_w"]),
    "mbb_16x8_mma": (["kind=0", "nx=16", "ny=8", "bc=mbb", "opt=1", "vf=0.4", "R=3"], 6, None),
    "mbb_48x24_mma": (["kind=0", "nx=48", "ny=24", "bc=mbb", "opt=1", "vf=0.4", "R=3"], 10,
                      ["f", "g", "rho", "s_after", "dfds", "n2g", "nb_ptr", "nb_idx", "nb_w"]),
    "heatsink_10x10_oc": (["kind=1", "nx=10", "ny=10", "bc=heatsink", "E0=1e-3", "patch_w=1",
                           "patch_i0=4"], 4, None),
    "cantilever_h8_6x3x3_oc": (["kind=2", "nx=6", "ny=3", "nz=3", "vf=0.3", "R=1.5"], 3, None),
    "cantilever_12x6_heaviside": (["kind=0", "nx=12", "ny=6", "bc=cantilever", "heaviside=1"], 4,
                                  None),
    "cantilever_60x40_conlin": (["kind=0", "nx=60", "ny=40", "bc=cantilever", "opt=2", "heaviside=1",
                                 "E1=210000", "E0=1e-4", "scale0=1e5", "move=0.2"], 6,
                                ["f", "g", "rho", "dfds", "s_after", "nb_ptr", "nb_idx", "nb_w"]),
}
TEST_MAINS = ["test_CG", "test_MMA", "test_MMA_3", "test_MMA_TOY2"]
# CONLIN replayed step by step on the optimiser test problems (ref_driver conlin)
CONLIN_PROBLEMS = {"mma": 30, "mma3": 30, "toy2": 30}


def read_vtk_vectors(path, name):
    """The POINT_DATA vectors called name of a legacy ASCII VTK file, as (npoints, 3)."""
    with open(path) as fh:
        words = fh.read().split()
    npts = int(words[words.index("POINT_DATA") + 1])
    k = next(i for i in range(len(words) - 1) if words[i] == "VECTORS" and words[i + 1] == name)
    return np.array(words[k + 3:k + 3 + 3 * npts], float).reshape(npts, 3)


def main():
    from oracle.build import REFERENCE_ROOT
    # usage: make_golden.py [path-to-PANSFEM2] [--only CASE]  (--only: regenerate one SIMP case and stop)
    argv = sys.argv[1:]
    only = None
    if "--only" in argv:
        k = argv.index("--only")
        only = argv[k + 1]
        argv = argv[:k] + argv[k + 2:]
    ref_root = argv[0] if argv else REFERENCE_ROOT
    obuild.build()
    if not obuild.build_reference(ref_root):
        raise SystemExit(f"reference tree not found at {ref_root}")
    tmp = os.path.join(ROOT, "oracle", "_ref", "dump.bin")
    for name, (args, iters, keep) in CASES.items():
        if only is not None and name != only:
            continue
        subprocess.run([os.path.join(REF, "ref_driver"), "simp", f"out={tmp}", f"iters={iters}"] + args,
                       check=True, stdout=subprocess.DEVNULL)
        d = read_dump(tmp)
        if keep is not None:
            d = {k: v for k, v in d.items() if k in keep or k in ("fix_node", "fix_dof", "load_node",
                                                                   "load_dof", "load_val")}
        d["iters"] = np.array([iters], np.int32)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(f"{name}: {sorted(d)}")
    if only is not None:
        return
    # iteration 0 of the 12x6 cantilever written by the reference's own VTK writer
    vtk = os.path.join(HERE, "ref_cantilever_12x6_it0.vtk")
    subprocess.run([os.path.join(REF, "ref_driver"), "simp", f"out={tmp}", "iters=1", "kind=0", "nx=12", "ny=6",
                    "bc=cantilever", f"vtk={vtk}"], check=True, stdout=subprocess.DEVNULL)
    print(f"{os.path.basename(vtk)}: {os.path.getsize(vtk)} bytes")
    # explicit meshes (tests/golden/fem_meshes.py): the general assembly path of the reference
    from tests.golden.fem_meshes import FEM_CASES, write_mesh  # noqa: E402
    mesh = os.path.join(ROOT, "oracle", "_ref", "mesh.txt")
    for name, mk in FEM_CASES.items():
        case = mk()
        write_mesh(case, mesh)
        solver = "cg" if name == "fem_planestrain_sample" else "scaling_cg"   # the sample uses CG
        subprocess.run([os.path.join(REF, "ref_driver"), "fem", f"mesh={mesh}", f"out={tmp}", f"solver={solver}"],
                       check=True, stdout=subprocess.DEVNULL)
        d = read_dump(tmp)
        d.update(kind=np.array([case["kind"]], np.int32), coords=np.asarray(case["coords"], float),
                 conn=np.asarray(case["conn"], np.int32), E=np.asarray(case["E"], float),
                 Vt=np.array([case["V"], case["t"]]),
                 fixed=np.array(case["fixed"], float).reshape(-1, 3), loads=np.array(case["loads"], float).reshape(-1, 3),
                 body=np.array(case.get("body") or (np.nan, np.nan), float),
                 edges=np.array(case.get("edges", []), np.int32).reshape(-1, 2),
                 traction=np.array(case.get("traction", (0.0, 0.0)), float),
                 solver=np.array([0 if solver == "scaling_cg" else 4], np.int32))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(f"{name}.npz")
    os.remove(mesh)
    # sample/solid/sample_linear.cpp: an H8 cantilever read from the reference's CSV files by its
    # own ImportFromCSV.h, with the displacements of its committed result_linear.vtk
    solid = os.path.join(ref_root, "sample", "solid")
    subprocess.run([os.path.join(REF, "ref_driver"), "fem", f"csvdir={solid}", "kind=2", "E=210000", "V=0.3",
                    f"out={tmp}"], check=True, stdout=subprocess.DEVNULL)
    d = read_dump(tmp)
    nn = len(d["read_coords"]) // 3
    d.update(kind=np.array([2], np.int32), coords=d["read_coords"].reshape(nn, 3),
             conn=d["read_conn"].reshape(-1, 8), E=np.full(len(d["read_conn"]) // 8, 210000.0),
             Vt=np.array([0.3, 1.0]),
             fixed=np.column_stack([d["read_fix"].reshape(-1, 2), d["read_fixval"]]),
             loads=np.column_stack([d["read_load"].reshape(-1, 2), d["read_loadval"]]),
             body=np.array([np.nan, np.nan]), edges=np.zeros((0, 2), np.int32), traction=np.zeros(2),
             solver=np.array([0], np.int32), vtk_u=read_vtk_vectors(os.path.join(solid, "result_linear.vtk"), "u"))
    np.savez_compressed(os.path.join(HERE, "fem_solid_sample.npz"), **d)
    print("fem_solid_sample.npz")
    # the reference's parse of the CSV grammar cases in tests/golden/csv_grammar/
    subprocess.run([os.path.join(REF, "ref_driver"), "csvread", f"csvdir={os.path.join(HERE, 'csv_grammar')}",
                    "nd=2", f"out={tmp}"], check=True, stdout=subprocess.DEVNULL)
    np.savez_compressed(os.path.join(HERE, "csv_grammar.npz"), **read_dump(tmp))
    print("csv_grammar.npz")
    for pb, iters in CONLIN_PROBLEMS.items():
        subprocess.run([os.path.join(REF, "ref_driver"), "conlin", f"out={tmp}", f"problem={pb}", f"iters={iters}"],
                       check=True, stdout=subprocess.DEVNULL)
        np.savez_compressed(os.path.join(HERE, f"conlin_{pb}.npz"), **read_dump(tmp))
        print(f"conlin_{pb}.npz")
    os.remove(tmp)
    for t in TEST_MAINS:
        out = subprocess.run([os.path.join(REF, t)], check=True, capture_output=True, text=True).stdout
        with open(os.path.join(HERE, f"ref_{t}.txt"), "w") as fh:
            fh.write(out)
        print(f"ref_{t}.txt: {len(out)} bytes")


if __name__ == "__main__":
    main()
