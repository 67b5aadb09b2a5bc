"""The CSV readers (ImportFromCSV.h:22-253) in Python (pansfem2_gb300.csvio) and C++
(pansfem2_gb300.hpp) against the reference's own readers: the grammar cases in
tests/golden/csv_grammar/ (CRLF, records split by spaces, empty ids, trailing commas, "free",
hex and prefix numbers, missing fields) parsed by the reference into csv_grammar.npz, and the
reference's H8 sample mesh (sample/solid) parsed into fem_solid_sample.npz."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle.build import REFERENCE_ROOT
from pansfem2_gb300 import csvio
from tests.cases import load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GRAMMAR = os.path.join(ROOT, "tests", "golden", "csv_grammar")
SOLID = os.path.join(REFERENCE_ROOT, "sample", "solid")


def _flat(rows):
    if isinstance(rows, np.ndarray):
        return rows.reshape(-1), [rows.shape[1]] * rows.shape[0]
    return (np.concatenate(rows) if rows else np.zeros(0)), [len(r) for r in rows]


def _pairs(conds):
    n, d, v = csvio.conditions_arrays(conds)
    return np.column_stack([n, d]).reshape(-1), v


def test_python_reader_matches_the_reference_on_the_grammar_cases():
    g = load("csv_grammar")
    x, xl = _flat(csvio.import_nodes_from_csv(os.path.join(GRAMMAR, "Node.csv")))
    assert np.array_equal(x, g["nodes"]) and np.array_equal(xl, g["node_len"])
    assert np.array_equal(np.signbit(x), np.signbit(g["nodes"]))   # "-0" stays negative zero
    c, cl = _flat(csvio.import_elements_from_csv(os.path.join(GRAMMAR, "Element.csv")))
    assert np.array_equal(c, g["conn"]) and np.array_equal(cl, g["conn_len"])
    i, v = _pairs(csvio.import_dirichlet_from_csv(os.path.join(GRAMMAR, "Dirichlet.csv")))
    assert np.array_equal(i, g["fix"]) and np.array_equal(v, g["fixval"])
    i, v = _pairs(csvio.import_neumann_from_csv(os.path.join(GRAMMAR, "Neumann.csv")))
    assert np.array_equal(i, g["load"]) and np.array_equal(v, g["loadval"])
    per = csvio.import_periodic_from_csv(os.path.join(GRAMMAR, "Periodic.csv"))
    assert np.array_equal(np.array(per).reshape(-1), g["periodic"])
    u = csvio.import_initial_from_csv(np.zeros((len(xl), 2)), os.path.join(GRAMMAR, "Initial.csv"))
    assert np.array_equal(u.reshape(-1), g["initial"])


@pytest.mark.parametrize("rows", ["std_vector", "reference_vector"])
def test_cpp_reader_matches_the_reference_on_the_grammar_cases(tmp_path, rows):
    """With std::vector<double> node rows, and with rows that have only the reference
    Vector<T>'s operator() and SIZE()."""
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "csv_check")
    flags = ["-DVECTOR_ROWS"] if rows == "reference_vector" else []
    subprocess.run(["g++", "-O1", "-std=c++17", *flags, "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "csv_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe, GRAMMAR, "2"], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        k, *vals = line.split()
        got[k] = vals
    g = load("csv_grammar")
    for k in ("node_len", "conn", "conn_len", "fix", "load", "periodic"):
        assert np.array_equal(np.array(got[k], int), g[k]), k
    for k in ("nodes", "fixval", "loadval", "initial"):
        assert np.array_equal(np.array(got[k], float), g[k]), k


def test_reader_errors(tmp_path):
    with pytest.raises(OSError, match="Node file .* open error!"):
        csvio.import_nodes_from_csv(str(tmp_path / "missing.csv"))
    with pytest.raises(OSError, match="Dirichlet Condition file"):   # the reference's message
        csvio.import_neumann_from_csv(str(tmp_path / "missing.csv"))
    for text, exc in ((b"id,x\n0,1e-310\n", OverflowError), (b"id,x\n0,1e999\n", OverflowError),
                      (b"id,x\n0,abc\n", ValueError), (b"id,x\n0,1,,2\n", ValueError)):
        p = tmp_path / "Node.csv"
        p.write_bytes(text)
        with pytest.raises(exc):
            csvio.import_nodes_from_csv(str(p))
    p = tmp_path / "Element.csv"
    p.write_bytes(b"id,n\n0,1,4294967296\n")
    with pytest.raises(OverflowError):
        csvio.import_elements_from_csv(str(p))


@pytest.mark.skipif(not os.path.isdir(SOLID), reason="the reference's sample files are not present")
def test_reference_sample_files():
    """sample/solid/{Node,Element,Dirichlet,Neumann}.csv read as the reference read them."""
    g = load("fem_solid_sample")
    x = csvio.import_nodes_from_csv(os.path.join(SOLID, "Node.csv"))
    assert np.array_equal(x.reshape(-1), g["read_coords"])
    e = csvio.import_elements_from_csv(os.path.join(SOLID, "Element.csv"))
    assert np.array_equal(e.reshape(-1), g["read_conn"])
    i, v = _pairs(csvio.import_dirichlet_from_csv(os.path.join(SOLID, "Dirichlet.csv")))
    assert np.array_equal(i, g["read_fix"]) and np.array_equal(v, g["read_fixval"])
    i, v = _pairs(csvio.import_neumann_from_csv(os.path.join(SOLID, "Neumann.csv")))
    assert np.array_equal(i, g["read_load"]) and np.array_equal(v, g["read_loadval"])


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE_ROOT, "src")),
                    reason="the reference's headers are not present")
def test_mirror_accepts_the_reference_vector_type(tmp_path):
    """The reference's own Vector<double> rows (as ImportNodesFromCSV and Delaunay::GenerateNodes
    return them) go into the mirror's readers and FemMesh unchanged: a compile check against
    the reference's Vector.h (no device call)."""
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    src = tmp_path / "refvec.cpp"
    src.write_text("""
#include <string>
#include <vector>
#include "src/LinearAlgebra/Models/Vector.h"
#include "pansfem2_gb300.hpp"
int run(const std::string &p) {
    std::vector<PANSFEM2::Vector<double> > x;
    PANSFEM2_GB300::ImportNodesFromCSV(x, p + "Node.csv");
    std::vector<std::vector<int> > el;
    PANSFEM2_GB300::ImportElementsFromCSV(el, p + "Element.csv");
    std::vector<PANSFEM2::Vector<double> > u(x.size(), PANSFEM2::Vector<double>(3));
    PANSFEM2_GB300::ImportInitialFromCSV(u, p + "Initial.csv");
    PANSFEM2_GB300::FemMesh m(PSF_H8_SOLID, x, el);
    return (int)m.nnodes();
}
""")
    subprocess.run(["g++", "-std=c++17", "-w", "-I", os.path.join(ROOT, "include"), "-I", REFERENCE_ROOT,
                    "-c", str(src), "-o", str(tmp_path / "refvec.o")], check=True)
