"""MMA<T> on the device for m > 1 and per-variable bounds (psf_mma_*), against the
oracle MMA (pinned bit for bit to the reference's test programs) one update at a
time from the same iterate, against the trajectory the reference's test_MMA_3
prints, and on a large problem with three constraints and per-variable bounds.
Tolerance: 1e-7 per update (the same bar as the m = 1 kernels); the printed
trajectory to its 6 significant digits."""
import os
import re

import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pansfem2_gb300 as P
    P.load()
    return P


def _mma5(s):
    C1, C2 = 0.0624, 1.0
    coef = np.array([61.0, 37.0, 19.0, 7.0, 1.0])
    f = C1 * np.sum(s)
    g = float(np.sum(coef * s ** -3.0) - C2)
    return f, [C1] * 5, [g], [list(-3.0 * coef * s ** -4.0)]


def _mma3(s):
    C1, C2 = 1.0, 0.124
    q = np.sqrt(1.0 + s[1] ** 2.0)
    f = C1 * s[0] * q
    df = [C1 * q, C1 * s[0] * s[1] / q]
    g0 = C2 * q * (8.0 * s[0] ** -1.0 + 1.0 * s[0] ** -1.0 * s[1] ** -1.0) - 1.0
    g1 = C2 * q * (8.0 * s[0] ** -1.0 - 1.0 * s[0] ** -1.0 * s[1] ** -1.0) - 1.0
    dg0 = [C2 * q * (-8.0 * s[0] ** -2.0 - 1.0 * s[0] ** -2.0 * s[1] ** -1.0),
           C2 * s[1] / q * (8.0 * s[0] ** -1.0 + 1.0 * s[0] ** -1.0 * s[1] ** -1.0)
           + C2 * q * (-1.0 * s[0] ** -1.0 * s[1] ** -2.0)]
    dg1 = [C2 * q * (-8.0 * s[0] ** -2.0 + 1.0 * s[0] ** -2.0 * s[1] ** -1.0),
           C2 * s[1] / q * (8.0 * s[0] ** -1.0 - 1.0 * s[0] ** -1.0 * s[1] ** -1.0)
           + C2 * q * (1.0 * s[0] ** -1.0 * s[1] ** -2.0)]
    return f, df, [g0, g1], [dg0, dg1]


def _toy2(s):
    f = float(np.sum(s ** 2.0))
    g0 = (s[0] - 5.0) ** 2.0 + (s[1] - 2.0) ** 2.0 + (s[2] - 1.0) ** 2.0 - 9.0
    g1 = (s[0] - 3.0) ** 2.0 + (s[1] - 4.0) ** 2.0 + (s[2] - 3.0) ** 2.0 - 9.0
    return (f, list(2.0 * s), [g0, g1],
            [[2.0 * (s[0] - 5.0), 2.0 * (s[1] - 2.0), 2.0 * (s[2] - 1.0)],
             [2.0 * (s[0] - 3.0), 2.0 * (s[1] - 4.0), 2.0 * (s[2] - 3.0)]])


# (n, m, x0, a0, a, c, d, xmin, xmax, iterations, functions): the reference's test mains
PROBLEMS = {
    "test_MMA (n 5, m 1)": (5, 1, [5.0] * 5, 1.0, [0.0], [1000.0], [1.0], [1.0] * 5, [10.0] * 5, 10, _mma5),
    "test_MMA_3 (n 2, m 2: the n <= m system)": (2, 2, [1.5, 0.5], 1.0, [0.0, 0.0], [1000.0, 1000.0], [1.0, 1.0],
                                                 [0.2, 0.1], [4.0, 1.6], 12, _mma3),
    "test_MMA_TOY2 (n 3, m 2)": (3, 2, [4.0, 3.0, 2.0], 1.0, [0.0, 0.0], [1000.0, 1000.0], [1.0, 1.0], [0.0] * 3,
                                 [5.0] * 3, 6, _toy2),
}
PARAMS = (1e-5, 0.1, 0.5, 0.5, 0.7, 1.2, 1e-5)


@pytest.mark.parametrize("name", list(PROBLEMS))
def test_updates_match_oracle_step_by_step(gpu, name):
    n, m, x0, a0, a, c, d, lo, hi, iters, fg = PROBLEMS[name]
    orc = O.MMA(n, m, a0, a, c, d, lo, hi)
    orc.set_parameters(*PARAMS)
    dev = gpu.DeviceMMA(n, m, a0, a, c, d, lo, hi)
    dev.set_parameters(*PARAMS)
    s = np.array(x0, float)
    for k in range(iters):
        f, df, g, dg = fg(s)
        x_o, _ = orc.update(s, f, df, g, dg)
        x_d, _ = dev.update(s, f, df, g, dg)
        assert np.max(np.abs(x_d - x_o)) <= 1e-7 * max(1.0, np.max(np.abs(x_o))), (k, x_d, x_o)
        s = x_o
    dev.close()


def test_n_le_m_trajectory_matches_the_reference_print(gpu):
    """The device MMA alone runs test_MMA_3's loop (IsConvergence exit included); its iterates
    equal the ones the reference prints (ref_test_MMA_3.txt) to their 6 digits."""
    n, m, x0, a0, a, c, d, lo, hi, _, fg = PROBLEMS["test_MMA_3 (n 2, m 2: the n <= m system)"]
    rows = [list(map(float, re.findall(r"[-+0-9.e]+", line.split("Constraints1:")[1])[1:]))
            for line in open(os.path.join(GOLDEN, "ref_test_MMA_3.txt")) if line.startswith("k = ")]
    dev = gpu.DeviceMMA(n, m, a0, a, c, d, lo, hi)
    dev.set_parameters(*PARAMS)
    s = np.array(x0, float)
    for k, ref in enumerate(rows):
        assert np.allclose(s, ref, rtol=1e-5, atol=1e-6), (k, s, ref)
        f, df, g, dg = fg(s)
        if dev.is_convergence(f):
            assert k == len(rows) - 1
            break
        s, _ = dev.update(s, f, df, g, dg)
    dev.close()


def test_large_problem_three_constraints_per_variable_bounds(gpu):
    """n = 20,000 variables, m = 3 linear constraints, a convex objective sum w_j / x_j, bounds
    that differ per variable; five updates in lockstep with the oracle."""
    rng = np.random.default_rng(4)
    n, m = 20000, 3
    w = rng.uniform(0.5, 2.0, n)
    Acon = rng.uniform(0.2, 1.0, (m, n))
    lo, hi = rng.uniform(0.05, 0.2, n), rng.uniform(0.7, 1.0, n)
    bvec = np.array([0.45, 0.5, 0.55]) * Acon.sum(1)

    def fg(x):
        return float(np.sum(w / x)), -w / x ** 2, Acon @ x - bvec, Acon

    orc = O.MMA(n, m, 1.0, [0.0] * m, [1000.0] * m, [1.0] * m, lo, hi)
    dev = gpu.DeviceMMA(n, m, 1.0, [0.0] * m, [1000.0] * m, [1.0] * m, lo, hi)
    for o in (orc, dev):
        o.set_parameters(1e-5, 0.1, 0.2, 0.5, 0.7, 1.2, 1e-5)
    s = 0.5 * (lo + hi)
    for k in range(5):
        f, df, g, dg = fg(s)
        x_o, _ = orc.update(s, f, df, g, dg)
        x_d, _ = dev.update(s, f, df, g, dg)
        assert np.max(np.abs(x_d - x_o)) <= 1e-7, (k, np.max(np.abs(x_d - x_o)))
        assert np.all(x_d >= lo - 1e-12) and np.all(x_d <= hi + 1e-12)
        s = x_o
    dev.close()


def test_cpp_mirror_runs_test_MMA_3(gpu, tmp_path):
    """tests/cpp/mma3_gpu.cpp: the reference's test_MMA_3 loop on the mirrored API with the
    reference's MMA constructor (two constraints, per-variable bounds) prints the reference's
    iterates to their 6 digits."""
    import subprocess
    from pansfem2_gb300 import _lib
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path / "mma3_gpu")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(root, "include"),
                    os.path.join(root, "tests", "cpp", "mma3_gpu.cpp"), "-o", exe,
                    "-L", libdir, "-lpansfem2_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    got = [list(map(float, l.split("\t")[1:3])) for l in out.splitlines() if l.startswith("k = ")]
    ref = [list(map(float, re.findall(r"[-+0-9.e]+", line.split("Constraints1:")[1])[1:]))
           for line in open(os.path.join(GOLDEN, "ref_test_MMA_3.txt")) if line.startswith("k = ")]
    assert len(got) == len(ref)
    assert np.allclose(got, ref, rtol=1e-5, atol=1e-6)
