"""The C++ bridge of include/gbilu_bridge.hpp, driven by tests/bridge_driver.cpp
as a simulator backend would use it: the pattern is analyzed once and only
re-analyzed when it changes; every call refactors; solves match the oracle."""
import os
import subprocess

import numpy as np
import pytest

from fpga_gb300.build import LIBDIR, ROOT
from fpga_gb300.synth import make_config
from oracle_lib import Prepared

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def driver(built_lib, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("bridge") / "bridge_driver")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "bridge_driver.cpp"), "-o", exe, "-L", LIBDIR, "-lgbilu",
                    "-Wl,-rpath," + LIBDIR], check=True)
    return exe


def run_driver(exe, tmp_path, s, device, precision=0, tol=1e-6, maxit=500):
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(fin, "wb") as f:
        np.array([s.nb, s.nnzb, precision], np.int32).tofile(f)
        np.asarray(s.rowptr, np.int32).tofile(f)
        np.asarray(s.colind, np.int32).tofile(f)
        np.asarray(s.vals, np.float64).reshape(-1).tofile(f)
        np.asarray(s.b, np.float64).tofile(f)
        np.array([tol], np.float64).tofile(f)
        np.array([maxit], np.int32).tofile(f)
    subprocess.run([exe, fin, fout, str(device)], check=True)
    raw = open(fout, "rb").read()
    head = np.frombuffer(raw, np.int32, 6)
    off = 24
    res = []
    for _ in range(2):
        iv = np.frombuffer(raw, np.int32, 4, off)
        red = np.frombuffer(raw, np.float64, 1, off + 16)[0]
        res.append(dict(iterations=int(iv[0]), half_iters=int(iv[1]), converged=bool(iv[2]),
                        status=int(iv[3]), reduction=float(red)))
        off += 24
    n = 3 * s.nb
    x1 = np.frombuffer(raw, np.float64, n, off)
    x2 = np.frombuffer(raw, np.float64, n, off + 8 * n)
    return head, res, x1, x2


def test_bridge_reanalyzes_only_on_new_pattern(driver, tmp_path):
    s = make_config("c1_20x20x10")
    head, _, _, _ = run_driver(driver, tmp_path, s, device=-1)
    st1, st2, st3, an2, fa2, an3 = (int(v) for v in head)
    assert (st1, st2, st3) == (0, 0, 0)       # SolverStatus::Success
    assert an2 == 1 and fa2 == 2              # one analysis, two factorizations
    assert an3 == 2                           # the changed pattern was analyzed


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_bridge_solves_match_oracle(driver, tmp_path, precision):
    s = make_config("c1_20x20x10")
    tol = 1e-8 if precision else 1e-6
    head, res, x1, x2 = run_driver(driver, tmp_path, s, device=0, precision=precision, tol=tol)
    assert tuple(int(v) for v in head[:3]) == (0, 0, 0)
    assert int(head[3]) == 1 and int(head[4]) == 2
    P = Prepared(s)
    x_ref, r_ref = P.solve(s.b, tol=tol, maxit=500)
    assert res[0]["converged"] and res[1]["converged"]
    assert np.linalg.norm(x1 - x_ref) <= 1e-6 * np.linalg.norm(x_ref)
    if precision == 0:
        assert res[0]["half_iters"] == r_ref.half_iters
    # step 2 solved 1.5 A x = b on the same pattern
    assert np.linalg.norm(x2 - x_ref / 1.5) <= 1e-6 * np.linalg.norm(x_ref)
    A = s.to_scipy()
    for x, r in ((x1, res[0]), (x2, res[1])):
        scale = 1.0 if x is x1 else 1.5
        rel = np.linalg.norm(s.b - scale * (A @ x)) / np.linalg.norm(s.b)
        assert rel <= tol * (1 + 1e-6) and abs(rel - r["reduction"]) <= 1e-3 * tol


@pytest.mark.gpu
@pytest.mark.parametrize("maxit", [0, 2, 5])
def test_bridge_mixed_honours_maxit(driver, tmp_path, maxit):
    """A simulator backend's iteration limit bounds a mixed-precision solve:
    the FP32 inner half-iterations of all refinement steps stop at
    2*maxit + 1, and the result reports MAXIT (not converged)."""
    s = make_config("c1_20x20x10")
    head, res, x1, _ = run_driver(driver, tmp_path, s, device=0, precision=1, tol=1e-13,
                                  maxit=maxit)
    assert tuple(int(v) for v in head[:3]) == (0, 0, 0)
    for r in res:
        assert r["status"] == 1 and not r["converged"]
        assert r["half_iters"] == 2 * maxit
    A = s.to_scipy()
    rel = np.linalg.norm(s.b - A @ x1) / np.linalg.norm(s.b)
    assert abs(rel - res[0]["reduction"]) <= 1e-6 * rel
