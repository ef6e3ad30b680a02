"""include/gbilu.h from plain C: tests/c_abi_driver.c is compiled as strict
C99 (-pedantic -Werror, no C++ and no CUDA headers) and linked against
libgbilu.so, the way the reference's host code or an FFI binding would use
the boundary. On the CPU it drives a host-only handle (analysis, ordering,
schedule, host factorization, statistics, error reporting); on a GPU it
also solves, and the solution must match a dense solve and, bit for bit,
the same solve through the Python binding."""
import os
import subprocess

import numpy as np
import pytest

from fpga_gb300 import GbIlu, native
from fpga_gb300.build import LIBDIR, ROOT

HERE = os.path.dirname(os.path.abspath(__file__))
NB = 50


@pytest.fixture(scope="module")
def driver(built_lib, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("c_abi") / "c_abi_driver")
    subprocess.run(["gcc", "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-O2",
                    "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "c_abi_driver.c"),
                    "-o", exe, "-L", LIBDIR, "-lgbilu", "-Wl,-rpath," + LIBDIR], check=True)
    return exe


def run(exe, tmp_path, device):
    out = tmp_path / f"out{device}.txt"
    subprocess.run([exe, str(device), str(out)], check=True)
    lines = out.read_text().split("\n")
    head = {}
    rest = []
    for ln in lines:
        parts = ln.split()
        if parts and parts[0].isalpha() or (parts and "_" in parts[0]):
            head[parts[0]] = parts[1:]
        elif parts:
            rest.append(float(parts[0]))
    return head, np.array(rest)


def chain_system():
    """The driver's system, built the same way."""
    rowptr, colind, vals = [0], [], []
    for i in range(NB):
        for k in (i - 1, i, i + 1):
            if k < 0 or k >= NB:
                continue
            colind.append(k)
            blk = np.empty(9)
            for e in range(9):
                r, c = divmod(e, 3)
                v = -1.0 if r == c else 0.1 * ((r + 2 * c + i) % 3 - 1)
                if k == i:
                    v = 4.0 + 0.01 * (i % 5) if r == c else 0.2
                blk[e] = v
            vals.append(blk)
        rowptr.append(len(colind))
    b = 1.0 + (np.arange(3 * NB) % 7)
    return (np.array(rowptr, np.int32), np.array(colind, np.int32),
            np.array(vals).reshape(-1, 3, 3), b)


def test_c_client_host_only(driver, tmp_path):
    head, _ = run(driver, tmp_path, -1)
    assert int(head["bad_analyze"][0]) == native.BAD_INPUT and head["bad_analyze"][1] == "1"
    assert int(head["ncolors"][0]) == 2
    assert int(head["steps"][0]) >= 2
    rowptr, colind, _, _ = chain_system()
    assert [int(v) for v in head["stats"]] == [NB, len(colind), 2]
    assert int(head["host_solve"][0]) == native.NO_DEVICE


@pytest.mark.gpu
def test_c_client_solves(driver, tmp_path):
    head, x = run(driver, tmp_path, 0)
    status, half, relres = int(head["solve"][0]), int(head["solve"][1]), float(head["solve"][2])
    assert status == 0 and relres <= 1e-8 and x.size == 3 * NB
    rowptr, colind, vals, b = chain_system()
    A = np.zeros((3 * NB, 3 * NB))
    for i in range(NB):
        for k in range(rowptr[i], rowptr[i + 1]):
            j = colind[k]
            A[3 * i:3 * i + 3, 3 * j:3 * j + 3] = vals[k]
    x_dense = np.linalg.solve(A, b)
    assert np.linalg.norm(x - x_dense) <= 1e-6 * np.linalg.norm(x_dense)
    with GbIlu(device=0) as g:
        g.analyze(rowptr, colind).factor(vals)
        xp, r = g.solve(b, tol=1e-8, maxit=200)
    assert r.half_iters == half and np.array_equal(xp, x)
