"""ctypes binding of the CPU oracle (oracle/gbilu_oracle.c) for the tests.

The oracle is the checker: tests compare the CUDA path (called through the
C-ABI library) against these functions on the same seeded inputs.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "_build", "liboracle.so")

_lib = None

I32P = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
F64P = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


class OrcResult(C.Structure):
    _fields_ = [("status", C.c_int), ("half_iters", C.c_int),
                ("norm0", C.c_double), ("norm", C.c_double),
                ("relres", C.c_double), ("norms", C.c_double * 4),
                ("last_norm_idx", C.c_int), ("nhist", C.c_int)]


def lib():
    global _lib
    if _lib is None:
        src = os.path.join(ORACLE_DIR, "gbilu_oracle.c")
        if (not os.path.exists(ORACLE_SO)
                or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src)):
            subprocess.check_call(["make", "-s", "-C", ORACLE_DIR])
        L = C.CDLL(ORACLE_SO)
        L.orc_color_greedy.argtypes = [C.c_int, I32P, I32P, I32P]
        L.orc_color_greedy.restype = C.c_int
        L.orc_color_parity.argtypes = [C.c_int, I32P, I32P, I32P]
        L.orc_color_parity.restype = C.c_int
        L.orc_color_order.argtypes = [C.c_int, I32P, I32P, I32P, C.c_int, I32P, I32P,
                                      I32P]
        L.orc_permute_bsr.argtypes = [C.c_int, I32P, I32P, F64P, I32P, I32P,
                                      I32P, F64P, I32P]
        L.orc_bilu0.argtypes = [C.c_int, I32P, I32P, F64P, F64P]
        L.orc_bilu0.restype = C.c_int
        L.orc_inv3.argtypes = [F64P, F64P]
        L.orc_inv3.restype = C.c_int
        for f in (L.orc_spmv, L.orc_spmv_t):
            f.argtypes = [C.c_int, I32P, I32P, F64P, F64P, F64P]
        for f in (L.orc_ilu_apply, L.orc_ilu_apply_t):
            f.argtypes = [C.c_int, I32P, I32P, F64P, F64P, F64P, F64P]
        L.orc_bicgstab.argtypes = [C.c_int, I32P, I32P, F64P, F64P, F64P, F64P,
                                   F64P, C.c_double, C.c_int, C.c_int, C.c_int,
                                   C.POINTER(OrcResult), C.c_void_p, C.c_int]
        L.orc_bicgstab.restype = C.c_int
        L.orc_grad_a.argtypes = [C.c_int, I32P, I32P, F64P, F64P, F64P]
        L.orc_bicgstab_omp.argtypes = [C.c_int, C.c_int, I32P, I32P, I32P, F64P,
                                       F64P, F64P, F64P, F64P, C.c_double,
                                       C.c_int, C.c_int, C.c_int,
                                       C.POINTER(OrcResult)]
        L.orc_bicgstab_omp.restype = C.c_int
        L.orc_bicgstab_omp_t.argtypes = L.orc_bicgstab_omp.argtypes
        L.orc_bicgstab_omp_t.restype = C.c_int
        L.orc_transpose_bsr.argtypes = [C.c_int, I32P, I32P, F64P, I32P, I32P, F64P]
        L.orc_mixed_ir.argtypes = [C.c_int, I32P, I32P, F64P, F64P, F64P, F64P,
                                   F64P, C.c_double, C.c_double, C.c_int, C.c_int,
                                   C.POINTER(OrcResult), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int)]
        L.orc_mixed_ir.restype = C.c_int
        _lib = L
    return _lib


class Prepared:
    """Colored, permuted and factored copy of a BlockSystem (oracle side)."""

    def __init__(self, sysm, coloring="parity"):
        L = lib()
        self.sys = sysm
        nb = sysm.nb
        self.nb = nb
        rp = np.ascontiguousarray(sysm.rowptr, dtype=np.int32)
        ci = np.ascontiguousarray(sysm.colind, dtype=np.int32)
        self.color = np.empty(nb, np.int32)
        color_fn = {"parity": L.orc_color_parity, "natural": L.orc_color_greedy}[coloring]
        self.ncolors = color_fn(nb, rp, ci, self.color)
        self.perm = np.empty(nb, np.int32)
        self.color_ptr = np.empty(self.ncolors + 1, np.int32)
        self.split = np.empty(self.ncolors, np.int32)
        L.orc_color_order(nb, rp, ci, self.color, self.ncolors, self.perm, self.color_ptr,
                          self.split)
        self.iperm = np.empty(nb, np.int32)
        self.iperm[self.perm] = np.arange(nb, dtype=np.int32)
        nnzb = int(rp[-1])
        self.rowptr = np.empty(nb + 1, np.int32)
        self.colind = np.empty(nnzb, np.int32)
        self.avals = np.empty(nnzb * 9, np.float64)
        self.src = np.empty(nnzb, np.int32)
        L.orc_permute_bsr(nb, rp, ci, np.ascontiguousarray(sysm.vals.reshape(-1)),
                          self.perm, self.rowptr, self.colind, self.avals, self.src)
        self.lu = self.avals.copy()
        self.dinv = np.empty(nb * 9, np.float64)
        self.ilu_status = L.orc_bilu0(nb, self.rowptr, self.colind, self.lu, self.dinv)
        # vector permutation helpers (3 unknowns per block row)
        self.vperm = (3 * self.perm[:, None] + np.arange(3)).reshape(-1)

    def to_perm(self, v):
        return np.ascontiguousarray(np.asarray(v, np.float64)[self.vperm])

    def from_perm(self, v):
        out = np.empty_like(v)
        out[self.vperm] = v
        return out

    # operators in the ORIGINAL numbering
    def spmv(self, x, transpose=False):
        y = np.empty(3 * self.nb)
        f = lib().orc_spmv_t if transpose else lib().orc_spmv
        f(self.nb, self.rowptr, self.colind, self.avals, self.to_perm(x), y)
        return self.from_perm(y)

    def ilu_apply(self, p, transpose=False):
        z = np.empty(3 * self.nb)
        f = lib().orc_ilu_apply_t if transpose else lib().orc_ilu_apply
        f(self.nb, self.rowptr, self.colind, self.lu, self.dinv, self.to_perm(p), z)
        return self.from_perm(z)

    def solve(self, b, x0=None, tol=1e-2, maxit=200, absolute=False,
              transpose=False, hist_cap=0):
        x = self.to_perm(np.zeros(3 * self.nb) if x0 is None else x0)
        res = OrcResult()
        hist = np.zeros(max(hist_cap, 1))
        lib().orc_bicgstab(self.nb, self.rowptr, self.colind, self.avals, self.lu,
                           self.dinv, self.to_perm(b), x, tol, int(absolute), maxit,
                           int(transpose), C.byref(res),
                           hist.ctypes.data if hist_cap else None, hist_cap)
        out = self.from_perm(x)
        if hist_cap:
            return out, res, hist[:min(res.nhist, hist_cap)]
        return out, res

    def transposes(self):
        """Explicit transposes of A and of the factored matrix (cached)."""
        if not hasattr(self, "_t"):
            nnz = self.colind.size
            t = []
            for v in (self.avals, self.lu):
                rp, ci, tv = np.empty(self.nb + 1, np.int32), np.empty(nnz, np.int32), \
                    np.empty(nnz * 9)
                lib().orc_transpose_bsr(self.nb, self.rowptr, self.colind, v, rp, ci, tv)
                t.append((rp, ci, tv))
            self._t = t
        return self._t

    def solve_omp(self, b, tol=1e-2, maxit=200, nthreads=0, transpose=False):
        x = np.zeros(3 * self.nb)
        res = OrcResult()
        if transpose:
            (rp, ci, ta), (_, _, tlu) = self.transposes()
            lib().orc_bicgstab_omp_t(self.nb, self.ncolors, self.color_ptr, rp, ci, ta, tlu,
                                     self.dinv, self.to_perm(b), x, tol, 0, maxit, nthreads,
                                     C.byref(res))
        else:
            lib().orc_bicgstab_omp(self.nb, self.ncolors, self.color_ptr, self.rowptr,
                                   self.colind, self.avals, self.lu, self.dinv,
                                   self.to_perm(b), x, tol, 0, maxit, nthreads,
                                   C.byref(res))
        return self.from_perm(x), res

    def mixed(self, b, tol=1e-8, inner_tol=1e-4, inner_maxit=500, max_outer=20):
        x = np.zeros(3 * self.nb)
        res = OrcResult()
        outer, inner = C.c_int(), C.c_int()
        lib().orc_mixed_ir(self.nb, self.rowptr, self.colind, self.avals, self.lu,
                           self.dinv, self.to_perm(b), x, tol, inner_tol, inner_maxit,
                           max_outer, C.byref(res), C.byref(outer), C.byref(inner))
        return self.from_perm(x), res, outer.value, inner.value

    def grad_a(self, lam, x):
        """dA on the ORIGINAL pattern/order: block k of the input BSR."""
        dA = np.empty(self.avals.size)
        lib().orc_grad_a(self.nb, self.rowptr, self.colind, self.to_perm(lam),
                         self.to_perm(x), dA)
        out = np.empty_like(dA).reshape(-1, 9)
        out[self.src] = dA.reshape(-1, 9)
        return out.reshape(-1, 3, 3)
