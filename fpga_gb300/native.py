"""ctypes binding of libgbilu.so (the C ABI declared in include/gbilu.h).

There is no fallback: if the library is missing or fails to load, every call
raises. Build it with ``fpga_gb300.build.build_library()`` (or
``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

from .build import LIB, ROOT

HEADER = os.path.join(ROOT, "include", "gbilu.h")

OK, MAXIT, ALREADY_CONVERGED, BREAKDOWN, NONFINITE, TIMEOUT = 0, 1, 2, 3, 4, 5
BAD_INPUT, SINGULAR, CUDA_ERROR, NOT_READY, NO_DEVICE = 6, 7, 8, 9, 10
FP64, MIXED = 0, 1


class Options(C.Structure):
    _fields_ = [("precision", C.c_int), ("absolute_tol", C.c_int), ("device", C.c_int),
                ("use_graph", C.c_int), ("timeout_ms", C.c_double),
                ("inner_tol", C.c_double), ("inner_maxit", C.c_int),
                ("max_outer", C.c_int), ("verbose", C.c_int), ("sweep_mode", C.c_int),
                ("factor_on_device", C.c_int), ("mixed_scheme", C.c_int),
                ("ru_delta", C.c_double), ("stage_small_steps", C.c_int),
                ("coloring", C.c_int), ("stream_large_steps", C.c_int),
                ("color_on_device", C.c_int)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int), ("half_iters", C.c_int), ("iterations", C.c_double),
                ("norm0", C.c_double), ("norm", C.c_double), ("relres", C.c_double),
                ("norms", C.c_double * 4), ("last_norm_idx", C.c_int),
                ("outer_iters", C.c_int), ("inner_half_iters", C.c_int),
                ("true_relres", C.c_double), ("device_ms", C.c_double),
                ("total_ms", C.c_double)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["norms"] = list(self.norms)
        return d


class Stats(C.Structure):
    _fields_ = [("nb", C.c_int), ("nnzb", C.c_int), ("ncolors", C.c_int),
                ("nnzb_lower", C.c_int), ("nnzb_upper", C.c_int), ("slices", C.c_int),
                ("slots_a", C.c_longlong), ("slots_l", C.c_longlong),
                ("slots_u", C.c_longlong), ("device_bytes", C.c_longlong),
                ("launches_per_iter", C.c_int), ("last_launches", C.c_longlong),
                ("factor_ms", C.c_double), ("analyze_ms", C.c_double),
                ("alg_bytes_spmv", C.c_double * 2), ("alg_bytes_ilu", C.c_double * 2),
                ("alg_bytes_iter", C.c_double * 2), ("ring_stages", C.c_int * 2),
                ("ring_stage_bytes", C.c_int * 2), ("apply_smem_bytes", C.c_int * 2),
                ("color_ms", C.c_double), ("color_on_device", C.c_int)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        for k in ("alg_bytes_spmv", "alg_bytes_ilu", "alg_bytes_iter", "ring_stages",
                  "ring_stage_bytes", "apply_smem_bytes"):
            d[k] = list(d[k])
        return d


class GbIluError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gbilu error {code}: {msg}")
        self.code = code


_lib = None
I32P = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
F64P = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
VP = C.c_void_p


def declared_symbols():
    """Function names declared in include/gbilu.h."""
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(r"^(?:int|const char \*)\s*(gbilu_\w+)\s*\(", text, re.M)))


def load():
    """Loads libgbilu.so; raises if it is absent (there is no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        raise RuntimeError(f"{LIB} is missing: build it with fpga_gb300.build.build_library()")
    L = C.CDLL(LIB)
    L.gbilu_default_options.argtypes = [C.POINTER(Options)]
    L.gbilu_create.argtypes = [C.POINTER(Options), C.POINTER(VP)]
    L.gbilu_destroy.argtypes = [VP]
    L.gbilu_analyze.argtypes = [VP, C.c_int, I32P, I32P]
    L.gbilu_get_ordering.argtypes = [VP, C.POINTER(C.c_int), VP, VP, VP]
    L.gbilu_device_order.argtypes = [VP, VP]
    L.gbilu_wait_probe.argtypes = [VP, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_double)]
    L.gbilu_factor.argtypes = [VP, F64P]
    L.gbilu_get_factors.argtypes = [VP, VP, VP]
    L.gbilu_solve.argtypes = [VP, VP, VP, C.c_double, C.c_int, C.POINTER(Result)]
    L.gbilu_solve_device.argtypes = [VP, VP, VP, C.c_double, C.c_int, C.POINTER(Result)]
    L.gbilu_apply_spmv.argtypes = [VP, F64P, F64P, C.c_int]
    L.gbilu_apply_ilu.argtypes = [VP, F64P, F64P, C.c_int]
    L.gbilu_adjoint.argtypes = [VP, F64P, F64P, F64P, VP, C.c_double, C.c_int,
                                C.POINTER(Result)]
    L.gbilu_adjoint_device.argtypes = [VP, VP, VP, VP, VP, C.c_double, C.c_int,
                                       C.POINTER(Result)]
    L.gbilu_dot_check.argtypes = [VP, C.c_int, VP, VP, C.POINTER(C.c_double),
                                  C.POINTER(C.c_double)]
    L.gbilu_fpga_export.argtypes = [VP, VP, VP, VP, VP, VP]
    L.gbilu_get_stats.argtypes = [VP, C.POINTER(Stats)]
    L.gbilu_bench_kernel.argtypes = [VP, C.c_int, C.c_int, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), C.POINTER(C.c_int)]
    L.gbilu_ilu_trace.argtypes = [VP, C.c_int, C.c_int, VP, VP, C.c_int, C.POINTER(C.c_int)]
    L.gbilu_schedule.argtypes = [VP, C.c_int, C.c_int, C.POINTER(C.c_int), VP]
    L.gbilu_status_string.argtypes = [C.c_int]
    L.gbilu_status_string.restype = C.c_char_p
    L.gbilu_last_error.argtypes = [VP]
    L.gbilu_last_error.restype = C.c_char_p
    _lib = L
    return L


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class GbIlu:
    """One solver handle: analyze a pattern once, factor values, solve.

    Mirrors the C ABI one to one; every failure raises GbIluError carrying
    the library's status code and message.
    """

    def __init__(self, precision="fp64", device=0, use_graph=True, absolute=False,
                 timeout_ms=0.0, inner_tol=1e-1, inner_maxit=500, max_outer=30,
                 verbose=0, sweep_mode=1, factor_on_device=False, mixed_scheme=0,
                 ru_delta=0.1, stage_small_steps=True, coloring="parity",
                 stream_large_steps=False, color_on_device=False):
        self.L = load()
        o = Options()
        self.L.gbilu_default_options(C.byref(o))
        o.precision = MIXED if precision == "mixed" else FP64
        o.device = device
        o.use_graph = int(use_graph)
        o.absolute_tol = int(absolute)
        o.timeout_ms = timeout_ms
        o.inner_tol = inner_tol
        o.inner_maxit = inner_maxit
        o.max_outer = max_outer
        o.verbose = verbose
        o.sweep_mode = sweep_mode
        o.factor_on_device = int(factor_on_device)
        o.mixed_scheme = mixed_scheme
        o.ru_delta = ru_delta
        o.stage_small_steps = int(stage_small_steps)
        o.coloring = {"parity": 0, "natural": 1}[coloring]
        o.stream_large_steps = int(stream_large_steps)
        o.color_on_device = int(color_on_device)
        self.h = VP()
        rc = self.L.gbilu_create(C.byref(o), C.byref(self.h))
        if rc:
            raise GbIluError(rc, "gbilu_create failed")
        self.nb = 0
        self.nnzb = 0

    def _check(self, rc):
        if rc:
            raise GbIluError(rc, self.L.gbilu_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.L.gbilu_destroy(self.h)
            self.h = VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # --- set-up
    def analyze(self, rowptr, colind):
        rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
        colind = np.ascontiguousarray(colind, dtype=np.int32)
        self.nb = rowptr.size - 1
        self.nnzb = int(rowptr[-1]) if rowptr.size else 0
        self._check(self.L.gbilu_analyze(self.h, self.nb, rowptr, colind))
        return self

    def factor(self, vals):
        v = _f64(vals).reshape(-1)
        if self.nb and v.size != 9 * self.nnzb:
            raise ValueError("vals must hold nnzb*9 doubles")
        self._check(self.L.gbilu_factor(self.h, v))
        return self

    def ordering(self):
        nc = C.c_int()
        self._check(self.L.gbilu_get_ordering(self.h, C.byref(nc), None, None, None))
        color = np.empty(self.nb, np.int32)
        perm = np.empty(self.nb, np.int32)
        cp = np.empty(nc.value + 1, np.int32)
        self._check(self.L.gbilu_get_ordering(self.h, C.byref(nc), color.ctypes.data,
                                              perm.ctypes.data, cp.ctypes.data))
        return nc.value, color, perm, cp

    def wait_probe(self, mode):
        """Runs a device wait that never completes (0: grid barrier, 1: data
        wait) and returns what its bounded timeout reported."""
        bf, st, ms = C.c_int(), C.c_int(), C.c_double()
        self._check(self.L.gbilu_wait_probe(self.h, int(mode), C.byref(bf), C.byref(st),
                                            C.byref(ms)))
        return {"bar_fail": bf.value, "status": st.value, "ms": ms.value}

    def device_order(self):
        """Input row held at each device row (the numbering of the device
        vectors and sliced layouts)."""
        order = np.empty(self.nb, np.int32)
        self._check(self.L.gbilu_device_order(self.h, order.ctypes.data))
        return order

    def factors(self):
        lu = np.empty(9 * self.nnzb)
        dinv = np.empty(9 * self.nb)
        self._check(self.L.gbilu_get_factors(self.h, lu.ctypes.data, dinv.ctypes.data))
        return lu, dinv

    # --- compute
    def solve(self, b, x0=None, tol=1e-2, maxit=200):
        b = _f64(b)
        x = np.zeros(3 * self.nb) if x0 is None else _f64(x0).copy()
        res = Result()
        self._check(self.L.gbilu_solve(self.h, b.ctypes.data, x.ctypes.data, tol, maxit,
                                       C.byref(res)))
        return x, res

    def solve_device(self, b_ptr, x_ptr, tol=1e-2, maxit=200):
        """b_ptr/x_ptr: device addresses (e.g. torch tensor .data_ptr())."""
        res = Result()
        self._check(self.L.gbilu_solve_device(self.h, VP(b_ptr), VP(x_ptr), tol, maxit,
                                              C.byref(res)))
        return res

    def solve_host_ptr(self, b_ptr, x_ptr, tol=1e-2, maxit=200):
        """As solve() on caller-owned (e.g. pinned) host buffers given by address."""
        res = Result()
        self._check(self.L.gbilu_solve(self.h, VP(b_ptr), VP(x_ptr), tol, maxit,
                                       C.byref(res)))
        return res

    def spmv(self, x, transpose=False):
        y = np.empty(3 * self.nb)
        self._check(self.L.gbilu_apply_spmv(self.h, _f64(x), y, int(transpose)))
        return y

    def ilu_apply(self, p, transpose=False):
        z = np.empty(3 * self.nb)
        self._check(self.L.gbilu_apply_ilu(self.h, _f64(p), z, int(transpose)))
        return z

    def adjoint(self, g, x, tol=1e-10, maxit=2000, want_dA=True):
        lam = np.empty(3 * self.nb)
        dA = np.empty(9 * self.nnzb) if want_dA else None
        res = Result()
        self._check(self.L.gbilu_adjoint(self.h, _f64(g), _f64(x), lam,
                                         dA.ctypes.data if want_dA else None, tol, maxit,
                                         C.byref(res)))
        return lam, (dA.reshape(-1, 3, 3) if want_dA else None), res

    def adjoint_device(self, g_ptr, x_ptr, lam_ptr, dA_ptr=None, tol=1e-10, maxit=2000):
        """As adjoint() on device arrays given by address (dA_ptr may be None)."""
        res = Result()
        self._check(self.L.gbilu_adjoint_device(self.h, VP(g_ptr), VP(x_ptr), VP(lam_ptr),
                                                VP(dA_ptr) if dA_ptr else None, tol, maxit,
                                                C.byref(res)))
        return res

    def dot_check(self, x, y):
        """(x, y) of two float32 vectors on the device: (double-float
        accumulation as in the mixed solve, FP64 accumulation)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        a, b = C.c_double(), C.c_double()
        self._check(self.L.gbilu_dot_check(self.h, x.size, x.ctypes.data, y.ctypes.data,
                                           C.byref(a), C.byref(b)))
        return a.value, b.value

    def fpga_export(self, b=None, x0=None):
        """The system as the Alveo kernel's input arrays (gbilu_fpga_export):
        a dict with vector_sizes[18], nnz_sizes[3] and per matrix A, L, U
        the color sizes (8-word header + 4 per part), P indices, values,
        column indices, new-row offsets; the block diagonal, rhs and x0
        (permuted); and 'pointers', the 21 vectorPointers (kept alive with
        the arrays)."""
        vs = np.zeros(18, np.int32)
        nz = np.zeros(3, np.int32)
        self._check(self.L.gbilu_fpga_export(self.h, None, None, vs.ctypes.data, nz.ctypes.data,
                                             None))
        out = {"vector_sizes": vs, "nnz_sizes": nz}
        vp = (C.c_void_p * 21)()
        keep = []
        for m, name in enumerate("ALU"):
            base = 6 * m
            arrs = {"sizes": np.zeros(8 + 4 * int(vs[base + 2]), np.uint32),
                    "pidx": np.zeros(int(vs[base + 3]), np.uint32),
                    "vals": np.zeros(int(nz[m]), np.float64),
                    "cols": np.zeros(int(vs[base + 1]), np.uint16),
                    "nrs": np.zeros(int(vs[base + 4]), np.uint8)}
            vptr = (C.c_void_p * 1)(arrs["vals"].ctypes.data)
            keep.append(vptr)
            vp[base + 0] = arrs["sizes"].ctypes.data
            vp[base + 1] = arrs["pidx"].ctypes.data
            vp[base + 2] = C.cast(vptr, C.c_void_p).value
            vp[base + 3] = arrs["cols"].ctypes.data
            vp[base + 4] = arrs["nrs"].ctypes.data
            out[name] = arrs
        n = int(vs[0])
        out["blkdiag"] = np.zeros(int(vs[5]), np.float64)
        out["rhs"] = np.zeros(n)
        out["x0"] = np.zeros(n)
        vp[18] = out["blkdiag"].ctypes.data
        vp[19] = out["rhs"].ctypes.data
        vp[20] = out["x0"].ctypes.data
        bb = None if b is None else _f64(b)
        xx = None if x0 is None else _f64(x0)
        self._check(self.L.gbilu_fpga_export(self.h, None if bb is None else bb.ctypes.data,
                                             None if xx is None else xx.ctypes.data,
                                             vs.ctypes.data, nz.ctypes.data, vp))
        out["pointers"] = vp
        out["_keep"] = keep
        return out

    def stats(self):
        s = Stats()
        self._check(self.L.gbilu_get_stats(self.h, C.byref(s)))
        return s.as_dict()

    KERNELS = {"spmv64": 0, "ilu64": 1, "spmv32": 2, "ilu32": 3,
               "spmv_alpha64": 4, "spmv_omega64": 5, "update_s64": 6, "update_r64": 7,
               "update_p64": 8, "spmv_alpha32": 9, "spmv_omega32": 10, "update_s32": 11,
               "update_r32": 12, "update_p32": 13}

    def ilu_trace(self, fp32=False, transpose=False):
        """[(rows, microseconds)] per color step of one single-launch ILU apply."""
        us = np.zeros(96)
        rows = np.zeros(96, np.int32)
        n = C.c_int()
        self._check(self.L.gbilu_ilu_trace(self.h, int(fp32), int(transpose), us.ctypes.data,
                                           rows.ctypes.data, 96, C.byref(n)))
        return [(int(rows[i]), float(us[i])) for i in range(n.value)]

    SCHEDULE_FIELDS = ("row0", "nrows", "slice0", "lane0", "mat", "has_d", "own_y", "nbr_hat",
                       "src_rows", "to_y", "final0", "final_d", "barrier_after")

    def schedule(self, transpose=False):
        """Steps of the single-launch ILU apply: a list of dicts (SCHEDULE_FIELDS)."""
        n = C.c_int()
        self._check(self.L.gbilu_schedule(self.h, int(transpose), 0, C.byref(n), None))
        buf = np.zeros(13 * max(n.value, 1), np.int32)
        self._check(self.L.gbilu_schedule(self.h, int(transpose), n.value, C.byref(n),
                                          buf.ctypes.data))
        return [dict(zip(self.SCHEDULE_FIELDS, map(int, buf[13 * q:13 * q + 13])))
                for q in range(n.value)]

    def bench_kernel(self, which, reps=20):
        """(avg ms, algorithmic bytes, launches) per application of a kernel family."""
        ms, by, la = C.c_double(), C.c_double(), C.c_int()
        self._check(self.L.gbilu_bench_kernel(self.h, self.KERNELS[which], reps, C.byref(ms),
                                               C.byref(by), C.byref(la)))
        return ms.value, by.value, la.value


def status_string(code):
    return load().gbilu_status_string(code).decode()
