"""The Alveo host-format interchange (gbilu_fpga_layout / _pack /
gbilu_status_lines) against the reference's own host library.

oracle/ref/Makefile compiles fpga_functions_bicgstab.cpp, bicgstab_utils.cpp
and bda_utils.cpp unmodified from the reference tree (with a stub OpenCL
header) into oracle/_ref/libfpgaref.so; these CPU tests compare the GB300
library's output with it byte for byte. They skip where neither the built
checker nor the reference tree is present.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from fpga_gb300 import load, native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libfpgaref.so")
# the reference tree (read only to build the checker); GBILU_REFERENCE_ROOT
# overrides where it is
REFERENCE_ROOT = os.environ.get("GBILU_REFERENCE_ROOT", "/root/reference")
REFERENCE = os.path.join(REFERENCE_ROOT, "linearalgebra/ilu0bicgstab/xilinx/src/sda_app")

I32P = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
U64P = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
U32P = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
I64P = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")


@pytest.fixture(scope="module")
def ref():
    if os.path.isdir(REFERENCE):
        subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"),
                               f"REF={REFERENCE}"])
    elif not os.path.exists(REF_SO):
        pytest.skip("reference host library not built and reference tree absent")
    L = C.CDLL(REF_SO)
    L.ref_setup_layout.argtypes = [C.c_int, C.c_uint, I32P, I32P, C.c_uint, U64P, U32P, I64P, U32P]
    L.ref_pack.argtypes = [C.c_uint, I32P, I32P, C.c_void_p, I32P, C.c_int, C.c_void_p]
    L.ref_decode.argtypes = [U64P, C.c_uint, C.POINTER(C.c_uint), C.POINTER(C.c_uint),
                             np.ctypeslib.ndpointer(np.float64), C.POINTER(C.c_ubyte), I32P]
    return L


@pytest.fixture(scope="module")
def gb(built_lib):
    L = load()
    L.gbilu_fpga_layout.argtypes = [C.c_uint, I32P, I32P, C.c_uint, U64P, U32P, I64P, U32P]
    L.gbilu_fpga_pack.argtypes = [C.c_uint, I32P, I32P, C.c_void_p, I32P, C.c_int, C.c_void_p]
    L.gbilu_status_lines.argtypes = [C.POINTER(native.Result), U64P, C.c_int]
    return L


def size_sets():
    rng = np.random.default_rng(0)
    yield np.array([4000, 26400, 2, 4016, 26560, 12000, 4000, 11200, 2, 2016, 11264, 12000,
                    4000, 11200, 2, 2016, 11264, 12000], np.int32), np.array([26400, 11200, 11200], np.int32)
    for _ in range(6):
        ps = rng.integers(1, 200000, 18).astype(np.int32)
        ps[[2, 8, 14]] = rng.integers(1, 256, 3)
        yield ps, rng.integers(1, 400000, 3).astype(np.int32)


def test_layout_matches_reference(ref, gb):
    for cfg_bits in (0, 2, 3):
        for ps, nz in size_sets():
            out = {}
            for name, L, f in (("ref", ref, ref.ref_setup_layout), ("gb", gb, gb.gbilu_fpga_layout)):
                setup = np.zeros(40, np.uint64)
                tot = np.zeros(5, np.uint32)
                offs = np.zeros(23, np.int64)
                ro = np.zeros(6, np.uint32)
                if name == "ref":
                    rc = f(0, cfg_bits, ps, nz, 64 * 16, setup, tot, offs, ro)
                else:
                    rc = f(cfg_bits, ps, nz, 64 * 16, setup, tot, offs, ro)
                assert rc == 0
                out[name] = (setup, tot, offs, ro)
            for a, b in zip(out["ref"], out["gb"]):
                assert np.array_equal(a, b)


def test_layout_rejects_partial_debug_line(ref, gb):
    ps, nz = next(size_sets())
    args = (np.zeros(40, np.uint64), np.zeros(5, np.uint32), np.zeros(23, np.int64), np.zeros(6, np.uint32))
    assert ref.ref_setup_layout(0, 0, ps, nz, 100, *args) == 1
    assert gb.gbilu_fpga_layout(0, ps, nz, 100, *args) == native.BAD_INPUT


def vector_pointers(ps, nz, rng):
    """Synthetic backend arrays of the sizes in ps (contents are arbitrary:
    the packer copies them)."""
    keep = []

    def arr(a):
        a = np.ascontiguousarray(a)
        keep.append(a)
        return a.ctypes.data

    vp = (C.c_void_p * 21)()
    for m, base in ((0, 0), (1, 6), (2, 12)):
        ncol = int(ps[base + 2])
        vp[base + 0] = arr(rng.integers(0, 2**31, 8 + 4 * ncol).astype(np.int32))
        vp[base + 1] = arr(rng.integers(0, 2**31, ps[base + 3]).astype(np.int32))
        vals = arr(rng.standard_normal(nz[m]))
        ptrs = (C.c_void_p * 1)(vals)
        keep.append(ptrs)
        vp[base + 2] = C.cast(ptrs, C.c_void_p).value
        vp[base + 3] = arr(rng.integers(0, 2**16, ps[base + 1]).astype(np.uint16))
        vp[base + 4] = arr(rng.integers(0, 256, ps[base + 4]).astype(np.uint8))
    vp[18] = arr(rng.standard_normal(ps[5]))
    vp[19] = arr(rng.standard_normal(ps[0]))
    vp[20] = arr(rng.standard_normal(ps[0]))
    return vp, keep


def test_pack_matches_reference(ref, gb):
    rng = np.random.default_rng(1)
    for ps, nz in list(size_sets())[:4]:
        ps = np.minimum(ps, 60000).astype(np.int32)
        nz = np.minimum(nz, 80000).astype(np.int32)
        vp, keep = vector_pointers(ps, nz, rng)
        tot = np.zeros(5, np.uint32)
        gb.gbilu_fpga_layout(0, ps, nz, 64, np.zeros(40, np.uint64), tot, np.zeros(23, np.int64),
                             np.zeros(6, np.uint32))
        for fill in (0, 1):
            banks = {k: [np.full(int(t), 0xAB, np.uint8) for t in tot] for k in ("ref", "gb")}
            ptrs = {k: (C.c_void_p * 5)(*[b.ctypes.data for b in banks[k]]) for k in banks}
            assert ref.ref_pack(2, ps, nz, C.cast(vp, C.c_void_p), ps, fill, C.cast(ptrs["ref"], C.c_void_p)) == 0
            assert gb.gbilu_fpga_pack(2, ps, nz, C.cast(vp, C.c_void_p), ps, fill, C.cast(ptrs["gb"], C.c_void_p)) == 0
            for b in range(5):
                assert np.array_equal(banks["ref"][b], banks["gb"][b]), (b, fill)


@pytest.mark.parametrize("status,half", [(0, 7), (0, 10), (1, 400), (2, -1), (5, 33)])
def test_status_lines_decoded_by_reference(ref, gb, status, half):
    r = native.Result()
    r.status = status
    r.half_iters = half
    r.device_ms = 2.5
    norms = [109.6, 1.49, 1.07, 2.45]
    for i in range(4):
        r.norms[i] = norms[i]
    lines = 8
    buf = np.zeros(lines * 8, np.uint64)
    assert gb.gbilu_status_lines(C.byref(r), buf, lines) == 0
    cyc, it = C.c_uint(), C.c_uint()
    out_norms = np.zeros(4)
    last = C.c_ubyte()
    flags = np.zeros(6, np.int32)
    rc = ref.ref_decode(buf, lines, C.byref(cyc), C.byref(it), out_norms, C.byref(last), flags)
    aborted, signature_err, overflow, noresults, wrafter, fifofull = flags
    assert signature_err == 0 and overflow == 0 and wrafter == 0 and fifofull == 0
    assert aborted == (status == 5) and rc == (1 if status == 5 else 0)
    assert noresults == (status == 2)
    if status != 5:
        assert cyc.value == 2500000
    assert it.value == (half & 0xFFFF)
    assert np.array_equal(out_norms, norms)
    assert last.value == ((half & 0xFFFF) % 3) + 1
