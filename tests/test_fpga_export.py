"""gbilu_fpga_export: the analyzed and factored system as the Alveo
kernel's input arrays (the backend's vectorPointers), CPU only.

* The arrays pack byte for byte as the reference's own host library packs
  them (fpga_copy_host_datamem, built from the reference sources under
  oracle/_ref; skipped when neither it nor the reference tree is there) and
  as gbilu_fpga_pack does.
* A CPU model of the kernel's reading of those packed bytes, written from
  its RTL (oracle/fpga_rtl_model.py), reproduces the oracle's SpMV and ILU0
  apply to 1e-12.
* Every color the kernel sees stays within its limits, and systems beyond
  them are refused with the limit named.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from fpga_gb300 import GbIlu, GbIluError, load, native
from fpga_gb300.synth import generate, make_config
from oracle_lib import Prepared

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from fpga_rtl_model import PackedSystem  # noqa: E402

I32P = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
U64P = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
U32P = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
I64P = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")

REF_SO = os.path.join(ROOT, "oracle", "_ref", "libfpgaref.so")
REFERENCE_ROOT = os.environ.get("GBILU_REFERENCE_ROOT", "/root/reference")
REFERENCE = os.path.join(REFERENCE_ROOT, "linearalgebra/ilu0bicgstab/xilinx/src/sda_app")

SYSTEMS = {
    "c1": lambda: make_config("c1_20x20x10"),
    "faults": lambda: generate(16, 14, 8, sigma=1.5, inactive_frac=0.05, fault_frac=0.02, seed=3),
    "small": lambda: generate(6, 5, 4, sigma=1.0, seed=1),
}


@pytest.fixture(scope="module")
def gb(built_lib):
    L = load()
    L.gbilu_fpga_layout.argtypes = [C.c_uint, I32P, I32P, C.c_uint, U64P, U32P, I64P, U32P]
    L.gbilu_fpga_pack.argtypes = [C.c_uint, I32P, I32P, C.c_void_p, I32P, C.c_int, C.c_void_p]
    return L


def exported(name, coloring="parity"):
    s = SYSTEMS[name]()
    g = GbIlu(device=-1, coloring=coloring)
    g.analyze(s.rowptr, s.colind).factor(s.vals)
    ex = g.fpga_export(s.b)
    return s, g, ex


def pack(L, ex, fill=1):
    ps = np.ascontiguousarray(ex["vector_sizes"], np.int32)
    nz = np.ascontiguousarray(ex["nnz_sizes"], np.int32)
    setup = np.zeros(40, np.uint64)
    tot = np.zeros(5, np.uint32)
    offs = np.zeros(23, np.int64)
    ro = np.zeros(6, np.uint32)
    assert L.gbilu_fpga_layout(0, ps, nz, 64, setup, tot, offs, ro) == 0
    banks = [np.full(int(t), 0xAB, np.uint8) for t in tot]
    ptrs = (C.c_void_p * 5)(*[b.ctypes.data for b in banks])
    assert L.gbilu_fpga_pack(0, ps, nz, C.cast(ex["pointers"], C.c_void_p), ps, fill,
                             C.cast(ptrs, C.c_void_p)) == 0
    return banks, offs, ps


@pytest.mark.parametrize("coloring", ["parity", "natural"])
@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_rtl_model_of_packed_bytes_matches_oracle(gb, name, coloring):
    s, g, ex = exported(name, coloring)
    banks, offs, ps = pack(gb, ex)
    model = PackedSystem(banks, offs, ps)
    P = Prepared(s, coloring=coloring)
    rng = np.random.default_rng(7)
    for _ in range(2):
        x = rng.standard_normal(s.n)
        y = P.from_perm(model.spmv(P.to_perm(x)))
        ref = P.spmv(x)
        assert np.linalg.norm(y - ref) <= 1e-12 * np.linalg.norm(ref)
        z = P.from_perm(model.ilu_apply(P.to_perm(x)))
        ref = P.ilu_apply(x)
        assert np.linalg.norm(z - ref) <= 1e-12 * np.linalg.norm(ref)
    # the right-hand side arrives permuted into R1
    r1 = np.frombuffer(banks[2], np.float64, s.n, int(offs[18]))
    assert np.array_equal(r1, P.to_perm(s.b))


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_every_color_within_kernel_limits(gb, name):
    s, g, ex = exported(name)
    vs = ex["vector_sizes"]
    assert vs[0] == 3 * s.nb <= 163840
    for m, key in enumerate("ALU"):
        nc = int(vs[6 * m + 2])
        assert 1 <= nc <= 256
        sizes = ex[key]["sizes"][8:].reshape(-1, 4).astype(np.int64)
        assert sizes.shape[0] == nc and int(sizes[:, 1].sum()) == 3 * s.nb
        assert (sizes[:, 1] <= 2048).all() and (sizes[:, 2] <= 8192).all()
        assert (sizes[:, 3] <= 32768).all()
        assert int(ex["nnz_sizes"][m]) <= 2 ** 21
        # every part's arrays padded to the line reads
        assert ex[key]["pidx"].size == sum(-(-int(c) // 16) * 16 for c in sizes[:, 2])
        assert ex[key]["vals"].size == sum(-(-int(v) // 8) * 8 for v in sizes[:, 3])
        assert ex[key]["cols"].size == sum(-(-int(v) // 32) * 32 for v in sizes[:, 3])
        assert ex[key]["nrs"].size == sum(-(-int(v) // 64) * 64 for v in sizes[:, 3])
    # the L values never read a later row, the U values never an earlier one
    # (the A, L and U colors are the same row ranges)
    assert np.array_equal(ex["L"]["sizes"][8:].reshape(-1, 4)[:, 1],
                          ex["U"]["sizes"][8:].reshape(-1, 4)[::-1, 1])


def test_long_runs_of_empty_rows_are_bridged(gb):
    """A color with more than 255 consecutive rows that have no L values
    (the new-row offset is 8 bits): zero values bridge the gap."""
    nb = 400
    rows = [[i] for i in range(nb)]
    # a path 0 - (nb-1): block row nb-1 (color 1) couples to row 0 only
    rows[0].append(nb - 1)
    rows[nb - 1].insert(0, 0)
    rowptr = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int32)
    colind = np.concatenate(rows).astype(np.int32)
    rng = np.random.default_rng(2)
    vals = 0.1 * rng.standard_normal((colind.size, 3, 3))
    for i in range(nb):
        vals[rowptr[i] + rows[i].index(i)] += 4.0 * np.eye(3)
    from fpga_gb300.synth import BlockSystem
    s = BlockSystem(nb, rowptr, colind, vals, rng.standard_normal(3 * nb), np.arange(nb), (nb, 1, 1))
    g = GbIlu(device=-1, coloring="natural")
    g.analyze(s.rowptr, s.colind).factor(s.vals)
    ex = g.fpga_export(s.b)
    assert (ex["A"]["nrs"] <= 255).all()
    banks, offs, ps = pack(gb, ex)
    model = PackedSystem(banks, offs, ps)
    P = Prepared(s, coloring="natural")
    x = rng.standard_normal(s.n)
    assert np.linalg.norm(P.from_perm(model.spmv(P.to_perm(x))) - P.spmv(x)) <= \
        1e-12 * np.linalg.norm(P.spmv(x))
    assert np.linalg.norm(P.from_perm(model.ilu_apply(P.to_perm(x))) - P.ilu_apply(x)) <= \
        1e-12 * np.linalg.norm(P.ilu_apply(x))


def test_systems_beyond_the_kernel_are_refused(built_lib):
    s = make_config("c4_60x60x30_adjoint")     # 324,000 unknowns > 163,840
    g = GbIlu(device=-1)
    g.analyze(s.rowptr, s.colind).factor(s.vals)
    with pytest.raises(GbIluError) as e:
        g.fpga_export(s.b)
    assert e.value.code == native.BAD_INPUT and "VECTOR_SIZE_ELEM" in str(e.value)


@pytest.fixture(scope="module")
def ref():
    if os.path.isdir(REFERENCE):
        subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"),
                               f"REF={REFERENCE}"])
    elif not os.path.exists(REF_SO):
        pytest.skip("reference host library not built and reference tree absent")
    L = C.CDLL(REF_SO)
    L.ref_pack.argtypes = [C.c_uint, I32P, I32P, C.c_void_p, I32P, C.c_int, C.c_void_p]
    return L


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_exported_arrays_pack_like_the_reference(gb, ref, name):
    s, g, ex = exported(name)
    ps = np.ascontiguousarray(ex["vector_sizes"], np.int32)
    nz = np.ascontiguousarray(ex["nnz_sizes"], np.int32)
    tot = np.zeros(5, np.uint32)
    gb.gbilu_fpga_layout(0, ps, nz, 64, np.zeros(40, np.uint64), tot, np.zeros(23, np.int64),
                         np.zeros(6, np.uint32))
    for fill in (0, 1):
        banks = {k: [np.full(int(t), 0xAB, np.uint8) for t in tot] for k in ("ref", "gb")}
        ptrs = {k: (C.c_void_p * 5)(*[b.ctypes.data for b in banks[k]]) for k in banks}
        vp = C.cast(ex["pointers"], C.c_void_p)
        assert ref.ref_pack(0, ps, nz, vp, ps, fill, C.cast(ptrs["ref"], C.c_void_p)) == 0
        assert gb.gbilu_fpga_pack(0, ps, nz, vp, ps, fill, C.cast(ptrs["gb"], C.c_void_p)) == 0
        for b in range(5):
            assert np.array_equal(banks["ref"][b], banks["gb"][b]), (b, fill)
