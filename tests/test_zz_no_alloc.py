"""The allocation-free SpMV + dot entry point, through the C ABI.

gbilu_bsr_spmv_dot_noalloc serves callers that cannot allocate device
memory (a fixed device arena handed out by a host framework, a callback in
which cudaMalloc's implicit synchronisation is not allowed). It works on
plain BSR arrays that already live on the device and keeps its reduction
scratch in a fixed array inside the library. This test checks it against
the handle-based SpMV entry point (gbilu_apply_spmv) and against the CPU
oracle's SpMV on two calls in a row, to the SpMV tolerance of the other GPU
tests, that the calls leave the device's free memory unchanged, and that it
rejects a system larger than its fixed scratch.

The file name sorts last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from fpga_gb300 import GbIlu, load
from fpga_gb300.synth import generate
from oracle_lib import Prepared

pytestmark = pytest.mark.gpu

KERNEL_TOL = 1e-12


def noalloc_fn():
    lib = load()
    f = lib.gbilu_bsr_spmv_dot_noalloc
    f.argtypes = [C.c_int] + [C.c_void_p] * 7 + [C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_matches_handle_spmv(built_lib):
    torch = pytest.importorskip("torch")
    s = generate(30, 24, 12, sigma=1.5, inactive_frac=0.05, fault_frac=0.01, seed=7)
    rng = np.random.default_rng(11)
    x = rng.standard_normal(s.n)
    w = rng.standard_normal(s.n)
    with GbIlu(device=0) as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        y_ref = g.spmv(x)
    y_orc = Prepared(s).spmv(x)
    assert np.linalg.norm(y_ref - y_orc) <= KERNEL_TOL * np.linalg.norm(y_orc)

    dev = torch.device("cuda:0")
    rp = torch.from_numpy(s.rowptr.astype(np.int32)).to(dev)
    ci = torch.from_numpy(s.colind.astype(np.int32)).to(dev)
    va = torch.from_numpy(np.ascontiguousarray(s.vals.reshape(-1))).to(dev)
    xd = torch.from_numpy(x).to(dev)
    wd = torch.from_numpy(w).to(dev)
    f = noalloc_fn()
    stream = torch.cuda.current_stream(dev).cuda_stream
    outs = [(torch.full((s.n,), float("nan"), dtype=torch.float64, device=dev),
             torch.full((1,), float("nan"), dtype=torch.float64, device=dev)) for _ in range(3)]
    torch.cuda.synchronize(dev)
    free = []
    for call, (yd, dot) in enumerate(outs):
        rc = f(s.nb, rp.data_ptr(), ci.data_ptr(), va.data_ptr(), xd.data_ptr(),
               yd.data_ptr(), wd.data_ptr(), dot.data_ptr(), stream)
        assert rc == 0, f"call {call}: status {rc}"
        torch.cuda.synchronize(dev)
        free.append(torch.cuda.mem_get_info(dev)[0])
    # the first call in a process may load the library's device code (and
    # with it the scratch array); the calls after it allocate nothing
    assert free[1] == free[0] and free[2] == free[0], free
    for call, (yd, dot) in enumerate(outs):
        y = yd.cpu().numpy()
        d = float(dot.cpu().item())
        for ref in (y_ref, y_orc):
            assert np.linalg.norm(y - ref) <= KERNEL_TOL * np.linalg.norm(ref), call
            assert abs(d - float(np.dot(ref, w))) <= \
                KERNEL_TOL * np.linalg.norm(ref) * np.linalg.norm(w), call


def test_noalloc_rejects_oversize(built_lib):
    f = noalloc_fn()
    one = C.c_void_p(1)
    # sizes are checked before any pointer is touched
    rc = f(4096 * 256 + 1, one, one, one, one, one, one, one, None)
    assert rc == 6
