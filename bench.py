"""Benchmark of the GB300 ILU0-BiCGSTAB solve (one JSON line on rank 0).

Metric: ILU0-BiCGSTAB solve time on the 100x100x50 (500k-cell, 1.425M
unknowns) system at relative residual 1e-2, FP64 (``value``, ms per solve,
inputs resident in HBM), the same through the host-buffer C-ABI call
(``e2e``), the mixed-precision form against FP64 at 1e-8 on the sigma=2.0
system, the adjoint/forward time ratio on the 60x60x30 system, and the
4,000-cell and 500k-cell systems at their tolerances in both forms.

A "step" is one solve of the 500k-cell system from x0 = 0. Inputs are larger
than L2 (the matrix values alone are 0.23 GB), so no L2 flush is inserted.
``--impl reference`` times the CPU restatement of the same algorithm (the
reference has no CPU solver; its arithmetic exists only as FPGA RTL) on all
host cores.

Multi-GPU: the solve does not shard without changing the preconditioner, so
N > 1 runs N independent replicas (one system per rank, seeded by rank):
value = the max over ranks of the per-solve device time (weak scaling: the
work per GPU is fixed), and ``replicas.solves_per_s`` the aggregate
throughput of all ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ILU0-BiCGSTAB solve ms @relres 1e-2: FP64 vs mixed; HBM GB/s; adjoint/fwd"
WORKLOAD = "c2_100x100x50"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"gbilu_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        try:
            rows = [l.split(",") for l in open(self.path) if l.strip()]
            os.remove(self.path)
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if len(r) >= 9]
        mx = [float(r[2]) for r in rows if len(r) >= 9]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows if len(r) >= 9 for i in range(4)
                          if r[5 + i].strip().lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(sm)}


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        if backend == "nccl":
            import torch
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier_max(world, value):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cpu" if dist.get_backend() == "gloo" else f"cuda:{torch.cuda.current_device()}"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def workload_config(s, cfg, nnzb, ncolors, world):
    """The config dict both arms print (same keys, same workload)."""
    return {"workload": WORKLOAD, "grid": list(cfg["grid"]), "nb": s.nb, "nnzb": nnzb,
            "colors": ncolors, "tol": cfg["tol"], "sigma": cfg["sigma"],
            "inactive": cfg["inactive"], "faults": cfg["faults"], "x0": "zero",
            "l2": "inputs larger than L2 (FP64 A 0.23 GB, L+U 0.19 GB)",
            "parallelism": f"replicas{world}" if world > 1 else "single"}


def host_cpu():
    """CPU model and thread count of the host running the CPU legs."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    return {"model": model, "nproc": os.cpu_count()}


def cpu_reference(args, world, rank):
    """The reference arm: the CPU restatement (oracle) on all host cores."""
    if rank != 0:
        return
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Prepared
    from fpga_gb300.synth import make_config, CONFIGS
    cores = os.cpu_count() or 1
    s = make_config(WORKLOAD)
    P = Prepared(s)
    cfg = CONFIGS[WORKLOAD]
    tol = cfg["tol"]
    for _ in range(max(1, args.warmup)):
        P.solve_omp(s.b, tol=tol, maxit=1000, nthreads=cores)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        x, r = P.solve_omp(s.b, tol=tol, maxit=1000, nthreads=cores)
        times.append((time.perf_counter() - t0) * 1e3)
    ms = statistics.mean(times)
    out = {"impl": "reference", "metric": METRIC, "value": ms, "unit": "ms", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded generator, no dataset)",
           "config": workload_config(s, cfg, s.nnzb, P.ncolors, world),
           "result": {"status": r.status, "half_iters": r.half_iters, "relres": r.relres},
           "cpu_baseline": {"value": ms, "unit": "ms", "cores": cores, "kind": "port",
                            "cpu": host_cpu(),
                            "sample": f"{args.steps} full solves of {WORKLOAD} to relres {tol} "
                                      "(OpenMP C restatement of the reference algorithm)"},
           "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def gpu_bench(args, world, rank, local):
    import numpy as np
    import torch
    from fpga_gb300 import GbIlu
    from fpga_gb300.synth import make_config, generate, CONFIGS, adjoint_selection

    torch.cuda.set_device(local)
    cfg = CONFIGS[WORKLOAD]
    s = make_config(WORKLOAD, seed=rank)
    tol, maxit = cfg["tol"], cfg["maxit"]
    g = GbIlu(device=local, precision="mixed")
    g.analyze(s.rowptr, s.colind).factor(s.vals)
    st = g.stats()
    n = s.n
    b_dev = torch.from_numpy(s.b).to(f"cuda:{local}")
    x_dev = torch.zeros(n, dtype=torch.float64, device=f"cuda:{local}")
    # FP64 run on device pointers: warm-up, then K timed solves
    g64 = GbIlu(device=local, precision="fp64", use_graph=not args.no_graph)
    g64.analyze(s.rowptr, s.colind).factor(s.vals)
    for _ in range(args.warmup):
        x_dev.zero_()
        g64.solve_device(b_dev.data_ptr(), x_dev.data_ptr(), tol, maxit)
    torch.cuda.synchronize()
    res = []
    launches = 0
    with ClockSampler(local) as clk:
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev_ms = 0.0
        for _ in range(args.steps):
            x_dev.zero_()
            r = g64.solve_device(b_dev.data_ptr(), x_dev.data_ptr(), tol, maxit)
            res.append(r)
            dev_ms += r.device_ms
            launches += g64.stats()["last_launches"]
        torch.cuda.synchronize()
        wall_ms = (time.perf_counter() - t0) * 1e3
        barrier(world)
    clocks = clk.summary()
    # device time of the solves (CUDA events on the library's stream), max over ranks
    # weak scaling: every rank solves its own system; the value is the
    # slowest rank's per-solve time, the aggregate rate is reported beside it
    ms_step = barrier_max(world, dev_ms / args.steps)
    value = ms_step
    r0 = res[-1]
    x_np = x_dev.cpu().numpy()
    true_relres = float(np.linalg.norm(s.b - s.to_scipy() @ x_np) / np.linalg.norm(s.b))

    # e2e: host pinned buffers through gbilu_solve (H2D b, x0; D2H x inside)
    b_pin = torch.from_numpy(s.b).pin_memory()
    x_pin = torch.zeros(n, dtype=torch.float64).pin_memory()
    for _ in range(max(2, args.warmup)):
        x_pin.zero_()
        g64.solve_host_ptr(b_pin.data_ptr(), x_pin.data_ptr(), tol, maxit)
    e2e_ms = []
    for _ in range(args.steps):
        x_pin.zero_()
        t0 = time.perf_counter()
        g64.solve_host_ptr(b_pin.data_ptr(), x_pin.data_ptr(), tol, maxit)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e = barrier_max(world, statistics.mean(e2e_ms))

    # dominant-kernel roofline: kernels timed back to back with CUDA events
    peak, peak_kind = peaks()
    kern = {}
    for name in ("spmv64", "ilu64", "spmv32", "ilu32"):
        ms, by, la = g.bench_kernel(name, reps=20)
        kern[name] = {"ms": ms, "alg_bytes": by, "launches": la, "gbs": by / ms / 1e6}
    trace = {"fp64": g.ilu_trace(fp32=False), "fp32": g.ilu_trace(fp32=True)}
    budget = iteration_budget(g, g64, st, b_dev, x_dev, local) if not args.quick else None
    it_ms = value / max(1, (r0.half_iters + 1) / 2.0)
    solve_gbs = st["alg_bytes_iter"][0] / it_ms / 1e6 if it_ms > 0 else None
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "ilu64_c2_traffic.txt")
    if os.path.exists(tfile):
        for line in open(tfile):
            if line.startswith("bytes_per_launch:"):
                traffic = float(line.split(":")[1])
    # the dominant kernel of the FP64 solve by device-time share (ncu launch
    # list, profiles/): the single-launch ILU0 apply
    dom = kern["ilu64"]
    # its FP64 floor: 9 FMA per block of L, U and D^-1 at the FP64 rate
    # measured on GB300 (1.68 FMA lanes per clock per SM, 2.07 GHz)
    fp64_fma_per_s = 1.68 * torch.cuda.get_device_properties(local).multi_processor_count * 2.07e9
    fp64_floor_us = 9 * (st["nnzb_lower"] + st["nnzb_upper"] + st["nb"]) / fp64_fma_per_s * 1e6
    roofline = {"bound": "hbm", "kernel": "k_ilu_coop<double> (ILU0 L+U sweeps, FP64)",
                "achieved": dom["gbs"], "peak": peak, "unit": "GB/s",
                "frac": dom["gbs"] / peak, "traffic": traffic,
                "peak_kind": peak_kind, "alg_bytes_per_launch": dom["alg_bytes"],
                "fp64_pipe_floor_us": fp64_floor_us,
                "fp64_floor_frac": fp64_floor_us / (dom["ms"] * 1e3)}

    extra = {}
    if not args.quick and rank == 0:
        extra = secondary(args, local, tol)

    cpu = None
    if rank == 0 and world == 1 and not args.quick:
        cpu = cpu_baseline(s, tol, maxit)

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "ms", "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
               "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
               "dtype": "f64", "data": "synthetic (seeded generator, no dataset)",
               "config": workload_config(s, cfg, st["nnzb"], st["ncolors"], world),
               "replicas": {"ranks": world, "solves_per_s": world * 1e3 / ms_step},
               "result": {"status": r0.status, "half_iters": r0.half_iters,
                          "relres": r0.relres, "true_relres": true_relres},
               "wall_ms_per_step": wall_ms / args.steps,
               "solve_gbs": solve_gbs,
               "solve_frac_of_peak": solve_gbs / peak if solve_gbs else None,
               "kernels": kern,
               "ilu_phases_rows_us": trace,
               "iteration_budget": budget,
               "analysis": analysis_timing(s, local) if not args.quick else None,
               "e2e": {"value": e2e, "unit": "ms", "h2d_bytes_per_step": 2 * n * 8,
                       "d2h_bytes_per_step": n * 8},
               "gpu_launches": int(launches),
               "roofline": roofline,
               "clocks": clocks}
        out.update(extra)
        if cpu:
            out["cpu_baseline"] = cpu
        print(json.dumps(out), flush=True)


FP64_FMA_LANES_PER_CLK_SM = 1.68   # measured on GB300 (independent DFMA chains)
SM_CLOCK_HZ = 2.07e9


def iteration_budget(g, g64, st, b_dev, x_dev, local):
    """Where one BiCGSTAB iteration's time goes: every kernel of the
    iteration timed alone (back to back, CUDA events), beside its HBM floor
    (algorithmic bytes at the measured copy peak) and, for FP64, its FP64
    floor (DFMA count at the measured FP64 rate); and the measured time per
    iteration of whole solves (the slope between maxit 4 and 12, tol 0)."""
    import torch
    peak, _ = peaks()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    fma_rate = FP64_FMA_LANES_PER_CLK_SM * sms * SM_CLOCK_HZ
    n, nb, nnzb = 3 * st["nb"], st["nb"], st["nnzb"]
    nlu = st["nnzb_lower"] + st["nnzb_upper"]
    # DFMA per launch (FP64): SpMV 9 per block (+ the fused dots), apply 9
    # per L, U and D block, update_s 2n, update_r 5n, update_p 2n
    fmas = {"ilu": 9 * (nlu + nb), "spmv_alpha": 9 * nnzb + n, "spmv_omega": 9 * nnzb + 2 * n,
            "update_s": 2 * n, "update_r": 5 * n, "update_p": 2 * n}
    out = {}
    for prec, suf in (("fp64", "64"), ("fp32", "32")):
        rows = {}
        for name, count in (("ilu", 2), ("spmv_alpha", 1), ("spmv_omega", 1), ("update_s", 1),
                            ("update_r", 1), ("update_p", 1)):
            ms, by, la = g.bench_kernel(name + suf, reps=20)
            r = {"per_iter": count, "us": ms * 1e3, "alg_bytes": by,
                 "hbm_floor_us": by / (peak * 1e9) * 1e6}
            if prec == "fp64":
                r["fp64_floor_us"] = fmas[name] / fma_rate * 1e6
            rows[name] = r
        tot = sum(r["us"] * r["per_iter"] for r in rows.values())
        out[prec] = {"kernels": rows, "sum_us": tot,
                     "hbm_floor_sum_us": sum(r["hbm_floor_us"] * r["per_iter"] for r in rows.values())}
        if prec == "fp64":
            out[prec]["fp64_floor_sum_us"] = sum(r["fp64_floor_us"] * r["per_iter"]
                                                 for r in rows.values())
    # measured per-iteration time of the FP64 graph loop
    t = {}
    for m in (4, 12):
        ms = []
        for _ in range(3):
            x_dev.zero_()
            ms.append(g64.solve_device(b_dev.data_ptr(), x_dev.data_ptr(), 0.0, m).device_ms)
        t[m] = statistics.median(ms)
    out["fp64"]["measured_us_per_iter"] = (t[12] - t[4]) / 8 * 1e3
    out["fp64"]["overhead_us_per_iter"] = out["fp64"]["measured_us_per_iter"] - out["fp64"]["sum_us"]
    return out


def analysis_timing(s, local):
    """Analysis (coloring, ordering, device layout and upload) and ILU0
    factorization of the headline system, timed separately: host-only
    analysis; the analysis of a device handle with the coloring on the host
    and on the GPU (the coloring's own time beside it); host factorization
    (with the upload) and device factorization."""
    from fpga_gb300 import GbIlu
    out = {}
    with GbIlu(device=-1) as h:
        h.analyze(s.rowptr, s.colind)
        out["analyze_ms_host_only"] = h.stats()["analyze_ms"]
    for dev in (False, True):
        with GbIlu(device=local, factor_on_device=dev, color_on_device=dev) as h:
            h.analyze(s.rowptr, s.colind)
            h.analyze(s.rowptr, s.colind)   # the second analysis (warm)
            h.factor(s.vals)
            h.factor(s.vals)                # the second factorization (warm)
            st = h.stats()
            key = "device" if dev else "host"
            out["analyze_ms_" + key + "_coloring"] = st["analyze_ms"]
            out["color_ms_" + key] = st["color_ms"]
            out["factor_ms_" + key] = st["factor_ms"]
    return out


def cpu_baseline(s, tol, maxit):
    """The oracle's OpenMP solver on the host cores, bounded samples: the
    headline system at its tolerance (the line's cpu_baseline) and, under
    ``others``, the other workloads and tolerances the GPU numbers are
    quoted on (median of 3 solves each, after one warm-up)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Prepared
    from fpga_gb300.synth import make_config, CONFIGS
    cores = os.cpu_count() or 1

    def timed(P, b, t, m, reps):
        P.solve_omp(b, tol=t, maxit=m, nthreads=cores)
        times = []
        for _ in range(reps):
            t0 = time.perf_counter()
            x, r = P.solve_omp(b, tol=t, maxit=m, nthreads=cores)
            times.append((time.perf_counter() - t0) * 1e3)
        return statistics.median(times), r

    P = Prepared(s)
    times = []
    P.solve_omp(s.b, tol=tol, maxit=maxit, nthreads=cores)
    t_end = time.perf_counter() + 10.0
    while len(times) < 3 or (time.perf_counter() < t_end and len(times) < 20):
        t0 = time.perf_counter()
        P.solve_omp(s.b, tol=tol, maxit=maxit, nthreads=cores)
        times.append((time.perf_counter() - t0) * 1e3)
    out = {"value": statistics.median(times), "unit": "ms", "cores": cores, "kind": "port",
           "cpu": host_cpu(),
           "sample": f"{len(times)} full solves of {WORKLOAD} to relres {tol} "
                     "(median; OpenMP C restatement, oracle/gbilu_oracle.c)"}
    others = []
    ms, r = timed(P, s.b, 1e-6, maxit, 3)
    others.append({"workload": WORKLOAD, "form": "fp64", "tol": 1e-6, "ms": ms,
                   "half_iters": r.half_iters})
    for wl, t in (("c1_20x20x10", 1e-2), ("c3_100x100x50_mixed", 1e-8),
                  ("c4_60x60x30_adjoint", 1e-10)):
        s2 = make_config(wl)
        P2 = Prepared(s2)
        ms, r = timed(P2, s2.b, t, CONFIGS[wl]["maxit"], 3)
        others.append({"workload": wl, "form": "fp64 forward", "tol": t, "ms": ms,
                       "half_iters": r.half_iters})
        if wl.startswith("c4"):
            # the adjoint's transposed solve, g = W^T (W x - d)
            from fpga_gb300.synth import adjoint_selection
            x, _ = P2.solve_omp(s2.b, tol=t, maxit=CONFIGS[wl]["maxit"], nthreads=cores)
            cells, d = adjoint_selection(s2.nb)
            idx = (3 * cells[:, None] + np.arange(3)).reshape(-1)
            gv = np.zeros(s2.n)
            gv[idx] = x[idx] - d
            P2.solve_omp(gv, tol=t, maxit=CONFIGS[wl]["maxit"], nthreads=cores, transpose=True)
            tt = []
            for _ in range(3):
                t0 = time.perf_counter()
                _, ra = P2.solve_omp(gv, tol=t, maxit=CONFIGS[wl]["maxit"], nthreads=cores,
                                     transpose=True)
                tt.append((time.perf_counter() - t0) * 1e3)
            others.append({"workload": wl, "form": "fp64 adjoint (transposed solve)", "tol": t,
                           "ms": statistics.median(tt), "half_iters": ra.half_iters})
    out["others"] = others
    return out


def secondary(args, local, tol64):
    """Mixed vs FP64 at 1e-8 (sigma=2.0 system) and adjoint/forward ratio."""
    import numpy as np
    from fpga_gb300 import GbIlu
    from fpga_gb300.synth import make_config, CONFIGS, adjoint_selection
    out = {}
    c3 = CONFIGS["c3_100x100x50_mixed"]
    s = make_config("c3_100x100x50_mixed")
    tol = c3["tol"]
    times = {}
    sols = {}
    for prec in ("fp64", "mixed"):
        g = GbIlu(device=local, precision=prec)
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        g.solve(s.b, tol=tol, maxit=c3["maxit"])
        ms = []
        for _ in range(3):
            x, r = g.solve(s.b, tol=tol, maxit=c3["maxit"])
            ms.append(r.device_ms)
        times[prec] = (statistics.median(ms), r)
        sols[prec] = x
        g.close()
    A = s.to_scipy()
    err = float(np.linalg.norm(sols["mixed"] - sols["fp64"]) / np.linalg.norm(sols["fp64"]))
    # against the CPU oracle's FP64 solve to the same tolerance (the checker)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Prepared
    x_orc, r_orc = Prepared(s).solve_omp(s.b, tol=tol, maxit=c3["maxit"],
                                         nthreads=os.cpu_count() or 1)
    err_orc = {p: float(np.linalg.norm(sols[p] - x_orc) / np.linalg.norm(x_orc)) for p in sols}
    tr = {p: float(np.linalg.norm(s.b - A @ sols[p]) / np.linalg.norm(s.b)) for p in sols}
    out["mixed"] = {"workload": "c3_100x100x50_mixed (sigma=2.0)", "tol": tol,
                    "fp64_ms": times["fp64"][0], "mixed_ms": times["mixed"][0],
                    "speedup": times["fp64"][0] / times["mixed"][0],
                    "fp64_half_iters": times["fp64"][1].half_iters,
                    "mixed_outer": times["mixed"][1].outer_iters,
                    "mixed_inner_half_iters": times["mixed"][1].inner_half_iters,
                    "true_relres": tr, "x_err_vs_fp64": err,
                    "x_err_vs_oracle": err_orc["mixed"],
                    "fp64_x_err_vs_oracle": err_orc["fp64"],
                    "oracle_half_iters": r_orc.half_iters}
    # the 4,000-cell system at 1e-2 and the 500k-cell one at 1e-2 and 1e-6,
    # FP64 and mixed
    rows = []
    for wl, tols in (("c1_20x20x10", (1e-2,)), (WORKLOAD, (1e-2, 1e-6))):
        s2 = make_config(wl)
        A2 = s2.to_scipy()
        for prec in ("fp64", "mixed"):
            g = GbIlu(device=local, precision=prec)
            g.analyze(s2.rowptr, s2.colind).factor(s2.vals)
            for tol2 in tols:
                g.solve(s2.b, tol=tol2, maxit=CONFIGS[wl]["maxit"])
                ms = []
                for _ in range(3):
                    x, r = g.solve(s2.b, tol=tol2, maxit=CONFIGS[wl]["maxit"])
                    ms.append(r.device_ms)
                rows.append({"workload": wl, "precision": prec, "tol": tol2,
                             "ms": statistics.median(ms),
                             "half_iters": r.half_iters if prec == "fp64" else r.inner_half_iters,
                             "outer": r.outer_iters,
                             "true_relres": float(np.linalg.norm(s2.b - A2 @ x) /
                                                  np.linalg.norm(s2.b))})
            g.close()
    out["tolerances"] = rows
    # adjoint / forward on the 60x60x30 system, device arrays: the forward
    # solve against the transposed solve alone and against the whole
    # backward pass (transposed solve, gathers and dL/dA on the pattern)
    import torch
    c4 = CONFIGS["c4_60x60x30_adjoint"]
    s = make_config("c4_60x60x30_adjoint")
    g = GbIlu(device=local, precision="fp64")
    g.analyze(s.rowptr, s.colind).factor(s.vals)
    cells, d = adjoint_selection(s.nb)
    idx = (3 * cells[:, None] + np.arange(3)).reshape(-1)
    dev = torch.device(f"cuda:{local}")
    bd = torch.from_numpy(s.b).to(dev)
    xd = torch.zeros(s.n, dtype=torch.float64, device=dev)
    ld = torch.zeros(s.n, dtype=torch.float64, device=dev)
    dAd = torch.zeros(s.nnzb * 9, dtype=torch.float64, device=dev)
    fw, bw, bw_full = [], [], []
    for rep in range(4):
        xd.zero_()
        r = g.solve_device(bd.data_ptr(), xd.data_ptr(), tol=c4["tol"], maxit=c4["maxit"])
        x = xd.cpu().numpy()
        gvec = np.zeros(s.n)
        gvec[idx] = x[idx] - d
        gd = torch.from_numpy(gvec).to(dev)
        ra = g.adjoint_device(gd.data_ptr(), xd.data_ptr(), ld.data_ptr(), None,
                              tol=c4["tol"], maxit=c4["maxit"])
        rf = g.adjoint_device(gd.data_ptr(), xd.data_ptr(), ld.data_ptr(), dAd.data_ptr(),
                              tol=c4["tol"], maxit=c4["maxit"])
        if rep:   # the first round is the warm-up
            fw.append(r.device_ms)
            bw.append(ra.device_ms)
            bw_full.append(rf.device_ms)
    f_ms = statistics.median(fw)
    out["adjoint"] = {"workload": "c4_60x60x30_adjoint", "tol": c4["tol"],
                      "forward_ms": f_ms, "adjoint_ms": statistics.median(bw),
                      "adjoint_ms_full": statistics.median(bw_full),
                      "ratio": statistics.median(bw) / f_ms,
                      "ratio_full": statistics.median(bw_full) / f_ms,
                      "forward_half_iters": r.half_iters, "adjoint_half_iters": rf.half_iters,
                      "timing": "device arrays, CUDA events; full = transposed solve + "
                                "gathers + dL/dA (nnzb*9 doubles written)"}
    g.close()
    out["adjoint_mixed_2m"] = mixed_adjoint_2m(local)
    return out


def mixed_adjoint_2m(local):
    """200x200x50 (2M cells, 6M unknowns): mixed forward + adjoint to 1e-8,
    time ratio, peak device memory, gradient error against the FP64 adjoint."""
    import numpy as np
    import torch
    from fpga_gb300 import GbIlu
    from fpga_gb300.synth import make_config, CONFIGS, adjoint_selection
    c5 = CONFIGS["c5_200x200x50_mixed_adjoint"]
    s = make_config("c5_200x200x50_mixed_adjoint")
    cells, d = adjoint_selection(s.nb)
    idx = (3 * cells[:, None] + np.arange(3)).reshape(-1)
    res = {"workload": "c5_200x200x50_mixed_adjoint", "nb": s.nb, "nnzb": s.nnzb, "tol": c5["tol"]}
    grads = {}
    dev = torch.device(f"cuda:{local}")
    for prec in ("mixed", "fp64"):
        # device arrays (allocated before the handle, so that the measured
        # device memory is the handle's): b, x, g, lambda and dL/dA
        bd = torch.from_numpy(s.b).to(dev)
        xd = torch.zeros(s.n, dtype=torch.float64, device=dev)
        gd = torch.zeros(s.n, dtype=torch.float64, device=dev)
        ld = torch.zeros(s.n, dtype=torch.float64, device=dev)
        dAd = torch.zeros(s.nnzb * 9, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        free0, total = torch.cuda.mem_get_info(local)
        g = GbIlu(device=local, precision=prec)
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        fw, bw, bw_full = [], [], []
        for rep in range(4):   # the first round builds the graphs: not timed
            xd.zero_()
            r = g.solve_device(bd.data_ptr(), xd.data_ptr(), tol=c5["tol"], maxit=c5["maxit"])
            if rep == 0:
                x = xd.cpu().numpy()
                gv = np.zeros(s.n)
                gv[idx] = x[idx] - d
                gd.copy_(torch.from_numpy(gv))
            ra0 = g.adjoint_device(gd.data_ptr(), xd.data_ptr(), ld.data_ptr(), None,
                                   tol=c5["tol"], maxit=c5["maxit"])
            ra = g.adjoint_device(gd.data_ptr(), xd.data_ptr(), ld.data_ptr(), dAd.data_ptr(),
                                  tol=c5["tol"], maxit=c5["maxit"])
            if rep:
                fw.append(r.device_ms)
                bw.append(ra0.device_ms)
                bw_full.append(ra.device_ms)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info(local)
        grads[prec] = (ld.cpu().numpy(), dAd.cpu().numpy())
        f_ms = statistics.median(fw)
        res[prec] = {"forward_ms": f_ms, "adjoint_ms": statistics.median(bw),
                     "ratio": statistics.median(bw) / f_ms,
                     "adjoint_ms_full": statistics.median(bw_full),
                     "ratio_full": statistics.median(bw_full) / f_ms,
                     "analyze_ms": g.stats()["analyze_ms"],
                     "factor_ms_host": g.stats()["factor_ms"],
                     "forward_status": r.status, "adjoint_status": ra.status,
                     "forward_true_relres": r.true_relres, "adjoint_true_relres": ra.true_relres,
                     "device_bytes_handle": g.stats()["device_bytes"],
                     "device_bytes_measured": free0 - free1,
                     "timing": "device arrays, CUDA events, median of 3 after a warm-up round; "
                               "full = transposed solve + gathers + dL/dA"}
        g.close()
        del bd, xd, gd, ld, dAd
    with GbIlu(device=local, precision="mixed", factor_on_device=True) as g:
        g.analyze(s.rowptr, s.colind)
        g.factor(s.vals)
        g.factor(s.vals)
        res["mixed"]["factor_ms_device"] = g.stats()["factor_ms"]
    res["lambda_rel_err_vs_fp64"] = float(np.linalg.norm(grads["mixed"][0] - grads["fp64"][0]) /
                                          np.linalg.norm(grads["fp64"][0]))
    res["dA_rel_err_vs_fp64"] = float(np.linalg.norm(grads["mixed"][1] - grads["fp64"][1]) /
                                      np.linalg.norm(grads["fp64"][1]))
    return res


def mixed_only(args):
    """Mixed solves of the 500k-cell system to 1e-8, timed alone (profiler target)."""
    from fpga_gb300 import GbIlu
    from fpga_gb300.synth import make_config
    s = make_config(WORKLOAD)
    g = GbIlu(device=0, precision="mixed", use_graph=not args.no_graph)
    g.analyze(s.rowptr, s.colind).factor(s.vals)
    for _ in range(args.warmup):
        g.solve(s.b, tol=1e-8, maxit=2000)
    ms = []
    for _ in range(args.steps):
        x, r = g.solve(s.b, tol=1e-8, maxit=2000)
        ms.append(r.device_ms)
    print(json.dumps({"mixed_ms": statistics.median(ms), "outer": r.outer_iters,
                      "inner_half_iters": r.inner_half_iters, "true_relres": r.true_relres}),
          flush=True)


def kernel_only(args):
    """One kernel family of the 500k-cell system timed alone (profiler target)."""
    from fpga_gb300 import GbIlu
    from fpga_gb300.synth import make_config
    s = make_config(WORKLOAD)
    g = GbIlu(device=0, precision="mixed" if args.kernel_only.endswith("32") else "fp64")
    g.analyze(s.rowptr, s.colind).factor(s.vals)
    ms, by, la = g.bench_kernel(args.kernel_only, reps=args.steps)
    print(json.dumps({"kernel": args.kernel_only, "ms": ms, "alg_bytes": by, "launches": la,
                      "gbs": by / ms / 1e6}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--quick", action="store_true",
                    help="only the FP64 500k-cell solve (for profiler runs)")
    ap.add_argument("--no-graph", action="store_true",
                    help="host-driven launches instead of the graph loop (profiler runs: "
                         "kernels inside a conditional graph node are not listed by ncu)")
    ap.add_argument("--kernel-only", default=None,
                    choices=["spmv64", "ilu64", "spmv32", "ilu32"],
                    help="time one kernel family alone (3 warm-up + --steps launches)")
    ap.add_argument("--mixed-only", action="store_true",
                    help="only mixed solves of the 500k-cell system to 1e-8 (profiler runs of "
                         "the FP32 iteration kernels; combine with --no-graph)")
    args = ap.parse_args()
    if args.mixed_only:
        mixed_only(args)
        return
    if args.kernel_only:
        kernel_only(args)
        return
    world, rank, local = dist_init(args)
    if args.impl == "reference":
        cpu_reference(args, world, rank)
    else:
        gpu_bench(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
