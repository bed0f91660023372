#!/usr/bin/env python
"""f(A)b engine benchmark (one JSON line on rank 0).

Workload (default): nonuniform FE fractional diffusion on a seeded Delaunay
mesh of the unit disk with ~1M nodes (997,710 interior rows, ~7.0M nnz),
A = M^{-1/2} K(kappa) M^{-1/2}, f(x) = x^-0.8, degree-8 Jacobi polynomial
preconditioner, m = 80, 20 deflated eigenvectors, 48 contour shifts, FP64.

A step is one f(A)b evaluation per right-hand side: deflation of a new b
(Z = Q^T b, U = b - Q Z, update = Q f(L) Z) plus the fused Lanczos + shifted
solves + lift launch.  ``value`` times steps with b already in HBM; ``e2e``
times the same steps through the C ABI with pinned host buffers (host->device
copy of b and device->host copy of f(A)b inside the timed region).

``--impl reference`` times the reference's CPU algorithm (nicksmethodcpu.m,
restated in C/OpenMP because MATLAB is not available) on the host cores.
Several GPUs run independent replicas (the path does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "f(A)b solves/sec + HBM GB/s at rel-err 1e-6 vs FP64 oracle; mixed/batched vs plain FP64"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="fe-disk-1M")
    ap.add_argument("--nrhs", type=int, default=1)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the mixed/batched and oracle checks")
    ap.add_argument("--no-config-extras", action="store_true",
                    help="skip the 256^3, batch-64 and adjoint-250k fields of the default line")
    ap.add_argument("--cpu-sample-s", type=float, default=30.0)
    ap.add_argument("--threads", type=int, default=0, help="threads per block (0: engine default)")
    ap.add_argument("--bps", type=int, default=0, help="resident blocks per SM (0: engine default)")
    ap.add_argument("--max-blocks", type=int, default=0, help="cap on the grid size (0: engine default)")
    ap.add_argument("--diag-compensation", type=int, default=0, choices=[0, 1],
                    help="mixed engine: 0 = diagonal-compensated FP32 matrix, 1 = plain FP32 values")
    ap.add_argument("--col-staging", type=int, default=0, choices=[0, 1, 2],
                    help="SELL column indices staged in shared memory by TMA: 0 auto (when the matrix is "
                         "not held in L2), 1 off, 2 on")
    ap.add_argument("--matrix-powers", type=int, default=None, choices=[0, 1],
                    help="1: two Horner levels of the polynomial per SpMV pass "
                         "(default: off for the f(A)b workloads, on for the adjoint)")
    ap.add_argument("--autotune", default="auto", choices=["auto", "on", "off"],
                    help="launch shape from the autotuner (auto: on for fd2d-* and batch-64, whose small "
                         "problems gain from it; off for the large FE and 3D workloads, where sweeps found the "
                         "engine default best)")
    ap.add_argument("--unfused", action="store_true",
                    help="step = build_subspace + lin_sys_solves + apply_V (three launches) instead of gm_solve")
    ap.add_argument("--val-prefetch", type=int, default=0, choices=[0, 1, 2],
                    help="L2 bulk prefetch of SELL values: 0 auto (matrix not L2-resident), 1 on, 2 off")
    ap.add_argument("--reorth", type=int, default=0, choices=[0, 1, 2],
                    help="Gram-Schmidt reorthogonalisation passes per Lanczos step (0: the reference's recurrence)")
    ap.add_argument("--l2-window", type=int, default=0, choices=[0, 1, 2],
                    help="0: keep the SELL matrix in L2 (persisting window) when it and one pass's vectors "
                         "fit, 1: off, 2: on whenever the matrix fits the persisting limit")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during a region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev: int):
        self.dev = dev
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        out, _ = self.p.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(workload: str, precision: str, nrhs: int):
    """DRAM bytes per fused launch of this workload from the committed ncu
    summaries: a line ``traffic[<workload>/<precision>/R<nrhs>]: <bytes>`` in
    profiles/*.md (measured on that launch, or scaled from a smaller capture
    of the same kernel, as the summary says)."""
    base = workload[:-len("-mixed")] if workload.endswith("-mixed") else workload
    base = base[:-len("-fp64")] if base.endswith("-fp64") else base
    key = f"traffic[{base}/{precision}/R{nrhs}]:"
    pdir = os.path.join(ROOT, "profiles")
    try:
        names = sorted(os.listdir(pdir))
    except OSError:
        return None
    for name in names:
        if not name.endswith(".md"):
            continue
        with open(os.path.join(pdir, name)) as fh:
            for line in fh:
                if line.startswith(key):
                    return float(line.split(":", 1)[1])
    return None


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    import platform
    import subprocess
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.machine()


def cpu_sample(P, U_defl, budget_s: float, threads: int):
    """Time the reference CPU algorithm on the host (bounded sample)."""
    from oracle import cpu_fab
    th = threads or cpu_fab.max_threads()
    t0 = time.perf_counter()
    cpu_fab.run(P.A, U_defl[:, :1], P.m, P.gamma, P.gs_re, P.gs_im, P.wts[:1], P.sigma, threads=th)
    t1 = time.perf_counter() - t0
    reps = 1
    while time.perf_counter() - t0 + t1 < budget_s and reps < 5:
        cpu_fab.run(P.A, U_defl[:, :1], P.m, P.gamma, P.gs_re, P.gs_im, P.wts[:1], P.sigma, threads=th)
        reps += 1
    dt = (time.perf_counter() - t0) / reps
    return dict(value=1.0 / dt, unit="solves/s", cores=int(th), kind="port", cpu_model=cpu_model(),
                host_cpus=os.cpu_count(),
                sample=f"{reps} full f(A)b solve(s) of 1 RHS (n={P.n}, m={P.m}, d={P.d}, C={P.C}) "
                       f"by the C/OpenMP restatement of nicksmethodcpu.m; {dt:.3f} s each")


def host_deflate(P, B):
    Q = P.Q
    if Q.shape[1] == 0:
        return B.copy()
    return B - Q @ (Q.T @ B)


def run_reference(args, P, rank):
    from gpumatfun_gb300 import replicas
    if not replicas.rank0_only(rank):
        return
    from oracle import cpu_fab
    th = cpu_fab.max_threads()
    U = host_deflate(P, P.U)
    t0 = time.perf_counter()
    cpu_fab.run(P.A, U[:, :1], P.m, P.gamma, P.gs_re, P.gs_im, P.wts[:1], P.sigma, threads=th)
    one = time.perf_counter() - t0
    budget = 150.0
    steps = max(1, min(args.steps, int(budget // max(one, 1e-9))))
    warm = min(args.warmup, max(0, int((budget - steps * one) // max(one, 1e-9))))
    for _ in range(warm):
        cpu_fab.run(P.A, U[:, :1], P.m, P.gamma, P.gs_re, P.gs_im, P.wts[:1], P.sigma, threads=th)
    t0 = time.perf_counter()
    for _ in range(steps):
        cpu_fab.run(P.A, U[:, :1], P.m, P.gamma, P.gs_re, P.gs_im, P.wts[:1], P.sigma, threads=th)
    dt = (time.perf_counter() - t0) / steps
    v = 1.0 / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": warm, "requested_steps": args.steps, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_of(args, P),
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": th, "kind": "port",
                             "cpu_model": cpu_model(), "host_cpus": os.cpu_count(),
                             "sample": f"{steps} full f(A)b solve(s) of 1 RHS by the C/OpenMP restatement of "
                                       "nicksmethodcpu.m (MATLAB CPU path); host-side deflation excluded"},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def use_autotune(args) -> bool:
    if args.autotune != "auto":
        return args.autotune == "on"
    return args.workload.startswith("fd2d-") or args.workload == "batch-64"


def config_of(args, P):
    return {"workload": P.name, "n": int(P.n), "nnz": int(P.A.nnz), "m": int(P.m), "C": int(P.C),
            "d": int(P.d), "k": int(P.k), "nrhs": int(args.nrhs), "precision": args.precision,
            "f": P.meta.get("f", "x^-0.8" if "disk" in P.name else "exp(-tau x^(alpha/2))"),
            "l2": "inputs larger than L2 (Krylov basis m x n x 8 B per RHS)",
            "l2_window": ["auto (SELL matrix persisting in L2 when it and one pass's vectors fit)", "off",
                          "on"][args.l2_window],
            "reorth": ["none (reference recurrence)", "CGS", "CGS2"][args.reorth],
            "parallelism": f"replicas x{args.gpus}"}


def run_ours(args, P, rank, world, local):
    import torch
    from gpumatfun_gb300 import Engine, replicas, roofline
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    R, K, W = args.nrhs, args.steps, args.warmup
    shape = dict(threads=args.threads, blocks_per_sm=args.bps, col_staging=args.col_staging,
                 matrix_powers=args.matrix_powers or 0)
    tuned = None
    if use_autotune(args):
        from gpumatfun_gb300 import autotune
        tuned = autotune.tune(P, args.precision, reps=3, device=torch.cuda.get_device_name(local))
        shape = {k: tuned[k] for k in ("threads", "blocks_per_sm", "col_staging", "sync_policy", "matrix_powers")}
        shape["sell_sigma"] = tuned.get("sell_sigma", 0)
    eng = Engine.from_problem(P, precision=args.precision, sync=False, l2_window=args.l2_window,
                              diag_compensation=args.diag_compensation, max_blocks=args.max_blocks,
                              reorth=args.reorth, val_prefetch=args.val_prefetch, **shape)
    eng.set_stream(stream.cuda_stream)
    n = P.n
    gen = torch.Generator(device=dev).manual_seed(1234 + rank)
    B = torch.rand((K + W, R, n), dtype=torch.float64, device=dev, generator=gen)
    B /= B.norm(dim=2, keepdim=True)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def step(i):
        eng.set_U_device(B[i].data_ptr())
        if args.unfused:
            eng.build_subspace()
            eng.lin_sys_solves()
            eng.apply_V()
        else:
            eng.solve()

    with torch.cuda.stream(stream):
        for i in range(W):
            step(i)
        torch.cuda.synchronize()
        barrier()
        clk = ClockSampler(local)
        clk.start()
        l0 = eng.info()["launches"]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for i in range(W, W + K):
            step(i)
        e1.record(stream)
        torch.cuda.synchronize()
        ms_step = e0.elapsed_time(e1) / K
        launches = eng.info()["launches"] - l0
        barrier()
        # dominant kernel alone: the fused Lanczos + solves + lift launch
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(K):
            eng.solve()
        f1.record(stream)
        torch.cuda.synchronize()
        ms_fused = f0.elapsed_time(f1) / K
        clocks = clk.stop()
    eng.sync()
    x_last = eng.get_solution()
    ms_step, ms_fused = replicas.max_over_ranks([ms_step, ms_fused], device=dev)
    value = world * R * 1e3 / ms_step

    # end to end through the C ABI with pinned host buffers
    Bh = torch.rand((K + 1, R, n), dtype=torch.float64, generator=torch.Generator().manual_seed(99 + rank))
    Bh /= Bh.norm(dim=2, keepdim=True)
    Bh = Bh.pin_memory()
    Xh = torch.empty((K + 1, R, n), dtype=torch.float64).pin_memory()
    lib, h = eng._lib, eng._h
    import ctypes as ct
    dp = ct.POINTER(ct.c_double)
    rc = lib.gm_solve_host(h, ct.cast(Bh[0].data_ptr(), dp), ct.cast(Xh[0].data_ptr(), dp))
    assert rc == 0, lib.gm_last_error(h)
    barrier()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    g0.record(stream)
    w0 = time.perf_counter()
    for i in range(1, K + 1):
        rc = lib.gm_solve_host(h, ct.cast(Bh[i].data_ptr(), dp), ct.cast(Xh[i].data_ptr(), dp))
        assert rc == 0, lib.gm_last_error(h)
    g1.record(stream)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - w0) / K
    ms_e2e = g0.elapsed_time(g1) / K
    ms_e2e, wall = replicas.max_over_ranks([ms_e2e, wall], device=dev)
    e2e = {"value": world * R * 1e3 / ms_e2e, "unit": "solves/s", "h2d_bytes_per_step": 8 * n * R,
           "d2h_bytes_per_step": 8 * n * R, "host_wall_ms_per_step": wall * 1e3}

    info = eng.info()
    sizes = roofline.Sizes(n=n, nnz=int(P.A.nnz), R=R, m=P.m, d=P.d, C=P.C, k=P.k, mixed=args.precision == "mixed",
                           reorth=args.reorth)
    alg = roofline.fused_solve_bytes(sizes)
    peak, peak_kind = measured_peaks()
    achieved = alg / (ms_fused * 1e-3) / 1e9
    # the committed ncu summary covers the FP64 single-RHS launch of this workload
    traffic = profiled_traffic(P.name, args.precision, R) if args.reorth == 0 else None
    roof = {"bound": "hbm", "kernel": "fab_kernel (fused Lanczos + shifted solves + lift)",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_kind": f"{peak_kind} copy bandwidth (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
            else "fallback 6.8 TB/s", "traffic": traffic, "algorithmic_bytes_per_launch": alg,
            "ms_per_launch": ms_fused,
            "frac_kind": ("effective: algorithmic bytes over the launch time; the SELL matrix is served from "
                          "the L2 persisting window on every pass after the first, so DRAM moves fewer bytes "
                          "(dram_frac)") if info["l2_window_bytes"] else
                         ("algorithmic bytes over the launch time; no L2 window: the SELL matrix streams from "
                          "HBM on every pass (column staging, value prefetch)"),
            "l2_window_bytes": info["l2_window_bytes"],
            "dram_achieved": traffic / (ms_fused * 1e-3) / 1e9 if traffic else None,
            "dram_frac": traffic / (ms_fused * 1e-3) / 1e9 / peak if traffic else None,
            "fp64_tflops": roofline.fused_solve_flops(sizes) / (ms_fused * 1e-3) / 1e12}
    if args.precision == "fp64":
        # the FP64 pipe is the binding unit on GB300 (2 FMA lanes per clock per
        # SM); its peak at the SM clock sampled during the timed region
        mhz = (clocks or {}).get("sm_mhz") or 0.0
        nsm = torch.cuda.get_device_properties(dev).multi_processor_count
        if mhz:
            peak64 = 2 * 2 * nsm * mhz * 1e6 / 1e12
            roof["fp64_peak_tflops"] = peak64
            roof["fp64_frac"] = roof["fp64_tflops"] / peak64

    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32-storage/f64-recurrence",
            "data": "synthetic (seeded disk mesh, Gaussian-field coefficient, uniform b)",
            "config": config_of(args, P), "e2e": e2e, "gpu_launches": int(launches),
            "roofline": roof, "clocks": clocks,
            "engine": {"grid_blocks": info["grid_blocks"], "threads": info["threads"],
                       "matrix_powers": info["matrix_powers"], "value_prefetch_bytes": info["value_prefetch_bytes"],
                       "launch_shape": dict(shape, autotuned=tuned is not None,
                                            cached=bool(tuned and tuned.get("cached"))),
                       "sell_padded": info["sell_padded"], "device_bytes": info["device_bytes"]}}
    eng.delete()
    del B
    torch.cuda.empty_cache()

    if rank == 0 and not args.no_extras:
        line["accuracy"] = accuracy_checks(P, args.precision)
        if args.precision == "fp64":
            line["mixed_batched"] = mixed_batched(P, K, W, dev, stream, x_ref_engine=None)
            if args.reorth == 0:
                line["reorth_cgs"] = reorth_extra(P, K, W, stream)
    if rank == 0 and not args.no_extras and not args.no_config_extras and P.name.startswith("fe-disk-1M"):
        # the other configurations of the metric, measured in the same run:
        # 256^3 mixed and FP64 (the largest single-GPU configuration), the
        # 64-problem batch against the plain FP64 single-solve engine, and the
        # 250k-node adjoint with its finite-difference checks
        ke, we = max(3, min(K, 10)), max(3, min(W, 3))
        line["fd3d_256"] = _extra("fd3d_256", fd3d_measure, 256, ke, we)
        line["fd2d_256"] = _extra("fd2d_256", fd2d_measure, 20, 5)
        line["batch_64"] = _extra("batch_64", batch_measure, ke, we, tune=False, monodomain=True)
        if "mixed_batched_over_fp64_single" in line["batch_64"]:
            line["mixed_batched_over_plain_fp64"] = {
                "batch_64": line["batch_64"]["mixed_batched_over_fp64_single"],
                "fe_disk_1M_R4": line.get("mixed_batched", {}).get("mixed_solves_per_s", 0.0) / (R * 1e3 / ms_fused),
                "note": "mixed engine, 4 right-hand sides per launch, over the plain FP64 engine with one "
                        "right-hand side per launch; fused launches on both sides"}
        line["adjoint_250k"] = _extra("adjoint_250k", adjoint_measure, 250_000, 3, 2)
        line["deflation_gpu"] = _extra("deflation_gpu", deflation_measure, P)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_sample(P, host_deflate(P, P.U), args.cpu_sample_s, 0)
    if rank == 0:
        print(json.dumps(line), flush=True)


def accuracy_checks(P, precision):
    """On the workload's own b: the FP64 engine against the FP64 oracle (when
    the oracle is affordable, n <= 2M) and, for the mixed engine, the mixed
    result against the FP64 engine run."""
    from gpumatfun_gb300 import Engine
    out = {}
    eng = Engine.from_problem(P, precision="fp64")
    eng.solve()
    x = eng.get_solution()
    eng.delete()
    if precision == "mixed":
        em = Engine.from_problem(P, precision="mixed")
        em.solve()
        xm = em.get_solution()
        em.delete()
        out["mixed_vs_fp64_engine_rel_err"] = float(np.linalg.norm(xm - x) / np.linalg.norm(x))
    if P.n <= 2_000_000:
        from oracle import fab
        t0 = time.perf_counter()
        ora = fab.OracleEngine(A=P.A, U0=P.U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                               flam=P.flam, wts=P.wts, shifts=P.shifts, col_scale=np.ones(P.R))
        want = ora.solve()
        out["fp64_vs_oracle_rel_err"] = float(np.linalg.norm(x - want) / np.linalg.norm(want))
        out["oracle_s"] = time.perf_counter() - t0
    return out


def reorth_extra(P, K, W, stream):
    """The same workload with classical Gram-Schmidt against the stored basis
    in every Lanczos step: fused-launch solves/s, algorithmic GB/s with the
    extra basis reads, and the change of f(A)b against the plain recurrence."""
    import torch
    from gpumatfun_gb300 import Engine, roofline
    eng = Engine.from_problem(P, precision="fp64", sync=False, reorth=1)
    eng.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        for _ in range(max(1, W)):
            eng.solve()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(K):
            eng.solve()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / K
    x = eng.get_solution()
    eng.delete()
    e = Engine.from_problem(P, precision="fp64", sync=False)
    e.solve()
    x0 = e.get_solution()
    e.delete()
    sz = roofline.Sizes(n=P.n, nnz=int(P.A.nnz), R=P.R, m=P.m, d=P.d, C=P.C, k=P.k, reorth=1)
    alg = roofline.fused_solve_bytes(sz)
    extra = sum(roofline.reorth_step_bytes(sz, j) for j in range(P.m))
    return {"solves_per_s": P.R * 1e3 / ms, "ms_per_launch": ms, "algorithmic_gb_per_s": alg / (ms * 1e-3) / 1e9,
            "reorth_bytes_per_launch": extra, "algorithmic_bytes_per_launch": alg,
            "rel_change_vs_plain_recurrence": float(np.linalg.norm(x - x0) / np.linalg.norm(x0)),
            "note": "fused launch, workload's own b, FP64 dots; reorth bytes are Gram-Schmidt reads/writes"}


def mixed_batched(P, K, W, dev, stream, x_ref_engine=None):
    """Mixed-precision engine with 4 right-hand sides per launch (and with the
    workload's own single right-hand side): solves/s and relative error
    against the FP64 engine on the same b."""
    import torch
    from gpumatfun_gb300 import Engine, workloads
    R = 4
    rng = np.random.default_rng(7)
    U = rng.random((P.n, R))
    U /= np.linalg.norm(U, axis=0, keepdims=True)
    P4 = workloads.make_problem(P.name, P.A, U, P.Q, P.lam, [P.funcs[0]] * R, P.m, P.C, P.l1, P.lN,
                                degree=P.d, prob_dim=P.lN / 4)
    out = {}
    for prec in ("fp64", "mixed", "mixed1"):
        eng = Engine.from_problem(P4 if prec != "mixed1" else P, precision=prec[:5], sync=False)
        eng.set_stream(stream.cuda_stream)
        with torch.cuda.stream(stream):
            for _ in range(max(1, W)):
                eng.solve()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(K):
                eng.solve()
            e1.record(stream)
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / K
        out[prec] = ((R if prec != "mixed1" else P.R) * 1e3 / ms, eng.get_solution())
        eng.delete()
    x64, xm = out["fp64"][1], out["mixed"][1]
    err = float(np.max(np.linalg.norm(xm - x64, axis=0) / np.linalg.norm(x64, axis=0)))
    return {"nrhs": R, "mixed_solves_per_s": out["mixed"][0], "fp64_batched_solves_per_s": out["fp64"][0],
            "mixed_rel_err_vs_fp64_engine": err, "mixed_single_rhs_solves_per_s": out["mixed1"][0],
            "note": "fused launch only (b resident, deflation excluded); same b for both precisions"}


def adjoint_measure(n_target: int, K: int, W: int, matrix_powers=None, fd_directions: int = 64) -> dict:
    """Adjoint workload: x = f(A(kappa)) b on the FE disk with ``n_target``
    nodes, loss L = 1/2 ||x - d||^2, one step = forward + backward
    (dL/dkappa per triangle and dL/db) through the same calls
    torch.autograd uses (the backward reuses the forward's stored Krylov
    state), in FP64 and with FP32 storage; then central finite differences of
    the loss on random directions (the configured check: white-noise
    directions v = kappa * N(0, 1) at step 1e-6, beside step 1e-3 and smooth
    Gaussian-field directions), in both precisions."""
    import torch
    from gpumatfun_gb300 import adjoint, workloads
    t0 = time.perf_counter()
    mesh, kappa, kstar, b = workloads.adjoint_case(n_target)
    prm = dict(workloads.ADJOINT_PARAMS)
    out = {}
    ops = {}
    for prec in ("fp64", "mixed"):
        mp = 1 if matrix_powers is None else matrix_powers
        ops[prec] = adjoint.FracFEOperator(mesh, kappa, precision=prec, matrix_powers=mp, **prm)
    setup_s = time.perf_counter() - t0
    op = ops["fp64"]
    dev = torch.device("cuda", 0)
    kt = torch.as_tensor(kappa, device=dev)
    bt = torch.as_tensor(b, device=dev)
    xs = op.forward(torch.as_tensor(kstar, device=dev), bt)
    gen = torch.Generator(device=dev).manual_seed(5)
    noise = torch.randn(xs.shape, generator=gen, device=dev, dtype=torch.float64)
    d = xs + 0.01 * xs.norm() / xs.numel() ** 0.5 * noise
    grads = {}
    for prec, o in ops.items():
        for _ in range(W):
            x = o.forward(kt, bt)
            o.backward(kt, bt, x - d)
        torch.cuda.synchronize()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        tf = tb = 0.0
        for _ in range(K):
            e[0].record()
            x = o.forward(kt, bt)
            g = x - d
            e[1].record()
            dk, db = o.backward(kt, bt, g)
            e[2].record()
            torch.cuda.synchronize()
            tf += e[0].elapsed_time(e[1])
            tb += e[1].elapsed_time(e[2])
        grads[prec] = (dk.clone(), db.cpu().numpy(), x.cpu().numpy())
        out[prec] = {"grad_evals_per_s": 1e3 * K / (tf + tb), "forward_ms": tf / K, "backward_ms": tb / K}
    # end to end with host buffers (numpy in, numpy out), FP64
    kh, bh = np.ascontiguousarray(kappa), np.ascontiguousarray(b)
    dh = d.cpu().numpy()
    xh = np.empty_like(bh)
    dkh = np.empty(op.ntri)
    dbh = np.empty_like(bh)
    op.engine.set_stream(None)
    t1 = time.perf_counter()
    for _ in range(K):
        op.engine.fe_forward(kh.ctypes.data, bh.ctypes.data, xh.ctypes.data)
        gh = xh - dh
        op.engine.fe_backward_stored(gh.ctypes.data, dkh.ctypes.data, dbh.ctypes.data)
    e2e_s = (time.perf_counter() - t1) / K
    op._stream = None
    dk64, db64, x64 = grads["fp64"]
    dkm, dbm, xm = grads["mixed"]
    rel = lambda a, r: float(np.linalg.norm(a - r) / np.linalg.norm(r))

    # Central finite differences of the loss.  The rounding noise of the loss
    # itself is measured by perturbing kappa by 1e-14 relative; noise / h
    # bounds what a step h can resolve.
    from gpumatfun_gb300 import problems as _pb
    cent = mesh.nodes[mesh.tris].mean(axis=1)
    t2 = time.perf_counter()
    fd_out = {"directions": fd_directions,
              "err": "|FD - adjoint| / rms(adjoint) over the directions; noise_bound = loss noise / h "
                     "in the same units"}
    for prec, o in ops.items():
        dkt = grads[prec][0]

        def loss(k):
            xx = o.forward(k, bt)
            return 0.5 * float(torch.sum((xx - d) ** 2))
        L0 = loss(kt)
        lnoise = max(abs(loss(kt * (1 + 1e-14 * torch.randn(kt.shape, generator=gen, device=dev,
                                                               dtype=torch.float64))) - L0) for _ in range(3))
        # the configured check: white-noise directions, step 1e-6 (and 1e-3)
        dirs = [kt * torch.randn(kt.shape, generator=gen, device=dev, dtype=torch.float64)
                for _ in range(fd_directions)]
        ads = np.array([float(torch.dot(dkt, v)) for v in dirs])
        rms = float(np.sqrt(np.mean(ads ** 2)))
        res = {"loss": L0, "loss_noise": lnoise}
        for h in (1e-6, 1e-3):
            fds = np.array([(loss(kt + h * v) - loss(kt - h * v)) / (2 * h) for v in dirs])
            err = np.abs(fds - ads) / rms
            res[f"white_h={h:g}"] = {"max_err": float(err.max()), "median_err": float(np.median(err)),
                                     "noise_bound": float(lnoise / h / rms)}
        # smooth directions v = kappa * g, g a Gaussian random field (sigma 1,
        # correlation length 0.1) at the triangle centroids: directional
        # derivatives large against the loss noise
        sdirs = [kt * torch.as_tensor(_pb.gaussian_random_field(cent, sigma=1.0, ell=0.1, seed=1000 + s),
                                      device=dev) for s in range(fd_directions)]
        sads = np.array([float(torch.dot(dkt, v)) for v in sdirs])
        srms = float(np.sqrt(np.mean(sads ** 2)))
        h = 1e-3
        c1 = np.array([(loss(kt + h * v) - loss(kt - h * v)) / (2 * h) for v in sdirs])
        serr = np.abs(c1 - sads) / srms
        res["smooth_h=0.001"] = {"max_err": float(serr.max()), "median_err": float(np.median(serr)),
                                 "noise_bound": float(lnoise / h / srms), "rms_directional_derivative": srms}
        fd_out[prec] = res
    fd_out["seconds"] = time.perf_counter() - t2
    res = {"config": {"n": int(op.n), "ntri": int(op.ntri), **prm, "l1": op.l1, "lN": op.lN,
                      "matrix_powers": int(op.engine.info()["matrix_powers"])},
           "fp64": out["fp64"], "mixed": out["mixed"],
           "e2e_grad_evals_per_s": 1.0 / e2e_s,
           "e2e_bytes": {"h2d_bytes_per_step": 8 * (2 * op.ntri + 3 * op.n), "d2h_bytes_per_step": 8 * (op.ntri + 2 * op.n)},
           "mixed_vs_fp64": {"x": rel(xm, x64), "dL_dkappa": rel(dkm.cpu().numpy(), dk64.cpu().numpy()),
                             "dL_db": rel(dbm, db64)},
           "finite_differences": fd_out, "setup_s": setup_s}
    for o in ops.values():
        o.delete()
    return res


def run_adjoint(args):
    """The adjoint workload's own JSON line (``--workload fe-adjoint-<n>k``)."""
    n_target = int(args.workload.split("-")[-1].replace("k", "000"))
    K, W = args.steps, args.warmup
    r = adjoint_measure(n_target, K, W, matrix_powers=args.matrix_powers)
    line = {"metric": "adjoint gradient evaluations/s (forward + backward: dL/dkappa per triangle and dL/db)",
            "value": r["fp64"]["grad_evals_per_s"], "unit": "grad-evals/s", "n_gpus": 1, "steps": K, "warmup": W,
            "ms_per_step": r["fp64"]["forward_ms"] + r["fp64"]["backward_ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded disk mesh, two Gaussian-field coefficients kappa and kappa*, uniform b, "
                    "d = f(A(kappa*)) b + 1% noise)",
            "config": {"workload": args.workload, **r["config"]},
            "e2e": {"value": r["e2e_grad_evals_per_s"], "unit": "grad-evals/s", **r["e2e_bytes"]},
            **{k: r[k] for k in ("fp64", "mixed", "mixed_vs_fp64", "finite_differences", "setup_s")}}
    print(json.dumps(line), flush=True)


def _timed_solves(eng, stream, K, W):
    """Device time of K back-to-back fused solves on ``stream`` (ms per solve)."""
    import torch
    eng.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        for _ in range(max(1, W)):
            eng.solve()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(K):
            eng.solve()
        e1.record(stream)
        torch.cuda.synchronize()
    return e0.elapsed_time(e1) / K


# Launch shape of the 256^2 FD solve when it is not autotuned: the one the
# autotuner chose on GB300 (256-thread blocks, one block per SM, no column
# staging, grid barriers between passes; the solve is latency-bound).
FD2D_SHAPE = dict(threads=256, blocks_per_sm=1, col_staging=1, sync_policy=1)


def fd2d_measure(K: int, W: int) -> dict:
    """Config 1 (2D 5-point Dirichlet Laplacian on 256^2, FP64, m = 60,
    C = 32, k = 10 analytic sine modes, no preconditioner): fused-launch
    solves/s with the engine's default launch shape and with the autotuner's
    shape, the error against the FP64 oracle, and against the exact DST-I
    solution (the Krylov truncation error of m = 60, as in the reference)."""
    import torch
    from gpumatfun_gb300 import Engine, workloads
    from oracle import fab, known
    P = workloads.cached_problem("fd2d-256")
    stream = torch.cuda.Stream()
    out = {"config": {"workload": "fd2d-256", "n": int(P.n), "nnz": int(P.A.nnz), "m": P.m, "C": P.C, "d": P.d,
                      "k": P.k, "nrhs": P.R, "precision": "fp64"}}
    x = None
    for tag, shape in (("default_shape", {}), ("autotuned_shape", FD2D_SHAPE)):
        eng = Engine.from_problem(P, precision="fp64", sync=False, **shape)
        ms = _timed_solves(eng, stream, K, W)
        x = eng.get_solution()
        info = eng.info()
        eng.delete()
        out[tag] = {"solves_per_s": P.R * 1e3 / ms, "ms_per_launch": ms, "grid_blocks": info["grid_blocks"],
                    "threads": info["threads"], **({"shape": shape} if shape else {})}
    ora = fab.OracleEngine(A=P.A, U0=P.U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                           flam=P.flam, wts=P.wts, shifts=P.shifts,
                           col_scale=P.col_scale if P.col_scale is not None else np.ones(P.R))
    want = ora.solve()
    out["rel_err_vs_fp64_oracle"] = float(np.linalg.norm(x - want) / np.linalg.norm(want))
    exact = known.dst_fab_2d(P.U[:, 0], int(P.meta["N"]), P.funcs[0], scale=float(P.meta["scale"]))
    xr = x.reshape(P.n, -1)[:, 0]
    out["rel_err_vs_exact_dst"] = float(np.linalg.norm(xr - exact) / np.linalg.norm(exact))
    return out


# Launch shape of the batch when it is not autotuned: the one the autotuner
# chose on GB300 for both precisions (256-thread blocks, grid barriers
# between passes, column staging on, residency from the occupancy limit).
BATCH_SHAPE = dict(threads=256, blocks_per_sm=0, col_staging=2, sync_policy=1)


def batch_measure(K: int, W: int, tune: bool, monodomain: bool = True) -> dict:
    """Batched serving-style workload: 64 fractional-diffusion problems of
    uneven size (N^2 grids, N log-uniform in [64, 1024]), 4 right-hand sides
    each, one persistent launch, in both precisions; against the plain FP64
    single-solve engine (one problem, one right-hand side per launch) on the
    same 256 solves.  Optionally the fractional monodomain time loop (512^2,
    200 steps, CUDA graph)."""
    import torch
    from gpumatfun_gb300 import BatchEngine, Engine, LanczosEngine, autotune, workloads
    t0 = time.perf_counter()
    probs = workloads.config5_batch()
    setup_s = time.perf_counter() - t0
    nsolves = sum(P.R for P in probs)
    stream = torch.cuda.Stream()
    res, sols = {}, {}
    shapes = {}
    e2e_ms = n_total = None
    for prec in ("mixed", "fp64"):
        shape = dict(BATCH_SHAPE)
        if tune:
            # row-block size, residency, staging and pass ordering tuned on this batch
            t = autotune.tune_batch(probs, precision=prec, reps=2, device=torch.cuda.get_device_name())
            shape = {k: t[k] for k in ("threads", "blocks_per_sm", "col_staging", "sync_policy")}
            default = [c for c in t.get("timed", []) if c["threads"] == 512 and c["blocks_per_sm"] == 0
                       and c["col_staging"] == 2 and c["sync_policy"] == 0]
            shapes[prec] = dict(shape, tuned_ms=t["ms"], default_shape_ms=default[0]["ms"] if default else None,
                                cached=t["cached"], candidates=t["trials"])
        else:
            shapes[prec] = dict(shape, autotuned=False)
        eng = BatchEngine(probs, precision=prec, sync=False, **shape)
        ms = _timed_solves(eng, stream, K, W)
        sols[prec] = eng.split(eng.get_solution())
        res[prec] = {"ms_per_launch": ms, "solves_per_s": nsolves * 1e3 / ms, "grid_blocks": eng.info()["grid_blocks"],
                     "device_bytes": eng.info()["device_bytes"]}
        if prec == "mixed":
            # end to end: host right-hand sides in, host solutions out, every step
            Uh = np.ascontiguousarray(np.concatenate([P.U for P in probs]))
            eng.set_stream(None)
            eng.set_U(Uh); eng.solve(); eng.get_solution()
            t1 = time.perf_counter()
            for _ in range(K):
                eng.set_U(Uh)
                eng.solve()
                eng.get_solution()
            e2e_ms = (time.perf_counter() - t1) * 1e3 / K
            n_total = int(Uh.shape[0])
        eng.delete()
    errs = [float(np.max(np.linalg.norm(a - b, axis=0) / np.linalg.norm(b, axis=0)))
            for a, b in zip(sols["mixed"], sols["fp64"])]
    # the plain FP64 single-solve engine: each problem alone, one right-hand side per launch
    single_ms = 0.0
    for P in probs:
        P1 = workloads.make_problem(P.name, P.A, P.U[:, :1], P.Q, P.lam, P.funcs[:1], P.m, P.C, P.l1, P.lN,
                                    degree=P.d)
        e = Engine.from_problem(P1, precision="fp64", sync=False)
        single_ms += P.R * _timed_solves(e, stream, max(2, K // 2), 1)
        e.delete()
    single = nsolves * 1e3 / single_ms
    sizes = [int(P.meta["N"]) for P in probs]
    out = {"config": {"workload": "batch-64", "problems": len(probs), "nrhs": probs[0].R,
                      "grid_N": [min(sizes), max(sizes)], "rows_total": int(sum(P.n for P in probs)),
                      "m": probs[0].m, "C": probs[0].C,
                      "f": "exp(-dt K_alpha lambda^0.75), dt 0.05, K_alpha 1e-4, side 2.5"},
           "mixed_batched": res["mixed"], "fp64_batched": res["fp64"], "launch_shape": shapes,
           "fp64_single_solve": {"solves_per_s": single, "note": "each problem alone, 1 RHS per launch"},
           "mixed_batched_over_fp64_single": res["mixed"]["solves_per_s"] / single,
           "mixed_vs_fp64_rel_err": {"worst": max(errs), "median": float(np.median(errs))},
           "e2e_solves_per_s": nsolves * 1e3 / e2e_ms,
           "e2e_bytes": {"h2d_bytes_per_step": 8 * n_total * probs[0].R, "d2h_bytes_per_step": 8 * n_total * probs[0].R},
           "setup_s": setup_s}
    if not monodomain:
        return out
    # fractional monodomain time loop, CUDA graph of 200 steps
    Pm, dt, ode, fhn = workloads.monodomain_problem(512)
    mono = {}
    Us = {}
    mono_shapes = {}
    for prec in ("mixed", "fp64"):
        mshape = {}
        if tune:
            t = autotune.tune(Pm, prec, reps=2, device=torch.cuda.get_device_name())
            mshape = {k: t[k] for k in ("threads", "blocks_per_sm", "col_staging", "sync_policy", "matrix_powers")}
            mshape["sell_sigma"] = t.get("sell_sigma", 0)
            mono_shapes[prec] = dict(mshape, tuned_ms=t["ms"])
        e = LanczosEngine(Pm.U, Pm.A, Pm.Q, Pm.lam, Pm.m, Pm.gamma, Pm.gs_re, Pm.gs_im, Pm.flam[:, 0],
                          Pm.flam[:, 1], dt, ode, fhn["aode"], fhn["bode"], fhn["code"], fhn["vrest"],
                          fhn["vamp"], fhn["vth"], fhn["vpeak"], fhn["c1ion"], fhn["c2ion"], np.ones(Pm.n),
                          Pm.wts[0], Pm.wts[1], Pm.shifts, precision=prec, sync=False, **mshape)
        e.set_stream(stream.cuda_stream)
        e.time_loop(200, monodomain=True, graph=True)   # capture + first replay
        Us[prec] = e.get_U()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        e.time_loop(200, monodomain=True, graph=True)
        e1.record(stream)
        torch.cuda.synchronize()
        mono[prec] = {"steps_per_s": 200e3 / e0.elapsed_time(e1), "ms_per_step": e0.elapsed_time(e1) / 200}
        e.delete()
    mono_err = float(np.linalg.norm(Us["mixed"][:, 0] - Us["fp64"][:, 0]) / np.linalg.norm(Us["fp64"][:, 0]))
    out["monodomain_512"] = {**{f"{p}_steps_per_s": mono[p]["steps_per_s"] for p in mono},
                             "steps": 200, "graph": True, "m": Pm.m, "C": Pm.C, "k": Pm.k,
                             "mixed_vs_fp64_after_200_steps": mono_err,
                             "launch_shape": mono_shapes or "engine default"}
    return out


def run_batch(args):
    """The batched workload's own JSON line (``--workload batch-64``)."""
    K, W = args.steps, args.warmup
    r = batch_measure(K, W, tune=use_autotune(args), monodomain=True)
    line = {"metric": "batched f(A)b solves/s (64 uneven fractional-diffusion problems x 4 RHS, one launch)",
            "value": r["mixed_batched"]["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "steps": K, "warmup": W,
            "ms_per_step": r["mixed_batched"]["ms_per_launch"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32-storage/f64-recurrence",
            "data": "synthetic (seeded grid sizes and right-hand sides)", "config": r["config"],
            "e2e": {"value": r["e2e_solves_per_s"], "unit": "solves/s", **r["e2e_bytes"]},
            **{k: v for k, v in r.items() if k not in ("config", "e2e_solves_per_s", "e2e_bytes")}}
    print(json.dumps(line), flush=True)


def fd3d_measure(N: int, K: int, W: int) -> dict:
    """Config 3 (3D 7-point variable-coefficient Laplacian on N^3, m = 100,
    f = exp(-5e-4 lambda^0.6)) in both precisions: fused-launch solves/s,
    algorithmic GB/s and its fraction of the measured HBM peak (the 1.4 GB
    FP32 / 2.3 GB FP64 matrix is streamed from HBM every pass, so this is a
    DRAM-level figure), the DRAM traffic of the committed ncu summary, and
    the mixed result's error against the FP64 engine on the same b."""
    import torch
    from gpumatfun_gb300 import Engine, roofline, workloads
    t0 = time.perf_counter()
    P = workloads.config3(N=N)
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.Stream()
    peak, _ = measured_peaks()
    out = {"config": {"workload": f"fd3d-{N}", "n": int(P.n), "nnz": int(P.A.nnz), "m": P.m, "C": P.C, "d": P.d,
                      "k": P.k, "nrhs": 1, "f": "exp(-5e-4 x^0.6)"}}
    xs = {}
    for prec in ("mixed", "fp64"):
        eng = Engine.from_problem(P, precision=prec, sync=False)
        ms = _timed_solves(eng, stream, K, W)
        xs[prec] = eng.get_solution()
        info = eng.info()
        eng.delete()
        sz = roofline.Sizes(n=P.n, nnz=int(P.A.nnz), R=1, m=P.m, d=P.d, C=P.C, k=P.k, mixed=prec == "mixed")
        alg = roofline.fused_solve_bytes(sz)
        ach = alg / (ms * 1e-3) / 1e9
        traffic = profiled_traffic(f"fd3d-{N}", prec, 1)
        out[prec] = {"solves_per_s": 1e3 / ms, "ms_per_launch": ms, "algorithmic_bytes_per_launch": alg,
                     "achieved_gb_s": ach, "peak_gb_s": peak, "frac": ach / peak,
                     "traffic": traffic,
                     "dram_frac": (traffic / (ms * 1e-3) / 1e9 / peak) if traffic else None,
                     "grid_blocks": info["grid_blocks"], "value_prefetch_bytes": info["value_prefetch_bytes"],
                     "l2_window_bytes": info["l2_window_bytes"], "col_stage_groups": info["col_stage_groups"]}
    out["mixed_rel_err_vs_fp64_engine"] = float(np.linalg.norm(xs["mixed"] - xs["fp64"]) / np.linalg.norm(xs["fp64"]))
    out["mixed_over_fp64"] = out["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    out["setup_s"] = setup_s
    return out


def deflation_measure(P) -> dict:
    """The workload's k deflation pairs computed on the GPU
    (gm_deflation_pairs: Chebyshev-filtered subspace iteration, FP64) against
    the host shift-invert eigsh pairs the workload was built with: time,
    eigenvalue agreement, residuals and the angle between the subspaces."""
    from gpumatfun_gb300 import eigs
    t0 = time.perf_counter()
    lam, Q, st = eigs.deflation_pairs(P.A, P.k)
    wall = time.perf_counter() - t0
    res = np.linalg.norm(P.A @ Q - Q * lam, axis=0) / np.abs(lam)
    cos = np.linalg.svd(P.Q.T @ Q, compute_uv=False)
    return {"k": int(P.k), "device_s": st["device_s"], "call_wall_s": wall, "iterations": st["iterations"],
            "block_spmvs": st["block_spmvs"], "block_width": 32,
            "max_rel_residual": float(res.max()), "eig_rel_err_vs_eigsh": float(np.max(np.abs(lam - P.lam) / P.lam)),
            "subspace_cos_min_vs_eigsh": float(cos.min()),
            "host_eigsh_s": P.meta.get("eigsh_s"),
            "note": "host_eigsh_s: scipy shift-invert eigsh (k + 1 pairs, sparse LU) when the workload was built "
                    "on this host"}


def _extra(name, fn, *a, **kw):
    """Run one extra measurement; a failure is recorded in the line instead of
    ending the run."""
    import torch
    t0 = time.perf_counter()
    try:
        r = fn(*a, **kw)
        r["wall_s"] = time.perf_counter() - t0
        return r
    except Exception as exc:  # noqa: BLE001 -- reported in the JSON line
        return {"error": f"{type(exc).__name__}: {exc}"[:400], "wall_s": time.perf_counter() - t0}
    finally:
        torch.cuda.empty_cache()


def main():
    args = parse()
    if args.workload == "batch-64":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "batched serving is not a reference workload"}))
        else:
            run_batch(args)
        return
    if args.workload.startswith("fe-adjoint-"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no adjoint"}))
        else:
            run_adjoint(args)
        return
    rank, world, local = dist_env()
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.init_process_group("nccl")
    from gpumatfun_gb300 import workloads
    P = workloads.cached_problem(args.workload, R=args.nrhs)
    if args.impl == "reference":
        run_reference(args, P, rank)
    else:
        run_ours(args, P, rank, world, local)
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
