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
    ap.add_argument("--cpu-sample-s", type=float, default=30.0)
    ap.add_argument("--l2-window", type=int, default=0, choices=[0, 1],
                    help="0: keep the SELL matrix in L2 (persisting window), 1: off")
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


def profiled_traffic(workload: str):
    """DRAM bytes per fused launch from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", f"fab_fused_{workload}.md")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


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
    return dict(value=1.0 / dt, unit="solves/s", cores=int(th), kind="port",
                sample=f"{reps} full f(A)b solve(s) of 1 RHS (n={P.n}, m={P.m}, d={P.d}, C={P.C}) "
                       f"by the C/OpenMP restatement of nicksmethodcpu.m; {dt:.3f} s each")


def host_deflate(P, B):
    Q = P.Q
    if Q.shape[1] == 0:
        return B.copy()
    return B - Q @ (Q.T @ B)


def run_reference(args, P, rank):
    if rank != 0:
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
                             "sample": f"{steps} full f(A)b solve(s) of 1 RHS by the C/OpenMP restatement of "
                                       "nicksmethodcpu.m (MATLAB CPU path); host-side deflation excluded"},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_of(args, P):
    return {"workload": P.name, "n": int(P.n), "nnz": int(P.A.nnz), "m": int(P.m), "C": int(P.C),
            "d": int(P.d), "k": int(P.k), "nrhs": int(args.nrhs), "precision": args.precision,
            "f": P.meta.get("f", "x^-0.8" if "disk" in P.name else "exp(-tau x^(alpha/2))"),
            "l2": "inputs larger than L2 (Krylov basis m x n x 8 B per RHS)",
            "l2_window": "SELL matrix persisting in L2" if args.l2_window == 0 else "off",
            "parallelism": f"replicas x{args.gpus}"}


def run_ours(args, P, rank, world, local):
    import torch
    from gpumatfun_gb300 import Engine, roofline
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    R, K, W = args.nrhs, args.steps, args.warmup
    eng = Engine.from_problem(P, precision=args.precision, sync=False, l2_window=args.l2_window)
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
    if world > 1:
        t = torch.tensor([ms_step, ms_fused], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_step, ms_fused = float(t[0]), float(t[1])
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
    if world > 1:
        t = torch.tensor([ms_e2e, wall], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_e2e, wall = float(t[0]), float(t[1])
    e2e = {"value": world * R * 1e3 / ms_e2e, "unit": "solves/s", "h2d_bytes_per_step": 8 * n * R,
           "d2h_bytes_per_step": 8 * n * R, "host_wall_ms_per_step": wall * 1e3}

    info = eng.info()
    sizes = roofline.Sizes(n=n, nnz=int(P.A.nnz), R=R, m=P.m, d=P.d, C=P.C, k=P.k, mixed=args.precision == "mixed")
    alg = roofline.fused_solve_bytes(sizes)
    peak, peak_kind = measured_peaks()
    achieved = alg / (ms_fused * 1e-3) / 1e9
    # the committed ncu summary covers the FP64 single-RHS launch of this workload
    traffic = profiled_traffic(P.name) if (args.precision == "fp64" and R == 1) else None
    roof = {"bound": "hbm", "kernel": "fab_kernel (fused Lanczos + shifted solves + lift)",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_kind": f"{peak_kind} copy bandwidth (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
            else "fallback 6.8 TB/s", "traffic": traffic, "algorithmic_bytes_per_launch": alg,
            "ms_per_launch": ms_fused,
            "fp64_tflops": roofline.fused_solve_flops(sizes) / (ms_fused * 1e-3) / 1e12}

    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32-storage/f64-recurrence",
            "data": "synthetic (seeded disk mesh, Gaussian-field coefficient, uniform b)",
            "config": config_of(args, P), "e2e": e2e, "gpu_launches": int(launches),
            "roofline": roof, "clocks": clocks,
            "engine": {"grid_blocks": info["grid_blocks"], "threads": info["threads"],
                       "sell_padded": info["sell_padded"], "device_bytes": info["device_bytes"]}}
    eng.delete()
    del B
    torch.cuda.empty_cache()

    if rank == 0 and not args.no_extras:
        line["accuracy"] = accuracy_checks(P, args.precision)
        if args.precision == "fp64":
            line["mixed_batched"] = mixed_batched(P, K, W, dev, stream, x_ref_engine=None)
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


def mixed_batched(P, K, W, dev, stream, x_ref_engine=None):
    """Mixed-precision engine with 4 right-hand sides per launch: solves/s and
    relative error against the FP64 engine on the same b."""
    import torch
    from gpumatfun_gb300 import Engine, workloads
    R = 4
    rng = np.random.default_rng(7)
    U = rng.random((P.n, R))
    U /= np.linalg.norm(U, axis=0, keepdims=True)
    P4 = workloads.make_problem(P.name, P.A, U, P.Q, P.lam, [P.funcs[0]] * R, P.m, P.C, P.l1, P.lN,
                                degree=P.d, prob_dim=P.lN / 4)
    out = {}
    for prec in ("fp64", "mixed"):
        eng = Engine.from_problem(P4, precision=prec, sync=False)
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
        out[prec] = (R * 1e3 / ms, eng.get_solution())
        eng.delete()
    x64, xm = out["fp64"][1], out["mixed"][1]
    err = float(np.max(np.linalg.norm(xm - x64, axis=0) / np.linalg.norm(x64, axis=0)))
    return {"nrhs": R, "mixed_solves_per_s": out["mixed"][0], "fp64_batched_solves_per_s": out["fp64"][0],
            "mixed_rel_err_vs_fp64_engine": err,
            "note": "fused launch only (b resident, deflation excluded); same b for both precisions"}


def main():
    args = parse()
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
