"""Autotuner for the engine's launch shape.

Times candidate launch shapes of the fused solve on the actual workload and
keeps the fastest.  The knobs are the ones the engine exposes at create time:
- threads per block (the row-block size: 32 SELL rows per warp);
- resident blocks per SM;
- TMA staging of SELL column indices on or off;
- neighbour waits vs grid barriers between SpMV passes;
- one or two Horner levels of the polynomial per SpMV pass (degree >= 2);
- the SELL-32 sorting window sigma, for matrices whose row lengths vary
  (sorting rows by length within a window cuts the slice padding).

Results are cached in a JSON file keyed by a signature of the workload:
- n, nnz, a row-length histogram and the number of right-hand sides;
- m, d, C and precision;
- the device name.

A repeated workload therefore reuses the tuned shape without timing again.
"""
from __future__ import annotations

import hashlib
import itertools
import json
import os
from typing import Callable

import numpy as np

__all__ = ["signature", "candidates", "tune", "default_cache_path", "batch_signature", "batch_candidates",
           "tune_batch"]


def default_cache_path() -> str:
    base = os.environ.get("GPUMATFUN_CACHE") or os.path.join(os.environ.get("TMPDIR", "/tmp"), "gpumatfun_cache")
    return os.path.join(base, "autotune.json")


def signature(P, precision: str, device: str = "") -> str:
    """Stable key of the quantities that decide the best launch shape."""
    lens = np.diff(P.A.indptr)
    hist = np.bincount(np.minimum(lens, 32), minlength=33)
    frac = np.round(hist / max(1, lens.size), 3).tolist()
    key = dict(n=int(P.n), nnz=int(P.A.nnz), rowlen=frac, R=int(P.R), m=int(P.m), d=int(P.d), C=int(P.C),
               precision=str(precision), device=device, space=2)
    return hashlib.sha1(json.dumps(key, sort_keys=True).encode()).hexdigest()[:16]


def candidates(R: int, degree: int = 0, ragged: bool = False) -> list:
    """The search space: row-block sizes, residency, staging, pass ordering;
    for a polynomial of degree >= 2, matrix-powers passes (neighbour waits
    only, unsorted slices); for ragged row lengths, sigma-sorted slices."""
    threads = (128, 256, 512)
    bps = (0, 1) if R >= 4 else (0, 1, 2)
    out = []
    for t, b, stg, pol in itertools.product(threads, bps, (1, 2), (0, 1)):
        out.append(dict(threads=t, blocks_per_sm=b, col_staging=stg, sync_policy=pol, matrix_powers=0, sell_sigma=0))
        if degree >= 2 and pol == 0:
            out.append(dict(threads=t, blocks_per_sm=b, col_staging=stg, sync_policy=pol, matrix_powers=1,
                            sell_sigma=0))
        if ragged:
            out.append(dict(threads=t, blocks_per_sm=b, col_staging=stg, sync_policy=pol, matrix_powers=0,
                            sell_sigma=SIGMA))
    return out


SIGMA = 256   # rows sorted by length within windows of 8 slices


def ragged(P) -> bool:
    """Row lengths vary enough that unsorted SELL-32 slices carry more than a
    quarter of padding (each slice is as long as its longest row)."""
    lens = np.diff(P.A.indptr)
    n = lens.size
    pad = np.zeros(-(-n // 32) * 32, dtype=np.int64)
    pad[:n] = lens
    per_slice = pad.reshape(-1, 32)
    rows = np.minimum(32, n - 32 * np.arange(per_slice.shape[0]))
    slots = int((per_slice.max(axis=1) * rows).sum())
    return bool(slots > 1.25 * max(1, int(lens.sum())))


def _measure_engine(P, precision: str, reps: int) -> Callable[[dict], float]:
    from .engine import Engine, GmError

    def run(cand: dict) -> float:
        try:
            eng = Engine.from_problem(P, precision=precision, sync=False, **cand)
        except GmError:
            return float("inf")
        try:
            eng.solve()
            eng.sync()
            ts = []
            for _ in range(reps):
                eng.solve()
                ts.append(eng.phase_times()["solve"])
            return float(np.median(ts))
        finally:
            eng.delete()
    return run


def _search(key: str, space: list, measure: Callable[[dict], float], cache_path: str, force: bool) -> dict:
    """Time every candidate (or reuse the cached winner for key) and cache the fastest."""
    cache = {}
    if os.path.exists(cache_path):
        try:
            with open(cache_path) as fh:
                cache = json.load(fh)
        except (OSError, ValueError):
            cache = {}
    if not force and key in cache:
        return dict(cache[key], cached=True)
    best, best_ms, timed = None, float("inf"), []
    for cand in space:
        ms = measure(cand)
        timed.append(dict(cand, ms=ms))
        if ms < best_ms:
            best, best_ms = cand, ms
    if best is None:
        raise RuntimeError("autotune: no candidate ran")
    result = dict(best, ms=best_ms, trials=len(timed), timed=timed)
    cache[key] = result
    os.makedirs(os.path.dirname(cache_path) or ".", exist_ok=True)
    tmp = f"{cache_path}.tmp{os.getpid()}"
    with open(tmp, "w") as fh:
        json.dump(cache, fh, indent=1)
    os.replace(tmp, cache_path)
    return dict(result, cached=False)


def tune(P, precision: str = "fp64", reps: int = 3, cache_path: str | None = None,
         space: list | None = None, measure: Callable[[dict], float] | None = None,
         device: str = "", force: bool = False) -> dict:
    """Best launch shape for workload P: a dict of Engine keyword arguments
    plus 'ms' (median fused-solve time).  ``measure`` replaces the GPU timing
    (tests); ``space`` replaces the candidate list."""
    return _search(signature(P, precision, device), space or candidates(P.R, P.d, ragged(P)),
                   measure or _measure_engine(P, precision, reps), cache_path or default_cache_path(), force)


def batch_signature(problems, precision: str, device: str = "") -> str:
    """Key of a batch: every problem's n and nnz in order, plus the shared
    nrhs, m, d, C and the precision."""
    P0 = problems[0]
    key = dict(sizes=[[int(P.n), int(P.A.nnz)] for P in problems], R=int(P0.R), m=int(P0.m), d=int(P0.d),
               C=int(P0.C), precision=str(precision), device=device, batch=True, space=2)
    return hashlib.sha1(json.dumps(key, sort_keys=True).encode()).hexdigest()[:16]


def batch_candidates(R: int) -> list:
    """Launch shapes of a batched engine: row-block size, residency, staging
    and pass ordering (each problem keeps its own barrier)."""
    bps = (0, 1) if R >= 4 else (0, 1, 2)
    return [dict(threads=t, blocks_per_sm=b, col_staging=stg, sync_policy=pol)
            for t, b, stg, pol in itertools.product((256, 512), bps, (1, 2), (0, 1))]


def _measure_batch(problems, precision: str, reps: int) -> Callable[[dict], float]:
    from .engine import BatchEngine, GmError

    def run(cand: dict) -> float:
        try:
            eng = BatchEngine(problems, precision=precision, sync=False, **cand)
        except GmError:
            return float("inf")
        try:
            eng.solve()
            eng.sync()
            ts = []
            for _ in range(reps):
                eng.solve()
                ts.append(eng.phase_times()["solve"])
            return float(np.median(ts))
        finally:
            eng.delete()
    return run


def tune_batch(problems, precision: str = "mixed", reps: int = 3, cache_path: str | None = None,
               space: list | None = None, measure: Callable[[dict], float] | None = None,
               device: str = "", force: bool = False) -> dict:
    """Best launch shape for a batch of problems in one engine: BatchEngine
    keyword arguments plus 'ms' (median time of the one launch that solves all
    of them)."""
    return _search(batch_signature(problems, precision, device), space or batch_candidates(problems[0].R),
                   measure or _measure_batch(problems, precision, reps), cache_path or default_cache_path(), force)
