"""Build recipe for the engine's shared library (sm_103a, in-tree).

``build()`` compiles ``csrc/engine.cu`` with nvcc into ``_lib/libgpumatfun.so``;
nothing is installed outside the source tree.  The library exports exactly the
C ABI declared in ``include/gpumatfun.h``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
LIB = Path(os.environ["GPUMATFUN_LIB"]) if os.environ.get("GPUMATFUN_LIB") else LIBDIR / "libgpumatfun.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["engine.cu", "kern_fp64.cu", "kern_mixed.cu", "kern_mixed_l2.cu", "noalloc.cu", "eigs.cu"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC"]
# Kernel shape overrides for tuning builds, e.g. "-DGM_MINB1=2 -DGM_CH1=4"
# (GM_MINB1 / GM_MINB / GM_MINB4: minimum resident 512-thread blocks per SM
# for 1 / 2 / 4 right-hand sides; GM_MINB1X: one right-hand side, matrix-powers
# and Gram-Schmidt entry points; GM_MINB1L2: one right-hand side, mixed, with
# the matrix in the L2 window; GM_MINB4M: four right-hand sides, mixed
# precision; GM_CH1/2/4/4F: SpMV chunk width for 1/2/4 right-hand sides, 4F the
# FP32-stored mixed engine).
EXTRA = os.environ.get("GPUMATFUN_NVCC_EXTRA", "").split()


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "gpumatfun.h"]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile the engine library if it is missing or older than its sources."""
    if not force and not _stale():
        return LIB
    LIB.parent.mkdir(parents=True, exist_ok=True)
    nvcc = nvcc_path()
    tag = f"{os.getpid()}"
    objs, procs = [], []
    # one translation unit per precision so the kernel instantiations compile in parallel
    for src in SOURCES:
        obj = LIB.parent / (Path(src).stem + f".{tag}.o")
        cmd = [nvcc, *ARCH, *FLAGS, *EXTRA, "-c", "-o", str(obj), str(CSRC / src)]
        if verbose:
            print(" ".join(cmd))
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True), src))
        objs.append(obj)
    errs = []
    for p, src in procs:
        out, err = p.communicate()
        if p.returncode != 0:
            errs.append(f"{src}: nvcc failed ({p.returncode}):\n{out}\n{err}")
    try:
        if errs:
            raise RuntimeError("\n".join(errs))
        tmp = LIB.with_suffix(f".so.tmp{tag}")
        cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed ({res.returncode}):\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    finally:
        for o in objs:
            if o.exists():
                o.unlink()
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
