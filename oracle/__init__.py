"""CPU oracle for the f(A)b engine (test infrastructure only).

This package restates, in FP64 numpy/scipy and in plain C, the algorithm of
GPUMatfun's f(A)b path so that the CUDA engine can be checked against it.
Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it; the product path never routes through it.

Modules
-------
fab      statement-by-statement restatement of the reference engine
         (``build_subspace``, ``lin_sys_solves``, ``apply_V``, deflation,
         ``update_U``/``update_U_monodomain``) and of ``nicksmethodcpu.m``.
known    analytic (DST-I) and dense-eigh known answers for f(A)b.
cpu_fab  ctypes loader for the C/OpenMP restatement used as the timed
         CPU baseline (``cpu_fab.c``).

Parity pinning: the reference cannot be built or run here (MATLAB, mex.h,
minlin and the cuSPARSE entry points it calls are all absent), so parity
against the reference's own binary outputs is unpinned.  The restatement is
pinned instead against the reference's own known-answer mechanisms: the DST
exact solution of the Dirichlet Laplacian (startup_nicksmethod_GPU.m:91-153)
and a dense eigendecomposition at small n, plus the circle FE meshes shipped
with the reference (circle1-3.mat) as fixtures.
"""
