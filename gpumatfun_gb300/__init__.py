"""GB300-native f(A)b engine (polynomial-preconditioned Lanczos, deflation and
contour-integral evaluation of f on the tridiagonal), with the reference's
handle API (``LanczosEngine``) over a C ABI (include/gpumatfun.h).

Modules: ``engine`` (handles: single problem, batch), ``adjoint`` (gradients
of a loss on f(A(kappa)) b, torch.autograd.Function), ``autotune`` (launch
shapes), ``replicas`` (multi-GPU timing), ``params`` (contour, polynomial,
shifts), ``problems``/``workloads`` (operators and benchmark workloads),
``roofline`` (algorithmic bytes and flops)."""
from .engine import Engine, LanczosEngine, BatchEngine, GmError, load_library  # noqa: F401
from . import params, problems, workloads  # noqa: F401

__version__ = "0.1.0"
