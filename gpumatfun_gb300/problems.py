"""Synthetic problem generators for the f(A)b engine.

The reference builds its test operators with the un-vendored ``laplacian.m``
(startup_nicksmethod_GPU.m:33-57) and FE matrices from meshes
(process_nonuniform.m:90-91).  These generators rebuild the same operators
from their definitions:

* finite-difference Laplacians as Kronecker sums of tridiag(-1, 2, -1)
  (Dirichlet) or its Neumann variant, with analytic eigenpairs
  4 sin^2(i pi / (2(N+1))) / 4 sin^2(i pi / (2N)) (startup_nicksmethod_GPU.m:92,111);
* a 3D 7-point variable-coefficient Laplacian (face-averaged coefficient);
* P1 finite elements on a seeded Delaunay mesh of the unit disk with a
  log-normal per-triangle coefficient, lumped mass and the symmetric scaling
  M^{-1/2} K M^{-1/2} of process_nonuniform.m:90-91.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp

__all__ = [
    "tridiag_1d", "laplacian_2d", "laplacian_2d_eigpairs", "laplacian_3d_var",
    "FEMesh", "disk_mesh", "gaussian_random_field", "p1_assemble", "fe_operator",
    "FEFixture", "load_fe_mat",
]


def tridiag_1d(N: int, bc: str = "D") -> sp.csr_matrix:
    """tridiag(-1, 2, -1) of size N; ``bc='N'`` sets the two corner entries to 1."""
    e = np.ones(N)
    T = sp.diags([-e[:-1], 2 * e, -e[:-1]], [-1, 0, 1], format="lil")
    if bc == "N":
        T[0, 0] = 1.0
        T[N - 1, N - 1] = 1.0
    return T.tocsr()


def laplacian_2d(N: int, bc: str = "D", scale: float = 1.0) -> sp.csr_matrix:
    """5-point Laplacian on an N x N interior grid, scale * (I kron T + T kron I).

    Row index i + N*j (x fastest), matching MATLAB's column-major reshape.
    """
    T = tridiag_1d(N, bc)
    I = sp.identity(N, format="csr")
    A = (sp.kron(I, T) + sp.kron(T, I)) * scale
    A = sp.csr_matrix(A)
    A.sort_indices()
    return A


def laplacian_2d_eigpairs(N: int, k: int, bc: str = "D", scale: float = 1.0):
    """The k smallest eigenpairs of ``laplacian_2d`` (analytic sine/cosine modes).

    Returns (lam (k,), Q (N^2, k)) with Q orthonormal, eigenvalues ascending
    (ties broken by (i, j) order).
    """
    if bc == "D":
        idx = np.arange(1, N + 1)
        lam1 = 4 * np.sin(idx * np.pi / (2 * (N + 1))) ** 2
        p = np.arange(1, N + 1)
        modes = np.sqrt(2.0 / (N + 1)) * np.sin(np.outer(p, idx) * np.pi / (N + 1))  # (N, N) [point, mode]
    else:
        idx = np.arange(0, N)
        lam1 = 4 * np.sin(idx * np.pi / (2 * N)) ** 2
        p = np.arange(N) + 0.5
        modes = np.cos(np.outer(p, idx) * np.pi / N) * np.sqrt(2.0 / N)
        modes[:, 0] = 1.0 / np.sqrt(N)
    L = (lam1[:, None] + lam1[None, :]) * scale  # [i (x-mode), j (y-mode)]
    order = np.lexsort((np.arange(N * N), L.ravel()))[:k]
    ii, jj = np.unravel_index(order, (N, N))
    Q = np.empty((N * N, k))
    for c, (a, b) in enumerate(zip(ii, jj)):
        Q[:, c] = np.kron(modes[:, b], modes[:, a])  # x index fastest
    return L.ravel()[order], Q


def laplacian_3d_var(N: int, h: float | None = None, amp: float = 0.5, dtype=np.float64) -> sp.csr_matrix:
    """7-point -div(kappa grad) on an N^3 interior grid of the unit cube, Dirichlet.

    kappa(x) = 1 + amp sin(2 pi x) sin(2 pi y) sin(2 pi z), evaluated at face
    midpoints; scaled by 1/h^2 with h = 1/(N+1).  Row index i + N j + N^2 k.
    """
    h = 1.0 / (N + 1) if h is None else h
    g = (np.arange(N) + 1) * h

    def kap(x, y, z):
        return 1.0 + amp * np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y) * np.sin(2 * np.pi * z)

    n = N ** 3
    I, J, K = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    I = I.ravel(order="F"); J = J.ravel(order="F"); K = K.ravel(order="F")
    row = I + N * J + N * N * K
    x, y, z = g[I], g[J], g[K]
    diag = np.zeros(n)
    rows, cols, vals = [], [], []
    for (di, dj, dk) in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
        kf = kap(x + 0.5 * di * h, y + 0.5 * dj * h, z + 0.5 * dk * h) / (h * h)
        diag += kf
        I2, J2, K2 = I + di, J + dj, K + dk
        ok = (I2 >= 0) & (I2 < N) & (J2 >= 0) & (J2 < N) & (K2 >= 0) & (K2 < N)
        rows.append(row[ok]); cols.append((I2 + N * J2 + N * N * K2)[ok]); vals.append(-kf[ok])
    rows.append(row); cols.append(row); vals.append(diag)
    A = sp.csr_matrix((np.concatenate(vals).astype(dtype), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    A.sort_indices()
    return A


@dataclass
class FEMesh:
    nodes: np.ndarray      # (nn, 2)
    tris: np.ndarray       # (nt, 3) int
    boundary: np.ndarray   # bool (nn,)


def disk_mesh(n_target: int, seed: int = 0) -> FEMesh:
    """Seeded Delaunay mesh of the unit disk with about ``n_target`` nodes.

    Boundary nodes are equispaced on the circle; interior nodes are a jittered
    hexagonal-ish lattice (spacing from the target count) so that triangles are
    well shaped.  The triangulation is scipy's Delaunay of the point set.
    """
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    hsp = math.sqrt(math.pi / (n_target * (math.sqrt(3) / 2)))  # lattice spacing
    nb = max(8, int(round(2 * math.pi / hsp)))
    th = np.arange(nb) * (2 * math.pi / nb)
    bnd = np.stack([np.cos(th), np.sin(th)], axis=1)
    ny = int(math.ceil(2.0 / (hsp * math.sqrt(3) / 2))) + 1
    ys = -1.0 + np.arange(ny) * hsp * math.sqrt(3) / 2
    nx = int(math.ceil(2.0 / hsp)) + 2
    xs = -1.0 + np.arange(nx) * hsp
    X, Y = np.meshgrid(xs, ys)
    X = X + (np.arange(ny)[:, None] % 2) * 0.5 * hsp
    P = np.stack([X.ravel(), Y.ravel()], axis=1)
    P = P + rng.uniform(-0.15, 0.15, size=P.shape) * hsp
    r = np.hypot(P[:, 0], P[:, 1])
    P = P[r < 1.0 - 0.6 * hsp]
    pts = np.concatenate([bnd, P], axis=0)
    tri = Delaunay(pts).simplices.astype(np.int64)
    # orient counter-clockwise
    a, b, c = pts[tri[:, 0]], pts[tri[:, 1]], pts[tri[:, 2]]
    area2 = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    flip = area2 < 0
    tri[flip, 1], tri[flip, 2] = tri[flip, 2].copy(), tri[flip, 1].copy()
    area2 = np.abs(area2)
    keep = area2 > 1e-14
    tri = tri[keep]
    boundary = np.zeros(pts.shape[0], dtype=bool)
    boundary[:nb] = True
    # reorder nodes along a space-filling order for locality (Morton on a grid)
    q = np.clip(((pts + 1.0) * 0.5 * 65535).astype(np.int64), 0, 65535)
    key = np.zeros(pts.shape[0], dtype=np.int64)
    for bit in range(16):
        key |= ((q[:, 0] >> bit) & 1) << (2 * bit)
        key |= ((q[:, 1] >> bit) & 1) << (2 * bit + 1)
    perm = np.argsort(key, kind="stable")
    inv = np.empty_like(perm)
    inv[perm] = np.arange(perm.size)
    return FEMesh(nodes=pts[perm], tris=inv[tri], boundary=boundary[perm])


def submesh(mesh: FEMesh, center=(0.0, 0.0), radius: float = 0.1) -> tuple:
    """The triangles of ``mesh`` whose three vertices lie within ``radius`` of
    ``center``, as a mesh of its own: nodes renumbered in their original
    order, and its boundary the nodes on an edge that only one kept triangle
    has (plus kept nodes of the original boundary), so that a homogeneous
    Dirichlet condition there gives an SPD operator.  Returns (submesh,
    indices of the kept triangles in ``mesh``)."""
    c = np.asarray(center, dtype=np.float64)
    inside = np.hypot(mesh.nodes[:, 0] - c[0], mesh.nodes[:, 1] - c[1]) < radius
    keep = np.flatnonzero(inside[mesh.tris].all(axis=1))
    tris = mesh.tris[keep]
    used = np.unique(tris)
    new_id = np.full(mesh.nodes.shape[0], -1, dtype=np.int64)
    new_id[used] = np.arange(used.size)
    t = new_id[tris]
    edges = np.sort(np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]]), axis=1)
    uniq, cnt = np.unique(edges, axis=0, return_counts=True)
    boundary = mesh.boundary[used].copy()
    boundary[uniq[cnt == 1].ravel()] = True
    return FEMesh(nodes=mesh.nodes[used], tris=t, boundary=boundary), keep


def gaussian_random_field(points: np.ndarray, sigma: float = 1.0, ell: float = 0.1,
                          seed: int = 0, grid: int = 512) -> np.ndarray:
    """Seeded stationary Gaussian field with squared-exponential covariance
    sigma^2 exp(-r^2/(2 ell^2)) on [-1,1]^2, by spectral synthesis on a periodic
    ``grid`` x ``grid`` lattice (domain padded to side 4 to limit wrap-around),
    sampled at ``points`` by bilinear interpolation."""
    rng = np.random.default_rng(seed)
    Lside = 4.0
    kx = np.fft.fftfreq(grid, d=Lside / grid) * 2 * np.pi
    KX, KY = np.meshgrid(kx, kx, indexing="ij")
    spec = (2 * np.pi * ell * ell) * np.exp(-0.5 * ell * ell * (KX ** 2 + KY ** 2))
    amp = np.sqrt(spec / (Lside * Lside)) * grid
    z = rng.standard_normal((grid, grid)) + 1j * rng.standard_normal((grid, grid))
    field = np.fft.ifft2(amp * z).real * grid
    field *= sigma / max(field.std(), 1e-300)
    u = (points[:, 0] + 2.0) / Lside * grid
    v = (points[:, 1] + 2.0) / Lside * grid
    i0 = np.floor(u).astype(np.int64) % grid
    j0 = np.floor(v).astype(np.int64) % grid
    fu = u - np.floor(u)
    fv = v - np.floor(v)
    i1 = (i0 + 1) % grid
    j1 = (j0 + 1) % grid
    return ((1 - fu) * (1 - fv) * field[i0, j0] + fu * (1 - fv) * field[i1, j0]
            + (1 - fu) * fv * field[i0, j1] + fu * fv * field[i1, j1])


def p1_element_grads(nodes: np.ndarray, tris: np.ndarray):
    """Per-triangle area and the gradients of the three P1 hat functions."""
    p = nodes[tris]  # (nt, 3, 2)
    d1 = p[:, 1] - p[:, 0]
    d2 = p[:, 2] - p[:, 0]
    area = 0.5 * (d1[:, 0] * d2[:, 1] - d1[:, 1] * d2[:, 0])
    # gradient of hat i: rot90(edge opposite i) / (2 area)
    e0 = p[:, 2] - p[:, 1]
    e1 = p[:, 0] - p[:, 2]
    e2 = p[:, 1] - p[:, 0]
    G = np.stack([np.stack([-e0[:, 1], e0[:, 0]], 1),
                  np.stack([-e1[:, 1], e1[:, 0]], 1),
                  np.stack([-e2[:, 1], e2[:, 0]], 1)], axis=1) / (2 * area)[:, None, None]
    return area, G


def p1_assemble(mesh: FEMesh, kappa: np.ndarray):
    """P1 stiffness K (kappa per triangle) and lumped mass diagonal M (area/3 per vertex)."""
    area, G = p1_element_grads(mesh.nodes, mesh.tris)
    Ke = np.einsum("tid,tjd->tij", G, G) * (area * kappa)[:, None, None]
    nn = mesh.nodes.shape[0]
    I = np.repeat(mesh.tris, 3, axis=1).ravel()
    J = np.tile(mesh.tris, (1, 3)).ravel()
    K = sp.csr_matrix((Ke.ravel(), (I, J)), shape=(nn, nn))
    K.sum_duplicates()
    M = np.bincount(mesh.tris.ravel(), weights=np.repeat(area / 3.0, 3), minlength=nn)
    return K, M


def fe_operator(mesh: FEMesh, kappa: np.ndarray):
    """A = M^{-1/2} K M^{-1/2} restricted to interior nodes (homogeneous Dirichlet
    on the disk boundary so that A is SPD).  Returns (A, msqrt, interior_index)."""
    K, M = p1_assemble(mesh, kappa)
    inner = np.flatnonzero(~mesh.boundary)
    K = K[inner][:, inner].tocsr()
    ms = np.sqrt(M[inner])
    D = sp.diags(1.0 / ms)
    A = sp.csr_matrix(D @ K @ D)
    A.sort_indices()
    return A, ms, inner


@dataclass
class FEFixture:
    """An FE problem read from a MATLAB mesh file of the reference's form."""
    A: sp.csr_matrix       # M^{-1/2} K M^{-1/2} on the kept nodes
    msqrt: np.ndarray      # sqrt of the lumped mass on the kept nodes
    nodes: np.ndarray      # (nn, dim) coordinates of all nodes
    elements: np.ndarray   # (ne, 3) zero-based node indices
    kept: np.ndarray       # zero-based indices of the kept nodes


def load_fe_mat(path: str, dirichlet: bool = True) -> FEFixture:
    """Read K, M, nodes and elements from a MATLAB v5 .mat mesh (the layout of
    the reference's circle1/2/3.mat, read by process_nonuniform.m:12) and form
    A = diag(1/sqrt(diag M)) K diag(1/sqrt(diag M)) as process_nonuniform.m:90-91
    does.  With ``dirichlet`` (default) the operator is restricted to the
    file's ``internal_nodes`` (homogeneous Dirichlet), which makes it SPD;
    otherwise every node is kept (the reference's Neumann operator, singular).
    The reference's symrcm reordering (process_nonuniform.m:15-20) is not
    applied: the engine partitions and orders rows itself."""
    import scipy.io as sio
    d = sio.loadmat(path)
    for key in ("K", "M", "nodes", "elements"):
        if key not in d:
            raise ValueError(f"{path}: no variable {key!r}")
    K = sp.csr_matrix(d["K"], dtype=np.float64)
    Mdiag = np.asarray(sp.csr_matrix(d["M"]).diagonal(), dtype=np.float64).ravel()
    n = K.shape[0]
    if dirichlet:
        if "internal_nodes" not in d:
            raise ValueError(f"{path}: no variable 'internal_nodes' for the Dirichlet restriction")
        kept = np.asarray(d["internal_nodes"]).ravel().astype(np.int64) - 1   # MATLAB is one-based
    else:
        kept = np.arange(n, dtype=np.int64)
    Kk = K[kept][:, kept]
    ms = np.sqrt(Mdiag[kept])
    D = sp.diags(1.0 / ms)
    A = sp.csr_matrix(D @ Kk @ D)
    A.sort_indices()
    elements = np.asarray(d["elements"]).astype(np.int64) - 1
    return FEFixture(A=A, msqrt=ms, nodes=np.asarray(d["nodes"], dtype=np.float64), elements=elements, kept=kept)
