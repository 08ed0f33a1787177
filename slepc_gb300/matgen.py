"""Synthetic sparse matrices and start vectors for the Krylov-Schur workloads.

Every generator returns a CSR triple ``(rowptr int32[n+1], colidx int32[nnz], vals float64[nnz])`` with the
column indices of each row in ascending order, i.e. exactly what ``MatCreateSeqAIJWithArrays`` takes.

Matrix families (the reference's own test matrices and the benchmark shapes):

* ``laplacian_1d(n)``: tridiagonal (2, -1), as in ``src/eps/tests/test2.c``.
* ``laplacian_2d(nx, ny)``: 5-point stencil (4 on the diagonal, -1 on neighbours, Dirichlet), as in
  ``src/eps/tutorials/ex2.c``.
* ``laplacian_3d(n)``: 7-point stencil (6, -1) on an n x n x n grid.
* ``convection_diffusion_2d(N, peclet)``: upwind 5-point convection-diffusion with c = Pe*h, h = 1/(N+1):
  diagonal 4+2c, west/south -1-c, east/north -1.  Diagonally similar to a symmetric matrix, so its spectrum is
  real and known in closed form (``convdiff_eigenvalues``).
* ``chung_lu(n, ...)``: normalised adjacency D^-1/2 A D^-1/2 of a power-law Chung-Lu graph with weights U(0,1].
* ``laplacian_2d_randdiag(n, seed)``: 5-point Laplacian on a near-square r x c grid plus diag(U[0,1]).

Random numbers come from counter-based splitmix64 so the same seed gives the same vector on every platform.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """The first ``count`` outputs of splitmix64 seeded with ``seed`` (skipping ``offset``), as uint64."""
    with np.errstate(over="ignore"):
        i = np.arange(offset + 1, offset + count + 1, dtype=np.uint64)
        z = np.uint64(seed) + i * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform_pm1(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """n doubles uniform in [-1, 1) from splitmix64 (53-bit mantissa); matches the oracle's generator."""
    u = splitmix64(seed, n, offset) >> np.uint64(11)
    return u.astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def uniform_01(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """n doubles uniform in [0, 1)."""
    u = splitmix64(seed, n, offset) >> np.uint64(11)
    return u.astype(np.float64) * (1.0 / 9007199254740992.0)


def start_vector(n: int, seed: int) -> np.ndarray:
    """Start vector uniform in [-1, 1], passed through EPSSetInitialSpace."""
    return uniform_pm1(seed, n)


def _stencil_csr(shape, diag, offsets):
    """CSR for a constant-coefficient stencil on a row-major grid with Dirichlet boundaries.

    ``offsets`` is a list of (axis, step, value).  Rows are grid points in C order; columns are sorted.
    """
    shape = tuple(int(s) for s in shape)
    n = int(np.prod(shape))
    idx = np.arange(n, dtype=np.int64).reshape(shape)
    strides = [int(np.prod(shape[a + 1:])) for a in range(len(shape))]
    cols = [idx.ravel()]
    vals = [np.broadcast_to(np.asarray(diag, dtype=np.float64), shape).ravel().astype(np.float64)]
    for axis, step, value in offsets:
        coord = np.indices(shape)[axis] if len(shape) > 1 else np.arange(n).reshape(shape)
        ok = (coord + step >= 0) & (coord + step < shape[axis])
        c = np.where(ok, idx + step * strides[axis], -1).ravel()
        v = np.where(ok, value, 0.0).ravel()
        cols.append(c)
        vals.append(v)
    C = np.stack(cols, axis=1)
    V = np.stack(vals, axis=1)
    order = np.argsort(np.where(C < 0, np.iinfo(np.int64).max, C), axis=1, kind="stable")
    C = np.take_along_axis(C, order, axis=1)
    V = np.take_along_axis(V, order, axis=1)
    mask = C >= 0
    counts = mask.sum(axis=1)
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=rowptr[1:])
    return rowptr.astype(np.int32), C[mask].astype(np.int32), V[mask].astype(np.float64)


def laplacian_1d(n: int):
    return _stencil_csr((n,), 2.0, [(0, -1, -1.0), (0, 1, -1.0)])


def laplacian_2d(nx: int, ny: int | None = None):
    """5-point Laplacian on an nx x ny grid (ex2.c numbering: row I = i*ny + j)."""
    ny = nx if ny is None else ny
    return _stencil_csr((nx, ny), 4.0, [(0, -1, -1.0), (0, 1, -1.0), (1, -1, -1.0), (1, 1, -1.0)])


def graph_laplacian_2d(nx: int, ny: int | None = None):
    """Graph Laplacian of an nx x ny mesh: -1 per mesh edge, the vertex degree on the diagonal (ex11.c's matrix,
    src/eps/tutorials/ex11.c:49-57).  Singular, with the constant vector as null space."""
    rowptr, colidx, vals = laplacian_2d(nx, ny)
    n = len(rowptr) - 1
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    vals = vals.copy()
    vals[colidx == rows] = np.diff(rowptr)[rows[colidx == rows]] - 1.0
    return rowptr, colidx, vals


def laplacian_3d(n: int):
    offs = [(a, s, -1.0) for a in range(3) for s in (-1, 1)]
    return _stencil_csr((n, n, n), 6.0, offs)


def convection_diffusion_2d(N: int, peclet: float):
    """Upwind convection-diffusion on an N x N grid, wind b = (1, 1), c = Pe * h with h = 1/(N+1).

    The stencil is scaled by h^2: diagonal 4 + 2c, upwind (west, south) neighbours -1 - c, downwind (east,
    north) neighbours -1.  Grid point (i, j) is row i*N + j; "west/south" are the -1 steps along both axes.
    """
    c = float(peclet) / (N + 1)
    return _stencil_csr((N, N), 4.0 + 2.0 * c,
                        [(0, -1, -1.0 - c), (0, 1, -1.0), (1, -1, -1.0 - c), (1, 1, -1.0)])


def laplacian_2d_randdiag(n_target: int, seed: int):
    """5-point Laplacian on an r x c grid (r = floor(sqrt n), c = ceil(n/r)) plus diag(U[0,1])."""
    r = int(math.isqrt(int(n_target)))
    c = -(-int(n_target) // r)
    rowptr, colidx, vals = laplacian_2d(r, c)
    n = r * c
    d = uniform_01(seed, n)
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    vals = vals.copy()
    vals[colidx == rows] += d
    return rowptr, colidx, vals


def laplacian_3d_randdiag(m: int, seed: int):
    rowptr, colidx, vals = laplacian_3d(m)
    n = m ** 3
    d = uniform_01(seed, n)
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    vals = vals.copy()
    vals[colidx == rows] += d
    return rowptr, colidx, vals


_NATIVE = None


def _native_lib():
    """ctypes handle of the C helpers (slepc_gb300/native/matgen_native.c), built on first use; None without gcc."""
    global _NATIVE
    if _NATIVE is None:
        try:
            from . import buildlib
            lib = ctypes.CDLL(buildlib.build_native())
            lib.chung_lu_build.argtypes = [ctypes.c_longlong, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_ulonglong,
                                           ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_void_p)]
            lib.chung_lu_build.restype = ctypes.c_longlong
            lib.chung_lu_fetch.argtypes = [ctypes.c_void_p] * 4
            lib.chung_lu_fetch.restype = None
            _NATIVE = lib
        except (OSError, RuntimeError):
            _NATIVE = False
    return _NATIVE or None


def chung_lu(n: int, mean_degree: float = 32.0, gamma: float = 2.1, max_degree: float = 1e5,
             seed: int = 4, weight_seed: int = 5, i0: float | None = None, native: bool | None = None):
    """Normalised adjacency D^-1/2 A D^-1/2 of a Chung-Lu power-law graph.

    Expected degrees w_i proportional to (i + i0)^(-1/(gamma-1)), scaled to the requested mean and capped at
    ``max_degree``; m = n*mean/2 edges drawn by weight-proportional endpoint sampling; self-loops dropped,
    duplicates merged, symmetrised; edge weights U(0,1]; zero-degree rows stay empty.
    """
    n = int(n)
    if i0 is None:
        i0 = max(1.0, n ** 0.05)
    i = np.arange(n, dtype=np.float64)
    w = (i + i0) ** (-1.0 / (gamma - 1.0))
    w *= mean_degree * n / w.sum()
    for _ in range(8):
        w = np.minimum(w, max_degree)
        w *= mean_degree * n / w.sum()
    w = np.minimum(w, max_degree)
    m = int(round(n * mean_degree / 2.0))
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    native = _native_lib() if native is None or native else None
    if native is not None:
        h = ctypes.c_void_p()
        cdf_c = np.ascontiguousarray(cdf, dtype=np.float64)
        nnz = native.chung_lu_build(n, cdf_c.ctypes.data_as(ctypes.c_void_p), m, seed, weight_seed, ctypes.byref(h))
        if nnz < 0:
            raise MemoryError("chung_lu: host allocation failed")
        rowptr = np.empty(n + 1, dtype=np.int32)
        cols = np.empty(nnz, dtype=np.int32)
        vals = np.empty(nnz, dtype=np.float64)
        native.chung_lu_fetch(h, rowptr.ctypes.data_as(ctypes.c_void_p), cols.ctypes.data_as(ctypes.c_void_p),
                              vals.ctypes.data_as(ctypes.c_void_p))
        return rowptr, cols, vals
    u = uniform_01(seed, 2 * m)
    ends = np.searchsorted(cdf, u, side="right").astype(np.int64)
    np.minimum(ends, n - 1, out=ends)
    a, b = ends[:m], ends[m:]
    keep = a != b
    a, b = a[keep], b[keep]
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    key = np.unique(lo * n + hi)
    lo, hi = key // n, key % n
    wt = 1.0 - uniform_01(weight_seed, key.size)  # (0, 1]
    rows = np.concatenate([lo, hi])
    cols = np.concatenate([hi, lo])
    ww = np.concatenate([wt, wt])
    deg = np.bincount(rows, weights=ww, minlength=n)
    dinv = np.where(deg > 0, 1.0 / np.sqrt(np.where(deg > 0, deg, 1.0)), 0.0)
    ww = ww * dinv[rows] * dinv[cols]
    order = np.lexsort((cols, rows))
    rows, cols, ww = rows[order], cols[order], ww[order]
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(rows, minlength=n), out=rowptr[1:])
    return rowptr.astype(np.int32), cols.astype(np.int32), ww.astype(np.float64)


# ---------------------------------------------------------------------------------------------------------
# Closed-form spectra (the 1e-10 pins for the Laplacian and convection-diffusion families)
# ---------------------------------------------------------------------------------------------------------

def laplacian_eigenvalues(dims) -> np.ndarray:
    """All eigenvalues of the Dirichlet Laplacian on a grid with the given dimensions (unsorted)."""
    lam = np.zeros(1)
    for N in dims:
        k = np.arange(1, N + 1)
        ev = 2.0 - 2.0 * np.cos(k * np.pi / (N + 1))
        lam = (lam[:, None] + ev[None, :]).ravel()
    return lam


def convdiff_eigenvalues(N: int, peclet: float) -> np.ndarray:
    """Eigenvalues of ``convection_diffusion_2d(N, peclet)``: sum over both axes of
    (2 + c - 2 sqrt(1+c) cos(k pi/(N+1)))."""
    c = float(peclet) / (N + 1)
    k = np.arange(1, N + 1)
    ev = 2.0 + c - 2.0 * np.sqrt(1.0 + c) * np.cos(k * np.pi / (N + 1))
    return (ev[:, None] + ev[None, :]).ravel()


def markov_walk(m: int):
    """CSR arrays of the random walk on a triangular grid of m points per side (G. W. Stewart, SRRIT, TR-514,
    University of Maryland, 1978): n = m(m+1)/2 states numbered along the grid's rows; from point (i, j) the walk
    moves up or right with probability pd = (i + j - 1) / (2(m - 1)) each (doubled on the boundary row/column) and
    down or left with pu = 1/2 - (i + j - 3) / (2(m - 1)).  The matrix is the transpose of the transition matrix,
    as the reference's ex5.c builds it; 1 is an exact eigenvalue."""
    cst = 0.5 / (m - 1)
    rows, cols, vals = [], [], []
    ix = 0
    for i in range(1, m + 1):
        jmax = m - i + 1
        for j in range(1, jmax + 1):
            ix += 1
            r = ix - 1
            if j != jmax:
                pd = cst * (i + j - 1)
                rows += [r, r]
                cols += [ix, ix + jmax - 1]
                vals += [2 * pd if i == 1 else pd, 2 * pd if j == 1 else pd]
            pu = 0.5 - cst * (i + j - 3)
            if j > 1:
                rows.append(r)
                cols.append(ix - 2)
                vals.append(pu)
            if i > 1:
                rows.append(r)
                cols.append(ix - jmax - 2)
                vals.append(pu)
    n = m * (m + 1) // 2
    rows, cols, vals = np.array(rows), np.array(cols), np.array(vals, dtype=np.float64)
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    rowptr = np.zeros(n + 1, dtype=np.int32)
    np.add.at(rowptr, rows + 1, 1)
    return np.cumsum(rowptr).astype(np.int32), cols.astype(np.int32), vals


def diagonal(d):
    """CSR arrays of diag(d) (the B of a generalised problem)."""
    d = np.asarray(d, dtype=np.float64)
    n = d.size
    return np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32), d.copy()


def log_mass(n: int) -> np.ndarray:
    """B(i,i) = 2 / log(i + 2): the diagonal B of the reference's generalised test (src/eps/tests/test1.c)."""
    return 2.0 / np.log(np.arange(n, dtype=np.float64) + 2.0)


def csr_to_dense(rowptr, colidx, vals, n=None) -> np.ndarray:
    n = len(rowptr) - 1 if n is None else n
    A = np.zeros((n, n))
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    np.add.at(A, (rows, colidx), vals)
    return A


def brusselator(N: int = 50, alpha: float = 2.0, beta: float = 5.45, delta1: float = 0.008,
                delta2: float = 0.004, L: float = 0.51302):
    """Brusselator wave model of ``src/eps/tutorials/ex9.c`` as an explicit CSR matrix of order 2N:
    A = [tau1*T + (beta-1) I, alpha^2 I; -beta I, tau2*T - alpha^2 I], T = tridiag(1, -2, 1),
    tau_i = delta_i / (h L)^2, h = 1/(N+1)."""
    h = 1.0 / (N + 1)
    tau1 = delta1 / ((h * L) ** 2)
    tau2 = delta2 / ((h * L) ** 2)
    n = 2 * N
    rows, cols, vals = [], [], []
    for i in range(N):
        for j, v in ((i - 1, tau1), (i, -2.0 * tau1 + beta - 1.0), (i + 1, tau1)):
            if 0 <= j < N:
                rows.append(i); cols.append(j); vals.append(v)
        rows.append(i); cols.append(N + i); vals.append(alpha * alpha)
    for i in range(N):
        rows.append(N + i); cols.append(i); vals.append(-beta)
        for j, v in ((i - 1, tau2), (i, -2.0 * tau2 - alpha * alpha), (i + 1, tau2)):
            if 0 <= j < N:
                rows.append(N + i); cols.append(N + j); vals.append(v)
    rows = np.asarray(rows); cols = np.asarray(cols); vals = np.asarray(vals, dtype=np.float64)
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(rows, minlength=n), out=rowptr[1:])
    return rowptr.astype(np.int32), cols.astype(np.int32), vals
