"""Seeded synthetic sparse symmetric-definite pencils (A, B) used by tests,
the benchmark and the fixture generator.

Every matrix is returned as a :class:`CSRMatrix`: int32 ``indptr``/``indices``
and float64 ``data``.  All matrices here are symmetric, so the same three
arrays are also the CCS layout the reference's ``app_ccs`` backend consumes
(``CCSMAT{data, i_row, j_col}``, app/app_ccs.h:20-24): ``j_col = indptr``,
``i_row = indices``.

Random numbers come from a counter-based SplitMix64 stream implemented here in
numpy integer arithmetic, so the inputs are identical on every machine and
numpy version (numpy's own distribution code may change between releases).

Workloads (no public dataset is involved; all are generated):

* ``laplace2d(128, 128)`` - 2D 5-point Dirichlet Laplacian, stencil 4/-1,
  n = 16384, B = I.
* ``laplace3d(64)`` + ``mass3d(64)`` - (1/h^2) 7-point stiffness (6/-1) on a
  64^3 grid, h = 1/65, and B = M x M x M with M = h*tridiag(1/6, 4/6, 1/6)
  (27 nonzeros per row), n = 262144.
* ``vardiff3d(128, seed)`` - cell-centred variable-coefficient diffusion,
  kappa = exp(N(0,1)) per cell, harmonic-mean face coefficients, Dirichlet,
  B = diag(h^3 (1 + 0.1 U[0,1])).
* ``aniso2d(nx, ny, eps)`` - anisotropic 5-point Laplacian, -eps on x faces
  and -1 on y faces; ``batch_problems`` draws the 512-problem batch.
* ``rgg_laplacian`` - shifted random-geometric-graph Laplacian L + 1e-3 I.
* ``multigrid_2d`` - a geometric hierarchy (linear interpolation, Galerkin
  coarse operators) of the 2D Laplacian for the block AMG solver.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

__all__ = [
    "CSRMatrix", "splitmix_uniform", "splitmix_normal", "laplace2d", "laplace3d",
    "mass3d", "identity_diag", "diag_matrix", "vardiff3d", "aniso2d", "rgg_laplacian",
    "initial_block", "config1", "config2", "config3", "batch_problems", "to_dense",
    "Transfer", "interpolation_1d", "multigrid_2d",
]


@dataclass
class CSRMatrix:
    n: int
    indptr: np.ndarray   # int32, n+1
    indices: np.ndarray  # int32, nnz
    data: np.ndarray     # float64, nnz

    @property
    def nnz(self) -> int:
        return int(self.indptr[-1])

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.data, self.indices, self.indptr), shape=(self.n, self.n))

    def diagonal(self) -> np.ndarray:
        rows = np.repeat(np.arange(self.n, dtype=np.int64), np.diff(self.indptr))
        d = np.zeros(self.n)
        m = rows == self.indices
        d[rows[m]] = self.data[m]
        return d


# --------------------------------------------------------------------------
# Deterministic random numbers
# --------------------------------------------------------------------------
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(counter: np.ndarray) -> np.ndarray:
    z = counter * np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def splitmix_uniform(seed: int, count: int, stream: int = 0) -> np.ndarray:
    """``count`` doubles uniform in [0, 1) from SplitMix64 at (seed, stream)."""
    with np.errstate(over="ignore"):
        base = (np.uint64(seed) * np.uint64(0x100000001B3)
                + np.uint64(stream) * np.uint64(0xD1B54A32D192ED03))
        ctr = base + np.arange(1, count + 1, dtype=np.uint64)
        bits = _splitmix64(ctr)
    return (bits >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def splitmix_normal(seed: int, count: int, stream: int = 0) -> np.ndarray:
    """Standard normal samples by the Box-Muller transform of two uniform streams."""
    u1 = splitmix_uniform(seed, count, 2 * stream + 1)
    u2 = splitmix_uniform(seed, count, 2 * stream + 2)
    u1 = np.maximum(u1, 1e-300)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


# --------------------------------------------------------------------------
# Assembly helpers
# --------------------------------------------------------------------------
def _from_coo(n: int, rows: np.ndarray, cols: np.ndarray, vals: np.ndarray) -> CSRMatrix:
    import scipy.sparse as sp
    m = sp.coo_matrix((vals, (rows, cols)), shape=(n, n)).tocsr()
    m.sum_duplicates()
    m.sort_indices()
    return CSRMatrix(n, m.indptr.astype(np.int32), m.indices.astype(np.int32),
                     m.data.astype(np.float64))


def _from_scipy(m) -> CSRMatrix:
    m = m.tocsr()
    m.sum_duplicates()
    m.sort_indices()
    return CSRMatrix(m.shape[0], m.indptr.astype(np.int32), m.indices.astype(np.int32),
                     m.data.astype(np.float64))


def _tridiag(k: int, lo: float, mid: float):
    import scipy.sparse as sp
    return sp.diags([np.full(k - 1, lo), np.full(k, mid), np.full(k - 1, lo)], [-1, 0, 1],
                    format="csr")


def laplace2d(nx: int, ny: int, scale: float = 1.0) -> CSRMatrix:
    """5-point Dirichlet Laplacian on an nx*ny grid, stencil scale*(4, -1)."""
    import scipy.sparse as sp
    tx = _tridiag(nx, -1.0, 2.0)
    ty = _tridiag(ny, -1.0, 2.0)
    m = sp.kron(sp.identity(ny), tx) + sp.kron(ty, sp.identity(nx))
    return _from_scipy(scale * m)


def laplace3d(k: int) -> CSRMatrix:
    """(1/h^2) * 7-point Dirichlet Laplacian (6, -1) on a k^3 grid, h = 1/(k+1)."""
    import scipy.sparse as sp
    h = 1.0 / (k + 1)
    t = _tridiag(k, -1.0, 2.0)
    i = sp.identity(k)
    m = sp.kron(sp.kron(i, i), t) + sp.kron(sp.kron(i, t), i) + sp.kron(sp.kron(t, i), i)
    return _from_scipy(m * (1.0 / (h * h)))


def mass3d(k: int) -> CSRMatrix:
    """B = M x M x M with the 1D consistent mass M = h * tridiag(1/6, 4/6, 1/6)."""
    import scipy.sparse as sp
    h = 1.0 / (k + 1)
    m1 = _tridiag(k, h / 6.0, 4.0 * h / 6.0)
    return _from_scipy(sp.kron(sp.kron(m1, m1), m1))


def identity_diag(n: int) -> CSRMatrix:
    return diag_matrix(np.ones(n))


def diag_matrix(d: np.ndarray) -> CSRMatrix:
    n = d.shape[0]
    return CSRMatrix(n, np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32),
                     np.asarray(d, dtype=np.float64).copy())


def vardiff3d(k: int, seed: int = 3):
    """Cell-centred variable-coefficient diffusion on a k^3 grid (h = 1/k).

    kappa = exp(N(0,1)) per cell; the face coefficient between two cells is the
    harmonic mean of their kappas; a Dirichlet face (on the boundary) uses the
    cell's own kappa at half distance (coefficient 2*kappa).  A is scaled by
    h (finite-volume: face area h^2 over distance h), B = diag(h^3 (1 + 0.1 U)).
    Returns (A, B) as CSRMatrix.
    """
    n = k ** 3
    h = 1.0 / k
    kap = np.exp(splitmix_normal(seed, n, 0)).reshape(k, k, k)  # [z, y, x]
    idx = np.arange(n, dtype=np.int64).reshape(k, k, k)
    diag = np.zeros((k, k, k))
    rows, cols, vals = [], [], []
    for axis in range(3):
        a = np.moveaxis(kap, axis, -1)
        ii = np.moveaxis(idx, axis, -1)
        d = np.moveaxis(diag, axis, -1)
        hm = 2.0 * a[..., :-1] * a[..., 1:] / (a[..., :-1] + a[..., 1:])
        d[..., :-1] += hm
        d[..., 1:] += hm
        d[..., 0] += 2.0 * a[..., 0]
        d[..., -1] += 2.0 * a[..., -1]
        rows += [ii[..., :-1].ravel(), ii[..., 1:].ravel()]
        cols += [ii[..., 1:].ravel(), ii[..., :-1].ravel()]
        vals += [-hm.ravel(), -hm.ravel()]
    rows.append(idx.ravel()); cols.append(idx.ravel()); vals.append(diag.ravel())
    A = _from_coo(n, np.concatenate(rows), np.concatenate(cols), np.concatenate(vals) * h)
    bd = h ** 3 * (1.0 + 0.1 * splitmix_uniform(seed, n, 1))
    return A, diag_matrix(bd)


def aniso2d(nx: int, ny: int, eps: float) -> CSRMatrix:
    """Anisotropic 5-point Dirichlet Laplacian: -eps on x faces, -1 on y faces."""
    import scipy.sparse as sp
    tx = _tridiag(nx, -eps, 2.0 * eps)
    ty = _tridiag(ny, -1.0, 2.0)
    return _from_scipy(sp.kron(sp.identity(ny), tx) + sp.kron(ty, sp.identity(nx)))


def rgg_laplacian(n: int, mean_degree: float, seed: int, shift: float = 1e-3) -> CSRMatrix:
    """Graph Laplacian L + shift*I of a random geometric graph in the unit square.

    The connection radius r gives an expected degree n*pi*r^2 = mean_degree.
    Neighbour search uses a uniform cell grid of side r.
    """
    pts = np.stack([splitmix_uniform(seed, n, 0), splitmix_uniform(seed, n, 1)], axis=1)
    r = np.sqrt(mean_degree / (np.pi * n))
    g = max(1, int(1.0 / r))
    cell = np.minimum((pts * g).astype(np.int64), g - 1)
    key = cell[:, 0] * g + cell[:, 1]
    order = np.argsort(key, kind="stable")
    skey = key[order]
    starts = np.searchsorted(skey, np.arange(g * g), side="left")
    ends = np.searchsorted(skey, np.arange(g * g), side="right")
    rows, cols = [], []
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            nb = cell + np.array([dx, dy])
            ok = (nb[:, 0] >= 0) & (nb[:, 0] < g) & (nb[:, 1] >= 0) & (nb[:, 1] < g)
            src = np.nonzero(ok)[0]
            nk = nb[src, 0] * g + nb[src, 1]
            cnt = ends[nk] - starts[nk]
            rep_src = np.repeat(src, cnt)
            off = np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)
            dst = order[np.repeat(starts[nk], cnt) + off]
            d2 = np.sum((pts[rep_src] - pts[dst]) ** 2, axis=1)
            m = (d2 <= r * r) & (rep_src != dst)
            rows.append(rep_src[m]); cols.append(dst[m])
    rows = np.concatenate(rows); cols = np.concatenate(cols)
    deg = np.bincount(rows, minlength=n).astype(np.float64)
    allr = np.concatenate([rows, np.arange(n)])
    allc = np.concatenate([cols, np.arange(n)])
    allv = np.concatenate([-np.ones(rows.shape[0]), deg + shift])
    return _from_coo(n, allr, allc, allv)


def initial_block(n: int, ncols: int, seed: int = 1) -> np.ndarray:
    """Seeded Gaussian N(0,1) initial block, column-major (Fortran order) n x ncols."""
    x = splitmix_normal(seed, n * ncols, 7).reshape(ncols, n).T
    return np.asfortranarray(x)


def to_dense(m: CSRMatrix) -> np.ndarray:
    return m.to_scipy().toarray()


# --------------------------------------------------------------------------
# Named workloads (sizes from the reference's benchmark configurations)
# --------------------------------------------------------------------------
def gcge_block_rule(nev: int):
    """Block size / nevInit / nevMax rule of the reference's SLEPc front end
    (gcge.c:394-431): bs = nev/3 (nev<20), nev/5 (nev<1000), ...;
    nevInit = 3 bs; nevMax = nevInit + nev; nev <= 6: bs = nev, nevInit = nevMax = 2 nev."""
    if nev > 6:
        if nev < 20:
            bs = nev // 3
        elif nev < 1000:
            bs = nev // 5
        elif nev < 4000:
            bs = 100
        else:
            bs = 200
        nev_init = 3 * bs
        nev_max = nev_init + nev
    else:
        bs = nev
        nev_init = 2 * nev
        nev_max = nev_init
    return bs, nev_init, nev_max


def config1():
    """2D 5-point Laplacian 128x128, B = I, nev = 20, bs = 20, nevInit = nevMax = 40."""
    A = laplace2d(128, 128)
    return dict(name="laplace2d_128x128", A=A, B=None, nev=20, block_size=20,
                nev_init=40, nev_max=40)


def config2(k: int = 64):
    """3D 7-point stiffness + Kronecker consistent mass on k^3, nev = 100, bs = 20/60/160."""
    A = laplace3d(k)
    B = mass3d(k)
    bs, ni, nm = gcge_block_rule(100)
    return dict(name=f"laplace3d_mass_{k}^3", A=A, B=B, nev=100, block_size=bs,
                nev_init=ni, nev_max=nm)


def config3(k: int = 128, seed: int = 3):
    A, B = vardiff3d(k, seed)
    bs, ni, nm = gcge_block_rule(200)
    return dict(name=f"vardiff3d_{k}^3", A=A, B=B, nev=200, block_size=bs,
                nev_init=ni, nev_max=nm)


def batch_problems(count: int = 512, seed: int = 4, nx_range=(40, 220), nev_range=(8, 64)):
    """The batched workload: anisotropic 2D Laplacians with diagonal B."""
    u = splitmix_uniform(seed, 4 * count, 0).reshape(count, 4)
    out = []
    for i in range(count):
        nx = nx_range[0] + int(u[i, 0] * (nx_range[1] - nx_range[0] + 1))
        ny = nx_range[0] + int(u[i, 1] * (nx_range[1] - nx_range[0] + 1))
        eps = float(np.exp(np.log(1.0) + u[i, 2] * (np.log(100.0) - np.log(1.0))))
        nev = nev_range[0] + int(u[i, 3] * (nev_range[1] - nev_range[0] + 1))
        A = aniso2d(nx, ny, eps)
        bd = 0.5 + 1.5 * splitmix_uniform(seed + 1000 + i, nx * ny, 0)
        bs, ni, nm = gcge_block_rule(nev)
        out.append(dict(name=f"aniso2d_{nx}x{ny}_eps{eps:.2f}", A=A, B=diag_matrix(bd), nev=nev,
                        block_size=bs, nev_init=ni, nev_max=nm))
    return out


def serving_requests(count: int = 64, seed: int = 5, rate: float = 8.0, max_n: int = 300_000):
    """The serving workload: a Poisson stream of generalized solve requests
    mixing three kinds -- (a) 2D/3D Dirichlet Laplacians, n from 1k to 300k;
    (b) shifted random-geometric-graph Laplacians L + 1e-3 I, n from 5k to
    200k, mean degree 8-12; (c) the variable-coefficient operator at 32^3 to
    96^3 -- with B = I or a lumped mass, nev from 10 to 100 and a relative
    tolerance from 1e-6 to 1e-10 per request.  `max_n` caps the sizes (for
    short runs).  Every request carries its arrival time in seconds
    (exponential gaps of mean 1/rate)."""
    u = splitmix_uniform(seed, 8 * count, 0).reshape(count, 8)
    out, t = [], 0.0
    for i in range(count):
        t += -np.log(max(1e-12, 1.0 - u[i, 0])) / rate
        kind = int(u[i, 1] * 3)
        nev = 10 + int(u[i, 2] * 91)
        tol = float(10.0 ** (-6.0 - 4.0 * u[i, 3]))
        lumped = u[i, 4] < 0.5
        if kind == 0:
            n = int(np.exp(np.log(1000) + u[i, 5] * (np.log(min(300_000, max_n)) - np.log(1000))))
            if u[i, 6] < 0.5:
                nx = max(32, int(np.sqrt(n)))
                A, name, h2 = laplace2d(nx, nx), f"lap2d_{nx}^2", 1.0 / (nx + 1) ** 2
            else:
                k = max(12, int(round(n ** (1.0 / 3.0))))
                A, name, h2 = laplace3d(k), f"lap3d_{k}^3", (1.0 / (k + 1)) ** 3
            B = (diag_matrix(h2 * (1.0 + 0.1 * splitmix_uniform(seed + 100 + i, A.n, 0)))
                 if lumped else None)
        elif kind == 1:
            n = int(np.exp(np.log(5000) + u[i, 5] * (np.log(min(200_000, max_n)) - np.log(5000))))
            deg = 8.0 + 4.0 * u[i, 6]
            A, name = rgg_laplacian(n, deg, seed + 200 + i), f"rgg_{n}_deg{deg:.1f}"
            B = (diag_matrix(1.0 + 0.1 * splitmix_uniform(seed + 300 + i, A.n, 0))
                 if lumped else None)
        else:
            kmax = max(32, min(96, int(max_n ** (1.0 / 3.0))))
            k = 32 + int(u[i, 5] * (kmax - 32 + 1))
            A, B = vardiff3d(k, seed + 400 + i)
            name = f"vardiff3d_{k}^3"
        nev = min(nev, A.n // 4)
        bs, ni, nm = gcge_block_rule(nev)
        out.append(dict(name=name, A=A, B=B, nev=nev, block_size=bs, nev_init=ni, nev_max=nm,
                        tol=(1e300, tol), arrival=t))
    return out


# --------------------------------------------------------------------------
# Multigrid hierarchies for the block AMG solver
# --------------------------------------------------------------------------
@dataclass
class Transfer:
    """Transfer operator P between adjacent levels: nrows fine rows by ncols
    coarse columns, in CCS (column pointers, row indices, values; int32 and
    float64), the layout of the reference's app_ccs matrices."""
    nrows: int
    ncols: int
    colptr: np.ndarray
    rowind: np.ndarray
    data: np.ndarray

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csc_matrix((self.data, self.rowind, self.colptr), shape=(self.nrows, self.ncols))

    def transpose(self) -> "Transfer":
        """P^T in CCS (its column pointers are P's row pointers)."""
        m = self.to_scipy().tocsr()
        m.sort_indices()
        return Transfer(self.ncols, self.nrows, m.indptr.astype(np.int32),
                        m.indices.astype(np.int32), m.data.astype(np.float64))


def interpolation_1d(nc: int):
    """(2 nc + 1) x nc linear interpolation: coarse point j sits on fine point
    2 j + 1 with weight 1 and spreads 1/2 to fine points 2 j and 2 j + 2 (the
    weights of the reference's test hierarchy, app/app_lapack.c:863-890)."""
    import scipy.sparse as sp
    j = np.arange(nc)
    rows = np.concatenate([2 * j + 1, 2 * j, 2 * j + 2])
    cols = np.concatenate([j, j, j])
    vals = np.concatenate([np.ones(nc), np.full(nc, 0.5), np.full(nc, 0.5)])
    return sp.csc_matrix((vals, (rows, cols)), shape=(2 * nc + 1, nc))


def multigrid_2d(nx: int, ny: int, levels: int):
    """Geometric hierarchy of the 5-point Laplacian (4, -1) on an nx x ny
    grid: P_l = interpolation in y (x) interpolation in x, A_{l+1} =
    P_l^T A_l P_l (Galerkin; the entries are dyadic rationals, so every
    machine computes the same coarse matrices exactly).  nx and ny must stay
    odd while halving: nx_{l+1} = (nx_l - 1) / 2.  Returns ([A_0 .. A_{L-1}]
    as CSRMatrix, [P_0 .. P_{L-2}] as Transfer)."""
    import scipy.sparse as sp
    A = [laplace2d(nx, ny)]
    P = []
    cx, cy = nx, ny
    for _ in range(levels - 1):
        if cx % 2 == 0 or cy % 2 == 0 or cx < 3 or cy < 3:
            raise ValueError(f"grid {cx} x {cy} cannot be coarsened")
        cx, cy = (cx - 1) // 2, (cy - 1) // 2
        p = sp.kron(interpolation_1d(cy), interpolation_1d(cx), format="csc")
        p.sort_indices()
        P.append(Transfer(p.shape[0], p.shape[1], p.indptr.astype(np.int32),
                          p.indices.astype(np.int32), p.data.astype(np.float64)))
        a = A[-1].to_scipy()
        A.append(_from_scipy((p.T @ a @ p).tocsr()))
    return A, P
