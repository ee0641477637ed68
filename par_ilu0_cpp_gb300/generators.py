"""Seeded synthetic sparse systems for the ILU(k)+GMRES solver.

Every matrix is returned as 0-based CSR with column-sorted rows and an explicit
diagonal in every row (the layout the reference's IlukSymbolic and IluSolver expect:
src/iluk.cpp:38-52, src/ilu_solver.cpp:276-289).  Natural (lexicographic) ordering
throughout, x fastest.  No dataset is involved: all inputs are generated in memory
from a seed.

Workloads (sizes as used by the tests and the benchmark):

* ``laplace2d(256)``      2D 5-point Laplacian [-1,-1,4,-1,-1], Dirichlet,
                           n = 65,536, nnz = 5n - 4*256 = 326,656.
* ``convdiff3d(128)``     3D 7-point convection-diffusion, D = 1, constant wind
                           (1, 0.5, 0.25) scaled to cell Peclet 0.5, first-order upwind,
                           n = 2,097,152, nnz = 7n - 6*128^2 = 14,581,760.
* ``lognormal27(64)``     3D 27-point operator with a lognormal coefficient field
                           (sigma = 1, correlation length 8 cells), n = 262,144,
                           nnz = 190^3 = 6,859,000.
* ``cdr2d(...)``          2D 5-point convection-diffusion-reaction with a negative
                           reaction shift (learned-shift stress set).
* ``batched_systems(...)`` many variable-coefficient 5-point systems of uneven size.
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "Csr",
    "laplace2d",
    "convdiff3d",
    "lognormal_field",
    "lognormal27",
    "cdr2d",
    "variable_poisson2d",
    "batched_systems",
    "random_rhs",
    "spmv",
]


class Csr:
    """Plain CSR triple (int32 row_ptr / col_idx, float64 values)."""

    __slots__ = ("n", "row_ptr", "col_idx", "values")

    def __init__(self, n, row_ptr, col_idx, values):
        self.n = int(n)
        self.row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int32)
        self.col_idx = np.ascontiguousarray(col_idx, dtype=np.int32)
        self.values = np.ascontiguousarray(values, dtype=np.float64)

    @property
    def nnz(self) -> int:
        return int(self.row_ptr[-1])

    def to_scipy(self):
        import scipy.sparse as sp

        return sp.csr_matrix((self.values, self.col_idx, self.row_ptr), shape=(self.n, self.n))

    def __repr__(self) -> str:
        return f"Csr(n={self.n}, nnz={self.nnz})"


def _from_coo(n, rows, cols, vals) -> Csr:
    """Assemble CSR from COO triplets (duplicates summed, columns sorted)."""
    import scipy.sparse as sp

    m = sp.coo_matrix((vals, (rows, cols)), shape=(n, n)).tocsr()
    m.sum_duplicates()
    m.sort_indices()
    return Csr(n, m.indptr, m.indices, m.data)


def _stencil(shape, offsets_coeffs):
    """Build a constant-coefficient stencil matrix on a Dirichlet box.

    ``offsets_coeffs`` is a list of ((dx, dy[, dz]), coeff); connections leaving the
    box are dropped (homogeneous Dirichlet)."""
    shape = tuple(int(s) for s in shape)
    n = int(np.prod(shape))
    grids = np.meshgrid(*[np.arange(s) for s in reversed(shape)], indexing="ij")
    # natural ordering: x fastest -> index = x + nx*(y + ny*z)
    coords = [g.ravel() for g in reversed(grids)]  # coords[0] = x, ...
    strides = [1]
    for s in shape[:-1]:
        strides.append(strides[-1] * s)
    idx = np.arange(n, dtype=np.int64)
    rows, cols, vals = [], [], []
    for off, coef in offsets_coeffs:
        mask = np.ones(n, dtype=bool)
        shift = 0
        for d, o in enumerate(off):
            c = coords[d] + o
            mask &= (c >= 0) & (c < shape[d])
            shift += o * strides[d]
        r = idx[mask]
        rows.append(r)
        cols.append(r + shift)
        vals.append(np.full(r.shape, coef, dtype=np.float64))
    return _from_coo(n, np.concatenate(rows), np.concatenate(cols), np.concatenate(vals))


def laplace2d(nx: int, ny: int | None = None) -> Csr:
    """2D 5-point Laplacian [-1,-1,4,-1,-1] with Dirichlet boundary."""
    ny = nx if ny is None else ny
    return _stencil((nx, ny), [((0, 0), 4.0), ((-1, 0), -1.0), ((1, 0), -1.0), ((0, -1), -1.0), ((0, 1), -1.0)])


def convdiff3d(nx: int, ny: int | None = None, nz: int | None = None, wind=(1.0, 0.5, 0.25),
               peclet: float = 0.5, diffusion: float = 1.0) -> Csr:
    """3D 7-point convection-diffusion, first-order upwind, Dirichlet box.

    Equation -D lap(u) + w . grad(u) on the unit cube, h = 1/(n+1), scaled by h^2.
    The wind direction ``wind`` is scaled so that the cell Peclet number
    Pe = max|w_d| h / (2 D) equals ``peclet``.  Upwinding (all wind components
    positive) adds w_d h to the diagonal and -w_d h to the upstream neighbour, so
    the matrix is nonsymmetric and (weakly) diagonally dominant."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    wind = np.asarray(wind, dtype=np.float64)
    # w_d * h for each direction: max component -> 2 D Pe
    wh = wind / np.max(np.abs(wind)) * (2.0 * diffusion * peclet)
    terms = [((0, 0, 0), 6.0 * diffusion + float(np.sum(np.abs(wh))))]
    for d in range(3):
        lo = [0, 0, 0]
        hi = [0, 0, 0]
        lo[d] = -1
        hi[d] = 1
        up = -diffusion - (wh[d] if wh[d] > 0 else 0.0)
        dn = -diffusion + (wh[d] if wh[d] < 0 else 0.0)
        terms.append((tuple(lo), up))
        terms.append((tuple(hi), dn))
    return _stencil((nx, ny, nz), terms)


def lognormal_field(shape, sigma: float, corr_len: float, seed: int) -> np.ndarray:
    """exp(sigma * g), g a zero-mean unit-variance Gaussian random field obtained by
    filtering seeded white noise with a Gaussian kernel exp(-r^2 / (2 l^2)) in Fourier
    space (periodic embedding on the box), l = corr_len cells."""
    rng = np.random.default_rng(seed)
    shape = tuple(int(s) for s in shape)
    noise = rng.standard_normal(shape)
    freqs = np.meshgrid(*[np.fft.fftfreq(s) for s in shape], indexing="ij")
    k2 = sum(f * f for f in freqs)
    # Fourier transform of a Gaussian of std l (in cells): exp(-2 pi^2 l^2 k^2)
    filt = np.exp(-2.0 * np.pi ** 2 * corr_len ** 2 * k2)
    g = np.real(np.fft.ifftn(np.fft.fftn(noise) * filt))
    g -= g.mean()
    std = g.std()
    if std > 0:
        g /= std
    return np.exp(sigma * g)


def lognormal27(nx: int, ny: int | None = None, nz: int | None = None, sigma: float = 1.0,
                corr_len: float = 8.0, seed: int = 0, shift: float = 1e-3) -> Csr:
    """3D 27-point operator from a lognormal cell field k.

    For every pair of neighbouring cells p, q (the 26 neighbours of the 3x3x3 box)
    the edge coefficient is the harmonic mean 2 k_p k_q / (k_p + k_q) divided by the
    squared offset length (1 face, 2 edge, 3 corner).  a_pq = -coef_pq and
    a_pp = sum_q coef_pq + ``shift``; neighbours outside the box are dropped."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    shape = (nx, ny, nz)
    k = lognormal_field((nz, ny, nx), sigma, corr_len, seed).ravel()  # index x + nx*(y + ny*z)
    n = nx * ny * nz
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    x = x.ravel()
    y = y.ravel()
    z = z.ravel()
    idx = np.arange(n, dtype=np.int64)
    rows, cols, vals = [], [], []
    diag = np.full(n, shift, dtype=np.float64)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                if dx == 0 and dy == 0 and dz == 0:
                    continue
                mask = ((x + dx >= 0) & (x + dx < nx) & (y + dy >= 0) & (y + dy < ny)
                        & (z + dz >= 0) & (z + dz < nz))
                p = idx[mask]
                q = p + dx + nx * (dy + ny * dz)
                kp = k[p]
                kq = k[q]
                coef = 2.0 * kp * kq / (kp + kq) / float(dx * dx + dy * dy + dz * dz)
                rows.append(p)
                cols.append(q)
                vals.append(-coef)
                np.add.at(diag, p, coef)
    rows.append(idx)
    cols.append(idx)
    vals.append(diag)
    del shape
    return _from_coo(n, np.concatenate(rows), np.concatenate(cols), np.concatenate(vals))


def variable_poisson2d(nx: int, ny: int | None = None, sigma: float = 1.0, corr_len: float = 8.0,
                       seed: int = 0, wind=(0.0, 0.0), reaction: float = 0.0) -> Csr:
    """2D 5-point variable-coefficient convection-diffusion-reaction.

    Face coefficients are harmonic means of a lognormal cell field (sigma, corr_len);
    ``wind`` = (w_x h, w_y h) adds first-order upwind convection; ``reaction`` is added
    to the diagonal (negative values make the operator indefinite)."""
    ny = nx if ny is None else ny
    n = nx * ny
    k = lognormal_field((ny, nx), sigma, corr_len, seed).ravel()
    y, x = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    x = x.ravel()
    y = y.ravel()
    idx = np.arange(n, dtype=np.int64)
    rows, cols, vals = [], [], []
    diag = np.full(n, float(reaction), dtype=np.float64)
    wx, wy = float(wind[0]), float(wind[1])
    for (dx, dy, w) in ((-1, 0, wx), (1, 0, -wx), (0, -1, wy), (0, 1, -wy)):
        # w > 0 on the upstream side (-1) is the upwind connection
        mask = (x + dx >= 0) & (x + dx < nx) & (y + dy >= 0) & (y + dy < ny)
        p_all = idx
        q_all = idx + dx + nx * dy
        kq = np.where(mask, k[np.clip(q_all, 0, n - 1)], k)
        coef = 2.0 * k * kq / (k + kq)
        conv = max(w, 0.0)
        # Dirichlet: the face to the boundary still contributes to the diagonal
        np.add.at(diag, p_all, coef + conv)
        p = p_all[mask]
        rows.append(p)
        cols.append(q_all[mask])
        vals.append(-(coef[mask] + conv))
    rows.append(idx)
    cols.append(idx)
    vals.append(diag)
    return _from_coo(n, np.concatenate(rows), np.concatenate(cols), np.concatenate(vals))


def _lambda_min_estimate(a: Csr, steps: int = 30, seed: int = 0) -> float:
    """Smallest eigenvalue estimate of the symmetric part (A + A^T)/2 from a few
    Lanczos steps (the Ritz value at the bottom of the tridiagonal spectrum)."""
    import scipy.sparse as sp

    m = a.to_scipy()
    s = ((m + m.T) * 0.5).tocsr()
    rng = np.random.default_rng(seed)
    q = rng.standard_normal(a.n)
    q /= np.linalg.norm(q)
    q_prev = np.zeros_like(q)
    alphas, betas = [], []
    beta = 0.0
    for _ in range(min(steps, a.n)):
        w = s @ q - beta * q_prev
        alpha = float(q @ w)
        w -= alpha * q
        beta = float(np.linalg.norm(w))
        alphas.append(alpha)
        if beta < 1e-14:
            break
        betas.append(beta)
        q_prev, q = q, w / beta
    t = np.diag(alphas)
    for i, b in enumerate(betas[: len(alphas) - 1]):
        t[i, i + 1] = t[i + 1, i] = b
    del sp
    return float(np.linalg.eigvalsh(t)[0])


def cdr2d(nx: int, seed: int, sigma: float = 1.5, max_peclet: float = 5.0, corr_len: float = 8.0,
          reaction_frac: float = 0.5) -> Csr:
    """Learned-shift stress matrix: 2D 5-point convection-diffusion-reaction.

    Lognormal diffusion (sigma = 1.5), a random wind direction with cell Peclet drawn
    uniformly up to ``max_peclet`` (relative to the mean face coefficient), and a
    negative reaction -s I with s ~ U[0, reaction_frac * lambda_min-estimate] of the
    operator's symmetric part, which makes the system mildly indefinite."""
    rng = np.random.default_rng(seed)
    pe = rng.uniform(0.0, max_peclet)
    ang = rng.uniform(0.0, 2.0 * np.pi)
    wdir = np.array([np.cos(ang), np.sin(ang)])
    # cell Peclet relative to a unit diffusion: |w| h / (2 D) = pe -> w h = 2 pe
    wind = 2.0 * pe * wdir
    a0 = variable_poisson2d(nx, nx, sigma=sigma, corr_len=corr_len, seed=int(rng.integers(1 << 31)),
                            wind=wind)
    lam = _lambda_min_estimate(a0, seed=int(rng.integers(1 << 31)))
    s = rng.uniform(0.0, reaction_frac * max(lam, 0.0))
    vals = a0.values.copy()
    rows = np.repeat(np.arange(a0.n), np.diff(a0.row_ptr))
    vals[a0.col_idx == rows] -= s
    return Csr(a0.n, a0.row_ptr, a0.col_idx, vals)


def batched_systems(count: int, seed: int, side_lo: int = 32, side_hi: int = 224, sigma: float = 1.0):
    """``count`` variable-coefficient 5-point Poisson systems with sides ~ U[lo, hi]."""
    rng = np.random.default_rng(seed)
    sides = rng.integers(side_lo, side_hi + 1, size=count)
    return [variable_poisson2d(int(s), int(s), sigma=sigma, seed=int(rng.integers(1 << 31))) for s in sides]


def random_rhs(a: Csr, seed: int, nrhs: int = 1):
    """x_true ~ U[-1, 1] from ``seed`` and b = A x_true (float64).  Returns (x, b);
    with nrhs > 1 both are (nrhs, n) arrays."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1.0, 1.0, size=(nrhs, a.n)) if nrhs > 1 else rng.uniform(-1.0, 1.0, size=a.n)
    b = spmv(a, x) if nrhs == 1 else np.stack([spmv(a, xi) for xi in x])
    return x, b


def spmv(a: Csr, x: np.ndarray) -> np.ndarray:
    """y = A x with each row summed in column order (as CsrMatVec does,
    src/csr_matrix.cpp:163-171), vectorised over rows."""
    rows = np.repeat(np.arange(a.n), np.diff(a.row_ptr))
    prod = a.values * x[a.col_idx]
    # np.add.reduceat sums each row's segment left to right
    out = np.zeros(a.n)
    nonempty = np.diff(a.row_ptr) > 0
    starts = a.row_ptr[:-1][nonempty]
    if starts.size:
        out[nonempty] = np.add.reduceat(prod, starts)
    del rows
    return out
