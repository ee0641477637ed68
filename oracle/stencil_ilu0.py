"""ORACLE — test infrastructure only.

CPU restatement (numpy float64, plain Python loop over rows) of ILU(0) for a full
7-point (3-D) or 5-point (2-D) stencil matrix in natural order, written as the scalar
recurrence on the diagonal that the reference's up-looking row elimination reduces to
on such a pattern (src/ilu_solver.cpp:555-589, `left_looking_col`: for each lower
entry k of row i in ascending column order, tmpa[k] /= u_kk, then tmpa[c] -= u_kc *
tmpa[k] over row k's upper entries c).

On a grid with nx >= 3 and ny >= 3 (ny >= 3 only when nz > 1) the only upper entry of
a lower neighbour k in {i - nx ny, i - nx, i - 1} that lies in row i's pattern is
(k, i) itself, so

    l_ik = a_ik / d_k,    d_i = a_ii - sum_k a_ki l_ik   (k ascending)

and the strictly upper entries of U are A's.  Each product and each difference is
rounded separately, as in the reference's expression.  Returns the factor values in
the CSR layout of the input (L strictly lower, U upper with its diagonal), comparable
entry by entry with the port's `factorize`.
"""
from __future__ import annotations

import numpy as np


def stencil_ilu0(a, nx: int, ny: int, nz: int = 1) -> np.ndarray:
    """ILU(0) factor values of the stencil matrix `a` (row_ptr, col_idx, values, n;
    columns ascending) on an nx x ny x nz grid in natural order."""
    n = a.n
    if n != nx * ny * nz:
        raise ValueError("grid does not match the matrix size")
    if nx < 3 or (ny < 3 and nz > 1) or (ny < 2 and nz == 1):
        raise ValueError("the diagonal recurrence needs nx >= 3 and ny >= 3 (3-D) or ny >= 2 (2-D)")
    rp = np.asarray(a.row_ptr, dtype=np.int64)
    ci = np.asarray(a.col_idx, dtype=np.int64)
    av = np.asarray(a.values, dtype=np.float64)
    lu = av.copy()
    d = np.empty(n)

    def entry(row, col):
        lo, hi = rp[row], rp[row + 1]
        p = lo + np.searchsorted(ci[lo:hi], col)
        if p >= hi or ci[p] != col:
            raise ValueError(f"pattern is not a full stencil: ({row}, {col}) missing")
        return p

    plane = nx * ny
    for i in range(n):
        x = i % nx
        y = (i // nx) % ny
        z = i // plane
        di = av[entry(i, i)]
        for k, present in ((i - plane, z > 0), (i - nx, y > 0), (i - 1, x > 0)):
            if not present:
                continue
            p = entry(i, k)
            lik = av[p] / d[k]
            lu[p] = lik
            di = di - av[entry(k, i)] * lik
        d[i] = di
        lu[entry(i, i)] = di
    return lu
