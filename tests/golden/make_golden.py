"""Generate the golden fixtures in tests/golden/ by running the REFERENCE itself.

The reference's own sources are compiled (unmodified, against the shim in
oracle/shim) by oracle/build_ref.sh into oracle/_ref/libref.so; this script calls
that library through ctypes on small seeded matrices and stores, per case:

  A (row_ptr, col_idx, values), lof
  F = IlukSymbolic(A, lof): row_ptr, col_idx, nzmap            (src/iluk.cpp:5-54)
  diag_ptr of F                                                 (src/ilu_solver.cpp:276-289)
  Liu etree parent of the L-DAG and the reversed U-DAG          (src/subtree.hpp:35-68)
  level depth of the L-DAG and the reversed U-DAG               (src/subtree.hpp:524-551)
  LU = Factorize(F)                                             (src/ilu_solver.cpp:553-671)
  x_true ~ U[-1,1] (seeded), b = A x_true via CsrMatVec         (src/csr_matrix.cpp:163-171)
  xs = Substitute(b) with 4 threads (descending U sweep)        (src/ilu_solver.cpp:704-734)
  GMRES(m) from x0 = 0 with tol = 1e-8 ||b||: ok flag, its, x   (src/gmres.cpp:138-288)

Run from the repository root (needs the reference checkout):
    python tests/golden/make_golden.py [REFERENCE_DIR]   (default: oracle.reference_dir())
"""
from __future__ import annotations

import os
import zlib
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from par_ilu0_cpp_gb300 import generators as g  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden", "golden_cases.npz")


def random_dd(n: int, density: float, seed: int, nonsym: bool = True) -> g.Csr:
    """Unstructured sparse matrix with a full diagonal, (mostly) diagonally dominant."""
    import scipy.sparse as sp

    rng = np.random.default_rng(seed)
    m = sp.random(n, n, density=density, random_state=rng, format="coo")
    m.data = rng.uniform(-1.0, 1.0, size=m.data.shape)
    if not nonsym:
        m = (m + m.T) * 0.5
    m = m.tocsr()
    rowsum = np.asarray(abs(m).sum(axis=1)).ravel()
    m = m + sp.diags(rowsum + rng.uniform(0.1, 1.0, size=n))
    m = m.tocsr()
    m.sum_duplicates()
    m.sort_indices()
    return g.Csr(n, m.indptr, m.indices, m.data)


def tridiag(n: int) -> g.Csr:
    import scipy.sparse as sp

    m = sp.diags([-1.0 * np.ones(n - 1), 2.5 * np.ones(n), -1.2 * np.ones(n - 1)], [-1, 0, 1]).tocsr()
    m.sort_indices()
    return g.Csr(n, m.indptr, m.indices, m.data)


def cases():
    yield "lap2d_24", g.laplace2d(24), 0, 30
    yield "convdiff3d_10", g.convdiff3d(10), 0, 50
    yield "lognormal27_8_k1", g.lognormal27(8, seed=3), 1, 30
    yield "lognormal27_8_k2", g.lognormal27(8, seed=3), 2, 30
    yield "lap2d_20_k3", g.laplace2d(20), 3, 30
    yield "random_300_k0", random_dd(300, 0.02, seed=11), 0, 20
    yield "random_300_k1", random_dd(300, 0.02, seed=11), 1, 20
    yield "random_sym_200_k2", random_dd(200, 0.03, seed=5, nonsym=False), 2, 20
    yield "tridiag_50", tridiag(50), 0, 10
    yield "cdr2d_16", g.cdr2d(16, seed=7), 0, 40
    yield "varpoisson_20x13", g.variable_poisson2d(20, 13, seed=2), 0, 30
    yield "single_1", g.Csr(1, [0, 1], [0], [3.0]), 0, 5


def main(ref_dir: str | None = None) -> None:
    oracle.build_ref(ref_dir)
    ref = oracle.Ref()
    store = {}
    names = []
    for name, a, lof, m in cases():
        f, nzmap = ref.iluk_symbolic(a, lof)
        diag = ref.diag_ptr(f)
        et_l = ref.etree(f, True)
        et_u = ref.etree(f, False)
        lv_l, nl_l = ref.levels(f, True)
        lv_u, nl_u = ref.levels(f, False)
        lu, _ = ref.factorize(f, nthreads=1)
        rng_seed = zlib.crc32(name.encode())
        rng = np.random.default_rng(rng_seed)
        x_true = rng.uniform(-1.0, 1.0, size=a.n)
        b = ref.matvec(a, x_true)
        xs, _ = ref.substitute(f, lu, b, nthreads=4)
        tol = 1e-8 * float(np.linalg.norm(b))
        res = ref.ilu_gmres(a, b, lof, tol, m, 1000, nthreads=1)
        p = name + "/"
        store.update({
            p + "a_rp": a.row_ptr, p + "a_ci": a.col_idx, p + "a_val": a.values,
            p + "lof": np.int32(lof), p + "restart": np.int32(m),
            p + "f_rp": f.row_ptr, p + "f_ci": f.col_idx, p + "nzmap": nzmap, p + "diag": diag,
            p + "etree_l": et_l, p + "etree_u": et_u, p + "level_l": lv_l, p + "level_u": lv_u,
            p + "nlev": np.array([nl_l, nl_u], dtype=np.int32),
            p + "lu": lu, p + "x_true": x_true, p + "b": b, p + "x_subs": xs,
            p + "tol": np.float64(tol), p + "gmres_ok": np.int32(res["ok"]), p + "gmres_iters": np.int32(res["iters"]),
            p + "gmres_x": res["x"],
        })
        names.append(name)
        print(f"{name}: n={a.n} nnz={a.nnz} knnz={f.nnz} levels={nl_l}/{nl_u} gmres ok={res['ok']} its={res['iters']}",
              file=sys.stderr)
    store["names"] = np.array(names)
    np.savez_compressed(OUT, **store)
    print("wrote", OUT, os.path.getsize(OUT), "bytes", file=sys.stderr)


if __name__ == "__main__":
    main(*sys.argv[1:])
