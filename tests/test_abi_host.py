"""Host-side checks of the drop-in library (no GPU needed): it loads, exports every
LLJBASH_* symbol the public headers declare, and its host logic — IlukSymbolic, the
pattern analysis, CsrMatVec, the CsrMatrix lifecycle, ReadCsrMatrixMM1 — matches the
reference bit for bit on the golden fixtures."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from par_ilu0_cpp_gb300 import api
from par_ilu0_cpp_gb300.generators import Csr


def declared_symbols():
    """Every exported name declared in include/*.h: LLJBASH_DECL(Name) macros of the
    reference-compatible headers and the LLJBASH_* prototypes of the extension header."""
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(inc, fn)).read()
        for m in re.finditer(r"#define\s+(\w+)\s+LLJBASH_DECL\(\1\)", text):
            names.add("LLJBASH_" + m.group(1))
        for m in re.finditer(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(LLJBASH_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    # types and inline helpers are not symbols
    for t in ("LLJBASH_CsrMatrix", "LLJBASH_GmresParameters", "LLJBASH_GmresStat", "LLJBASH_IluSolverHdl",
              "LLJBASH_GmresHdl", "LLJBASH_GetCsrNonzeros", "LLJBASH_DECL", "LLJBASH_DEFAULT_VALUE",
              "LLJBASH_STRUCT_TYPEDEF"):
        names.discard(t)
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = api.load()
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_reference_abi_names_present():
    """The names of the reference's C ABI (include_c/*.h, include/csr_matrix.h, iluk.h)."""
    lib = api.load()
    ref_names = ["IluSolverCreate", "IluSolverDestroy", "IluSolverGetMatrix", "IluSolverSetup", "IluSolverFactorize",
                 "GmresCreate", "GmresDestroy", "GmresGetParameters", "GmresGetStat", "GmresSetPreconditioner",
                 "GmresSolve", "SetupCsrMatrix", "CopyCsrMatrix", "CopyCsrMatrixValues", "DestroyCsrMatrix",
                 "ReadCsrMatrixMM1", "CsrMatVec", "CsrAmdOrder", "CsrNdOrder", "IlukSymbolic", "CSR_MATRIX_DEFAULT"]
    for n in ref_names:
        assert hasattr(lib, "LLJBASH_" + n), n
    d = api.CsrMatrix.in_dll(lib, "LLJBASH_CSR_MATRIX_DEFAULT")
    assert d.size == -1 and d.max_nnz == 0 and not d.row_ptr


def test_struct_layouts():
    assert ctypes.sizeof(api.GmresParameters) == 16
    assert ctypes.sizeof(api.GmresStat) == 32
    assert ctypes.sizeof(api.CsrMatrix) == 32


def test_iluk_symbolic_bit_exact(golden):
    f, nzmap = api.iluk_symbolic(golden.a, golden.lof)
    assert np.array_equal(f.row_ptr, golden.f_rp)
    assert np.array_equal(f.col_idx, golden.f_ci)
    assert np.array_equal(nzmap, golden.nzmap)
    ref_vals = np.zeros(len(golden.f_ci))
    ref_vals[golden.nzmap] = golden.a.values
    assert np.array_equal(f.values, ref_vals)


def test_analysis_bit_exact(golden):
    out = api.analyze_pattern(golden.f_csr())
    assert np.array_equal(out["diag"], golden.diag)
    assert np.array_equal(out["etree_l"], golden.etree_l)
    assert np.array_equal(out["etree_u"], golden.etree_u)
    assert np.array_equal(out["depth_l"], golden.level_l)
    assert np.array_equal(out["depth_u"], golden.level_u)
    assert list(out["nlev"]) == list(golden.nlev)


def test_missing_diagonal_reported():
    a = Csr(2, [0, 1, 2], [1, 1], [1.0, 2.0])  # row 0 has no diagonal
    with pytest.raises(RuntimeError):
        api.analyze_pattern(a)
    lib = api.load()
    rc = lib.LLJBASH_Gb300AnalyzePattern(2, a.row_ptr.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                         a.col_idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), None, None, None,
                                         None, None, None)
    assert rc == -2


def test_csr_matvec_matches_golden(golden):
    y = api.csr_matvec(golden.a, golden.x_true)
    assert np.allclose(y, golden.b, rtol=1e-14, atol=1e-14)


def test_csr_lifecycle():
    lib = api.load()
    a = Csr(3, [0, 2, 3, 5], [0, 2, 1, 0, 2], [1.0, 2.0, 3.0, 4.0, 5.0])
    view = api.HostCsrView(a)
    dst = api.CsrMatrix(-1, 0, None, None, None)
    lib.LLJBASH_CopyCsrMatrix(ctypes.byref(dst), view.ref)
    assert dst.size == 3 and dst.max_nnz == 5
    assert [dst.col_idx[i] for i in range(5)] == [0, 2, 1, 0, 2]
    a2 = Csr(3, a.row_ptr, a.col_idx, a.values * 2)
    lib.LLJBASH_CopyCsrMatrixValues(ctypes.byref(dst), api.HostCsrView(a2).ref)
    assert [dst.value[i] for i in range(5)] == [2.0, 4.0, 6.0, 8.0, 10.0]
    assert dst.row_ptr.contents.value == 0 and ctypes.addressof(dst.value.contents) % 64 == 0
    lib.LLJBASH_DestroyCsrMatrix(ctypes.byref(dst))
    assert dst.size == -1 and not dst.row_ptr and not dst.value


def _order(a, nd):
    lib = api.load()
    p = np.zeros(a.n, np.int32)
    ip = np.zeros(a.n, np.int32)
    ptr = lambda v: v.ctypes.data_as(ctypes.POINTER(ctypes.c_int))  # noqa: E731
    f = lib.LLJBASH_CsrNdOrder if nd else lib.LLJBASH_CsrAmdOrder
    return f(api.HostCsrView(a).ref, ptr(p), ptr(ip)), p, ip


@pytest.mark.parametrize("make", [lambda: Csr(3, [0, 1, 2, 3], [0, 1, 2], [1.0, 1.0, 1.0]),
                                  lambda: __import__("par_ilu0_cpp_gb300.generators").generators.laplace2d(40),
                                  lambda: __import__("par_ilu0_cpp_gb300.generators").generators.convdiff3d(14)],
                         ids=["diagonal", "laplace2d_40", "convdiff3d_14"])
def test_fill_reducing_orderings(make):
    """CsrAmdOrder / CsrNdOrder (the library's own AMD and nested dissection): valid
    permutations with the reference's return codes (AMD 0, ND 1 on success), p[k] the
    row placed k-th and ip its inverse, and far less LU fill than the natural order."""
    import scipy.sparse.linalg as sla

    a = make()
    m = a.to_scipy()

    def fill(perm):
        lu = sla.splu(m[perm][:, perm].tocsc(), permc_spec="NATURAL", diag_pivot_thresh=0.0,
                      options=dict(SymmetricMode=True))
        return lu.L.nnz + lu.U.nnz

    natural = fill(np.arange(a.n))
    for nd in (False, True):
        rc, p, ip = _order(a, nd)
        assert rc == (1 if nd else 0)
        assert np.array_equal(np.sort(p), np.arange(a.n)) and np.array_equal(ip[p], np.arange(a.n))
        if a.n > 100:
            assert fill(p) < 0.5 * natural, (nd, fill(p), natural)


def test_ordering_rejects_invalid_input():
    bad = Csr(3, [0, 1, 3, 3], [0, 5, 1], [1.0, 1.0, 1.0])
    rc, _, _ = _order(bad, False)
    assert rc == -1
    rc, _, _ = _order(bad, True)
    assert rc == 0


def _write_mm(path, n, entries):
    with open(path, "w") as fh:
        fh.write("%%MatrixMarket matrix coordinate real general\n% comment\n")
        fh.write(f"{n} {n} {len(entries)}\n")
        for i, j, v in entries:
            fh.write(f"{i + 1} {j + 1} {v!r}\n")


def _read_mm(path):
    lib = api.load()
    m = api.CsrMatrix(-1, 0, None, None, None)
    lib.LLJBASH_ReadCsrMatrixMM1(ctypes.byref(m), path.encode())
    out = api._owned_to_numpy(m)
    lib.LLJBASH_DestroyCsrMatrix(ctypes.byref(m))
    return out


def test_read_mm_row_matching_known_answer(tmp_path):
    # Rows 0 and 1 lack a usable diagonal; the maximum matching swaps them.
    entries = [(0, 1, 2.0), (1, 0, 3.0), (2, 2, 4.0), (0, 2, 1.0)]
    p = str(tmp_path / "swap.mtx")
    _write_mm(p, 3, entries)
    m = _read_mm(p)
    assert list(m.row_ptr) == [0, 1, 3, 4]
    assert list(m.col_idx) == [0, 1, 2, 2]
    assert list(m.values) == [3.0, 2.0, 1.0, 4.0]


def test_read_mm_matches_reference(tmp_path):
    """Against the reference's own ReadCsrMatrixMM1 (needs oracle/_ref)."""
    import oracle

    if not os.path.isfile(oracle.REF_SO):
        pytest.skip("reference library not built here")
    ref = ctypes.CDLL(oracle.REF_SO)
    rng = np.random.default_rng(3)
    n = 60
    entries = []
    for i in range(n):
        cols = rng.choice(n, size=4, replace=False)
        for j in cols:
            entries.append((i, int(j), float(rng.uniform(-2, 2))))
    # a full permutation guarantees a perfect matching
    perm = rng.permutation(n)
    have = {(i, j) for i, j, _ in entries}
    for i in range(n):
        if (i, int(perm[i])) not in have:
            entries.append((i, int(perm[i]), float(rng.uniform(1, 2))))
    rng.shuffle(entries)
    p = str(tmp_path / "rand.mtx")
    _write_mm(p, n, entries)
    mine = _read_mm(p)
    m = api.CsrMatrix(-1, 0, None, None, None)
    ref.LLJBASH_ReadCsrMatrixMM1(ctypes.byref(m), p.encode())
    theirs = api._owned_to_numpy(m)
    assert np.array_equal(mine.row_ptr, theirs.row_ptr)
    assert np.array_equal(mine.col_idx, theirs.col_idx)
    assert np.array_equal(mine.values, theirs.values)


def test_ilu_option_values_checked():
    """Option values are validated on the host, before any device work."""
    ilu = api.IluSolver()
    for v in (0, 1, 2, 4, 8, 16, 32):
        ilu.set_option(api.ILU_OPT_ROW_LANES, v)
    for v in (3, 64, -1, 2.5):
        with pytest.raises(RuntimeError):
            ilu.set_option(api.ILU_OPT_ROW_LANES, v)
    for v in (0, 1, 4000000):
        ilu.set_option(api.ILU_OPT_WAIT_LIMIT_US, v)
    for v in (-1, 0.5, 3e9):
        with pytest.raises(RuntimeError):
            ilu.set_option(api.ILU_OPT_WAIT_LIMIT_US, v)
    for v in (-2, -1, 0, 16384):
        ilu.set_option(api.ILU_OPT_BLOCK_ROWS, v)
    with pytest.raises(RuntimeError):
        ilu.set_option(api.ILU_OPT_BLOCK_ROWS, -3)
    for v in (-1, 0, 1):
        ilu.set_option(api.ILU_OPT_GRID, v)
    for v in (2, -2, 0.5):
        with pytest.raises(RuntimeError):
            ilu.set_option(api.ILU_OPT_GRID, v)
    for v in (0, 1, 4, 8):
        ilu.set_option(api.ILU_OPT_GRID_WARP_Y, v)
    for v in (2, 3, 16, 32, 64, -1):
        with pytest.raises(RuntimeError):
            ilu.set_option(api.ILU_OPT_GRID_WARP_Y, v)
    for opt in (api.ILU_OPT_GRID_CTA_Y, api.ILU_OPT_GRID_CTA_Z):
        ilu.set_option(opt, 0)
        ilu.set_option(opt, 7)
        for v in (-3, 9, 1.5):
            with pytest.raises(RuntimeError):
                ilu.set_option(opt, v)
    for v in (0, 1, 2, 8, 16):
        ilu.set_option(api.ILU_OPT_GRID_CLUSTER, v)
    for v in (-1, 17, 2.5):
        with pytest.raises(RuntimeError):
            ilu.set_option(api.ILU_OPT_GRID_CLUSTER, v)
    for v in (0, 1):
        ilu.set_option(api.ILU_OPT_SWEEP_TIMELINE, v)
        ilu.set_option(api.ILU_OPT_GRID_ONE_CTA_PER_SM, v)
    with pytest.raises(RuntimeError):
        ilu.set_option(api.ILU_OPT_GRID_ONE_CTA_PER_SM, 2)
    for v in (2, -1):
        with pytest.raises(RuntimeError):
            ilu.set_option(api.ILU_OPT_SWEEP_TIMELINE, v)
    with pytest.raises(RuntimeError):  # nothing recorded before SetupMatrix
        ilu.sweep_timeline(False, False)
    for v in (0, 1, 2):
        ilu.set_option(api.ILU_OPT_TICKET_ORDER, v)
    with pytest.raises(RuntimeError):
        ilu.set_option(api.ILU_OPT_TICKET_ORDER, 3)
    with pytest.raises(RuntimeError):
        ilu.set_option(12345, 1)
