"""Structural checks of caller CSR matrices.

A corrupted CSR from a C caller (row pointers that decrease or do not start at 0,
column indices outside [0, n), rows not strictly ascending) must be refused with -1 and
a message before any of it reaches a kernel, where an out-of-range index would make the
kernel read or write outside its buffers.  The host entry points (IluSolverSetup,
Gb300AnalyzePattern, BatchCreate, GmresSolve's array bounds) are checked here on the
CPU; GmresSolve's column check (which overlaps the host->device copies) and
GmresSolveDevice's device-side check need a GPU and are marked ``gpu``.
"""
import ctypes

import numpy as np
import pytest

from par_ilu0_cpp_gb300 import api
from par_ilu0_cpp_gb300 import generators as g
from par_ilu0_cpp_gb300.generators import Csr


def _good():
    # 4x4 with a full diagonal and a few off-diagonal entries
    rp = [0, 2, 5, 7, 9]
    ci = [0, 1, 0, 1, 3, 2, 3, 1, 3]
    va = [4.0, -1.0, -1.0, 4.0, -1.0, 4.0, -1.0, -1.0, 4.0]
    return rp, ci, va


def _corrupted():
    """(name, rp, ci) with rp[n] == len(ci) in every case, so that the arrays really
    hold the entries the row pointers name (only their structure is wrong)."""
    rp, ci, _ = _good()
    out = []
    c = list(ci)
    c[4] = 4  # row 1: column 4 of a 4x4 matrix
    out.append(("column_out_of_range", rp, c))
    c = list(ci)
    c[0] = -1
    out.append(("negative_column", rp, c))
    c = list(ci)
    c[3], c[4] = c[4], c[3]  # row 1: 0, 3, 1
    out.append(("columns_not_ascending", rp, c))
    c = list(ci)
    c[6] = 2  # row 2: 2, 2
    out.append(("duplicate_column", rp, c))
    r = list(rp)
    r[2] = 1  # 0, 2, 1, 7, 9
    out.append(("row_ptr_decreasing", r, ci))
    return out


CORRUPTED = _corrupted()


def _analyze(n, rp, ci):
    lib = api.load()
    rpa = np.asarray(rp, dtype=np.int32)
    cia = np.asarray(ci, dtype=np.int32)
    ip = ctypes.POINTER(ctypes.c_int)
    return lib.LLJBASH_Gb300AnalyzePattern(n, rpa.ctypes.data_as(ip), cia.ctypes.data_as(ip), None, None, None, None,
                                          None, None)


def test_good_matrix_passes():
    rp, ci, va = _good()
    assert _analyze(4, rp, ci) == 0
    an = api.analyze_pattern(Csr(4, rp, ci, va))
    assert list(an["diag"]) == [0, 3, 5, 8]


@pytest.mark.parametrize("name,rp,ci", CORRUPTED, ids=[c[0] for c in CORRUPTED])
def test_analyze_pattern_rejects(name, rp, ci):
    assert _analyze(4, rp, ci) == -1
    assert "invalid CSR matrix" in api.last_error()


@pytest.mark.parametrize("name,rp,ci", CORRUPTED, ids=[c[0] for c in CORRUPTED])
def test_ilu_setup_rejects_before_device_work(name, rp, ci):
    """Setup returns -1 with the message and does no device work (this runs on CPU-only
    machines, where any device call would fail with a different message)."""
    ilu = api.IluSolver()
    ilu.set_matrix(Csr(4, rp, ci, np.ones(len(ci))))
    assert ilu.setup() == -1
    assert "invalid CSR matrix (ILU matrix)" in api.last_error()


def test_ilu_setup_rejects_row_ptr_not_starting_at_zero():
    # rp[0] = 1: the arrays hold rp[n] = 10 entries, the first one never named by a row
    ilu = api.IluSolver()
    m = ilu.matrix_ptr()
    lib = api.load()
    lib.LLJBASH_SetupCsrMatrix(m, 4, 10)
    rp = np.array([1, 3, 6, 8, 10], dtype=np.int32)
    ci = np.array([0, 0, 1, 0, 1, 3, 2, 3, 1, 3], dtype=np.int32)
    ctypes.memmove(m.contents.row_ptr, rp.ctypes.data, 4 * 5)
    ctypes.memmove(m.contents.col_idx, ci.ctypes.data, 4 * 10)
    assert ilu.setup() == -1
    assert "row_ptr[0]" in api.last_error()


def test_ilu_setup_rejects_row_ptr_beyond_capacity():
    ilu = api.IluSolver()
    m = ilu.matrix_ptr()
    lib = api.load()
    lib.LLJBASH_SetupCsrMatrix(m, 4, 9)
    rp = np.array([0, 2, 5, 7, 9], dtype=np.int32)
    ci = np.array([0, 1, 0, 1, 3, 2, 3, 1, 3], dtype=np.int32)
    ctypes.memmove(m.contents.row_ptr, rp.ctypes.data, 4 * 5)
    ctypes.memmove(m.contents.col_idx, ci.ctypes.data, 4 * 9)
    m.contents.max_nnz = 8  # the arrays claim to hold fewer entries than row_ptr[n]
    assert ilu.setup() == -1
    assert "exceeds" in api.last_error()


def test_gmres_rejects_bad_row_ptr_before_device_work():
    rp, ci, va = _good()
    bad = api.CsrMatrix(4, 9, None, None, None)
    rpa = np.array([2, 2, 5, 7, 9], dtype=np.int32)  # row_ptr[0] != 0
    cia = np.asarray(ci, dtype=np.int32)
    vaa = np.asarray(va)
    ip, dp = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
    bad.row_ptr = rpa.ctypes.data_as(ip)
    bad.col_idx = cia.ctypes.data_as(ip)
    bad.value = vaa.ctypes.data_as(dp)
    gm = api.Gmres(1e-8, 10, 100)
    b = np.ones(4)
    x = np.zeros(4)
    its = ctypes.c_int(-7)
    ok = gm.lib.LLJBASH_GmresSolve(gm.h, ctypes.byref(bad), b.ctypes.data_as(dp), x.ctypes.data_as(dp),
                                   ctypes.byref(its))
    assert not ok and its.value == 0
    assert "invalid CSR matrix (GMRES matrix)" in api.last_error()


def test_batch_create_rejects_bad_system():
    a0 = g.laplace2d(4)
    rp, ci, va = _good()
    c = list(ci)
    c[4] = 9
    n = np.array([a0.n, 4], dtype=np.int32)
    rp_all = np.concatenate([a0.row_ptr, np.asarray(rp)]).astype(np.int32)
    ci_all = np.concatenate([a0.col_idx, np.asarray(c)]).astype(np.int32)
    va_all = np.concatenate([a0.values, np.asarray(va)])
    lib = api.load()
    ip, dp = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
    h = lib.LLJBASH_BatchCreate(2, n.ctypes.data_as(ip), rp_all.ctypes.data_as(ip), ci_all.ctypes.data_as(ip),
                                va_all.ctypes.data_as(dp), 1, 10, 1e-8, 100)
    assert not h
    assert "invalid CSR matrix (batched system 1)" in api.last_error()


# ---- GPU: the checks that run next to device work -------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("name,rp,ci", CORRUPTED, ids=[c[0] for c in CORRUPTED])
def test_gmres_host_arrays_rejected_on_gpu(name, rp, ci):
    """GmresSolve copies A while the host checks it; a failed check returns false before
    any kernel runs, and the solver works afterwards."""
    a_good = Csr(4, *_good())
    ilu = api.IluSolver()
    ilu.set_matrix(a_good)
    assert ilu.setup() == 0 and ilu.factorize() == 0
    gm = api.Gmres(1e-10, 10, 100)
    gm.set_preconditioner(ilu)
    res = gm.solve(Csr(4, rp, ci, np.ones(len(ci))), np.ones(4))
    assert not res.ok
    assert "invalid CSR matrix (GMRES matrix)" in api.last_error()
    res = gm.solve(a_good, np.ones(4))
    assert res.ok


@pytest.mark.gpu
@pytest.mark.parametrize("name,rp,ci", CORRUPTED, ids=[c[0] for c in CORRUPTED])
def test_gmres_device_arrays_rejected_on_gpu(name, rp, ci):
    """GmresSolveDevice checks the device arrays with a kernel that reads a row's
    columns only after its bounds have passed; the arrays here hold exactly n + 1 row
    pointers and row_ptr[n] entries."""
    torch = pytest.importorskip("torch")
    a_good = Csr(4, *_good())
    ilu = api.IluSolver()
    ilu.set_matrix(a_good)
    assert ilu.setup() == 0 and ilu.factorize() == 0
    gm = api.Gmres(1e-10, 10, 100)
    gm.set_preconditioner(ilu)
    d_rp = torch.tensor(rp, dtype=torch.int32, device="cuda")
    d_ci = torch.tensor(ci, dtype=torch.int32, device="cuda")
    d_v = torch.ones(len(ci), dtype=torch.float64, device="cuda")
    d_b = torch.ones(4, dtype=torch.float64, device="cuda")
    d_x = torch.zeros(4, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    ok, its = gm.solve_device(4, d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr(), d_b.data_ptr(), d_x.data_ptr())
    assert not ok and its == 0
    assert "invalid CSR matrix (GMRES matrix)" in api.last_error()
    g_rp = torch.tensor(a_good.row_ptr, dtype=torch.int32, device="cuda")
    g_ci = torch.tensor(a_good.col_idx, dtype=torch.int32, device="cuda")
    g_v = torch.tensor(a_good.values, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    ok, its = gm.solve_device(4, g_rp.data_ptr(), g_ci.data_ptr(), g_v.data_ptr(), d_b.data_ptr(), d_x.data_ptr())
    assert ok
