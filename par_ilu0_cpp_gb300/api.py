"""Python mirror of the reference's ILU/GMRES interface over the LLJBASH_* C ABI.

The classes follow lljbash::IluSolver / lljbash::PreconditionedGmres
(include/ilu_solver.hpp:8-30, include/gmres.hpp:9-22 of the reference) and call the
native library ``lib/libpar-ilu0-gmres_c.so`` through ctypes; every computation runs
in that library (CUDA kernels for the numeric work, host C++ for the symbolic
analysis).  There is no Python or CPU fallback: if the library is missing, loading it
raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from .generators import Csr

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(PKG, "lib")
C_LIB_PATH = os.path.join(LIB_DIR, "libpar-ilu0-gmres_c.so")
CORE_LIB_PATH = os.path.join(LIB_DIR, "libpar-ilu0-gmres.so")

_I = ctypes.POINTER(ctypes.c_int)
_D = ctypes.POINTER(ctypes.c_double)
_F = ctypes.POINTER(ctypes.c_float)


class CsrMatrix(ctypes.Structure):
    """struct LLJBASH_CsrMatrix (include/csr_matrix.h)."""

    _fields_ = [("size", ctypes.c_int), ("max_nnz", ctypes.c_int), ("row_ptr", _I), ("col_idx", _I),
                ("value", _D)]


class GmresParameters(ctypes.Structure):
    _fields_ = [("tolerance", ctypes.c_double), ("krylov_subspace_dimension", ctypes.c_int),
                ("max_iterations", ctypes.c_int)]


class GmresStat(ctypes.Structure):
    _fields_ = [("total_init_time", ctypes.c_double), ("total_fgmr_time", ctypes.c_double),
                ("total_mv_time", ctypes.c_double), ("total_precon_time", ctypes.c_double)]


class IluInfo(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("nnz", ctypes.c_int), ("levels_lower", ctypes.c_int),
                ("levels_upper", ctypes.c_int), ("breakdowns", ctypes.c_int), ("first_breakdown", ctypes.c_int),
                ("factor_ms", ctypes.c_double), ("kernel_launches", ctypes.c_longlong), ("shift_applied", ctypes.c_int),
                ("block_rows_fp64", ctypes.c_int), ("block_rows_fp32", ctypes.c_int),
                ("block_cluster_fp64", ctypes.c_int), ("block_cluster_fp32", ctypes.c_int),
                ("row_lanes_lower", ctypes.c_int), ("row_lanes_upper", ctypes.c_int),
                ("factor_lane", ctypes.c_int), ("grid_fp64", ctypes.c_int), ("grid_fp32", ctypes.c_int),
                ("grid_nx", ctypes.c_int),
                ("grid_ny", ctypes.c_int), ("grid_nz", ctypes.c_int), ("grid_warp_y", ctypes.c_int),
                ("grid_warp_z", ctypes.c_int), ("grid_cta_y", ctypes.c_int), ("grid_cta_z", ctypes.c_int),
                ("grid_blocks", ctypes.c_int), ("grid_cluster", ctypes.c_int), ("factor_subtree_parts", ctypes.c_int),
                ("factor_subtree_rows", ctypes.c_int)]


class GmresReport(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("iterations", ctypes.c_int), ("cycles", ctypes.c_int),
                ("converged", ctypes.c_int), ("residual", ctypes.c_double), ("solve_ms", ctypes.c_double),
                ("kernel_launches", ctypes.c_longlong)]


ILU_OPT_COPY_BACK = 1
ILU_OPT_BLOCK_ROWS = 2
ILU_OPT_SOLVE_WARPS = 3
ILU_OPT_ROW_LANES = 4
ILU_OPT_WAIT_LIMIT_US = 5
ILU_OPT_GRID = 6
ILU_OPT_GRID_WARP_Y = 7
ILU_OPT_GRID_CTA_Y = 8
ILU_OPT_GRID_CTA_Z = 9
ILU_OPT_GRID_CLUSTER = 13
ILU_OPT_SWEEP_TIMELINE = 14
ILU_OPT_GRID_ONE_CTA_PER_SM = 15
LINE_TIMELINE_WORDS = 12  # values per block of a sweep timeline
ILU_OPT_TICKET_ORDER = 11
ILU_OPT_FACTOR_KERNEL = 12
GMRES_OPT_MODE = 1
GMRES_OPT_TAU = 2
GMRES_OPT_USE_GRAPH = 3
GMRES_OPT_PROFILE = 4
GMRES_OPT_KEEP_MATRIX = 5
GMRES_OPT_VERIFY = 6
KERNEL_KINDS = ("residual", "sptrsv_lower", "sptrsv_upper", "spmv", "cgs_dot", "cgs_axpy_dot", "cgs_axpy_norm",
                "update")

_LIB = None


def library_path() -> str:
    return C_LIB_PATH


def load() -> ctypes.CDLL:
    """Loads the C-ABI library (raises OSError / FileNotFoundError if it is not built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.isfile(C_LIB_PATH):
        raise FileNotFoundError(f"native library not built: {C_LIB_PATH} (run __graft_entry__.build())")
    lib = ctypes.CDLL(C_LIB_PATH)
    sig = {
        "LLJBASH_SetupCsrMatrix": (None, [ctypes.POINTER(CsrMatrix), ctypes.c_int, ctypes.c_int]),
        "LLJBASH_CopyCsrMatrix": (None, [ctypes.POINTER(CsrMatrix), ctypes.POINTER(CsrMatrix)]),
        "LLJBASH_CopyCsrMatrixValues": (None, [ctypes.POINTER(CsrMatrix), ctypes.POINTER(CsrMatrix)]),
        "LLJBASH_DestroyCsrMatrix": (None, [ctypes.POINTER(CsrMatrix)]),
        "LLJBASH_ReadCsrMatrixMM1": (None, [ctypes.POINTER(CsrMatrix), ctypes.c_char_p]),
        "LLJBASH_CsrMatVec": (None, [ctypes.POINTER(CsrMatrix), _D, _D]),
        "LLJBASH_CsrAmdOrder": (ctypes.c_int, [ctypes.POINTER(CsrMatrix), _I, _I]),
        "LLJBASH_CsrNdOrder": (ctypes.c_int, [ctypes.POINTER(CsrMatrix), _I, _I]),
        "LLJBASH_IlukSymbolic": (ctypes.c_int, [ctypes.POINTER(CsrMatrix), ctypes.c_int, ctypes.POINTER(CsrMatrix), _I]),
        "LLJBASH_IluSolverCreate": (ctypes.c_void_p, [ctypes.c_int]),
        "LLJBASH_IluSolverDestroy": (None, [ctypes.c_void_p]),
        "LLJBASH_IluSolverGetMatrix": (ctypes.POINTER(CsrMatrix), [ctypes.c_void_p]),
        "LLJBASH_IluSolverSetup": (ctypes.c_int, [ctypes.c_void_p]),
        "LLJBASH_IluSolverFactorize": (ctypes.c_int, [ctypes.c_void_p]),
        "LLJBASH_GmresCreate": (ctypes.c_void_p, []),
        "LLJBASH_GmresDestroy": (None, [ctypes.c_void_p]),
        "LLJBASH_GmresGetParameters": (ctypes.POINTER(GmresParameters), [ctypes.c_void_p]),
        "LLJBASH_GmresGetStat": (ctypes.POINTER(GmresStat), [ctypes.c_void_p]),
        "LLJBASH_GmresSetPreconditioner": (None, [ctypes.c_void_p, ctypes.c_void_p]),
        "LLJBASH_GmresSolve": (ctypes.c_bool, [ctypes.c_void_p, ctypes.POINTER(CsrMatrix), _D, _D, _I]),
        "LLJBASH_Gb300LastError": (ctypes.c_char_p, []),
        "LLJBASH_IluSolverSubstitute": (ctypes.c_int, [ctypes.c_void_p, _D, _D]),
        "LLJBASH_IluSolverFactorizeDevice": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
        "LLJBASH_IluSolverSubstituteDeviceNoAlloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
        "LLJBASH_GmresSolveDevice": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _I]),
        "LLJBASH_IluSolverSetOption": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]),
        "LLJBASH_IluSolverSetShift": (ctypes.c_int, [ctypes.c_void_p, _D]),
        "LLJBASH_IluSolverGetInfo": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(IluInfo)]),
        "LLJBASH_IluSolverGetAnalysis": (ctypes.c_int, [ctypes.c_void_p, _I, _I, _I, _I, _I]),
        "LLJBASH_IluSolverGetSweepTimeline": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                             ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int]),
        "LLJBASH_Gb300AnalyzePattern": (ctypes.c_int, [ctypes.c_int, _I, _I, _I, _I, _I, _I, _I, _I]),
        "LLJBASH_Gb300TreeSchedule": (ctypes.c_int, [ctypes.c_int, _I, _I, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                     ctypes.c_double, _I, _I, _I, _I, _I, _I]),
        "LLJBASH_GmresSetOption": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]),
        "LLJBASH_GmresGetReport": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(GmresReport)]),
        "LLJBASH_GmresGetKernelTimes": (ctypes.c_int, [ctypes.c_void_p, _D, ctypes.POINTER(ctypes.c_longlong),
                                                       ctypes.c_int]),
        "LLJBASH_GmresResetKernelTimes": (ctypes.c_int, [ctypes.c_void_p]),
        "LLJBASH_IluSolverSetShiftModel": (ctypes.c_int, [ctypes.c_void_p, _F, ctypes.c_int, ctypes.c_double]),
        "LLJBASH_ShiftModelNumParams": (ctypes.c_int, []),
        "LLJBASH_ShiftFeatures": (ctypes.c_int, [ctypes.c_int, _I, _I, _D, _I, ctypes.c_int, _F, _F, _F]),
        "LLJBASH_ShiftTrainerCreate": (ctypes.c_void_p, [ctypes.c_uint]),
        "LLJBASH_ShiftTrainerDestroy": (None, [ctypes.c_void_p]),
        "LLJBASH_ShiftTrainerSetData": (ctypes.c_int, [ctypes.c_void_p, _F, _F, ctypes.c_int]),
        "LLJBASH_ShiftTrainerSetParams": (ctypes.c_int, [ctypes.c_void_p, _F]),
        "LLJBASH_ShiftTrainerGetParams": (ctypes.c_int, [ctypes.c_void_p, _F]),
        "LLJBASH_ShiftTrainerStep": (ctypes.c_int, [ctypes.c_void_p, _I, ctypes.c_int, ctypes.c_float,
                                                    ctypes.POINTER(ctypes.c_double)]),
        "LLJBASH_ShiftTrainerGradient": (ctypes.c_int, [ctypes.c_void_p, _F, ctypes.POINTER(ctypes.c_double)]),
        "LLJBASH_ShiftTrainerPredict": (ctypes.c_int, [ctypes.c_void_p, _F]),
        "LLJBASH_BatchCreate": (ctypes.c_void_p, [ctypes.c_int, _I, _I, _I, _D, ctypes.c_int, ctypes.c_int,
                                                  ctypes.c_double, ctypes.c_int]),
        "LLJBASH_BatchCreateEx": (ctypes.c_void_p, [ctypes.c_int, _I, _I, _I, _D, _D, ctypes.c_int, ctypes.c_int,
                                                    ctypes.c_double, ctypes.c_int]),
        "LLJBASH_BatchDestroy": (None, [ctypes.c_void_p]),
        "LLJBASH_BatchSetShiftModel": (ctypes.c_int, [ctypes.c_void_p, _F, ctypes.c_int, ctypes.c_double]),
        "LLJBASH_BatchAutotune": (ctypes.c_int, [ctypes.c_void_p, _I, _I]),
        "LLJBASH_BatchGetShape": (ctypes.c_int, [ctypes.c_void_p, _I, _I, _I]),
        "LLJBASH_BatchSetShape": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
        "LLJBASH_BatchGetTrials": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _I, _I, _I, _D]),
        "LLJBASH_BatchSolve": (ctypes.c_int, [ctypes.c_void_p, _D, _D, _I, _D, _I, ctypes.POINTER(ctypes.c_double)]),
    }
    for name, (res, args) in sig.items():
        if hasattr(lib, name):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
    _LIB = lib
    return lib


def last_error() -> str:
    return load().LLJBASH_Gb300LastError().decode()


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ip(a):
    return a.ctypes.data_as(_I)


def _dp(a):
    return a.ctypes.data_as(_D)


def _fp(a):
    return a.ctypes.data_as(_F) if a is not None else None


class HostCsrView:
    """A CsrMatrix struct pointing at numpy arrays (no copy).  Keep it alive while the
    library uses it."""

    def __init__(self, a: Csr):
        self._rp = _i32(a.row_ptr)
        self._ci = _i32(a.col_idx)
        self._v = _f64(a.values)
        self.s = CsrMatrix(a.n, int(self._rp[-1]), _ip(self._rp), _ip(self._ci), _dp(self._v))

    @property
    def ref(self):
        return ctypes.byref(self.s)


def _fill_owned(dst_ptr, a: Csr) -> None:
    """SetupCsrMatrix(dst, n, nnz) and copy a's arrays into the library-owned storage."""
    lib = load()
    lib.LLJBASH_SetupCsrMatrix(dst_ptr, a.n, a.nnz)
    m = dst_ptr.contents
    ctypes.memmove(m.row_ptr, _i32(a.row_ptr).ctypes.data, 4 * (a.n + 1))
    if a.nnz:
        ctypes.memmove(m.col_idx, _i32(a.col_idx).ctypes.data, 4 * a.nnz)
        ctypes.memmove(m.value, _f64(a.values).ctypes.data, 8 * a.nnz)


class OwnedCsr:
    """A CsrMatrix whose arrays the library allocates (SetupCsrMatrix: page-locked where
    a GPU is usable, so host<->device copies run at full link speed), holding a copy of
    ``a``.  Usable wherever a HostCsrView is."""

    def __init__(self, a: Csr):
        self.lib = load()
        self.s = CsrMatrix()
        _fill_owned(ctypes.pointer(self.s), a)

    @property
    def ref(self):
        return ctypes.byref(self.s)

    def __del__(self):
        try:
            self.lib.LLJBASH_DestroyCsrMatrix(ctypes.byref(self.s))
        except Exception:
            pass


def _owned_to_numpy(m: CsrMatrix) -> Csr:
    n = m.size
    rp = np.ctypeslib.as_array(m.row_ptr, shape=(n + 1,)).copy()
    nnz = int(rp[-1])
    ci = np.ctypeslib.as_array(m.col_idx, shape=(nnz,)).copy() if nnz else np.zeros(0, np.int32)
    v = np.ctypeslib.as_array(m.value, shape=(nnz,)).copy() if nnz else np.zeros(0)
    return Csr(n, rp, ci, v)


def iluk_symbolic(a: Csr, lof: int):
    """IlukSymbolic through the C ABI: returns (F, nzmap) with F's values = A scattered."""
    lib = load()
    view = HostCsrView(a)
    f = CsrMatrix(-1, 0, None, None, None)
    nzmap = np.empty(a.nnz, dtype=np.int32)
    knnz = lib.LLJBASH_IlukSymbolic(view.ref, int(lof), ctypes.byref(f), _ip(nzmap))
    if knnz < 0:
        raise RuntimeError("IlukSymbolic failed")
    out = _owned_to_numpy(f)
    lib.LLJBASH_DestroyCsrMatrix(ctypes.byref(f))
    return out, nzmap


def csr_matvec(a: Csr, x) -> np.ndarray:
    lib = load()
    view = HostCsrView(a)
    xx = _f64(x)
    y = np.empty(a.n)
    lib.LLJBASH_CsrMatVec(view.ref, _dp(xx), _dp(y))
    return y


def analyze_pattern(a: Csr):
    """Host analysis: dict(diag, etree_l, etree_u, depth_l, depth_u, nlev)."""
    lib = load()
    n = a.n
    outs = {k: np.empty(n, dtype=np.int32) for k in ("diag", "etree_l", "etree_u", "depth_l", "depth_u")}
    nlev = np.zeros(2, dtype=np.int32)
    rc = lib.LLJBASH_Gb300AnalyzePattern(n, _ip(_i32(a.row_ptr)), _ip(_i32(a.col_idx)), _ip(outs["diag"]),
                                         _ip(outs["etree_l"]), _ip(outs["etree_u"]), _ip(outs["depth_l"]),
                                         _ip(outs["depth_u"]), _ip(nlev))
    if rc != 0:
        raise RuntimeError(f"analysis failed ({rc}): {last_error()}")
    outs["nlev"] = nlev
    return outs


def tree_schedule(a: Csr, upper: bool, nproc: int, granularity: int = 1, relax: float = 1.0):
    """The reference's subtree scheduler on a's pattern: dict(part_ptr, partitions,
    task_queue, subtree_size, subtree_weight)."""
    lib = load()
    n = a.n
    out = {"part_ptr": np.zeros(nproc + 2, dtype=np.int32), "partitions": np.zeros(n, dtype=np.int32),
           "task_queue": np.zeros(n + 1, dtype=np.int32), "subtree_size": np.zeros(n + 1, dtype=np.int32),
           "subtree_weight": np.zeros(n + 1, dtype=np.int32)}
    nt = ctypes.c_int(0)
    rc = lib.LLJBASH_Gb300TreeSchedule(n, _ip(_i32(a.row_ptr)), _ip(_i32(a.col_idx)), int(upper), int(nproc),
                                       int(granularity), float(relax), _ip(out["part_ptr"]), _ip(out["partitions"]),
                                       _ip(out["task_queue"]), ctypes.byref(nt), _ip(out["subtree_size"]),
                                       _ip(out["subtree_weight"]))
    if rc != 0:
        raise RuntimeError(f"tree schedule failed ({rc}): {last_error()}")
    out["task_queue"] = out["task_queue"][: nt.value + 1] if nt.value else out["task_queue"][:0]
    return out


class IluSolver:
    """lljbash::IluSolver over the C ABI (LLJBASH_IluSolver*)."""

    def __init__(self, nthreads: int = 0):
        self.lib = load()
        self.h = self.lib.LLJBASH_IluSolverCreate(int(nthreads))
        self.n = -1

    def close(self):
        if self.h:
            self.lib.LLJBASH_IluSolverDestroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def matrix_ptr(self):
        return self.lib.LLJBASH_IluSolverGetMatrix(self.h)

    def set_matrix(self, f: Csr) -> None:
        """GetMatrix() + SetupCsrMatrix + copy (the test/test.c:16-17 pattern)."""
        _fill_owned(self.matrix_ptr(), f)
        self.n = f.n

    def set_values(self, values) -> None:
        m = self.matrix_ptr().contents
        v = _f64(values)
        ctypes.memmove(m.value, v.ctypes.data, 8 * v.size)

    def values(self) -> np.ndarray:
        m = self.matrix_ptr().contents
        nnz = int(m.row_ptr[m.size])
        return np.ctypeslib.as_array(m.value, shape=(nnz,)).copy()

    def setup(self) -> int:
        return self.lib.LLJBASH_IluSolverSetup(self.h)

    def factorize(self) -> int:
        return self.lib.LLJBASH_IluSolverFactorize(self.h)

    def factorize_device(self, d_values: int) -> int:
        """Factorize from a device pointer (int address) holding nnz(F) doubles."""
        return self.lib.LLJBASH_IluSolverFactorizeDevice(self.h, ctypes.c_void_p(d_values))

    def substitute(self, b) -> np.ndarray:
        bb = _f64(b).copy()
        x = np.empty_like(bb)
        rc = self.lib.LLJBASH_IluSolverSubstitute(self.h, _dp(bb), _dp(x))
        if rc != 0:
            raise RuntimeError(f"substitute failed ({rc}): {last_error()}")
        return x

    def set_option(self, option: int, value: float) -> None:
        if self.lib.LLJBASH_IluSolverSetOption(self.h, int(option), float(value)) != 0:
            raise RuntimeError(last_error())

    def set_shift(self, shift) -> None:
        if shift is None:
            rc = self.lib.LLJBASH_IluSolverSetShift(self.h, None)
        else:
            s = _f64(shift)
            rc = self.lib.LLJBASH_IluSolverSetShift(self.h, _dp(s))
        if rc != 0:
            raise RuntimeError(last_error())

    def set_shift_model(self, params, min_shift: float = 0.0) -> None:
        """Learned-shift MLP parameters (369 floats) for later factorisations; None removes it."""
        if params is None:
            rc = self.lib.LLJBASH_IluSolverSetShiftModel(self.h, None, 0, 0.0)
        else:
            p = np.ascontiguousarray(params, dtype=np.float32)
            rc = self.lib.LLJBASH_IluSolverSetShiftModel(self.h, _fp(p), int(p.size), float(min_shift))
        if rc != 0:
            raise RuntimeError(last_error())

    def info(self) -> IluInfo:
        inf = IluInfo()
        self.lib.LLJBASH_IluSolverGetInfo(self.h, ctypes.byref(inf))
        return inf

    def analysis(self):
        n = self.info().n
        outs = {k: np.empty(n, dtype=np.int32) for k in ("diag", "etree_l", "etree_u", "depth_l", "depth_u")}
        rc = self.lib.LLJBASH_IluSolverGetAnalysis(self.h, _ip(outs["diag"]), _ip(outs["etree_l"]),
                                                   _ip(outs["etree_u"]), _ip(outs["depth_l"]), _ip(outs["depth_u"]))
        if rc != 0:
            raise RuntimeError(last_error())
        return outs

    def sweep_timeline(self, upper: bool, fp32: bool) -> np.ndarray:
        """Per-block timeline [nblocks, 12] (uint64) of the last line-pipeline sweep of
        this kind: compute start (ns), SM id, end of each compute warp, end of the halo
        warp (LLJBASH_IluSolverGetSweepTimeline)."""
        nblk = self.lib.LLJBASH_IluSolverGetSweepTimeline(self.h, int(upper), int(fp32), None, 0)
        if nblk < 0:
            raise RuntimeError(last_error())
        out = np.zeros((nblk, LINE_TIMELINE_WORDS), dtype=np.uint64)
        rc = self.lib.LLJBASH_IluSolverGetSweepTimeline(
            self.h, int(upper), int(fp32), out.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong)), out.size)
        if rc < 0:
            raise RuntimeError(last_error())
        return out


@dataclass
class SolveResult:
    ok: bool
    iterations: int
    x: np.ndarray
    report: GmresReport


class Gmres:
    """lljbash::PreconditionedGmres over the C ABI (LLJBASH_Gmres*)."""

    def __init__(self, tolerance: float = 1e-8, restart: int = 60, max_iterations: int = 200):
        self.lib = load()
        self.h = self.lib.LLJBASH_GmresCreate()
        p = self.params
        p.tolerance = tolerance
        p.krylov_subspace_dimension = restart
        p.max_iterations = max_iterations

    def close(self):
        if self.h:
            self.lib.LLJBASH_GmresDestroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self) -> GmresParameters:
        return self.lib.LLJBASH_GmresGetParameters(self.h).contents

    @property
    def stat(self) -> GmresStat:
        return self.lib.LLJBASH_GmresGetStat(self.h).contents

    def set_preconditioner(self, ilu: IluSolver | None) -> None:
        self.lib.LLJBASH_GmresSetPreconditioner(self.h, ilu.h if ilu is not None else None)

    def set_option(self, option: int, value: float) -> None:
        if self.lib.LLJBASH_GmresSetOption(self.h, int(option), float(value)) != 0:
            raise RuntimeError(last_error())

    def solve(self, a: Csr, rhs, x0=None) -> SolveResult:
        view = HostCsrView(a)
        b = _f64(rhs).copy()
        x = np.zeros(a.n) if x0 is None else _f64(x0).copy()
        its = ctypes.c_int(0)
        ok = self.lib.LLJBASH_GmresSolve(self.h, view.ref, _dp(b), _dp(x), ctypes.byref(its))
        return SolveResult(bool(ok), int(its.value), x, self.report())

    def solve_buffers(self, matrix, rhs: np.ndarray, x: np.ndarray):
        """GmresSolve on caller-owned host buffers, without copies: ``matrix`` a
        HostCsrView or OwnedCsr, ``rhs`` and ``x`` contiguous float64 arrays (``x`` holds
        the initial guess and receives the solution).  Returns (ok, its)."""
        assert rhs.dtype == np.float64 and x.dtype == np.float64
        assert rhs.flags.c_contiguous and x.flags.c_contiguous
        its = ctypes.c_int(0)
        ok = self.lib.LLJBASH_GmresSolve(self.h, matrix.ref, _dp(rhs), _dp(x), ctypes.byref(its))
        return bool(ok), int(its.value)

    def solve_device(self, n: int, d_rp: int, d_ci: int, d_val: int, d_rhs: int, d_sol: int):
        """GMRES on device-resident operands (int device addresses); returns (ok, its)."""
        its = ctypes.c_int(0)
        ok = self.lib.LLJBASH_GmresSolveDevice(self.h, int(n), ctypes.c_void_p(d_rp), ctypes.c_void_p(d_ci),
                                               ctypes.c_void_p(d_val), ctypes.c_void_p(d_rhs), ctypes.c_void_p(d_sol),
                                               ctypes.byref(its))
        return bool(ok), int(its.value)

    def report(self) -> GmresReport:
        r = GmresReport()
        self.lib.LLJBASH_GmresGetReport(self.h, ctypes.byref(r))
        return r

    def kernel_times(self):
        k = len(KERNEL_KINDS)
        ms = np.zeros(k)
        cnt = np.zeros(k, dtype=np.int64)
        self.lib.LLJBASH_GmresGetKernelTimes(self.h, _dp(ms), cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), k)
        return {name: (float(ms[i]), int(cnt[i])) for i, name in enumerate(KERNEL_KINDS)}

    def reset_kernel_times(self) -> None:
        self.lib.LLJBASH_GmresResetKernelTimes(self.h)


def ilu_gmres(a: Csr, b, lof: int = 0, tol: float = 1e-8, restart: int = 30, maxit: int = 1000, mode: int = 0,
              relative: bool = True, x0=None):
    """The test/benchmark.cpp:89-131 sequence through the C ABI: IlukSymbolic -> set F
    values -> Setup -> Factorize -> GMRES.  With ``relative`` the absolute tolerance
    passed to GMRES is tol * ||b||_2 (the reference's test is absolute)."""
    f, _ = iluk_symbolic(a, lof)
    ilu = IluSolver()
    ilu.set_matrix(f)
    rc = ilu.setup()
    if rc != 0:
        raise RuntimeError(f"setup failed ({rc}): {last_error()}")
    rc = ilu.factorize()
    if rc != 0:
        raise RuntimeError(f"factorize failed ({rc}): {last_error()}")
    g = Gmres(tol * (float(np.linalg.norm(b)) if relative else 1.0), restart, maxit)
    g.set_preconditioner(ilu)
    g.set_option(GMRES_OPT_MODE, mode)
    res = g.solve(a, b, x0)
    return res, ilu, g


def shift_features(a: Csr, depth=None, nlev: int = 1, params=None):
    """Per-row MLP features X[n, 4] (and MLP outputs y[n] with params), on the device."""
    lib = load()
    X = np.empty((a.n, 4), dtype=np.float32)
    y = np.empty(a.n, dtype=np.float32) if params is not None else None
    p = np.ascontiguousarray(params, dtype=np.float32) if params is not None else None
    d = _i32(depth) if depth is not None else None
    rc = lib.LLJBASH_ShiftFeatures(a.n, _ip(_i32(a.row_ptr)), _ip(_i32(a.col_idx)), _dp(_f64(a.values)),
                                   _ip(d) if d is not None else None, int(nlev), _fp(X), _fp(p), _fp(y))
    if rc != 0:
        raise RuntimeError(last_error())
    return (X, y) if params is not None else X


class ShiftTrainer:
    """GPU trainer of the shift MLP (hand-written forward / backward / Adam kernels)."""

    def __init__(self, seed: int = 0):
        self.lib = load()
        self.h = self.lib.LLJBASH_ShiftTrainerCreate(int(seed))
        if not self.h:
            raise RuntimeError(last_error())
        self.nparams = self.lib.LLJBASH_ShiftModelNumParams()

    def close(self):
        if self.h:
            self.lib.LLJBASH_ShiftTrainerDestroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_data(self, X, targets):
        self._X = np.ascontiguousarray(X, dtype=np.float32)
        self._T = np.ascontiguousarray(targets, dtype=np.float32)
        self.n = self._T.size
        if self.lib.LLJBASH_ShiftTrainerSetData(self.h, _fp(self._X), _fp(self._T), int(self.n)) != 0:
            raise RuntimeError(last_error())

    @property
    def params(self) -> np.ndarray:
        p = np.empty(self.nparams, dtype=np.float32)
        if self.lib.LLJBASH_ShiftTrainerGetParams(self.h, _fp(p)) != 0:
            raise RuntimeError(last_error())
        return p

    @params.setter
    def params(self, p):
        q = np.ascontiguousarray(p, dtype=np.float32)
        if self.lib.LLJBASH_ShiftTrainerSetParams(self.h, _fp(q)) != 0:
            raise RuntimeError(last_error())

    def step(self, idx, lr: float) -> float:
        ii = _i32(idx)
        loss = ctypes.c_double(0.0)
        if self.lib.LLJBASH_ShiftTrainerStep(self.h, _ip(ii), int(ii.size), float(lr), ctypes.byref(loss)) != 0:
            raise RuntimeError(last_error())
        return float(loss.value)

    def gradient(self):
        g = np.empty(self.nparams, dtype=np.float32)
        loss = ctypes.c_double(0.0)
        if self.lib.LLJBASH_ShiftTrainerGradient(self.h, _fp(g), ctypes.byref(loss)) != 0:
            raise RuntimeError(last_error())
        return g, float(loss.value)

    def predict(self) -> np.ndarray:
        y = np.empty(self.n, dtype=np.float32)
        if self.lib.LLJBASH_ShiftTrainerPredict(self.h, _fp(y)) != 0:
            raise RuntimeError(last_error())
        return y


def fill_reducing_order(a: Csr, method: str = "nd"):
    """CsrNdOrder ("nd") or CsrAmdOrder ("amd") of a's pattern: (p, ip), p[k] the row
    placed k-th and ip its inverse."""
    lib = load()
    p = np.zeros(a.n, np.int32)
    ip = np.zeros(a.n, np.int32)
    f = lib.LLJBASH_CsrNdOrder if method == "nd" else lib.LLJBASH_CsrAmdOrder
    rc = f(HostCsrView(a).ref, _ip(p), _ip(ip))
    if rc != (1 if method == "nd" else 0):
        raise RuntimeError(last_error())
    return p, ip


def reorder(a: Csr, method: str = "nd") -> Csr:
    """P A P^T with the fill-reducing order of `method` (rows sorted by column)."""
    p, _ = fill_reducing_order(a, method)
    sp = a.to_scipy()[p][:, p].tocsr()
    sp.sort_indices()
    return Csr(a.n, sp.indptr.astype(np.int32), sp.indices.astype(np.int32), sp.data.astype(np.float64))


class BatchSolver:
    """Batched persistent ILU(0) + GMRES over many systems x right-hand sides (one launch)."""

    def __init__(self, systems, nrhs: int, restart: int = 30, rtol: float = 1e-8, maxit: int = 1000,
                 factor_values=None):
        """factor_values (optional): per system, the values to factorise (e.g. A plus a
        diagonal shift); GMRES iterates on A."""
        self.lib = load()
        self.systems = systems
        self.nrhs = nrhs
        n = np.array([a.n for a in systems], dtype=np.int32)
        rp = np.concatenate([a.row_ptr for a in systems]).astype(np.int32)
        ci = np.concatenate([a.col_idx for a in systems]).astype(np.int32)
        val = np.concatenate([a.values for a in systems]).astype(np.float64)
        if factor_values is None:
            self.h = self.lib.LLJBASH_BatchCreate(len(systems), _ip(n), _ip(rp), _ip(ci), _dp(val), int(nrhs),
                                                  int(restart), float(rtol), int(maxit))
        else:
            fv = np.concatenate(factor_values).astype(np.float64)
            self.h = self.lib.LLJBASH_BatchCreateEx(len(systems), _ip(n), _ip(rp), _ip(ci), _dp(val), _dp(fv),
                                                    int(nrhs), int(restart), float(rtol), int(maxit))
        if not self.h:
            raise RuntimeError(last_error())
        self.total = int(sum(a.n for a in systems)) * nrhs

    def close(self):
        if self.h:
            self.lib.LLJBASH_BatchDestroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_shift_model(self, params, min_shift: float = 0.0):
        p = np.ascontiguousarray(params, dtype=np.float32) if params is not None else None
        rc = self.lib.LLJBASH_BatchSetShiftModel(self.h, _fp(p), int(p.size) if p is not None else 0, float(min_shift))
        if rc != 0:
            raise RuntimeError(last_error())

    def autotune(self):
        c = ctypes.c_int(0)
        lf = ctypes.c_int(0)
        if self.lib.LLJBASH_BatchAutotune(self.h, ctypes.byref(c), ctypes.byref(lf)) != 0:
            raise RuntimeError(last_error())
        return int(c.value), bool(lf.value)

    def shape(self):
        """(CTAs per SM, largest first, right-hand sides per item) in use."""
        c, lf, g = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        if self.lib.LLJBASH_BatchGetShape(self.h, ctypes.byref(c), ctypes.byref(lf), ctypes.byref(g)) != 0:
            raise RuntimeError(last_error())
        return int(c.value), bool(lf.value), int(g.value)

    def set_shape(self, ctas_per_sm: int, largest_first: bool, rhs_per_cta: int):
        if self.lib.LLJBASH_BatchSetShape(self.h, int(ctas_per_sm), int(bool(largest_first)), int(rhs_per_cta)) != 0:
            raise RuntimeError(last_error())

    def trials(self):
        """The autotuner's trials: list of dicts (ctas_per_sm, largest_first, rhs_per_cta, ms)."""
        k = self.lib.LLJBASH_BatchGetTrials(self.h, 0, None, None, None, None)
        c = np.zeros(max(k, 1), dtype=np.int32)
        lf = np.zeros_like(c)
        g = np.zeros_like(c)
        ms = np.zeros(max(k, 1))
        self.lib.LLJBASH_BatchGetTrials(self.h, k, _ip(c), _ip(lf), _ip(g), _dp(ms))
        return [dict(ctas_per_sm=int(c[i]), largest_first=bool(lf[i]), rhs_per_cta=int(g[i]), ms=float(ms[i]))
                for i in range(k)]

    def solve(self, rhs):
        """rhs: flat array (systems in order, nrhs vectors each).  Returns dict."""
        b = np.ascontiguousarray(rhs, dtype=np.float64)
        assert b.size == self.total
        x = np.empty_like(b)
        k = len(self.systems) * self.nrhs
        its = np.empty(k, dtype=np.int32)
        res = np.empty(k)
        conv = np.empty(k, dtype=np.int32)
        ms = ctypes.c_double(0.0)
        if self.lib.LLJBASH_BatchSolve(self.h, _dp(b), _dp(x), _ip(its), _dp(res), _ip(conv), ctypes.byref(ms)) != 0:
            raise RuntimeError(last_error())
        return dict(x=x, iterations=its, residual=res, converged=conv.astype(bool), ms=float(ms.value))
