"""ORACLE — test infrastructure only.

Python bindings for the two CPU checkers of the ILU(k)+GMRES path:

* ``port``: oracle/port/ilu_port.cpp, a plain C++ restatement of the reference's
  algorithm (built by oracle/build_port.sh into oracle/_build/libport.so; builds on
  any host, so it is also the CPU baseline on machines without the reference).
* ``ref``: the reference's own unmodified sources compiled against the shim in
  oracle/shim (oracle/build_ref.sh -> oracle/_ref/libref.so, libref_strict.so and the
  threaded-BLAS timing build libref_omp.so); available where the reference checkout is
  present, or where oracle/_ref/src holds the copy staged by build_ref.sh (oracle/_ref
  is git-ignored and travels with the working tree).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
package.  The product library never does.
"""
from __future__ import annotations

import contextlib
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libport.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")
REF_STRICT_SO = os.path.join(HERE, "_ref", "libref_strict.so")
REF_OMP_SO = os.path.join(HERE, "_ref", "libref_omp.so")
REF_STAGE = os.path.join(HERE, "_ref", "src")
# where the reference checkout is read from (PAR_ILU0_REFERENCE_DIR overrides)
DEFAULT_REFERENCE_DIR = "/root/reference"


def reference_dir() -> str:
    return os.environ.get("PAR_ILU0_REFERENCE_DIR", DEFAULT_REFERENCE_DIR)

_I = ctypes.POINTER(ctypes.c_int)
_D = ctypes.POINTER(ctypes.c_double)


def _ip(a):
    return a.ctypes.data_as(_I) if a is not None else None


def _dp(a):
    return a.ctypes.data_as(_D) if a is not None else None


def build_port() -> str:
    subprocess.run([os.path.join(HERE, "build_port.sh")], check=True, stdout=subprocess.DEVNULL)
    return PORT_SO


def reference_file(rel: str) -> str | None:
    """Path of a reference source file (e.g. "test/test.c") in the checkout, else in the
    copy staged by build_ref.sh; None when neither has it."""
    for base in (reference_dir(), REF_STAGE):
        path = os.path.join(base, rel)
        if os.path.isfile(path):
            return path
    return None


def build_ref(ref_dir: str | None = None) -> str | None:
    """Builds oracle/_ref from the reference checkout, or from the staged copy in
    oracle/_ref/src where the checkout is absent; None when neither exists."""
    ref_dir = ref_dir or reference_dir()
    have = os.path.isfile(os.path.join(ref_dir, "src", "ilu_solver.cpp"))
    staged = os.path.isfile(os.path.join(REF_STAGE, "src", "ilu_solver.cpp"))
    if not (have or staged):
        return None
    subprocess.run([os.path.join(HERE, "build_ref.sh"), ref_dir if have else REF_STAGE], check=True,
                   stdout=subprocess.DEVNULL)
    return REF_SO


@contextlib.contextmanager
def c_stdout_to_stderr():
    """Sends what native code prints to stdout (the reference prints its setup times
    there) to stderr for the duration, so that a caller's own stdout (one JSON line)
    stays clean."""
    import sys

    libc = ctypes.CDLL(None)
    sys.stdout.flush()
    libc.fflush(None)
    saved = os.dup(1)
    try:
        os.dup2(2, 1)
        yield
    finally:
        libc.fflush(None)
        os.dup2(saved, 1)
        os.close(saved)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class _Lib:
    """Common wrappers; ``prefix`` is 'port_' or 'ref_'."""

    def __init__(self, path: str, prefix: str):
        if not os.path.isfile(path):
            raise FileNotFoundError(path)
        self.path = path
        self.lib = ctypes.CDLL(path)
        self.p = prefix

    def _f(self, name):
        return getattr(self.lib, self.p + name)

    def diag_ptr(self, a):
        d = np.empty(a.n, dtype=np.int32)
        self._f("diag_ptr")(a.n, _ip(_i32(a.row_ptr)), _ip(_i32(a.col_idx)), _ip(d))
        return d

    def etree(self, a, lower: bool):
        rp, ci = _i32(a.row_ptr), _i32(a.col_idx)
        d = self.diag_ptr(a)
        parent = np.empty(a.n, dtype=np.int32)
        self._f("etree")(a.n, _ip(rp), _ip(ci), _ip(d), int(lower), _ip(parent))
        return parent

    def levels(self, a, lower: bool):
        rp, ci = _i32(a.row_ptr), _i32(a.col_idx)
        d = self.diag_ptr(a)
        depth = np.empty(a.n, dtype=np.int32)
        f = self._f("levels")
        f.restype = ctypes.c_int
        nlev = f(a.n, _ip(rp), _ip(ci), _ip(d), int(lower), _ip(depth))
        return depth, int(nlev)


class Port(_Lib):
    def __init__(self, path: str = PORT_SO):
        super().__init__(path, "port_")
        self.lib.port_factorize.restype = ctypes.c_double
        self.lib.port_iluk_symbolic.restype = ctypes.c_int
        self.lib.port_gmres.restype = ctypes.c_int

    def iluk_symbolic(self, a, lof: int):
        """Returns (f_row_ptr, f_col_idx, f_values(A scattered, fill 0), nzmap)."""
        from par_ilu0_cpp_gb300.generators import Csr

        rp, ci = _i32(a.row_ptr), _i32(a.col_idx)
        knnz = self.lib.port_iluk_symbolic(a.n, _ip(rp), _ip(ci), int(lof))
        frp = np.empty(a.n + 1, dtype=np.int32)
        fci = np.empty(knnz, dtype=np.int32)
        fv = np.empty(knnz, dtype=np.float64)
        nz = np.empty(a.nnz, dtype=np.int32)
        self.lib.port_iluk_fetch(_dp(_f64(a.values)), _ip(frp), _ip(fci), _dp(fv), _ip(nz))
        return Csr(a.n, frp, fci, fv), nz

    def factorize(self, f, nthreads: int = 1):
        vals = _f64(f.values).copy()
        secs = self.lib.port_factorize(f.n, _ip(_i32(f.row_ptr)), _ip(_i32(f.col_idx)), _dp(vals), int(nthreads))
        return vals, float(secs)

    def substitute(self, f, lu, b):
        x = np.empty(f.n)
        self.lib.port_substitute(f.n, _ip(_i32(f.row_ptr)), _ip(_i32(f.col_idx)), _dp(_f64(lu)), _dp(_f64(b)), _dp(x))
        return x

    def matvec(self, a, x):
        y = np.empty(a.n)
        self.lib.port_csr_matvec(a.n, _ip(_i32(a.row_ptr)), _ip(_i32(a.col_idx)), _dp(_f64(a.values)),
                                 _dp(_f64(x)), _dp(y))
        return y

    def gmres(self, a, f, lu, b, tol, restart, maxit, x0=None, nthreads: int = 1):
        """Returns (ok, iters, x, precon_seconds); tol is absolute."""
        x = np.zeros(a.n) if x0 is None else _f64(x0).copy()
        its = ctypes.c_int(0)
        tp = ctypes.c_double(0.0)
        ok = self.lib.port_gmres(a.n, _ip(_i32(a.row_ptr)), _ip(_i32(a.col_idx)), _dp(_f64(a.values)),
                                 _ip(_i32(f.row_ptr)), _ip(_i32(f.col_idx)), _dp(_f64(lu)), _dp(_f64(b)), _dp(x),
                                 ctypes.c_double(tol), int(restart), int(maxit), int(nthreads), ctypes.byref(its),
                                 ctypes.byref(tp))
        return bool(ok), int(its.value), x, float(tp.value)


class Ref(_Lib):
    """The reference itself (compiled from its own sources)."""

    def __init__(self, path: str = REF_SO):
        super().__init__(path, "ref_")
        self.lib.ref_iluk_symbolic.restype = ctypes.c_int
        self.lib.ref_ilu_gmres.restype = ctypes.c_int

    def iluk_symbolic(self, a, lof: int):
        from par_ilu0_cpp_gb300.generators import Csr

        rp, ci, v = _i32(a.row_ptr), _i32(a.col_idx), _f64(a.values)
        knnz = self.lib.ref_iluk_symbolic(a.n, _ip(rp), _ip(ci), _dp(v), int(lof))
        frp = np.empty(a.n + 1, dtype=np.int32)
        fci = np.empty(knnz, dtype=np.int32)
        fv = np.empty(knnz, dtype=np.float64)
        nz = np.empty(a.nnz, dtype=np.int32)
        self.lib.ref_iluk_fetch(_ip(frp), _ip(fci), _dp(fv), _ip(nz))
        return Csr(a.n, frp, fci, fv), nz

    def factorize(self, f, nthreads: int = 1):
        vals = _f64(f.values).copy()
        times = np.zeros(2)
        self.lib.ref_factorize(f.n, _ip(_i32(f.row_ptr)), _ip(_i32(f.col_idx)), _dp(vals), int(nthreads), _dp(times))
        return vals, times

    def substitute(self, f, lu, b, nthreads: int = 1, reps: int = 1):
        x = np.empty(f.n)
        secs = ctypes.c_double(0.0)
        self.lib.ref_substitute(f.n, _ip(_i32(f.row_ptr)), _ip(_i32(f.col_idx)), _dp(_f64(lu)), _dp(_f64(b)),
                                _dp(x), int(nthreads), int(reps), ctypes.byref(secs))
        return x, float(secs.value)

    def matvec(self, a, x):
        y = np.empty(a.n)
        self.lib.ref_csr_matvec(a.n, _ip(_i32(a.row_ptr)), _ip(_i32(a.col_idx)), _dp(_f64(a.values)),
                                _dp(_f64(x)), _dp(y))
        return y

    def ilu_gmres(self, a, b, lof, tol, restart, maxit, nthreads: int = 1, x0=None):
        """Full benchmark.cpp sequence.  Returns dict(ok, iters, x, times, stat)."""
        x = np.zeros(a.n) if x0 is None else _f64(x0).copy()
        its = ctypes.c_int(0)
        times = np.zeros(4)
        stat = np.zeros(2)
        ok = self.lib.ref_ilu_gmres(a.n, _ip(_i32(a.row_ptr)), _ip(_i32(a.col_idx)), _dp(_f64(a.values)), int(lof),
                                    _dp(_f64(b)), _dp(x), ctypes.c_double(tol), int(restart), int(maxit),
                                    int(nthreads), ctypes.byref(its), _dp(times), _dp(stat))
        return dict(ok=bool(ok), iters=int(its.value), x=x, times=times, stat=stat)

    def tree_schedule(self, a, upper, nproc, granularity=1, relax=1.0):
        """The reference's tree_schedule on a's pattern (see ref_driver.cpp)."""
        n = a.n
        rp, ci = _i32(a.row_ptr), _i32(a.col_idx)
        d = self.diag_ptr(a)
        out = {"part_ptr": np.zeros(nproc + 2, dtype=np.int32), "partitions": np.zeros(n, dtype=np.int32),
               "task_queue": np.zeros(n + 1, dtype=np.int32), "subtree_size": np.zeros(n + 1, dtype=np.int32),
               "subtree_weight": np.zeros(n + 1, dtype=np.int32)}
        f = self.lib.ref_tree_schedule
        f.restype = ctypes.c_int
        with c_stdout_to_stderr():
            nt = f(n, _ip(rp), _ip(ci), _ip(d), int(not upper), int(nproc), int(granularity), ctypes.c_double(relax),
                   _ip(out["part_ptr"]), _ip(out["partitions"]), _ip(out["task_queue"]), _ip(out["subtree_size"]),
                   _ip(out["subtree_weight"]))
        out["task_queue"] = out["task_queue"][: nt + 1] if nt else out["task_queue"][:0]
        return out

    def solve_system(self, a, rhs, lof, rtol, restart, maxit, nthreads: int = 1):
        """One system of a batch: symbolic + setup, one Factorize, then a GMRES solve
        from x0 = 0 per row of rhs (nrhs x n) to rtol * ||b_r||_2, all on the calling
        thread (ctypes releases the GIL, so a thread pool runs systems side by side).
        The reference prints to stdout: wrap calls in c_stdout_to_stderr.  Returns
        dict(converged, iters, x, times = [symbolic + setup, factorize, solves] in s)."""
        rhs = np.ascontiguousarray(np.atleast_2d(rhs), dtype=np.float64)
        nrhs = rhs.shape[0]
        x = np.empty_like(rhs)
        its = np.zeros(nrhs, dtype=np.int32)
        times = np.zeros(3)
        f = self.lib.ref_solve_system
        f.restype = ctypes.c_int
        conv = f(a.n, _ip(_i32(a.row_ptr)), _ip(_i32(a.col_idx)), _dp(_f64(a.values)), int(lof), int(restart),
                 int(maxit), ctypes.c_double(rtol), int(nthreads), int(nrhs), _dp(rhs), _dp(x), _ip(its), _dp(times))
        return dict(converged=int(conv), iters=its, x=x, times=times)

    def session(self, a, lof, tol, restart, maxit, nthreads):
        """The test/benchmark.cpp repetition loop: symbolic + first setup now, then
        RefSession.step() = one repetition (Factorize + GMRES timed)."""
        return RefSession(self, a, lof, tol, restart, maxit, nthreads)


class RefSession:
    def __init__(self, ref, a, lof, tol, restart, maxit, nthreads):
        lib = ref.lib
        lib.ref_session_create.restype = ctypes.c_void_p
        lib.ref_session_set_threads.restype = ctypes.c_double
        lib.ref_session_set_threads.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.ref_session_step.argtypes = [ctypes.c_void_p, _D, _D, _I, _D]
        lib.ref_session_destroy.argtypes = [ctypes.c_void_p]
        self.lib = lib
        self.n = a.n
        self._keep = (_i32(a.row_ptr), _i32(a.col_idx), _f64(a.values))
        times = np.zeros(2)
        with c_stdout_to_stderr():
            self.h = lib.ref_session_create(a.n, _ip(self._keep[0]), _ip(self._keep[1]), _dp(self._keep[2]), int(lof),
                                            int(restart), int(maxit), ctypes.c_double(tol), int(nthreads),
                                            _dp(times))
        self.symbolic_s, self.setup_s = float(times[0]), float(times[1])
        self.threads = int(nthreads)

    def set_threads(self, nthreads: int) -> float:
        self.threads = int(nthreads)
        with c_stdout_to_stderr():
            return float(self.lib.ref_session_set_threads(self.h, int(nthreads)))

    def step(self, b):
        """Returns (ok, iters, x, factorize_s, gmres_s)."""
        bb = _f64(b)
        x = np.empty(self.n)
        its = ctypes.c_int(0)
        times = np.zeros(2)
        with c_stdout_to_stderr():
            ok = self.lib.ref_session_step(self.h, _dp(bb), _dp(x), ctypes.byref(its), _dp(times))
        return bool(ok), int(its.value), x, float(times[0]), float(times[1])

    def close(self):
        if self.h:
            self.lib.ref_session_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
