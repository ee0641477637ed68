"""ORACLE — test infrastructure only.

Python bindings for the two CPU checkers of the ILU(k)+GMRES path:

* ``port``: oracle/port/ilu_port.cpp, a plain C++ restatement of the reference's
  algorithm (built by oracle/build_port.sh into oracle/_build/libport.so; builds on
  any host, so it is also the CPU baseline on machines without the reference).
* ``ref``: the reference's own unmodified sources compiled against the shim in
  oracle/shim (oracle/build_ref.sh -> oracle/_ref/libref.so); only available where
  the reference checkout is present.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
package.  The product library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libport.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")
REF_STRICT_SO = os.path.join(HERE, "_ref", "libref_strict.so")

_I = ctypes.POINTER(ctypes.c_int)
_D = ctypes.POINTER(ctypes.c_double)


def _ip(a):
    return a.ctypes.data_as(_I) if a is not None else None


def _dp(a):
    return a.ctypes.data_as(_D) if a is not None else None


def build_port() -> str:
    subprocess.run([os.path.join(HERE, "build_port.sh")], check=True, stdout=subprocess.DEVNULL)
    return PORT_SO


def build_ref(reference_dir: str = "/root/reference") -> str | None:
    if not os.path.isfile(os.path.join(reference_dir, "src", "ilu_solver.cpp")):
        return None
    subprocess.run([os.path.join(HERE, "build_ref.sh"), reference_dir], check=True, stdout=subprocess.DEVNULL)
    return REF_SO


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
