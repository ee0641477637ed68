"""The allocation-free substitution entry point (LLJBASH_IluSolverSubstituteDeviceNoAlloc).

It exists for callers that cannot call cudaMalloc when they apply the preconditioner —
an application that reserved all device memory for its own pool, or one that must not
let a library allocate (and possibly synchronise the device) inside its pipelined
work.  Its scratch lives in a static device array of the library, so it is limited to
2,097,152 rows.

This file is collected last on purpose: if it fails, a run that stops at the first
failure has already run every other test.  It needs no state from other tests and
passes in a fresh process as well as after the rest of the suite.  The test itself
allocates its input/output buffers through the CUDA runtime (only the entry point under
test must not allocate) and compares two consecutive calls against the existing
LLJBASH_IluSolverSubstitute on the same factors, within the substitution tolerance used
by the parity tests (1e-12)."""
import ctypes
import os

import numpy as np
import pytest

from conftest import rel_err
from par_ilu0_cpp_gb300 import api
from par_ilu0_cpp_gb300 import build as nb
from par_ilu0_cpp_gb300 import generators as g

pytestmark = pytest.mark.gpu

_H2D, _D2H = 1, 2


def _cudart():
    path = os.path.join(nb._cuda_lib_dir(nb._nvcc()), "libcudart.so")
    rt = ctypes.CDLL(path)
    rt.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
    rt.cudaFree.argtypes = [ctypes.c_void_p]
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    return rt


class _DeviceArray:
    def __init__(self, rt, n):
        self.rt = rt
        self.n = n
        self.ptr = ctypes.c_void_p()
        assert rt.cudaMalloc(ctypes.byref(self.ptr), 8 * n) == 0

    def put(self, host):
        h = np.ascontiguousarray(host, dtype=np.float64)
        assert self.rt.cudaMemcpy(self.ptr, h.ctypes.data, 8 * self.n, _H2D) == 0

    def get(self):
        h = np.empty(self.n)
        assert self.rt.cudaMemcpy(h.ctypes.data, self.ptr, 8 * self.n, _D2H) == 0
        return h

    def free(self):
        self.rt.cudaFree(self.ptr)


@pytest.mark.parametrize("make", [lambda: g.laplace2d(64), lambda: g.convdiff3d(20),
                                  lambda: g.lognormal27(8, seed=2)])
def test_no_alloc_substitution_matches_existing_entry_point(make):
    lib = api.load()
    rt = _cudart()
    a = make()
    f, _ = api.iluk_symbolic(a, 0)
    ilu = api.IluSolver()
    ilu.set_matrix(f)
    assert ilu.setup() == 0
    assert ilu.factorize() == 0
    rng = np.random.default_rng(11)
    rhs = [rng.uniform(-1, 1, a.n), rng.uniform(-1, 1, a.n)]
    expected = [ilu.substitute(b) for b in rhs]
    d_b = _DeviceArray(rt, a.n)
    d_x = _DeviceArray(rt, a.n)
    try:
        for b, ref in zip(rhs, expected):  # two calls in a row share the static scratch
            d_b.put(b)
            rc = lib.LLJBASH_IluSolverSubstituteDeviceNoAlloc(ctypes.c_void_p(ilu.h), d_b.ptr, d_x.ptr)
            assert rc == 0, api.last_error()
            assert rel_err(d_x.get(), ref) <= 1e-12
            assert np.array_equal(d_b.get(), b)  # the input is left untouched
    finally:
        d_b.free()
        d_x.free()


def test_no_alloc_rejects_sizes_beyond_its_limit():
    lib = api.load()
    n = (1 << 21) + 1
    a = g.Csr(n, np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32), np.full(n, 2.0))
    ilu = api.IluSolver()
    ilu.set_matrix(a)
    assert ilu.setup() == 0
    assert ilu.factorize() == 0
    rc = lib.LLJBASH_IluSolverSubstituteDeviceNoAlloc(ctypes.c_void_p(ilu.h), ctypes.c_void_p(0), ctypes.c_void_p(0))
    assert rc == -1
    assert "2097152" in api.last_error()
