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

from conftest import banded, rel_err
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


def _solver(a, block_rows=0, solve_warps=0, grid=0):
    f, _ = api.iluk_symbolic(a, 0)
    ilu = api.IluSolver()
    ilu.set_option(api.ILU_OPT_BLOCK_ROWS, block_rows)
    ilu.set_option(api.ILU_OPT_GRID, grid)
    if solve_warps:
        ilu.set_option(api.ILU_OPT_SOLVE_WARPS, solve_warps)
    ilu.set_matrix(f)
    assert ilu.setup() == 0, api.last_error()
    assert ilu.factorize() == 0, api.last_error()
    return ilu


def _no_alloc(lib, ilu, d_b, d_x):
    return lib.LLJBASH_IluSolverSubstituteDeviceNoAlloc(ctypes.c_void_p(ilu.h), d_b.ptr, d_x.ptr)


# Both substitution schedules: the automatic choice (block-local kernels with clusters on
# the 3-D grid, block-local on the 2-D one), the block-local kernel forced with an
# explicit block size, and the level-ordered kernel (-1) on every matrix.
CASES = [("laplace2d_64_auto", lambda: g.laplace2d(64), 0),
         ("laplace2d_64_level", lambda: g.laplace2d(64), -1),
         ("convdiff3d_20_auto", lambda: g.convdiff3d(20), 0),
         ("convdiff3d_20_block", lambda: g.convdiff3d(20), 800),
         ("convdiff3d_20_level", lambda: g.convdiff3d(20), -1),
         ("lognormal27_8_auto", lambda: g.lognormal27(8, seed=2), 0),
         ("lognormal27_8_level", lambda: g.lognormal27(8, seed=2), -1),
         # line-pipeline sweeps forced for both sweeps (no block-local or level packs)
         ("laplace2d_64_line", lambda: g.laplace2d(64), "line"),
         ("convdiff3d_20_line", lambda: g.convdiff3d(20), "line")]


@pytest.mark.parametrize("name,make,block_rows", CASES, ids=[c[0] for c in CASES])
def test_no_alloc_substitution_matches_existing_entry_point(name, make, block_rows):
    lib = api.load()
    rt = _cudart()
    a = make()
    ilu = _solver(a, 0, grid=1) if block_rows == "line" else _solver(a, block_rows)
    info = ilu.info()
    if block_rows == "line":
        assert info.grid_fp64 == 3
    if block_rows == -1:
        assert info.block_rows_fp64 == 0  # level-ordered kernel
    elif block_rows != "line" and block_rows > 0:
        assert info.block_rows_fp64 == block_rows  # block-local kernel
    rng = np.random.default_rng(11)
    rhs = [rng.uniform(-1, 1, a.n), rng.uniform(-1, 1, a.n)]
    expected = [ilu.substitute(b) for b in rhs]
    d_b = _DeviceArray(rt, a.n)
    d_x = _DeviceArray(rt, a.n)
    try:
        for b, ref in zip(rhs, expected):  # two calls in a row share the static scratch
            d_b.put(b)
            rc = _no_alloc(lib, ilu, d_b, d_x)
            assert rc == 0, api.last_error()
            assert rel_err(d_x.get(), ref) <= 1e-12
            assert np.array_equal(d_b.get(), b)  # the input is left untouched
    finally:
        d_b.free()
        d_x.free()


def test_no_alloc_recovers_after_a_wait_gives_up():
    """A call whose device-side wait reaches its limit returns -1 and leaves the shared
    scratch with a set status word; the next call with the normal limit must clear it
    and match the existing entry point.  A 1 us limit cuts short the real waits of the
    1,500-level chain of a banded matrix solved by 1,024 warps (the level-ordered kernel
    takes tasks far ahead of the critical path)."""
    lib = api.load()
    rt = _cudart()
    a = banded(1500, 100, 4)
    ilu = api.IluSolver()
    ilu.set_option(api.ILU_OPT_SOLVE_WARPS, 1024)
    ilu.set_matrix(a)
    assert ilu.setup() == 0, api.last_error()
    assert ilu.factorize() == 0, api.last_error()
    b = np.random.default_rng(8).uniform(-1, 1, a.n)
    ref = ilu.substitute(b)
    d_b = _DeviceArray(rt, a.n)
    d_x = _DeviceArray(rt, a.n)
    try:
        d_b.put(b)
        ilu.set_option(api.ILU_OPT_WAIT_LIMIT_US, 1)
        assert _no_alloc(lib, ilu, d_b, d_x) == -1
        assert "timed out" in api.last_error()
        ilu.set_option(api.ILU_OPT_WAIT_LIMIT_US, 0)
        for _ in range(2):
            assert _no_alloc(lib, ilu, d_b, d_x) == 0, api.last_error()
            assert rel_err(d_x.get(), ref) <= 1e-12
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
