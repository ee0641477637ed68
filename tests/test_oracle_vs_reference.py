"""The oracle port (oracle/port, the restatement of the reference's algorithm) against the
reference's own code, compiled from its sources into oracle/_ref, on inputs the golden
fixtures do not cover: ragged random patterns (rows of 0 .. 40 off-diagonal entries at
random columns, ILU(0) and ILU(1) with rows up to ~500 entries), a 27-point ILU(2)
factor, banded rows of 201 entries, a single row and a diagonal-only matrix.  These are
the inputs the GPU edge-case tests check the CUDA path on, against the port.  Runs where
the reference build loads (the machine it was built on)."""
import numpy as np
import pytest

import oracle
from conftest import banded, csr_from_rows, ragged, rel_err
from par_ilu0_cpp_gb300 import generators as g


@pytest.fixture(scope="module")
def port():
    oracle.build_port()
    return oracle.Port()


@pytest.fixture(scope="module")
def ref():
    try:
        return oracle.Ref(oracle.REF_STRICT_SO)
    except OSError as e:
        pytest.skip(f"reference build not loadable here: {e}")


CASES = [
    ("ragged_ilu0", lambda: ragged(2000, 40, seed=21), 0),
    ("ragged_ilu1", lambda: ragged(2000, 40, seed=22), 1),
    ("lognormal27_10_ilu2", lambda: g.lognormal27(10, seed=4), 2),
    ("banded_100", lambda: banded(600, 100, 5), 0),
    ("single_row", lambda: csr_from_rows(1, [[0]], [[3.0]]), 0),
    ("diagonal_only", lambda: csr_from_rows(50, [[i] for i in range(50)], [[1.0 + i] for i in range(50)]), 0),
]


@pytest.mark.parametrize("name,make,lof", CASES, ids=[c[0] for c in CASES])
def test_port_matches_reference_build(port, ref, name, make, lof):
    a = make()
    f_ref, nz_ref = ref.iluk_symbolic(a, lof)
    f, nz = port.iluk_symbolic(a, lof)
    assert np.array_equal(f.row_ptr, f_ref.row_ptr) and np.array_equal(f.col_idx, f_ref.col_idx)
    assert np.array_equal(nz, nz_ref)
    assert np.array_equal(port.diag_ptr(f), port.diag_ptr(f_ref))
    lu_ref, _ = ref.factorize(f_ref, nthreads=1)
    lu, _ = port.factorize(f, nthreads=1)
    assert rel_err(lu, lu_ref, floor=1e-300) <= 1e-12
    _, b = g.random_rhs(a, seed=31)
    # the reference's multi-threaded substitution order (descending U), which the port follows
    x_ref, _ = ref.substitute(f_ref, lu_ref, b, nthreads=4)
    x = port.substitute(f, lu, b)
    assert rel_err(x, x_ref) <= 1e-12


# ---- the benchmark configurations at full size ---------------------------------------
# The host integer output (ILU(k) pattern, nzmap, diagonal pointers, both elimination
# trees and both level-depth arrays) of the library against the reference build on the
# 128^3 7-point ILU(0) factor and the 64^3 27-point ILU(1) / ILU(2) factors (15.7M and
# 24.0M entries), bit for bit.
FULL = [
    ("convdiff3d_128_ilu0", lambda: g.convdiff3d(128), 0),
    ("lognormal27_64_ilu1", lambda: g.lognormal27(64, seed=0), 1),
    ("lognormal27_64_ilu2", lambda: g.lognormal27(64, seed=0), 2),
]


@pytest.fixture(scope="module")
def ref_fast():
    try:
        return oracle.Ref(oracle.REF_SO)
    except OSError as e:
        pytest.skip(f"reference build not loadable here: {e}")


@pytest.mark.parametrize("name,make,lof", FULL, ids=[c[0] for c in FULL])
def test_host_analysis_bit_exact_at_benchmark_sizes(ref_fast, name, make, lof):
    from par_ilu0_cpp_gb300 import api

    a = make()
    f_ref, nz_ref = ref_fast.iluk_symbolic(a, lof)
    f, nz = api.iluk_symbolic(a, lof)
    assert np.array_equal(f.row_ptr, f_ref.row_ptr)
    assert np.array_equal(f.col_idx, f_ref.col_idx)
    assert np.array_equal(nz, nz_ref)
    an = api.analyze_pattern(f)
    assert np.array_equal(an["diag"], ref_fast.diag_ptr(f_ref))
    assert np.array_equal(an["etree_l"], ref_fast.etree(f_ref, True))
    assert np.array_equal(an["etree_u"], ref_fast.etree(f_ref, False))
    depth_l, nl = ref_fast.levels(f_ref, True)
    depth_u, nu = ref_fast.levels(f_ref, False)
    assert np.array_equal(an["depth_l"], depth_l) and np.array_equal(an["depth_u"], depth_u)
    assert list(an["nlev"]) == [nl, nu]


def test_reference_batch_entry_matches_single_solves():
    """ref_solve_system (one factorisation, a GMRES solve per right-hand side, the batched
    CPU baseline's unit of work) gives the same iterations and solutions as the
    benchmark sequence run once per right-hand side, also from several threads at once."""
    import concurrent.futures

    try:
        ref = oracle.Ref(oracle.REF_OMP_SO)
    except OSError as e:
        pytest.skip(f"reference timing build not loadable here: {e}")
    systems = g.batched_systems(4, 7)
    rhs = [np.atleast_2d(g.random_rhs(a, seed=40 + k, nrhs=3)[1]) for k, a in enumerate(systems)]
    with oracle.c_stdout_to_stderr():
        with concurrent.futures.ThreadPoolExecutor(max_workers=4) as ex:
            out = list(ex.map(lambda k: ref.solve_system(systems[k], rhs[k], 0, 1e-8, 30, 1000, 1), range(4)))
        for k, a in enumerate(systems):
            assert out[k]["converged"] == 3
            for r in range(3):
                b = rhs[k][r]
                one = ref.ilu_gmres(a, b, 0, 1e-8 * float(np.linalg.norm(b)), 30, 1000, nthreads=1)
                assert one["ok"] and one["iters"] == out[k]["iters"][r]
                assert rel_err(out[k]["x"][r], one["x"]) <= 1e-12
