"""The CPU oracle (oracle/port, a restatement of the reference's algorithm) against the
golden fixtures produced by the reference itself (tests/golden/make_golden.py)."""
import numpy as np
import pytest

import oracle
from conftest import rel_err


@pytest.fixture(scope="module")
def port():
    oracle.build_port()
    return oracle.Port()


def test_symbolic_bit_exact(port, golden):
    f, nzmap = port.iluk_symbolic(golden.a, golden.lof)
    assert np.array_equal(f.row_ptr, golden.f_rp)
    assert np.array_equal(f.col_idx, golden.f_ci)
    assert np.array_equal(nzmap, golden.nzmap)


def test_analysis_bit_exact(port, golden):
    f = golden.f_csr()
    assert np.array_equal(port.diag_ptr(f), golden.diag)
    assert np.array_equal(port.etree(f, True), golden.etree_l)
    assert np.array_equal(port.etree(f, False), golden.etree_u)
    dl, nl = port.levels(f, True)
    du, nu = port.levels(f, False)
    assert np.array_equal(dl, golden.level_l) and nl == golden.nlev[0]
    assert np.array_equal(du, golden.level_u) and nu == golden.nlev[1]


def test_factorize_matches_reference(port, golden):
    lu, _ = port.factorize(golden.f_csr(), nthreads=1)
    assert rel_err(lu, golden.lu, floor=1e-300) <= 1e-12
    lu4, _ = port.factorize(golden.f_csr(), nthreads=4)
    assert np.array_equal(lu, lu4)  # the queue schedule does not change any operation


def test_substitute_matches_reference(port, golden):
    x = port.substitute(golden.f_csr(), golden.lu, golden.b)
    assert rel_err(x, golden.x_subs) <= 1e-12


def test_gmres_matches_reference(port, golden):
    f = golden.f_csr()
    lu, _ = port.factorize(f)
    ok, its, x, _ = port.gmres(golden.a, f, lu, golden.b, golden.tol, golden.restart, 1000)
    assert ok == golden.gmres_ok
    assert abs(its - golden.gmres_iters) <= 1
    r = golden.b - port.matvec(golden.a, x)
    assert np.linalg.norm(r) <= golden.tol * 1.0001
