"""The diagonal recurrence of ILU(0) on full 7-point / 5-point stencils (oracle, CPU)
against the port of the reference's row elimination and against the reference's own
code (its build without contraction or fast-math, where it loads): the same factor
values, entry by entry, so a line-pipeline factorisation of such matrices (the sweep's
dependency structure, one division per step) computes the reference's factors."""
import platform

import numpy as np
import pytest

import oracle
from oracle.stencil_ilu0 import stencil_ilu0
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
    ("convdiff3d_12x10x9", lambda: g.convdiff3d(12, 10, 9), (12, 10, 9)),
    ("convdiff3d_3x3x5", lambda: g.convdiff3d(3, 3, 5), (3, 3, 5)),
    ("laplace2d_15x11", lambda: g.laplace2d(15, 11), (15, 11, 1)),
    ("laplace2d_4x2", lambda: g.laplace2d(4, 2), (4, 2, 1)),
]


@pytest.mark.parametrize("name,make,dims", CASES, ids=[c[0] for c in CASES])
def test_diagonal_recurrence_matches_row_elimination(port, name, make, dims):
    a = make()
    lu_port, _ = port.factorize(a)
    lu = stencil_ilu0(a, *dims)
    if platform.machine() in ("x86_64", "AMD64"):
        # no contraction of a*b - c on this host's build of the port: bit-exact
        assert np.array_equal(lu, lu_port), name
    else:
        np.testing.assert_allclose(lu, lu_port, rtol=1e-14, atol=0)
    # the strictly upper entries of U are A's
    rp, ci = a.row_ptr, a.col_idx
    rows = np.repeat(np.arange(a.n), np.diff(rp))
    upper = ci > rows
    assert np.array_equal(lu[upper], a.values[upper])


@pytest.mark.parametrize("name,make,dims", CASES, ids=[c[0] for c in CASES])
def test_diagonal_recurrence_matches_the_reference_build(ref, name, make, dims):
    a = make()
    lu_ref, _ = ref.factorize(a)
    assert np.array_equal(stencil_ilu0(a, *dims), lu_ref), name


def test_recurrence_rejects_other_shapes():
    a = g.convdiff3d(6)
    with pytest.raises(ValueError):
        stencil_ilu0(a, 6, 6, 5)  # wrong size
    with pytest.raises(ValueError):
        stencil_ilu0(g.convdiff3d(6, 2, 4), 6, 2, 4)  # ny = 2: more entries change
