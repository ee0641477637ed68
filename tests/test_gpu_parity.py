"""GPU parity: the CUDA path, called through the LLJBASH_* C ABI, against the
reference's own outputs (golden fixtures) and the CPU oracle on larger seeded inputs.

Tolerances (from the task's correctness bar):
* factors: 1e-12 relative per entry;
* substitution: 1e-12, relative per entry with a floor of 1e-3 * max|x| for entries
  near zero (the reference's sums may be reassociated by -ffast-math);
* GMRES: iteration count within +-1 of the reference, FP64 true residual <= tol.
"""
import numpy as np
import pytest

import oracle
from conftest import banded, csr_from_rows, ragged, rel_err
from par_ilu0_cpp_gb300 import api
from par_ilu0_cpp_gb300 import generators as g

pytestmark = pytest.mark.gpu


def factorize(f):
    ilu = api.IluSolver()
    ilu.set_matrix(f)
    assert ilu.setup() == 0, api.last_error()
    assert ilu.factorize() == 0, api.last_error()
    return ilu


def true_residual(a, b, x):
    return float(np.linalg.norm(b - g.spmv(a, x)))


@pytest.fixture(scope="module")
def port():
    oracle.build_port()
    return oracle.Port()


def test_golden_factors(golden):
    ilu = factorize(golden.f_csr())
    assert rel_err(ilu.values(), golden.lu, floor=1e-300) <= 1e-12
    an = ilu.analysis()
    assert np.array_equal(an["diag"], golden.diag)
    assert np.array_equal(an["etree_l"], golden.etree_l)
    assert np.array_equal(an["depth_u"], golden.level_u)
    info = ilu.info()
    assert info.levels_lower == golden.nlev[0] and info.breakdowns == 0


def test_golden_substitution(golden):
    ilu = factorize(golden.f_csr())
    x = ilu.substitute(golden.b)
    assert rel_err(x, golden.x_subs) <= 1e-12
    x2 = ilu.substitute(golden.b)  # sentinel state is restored between calls
    assert np.array_equal(x, x2)


def test_golden_gmres(golden):
    res, ilu, gm = api.ilu_gmres(golden.a, golden.b, lof=golden.lof, tol=golden.tol, restart=golden.restart,
                                 maxit=1000, relative=False)
    assert res.ok == golden.gmres_ok
    assert abs(res.iterations - golden.gmres_iters) <= 1, (res.iterations, golden.gmres_iters)
    assert true_residual(golden.a, golden.b, res.x) <= golden.tol * 1.0001
    assert res.report.converged == 1
    assert np.max(np.abs(res.x - golden.gmres_x)) <= 1e-6 * max(1.0, np.max(np.abs(golden.gmres_x)))


LARGE = [
    ("laplace2d_256", lambda: g.laplace2d(256), 0, 30),
    ("convdiff3d_32", lambda: g.convdiff3d(32), 0, 50),
    ("lognormal27_16_k1", lambda: g.lognormal27(16, seed=1), 1, 30),
    ("lognormal27_16_k2", lambda: g.lognormal27(16, seed=1), 2, 30),
]


@pytest.mark.parametrize("name,make,lof,m", LARGE, ids=[c[0] for c in LARGE])
def test_large_against_oracle(port, name, make, lof, m):
    a = make()
    f, _ = port.iluk_symbolic(a, lof)
    lu_ref, _ = port.factorize(f)
    ilu = factorize(f)
    assert rel_err(ilu.values(), lu_ref, floor=1e-300) <= 1e-12
    x_true, b = g.random_rhs(a, seed=5)
    xs = ilu.substitute(b)
    assert rel_err(xs, port.substitute(f, lu_ref, b)) <= 1e-12
    tol = 1e-8 * float(np.linalg.norm(b))
    ok, its, x_ref, _ = port.gmres(a, f, lu_ref, b, tol, m, 1000)
    gm = api.Gmres(tol, m, 1000)
    gm.set_preconditioner(ilu)
    res = gm.solve(a, b)
    assert res.ok and ok
    assert abs(res.iterations - its) <= 1, (res.iterations, its)
    assert true_residual(a, b, res.x) <= tol * 1.0001


# The benchmark configurations at full size: 128^3 7-point convection-diffusion with
# ILU(0) + GMRES(50) (the configuration the headline is measured on: FP64 blocks of
# 16,384 rows, FP32 clusters over 32,768-row blocks) and the 64^3 27-point lognormal
# operator with ILU(1) / ILU(2) + GMRES(30) (lane-group sweeps).  Factors and one FP64
# substitution against the oracle port to 1e-12, plain FP64 GMRES iterations within +-1
# of the port's, and the FP64 true residual of the plain and mixed-precision solves.
FULL = [
    ("convdiff3d_128_ilu0", lambda: g.convdiff3d(128), 0, 50),
    ("lognormal27_64_ilu1", lambda: g.lognormal27(64, seed=0), 1, 30),
    ("lognormal27_64_ilu2", lambda: g.lognormal27(64, seed=0), 2, 30),
]


@pytest.mark.parametrize("name,make,lof,m", FULL, ids=[c[0] for c in FULL])
def test_benchmark_configuration_against_oracle(port, name, make, lof, m):
    import os

    threads = os.cpu_count() or 1
    a = make()
    f, _ = api.iluk_symbolic(a, lof)  # bit-exact with the reference (CPU test)
    lu_ref, _ = port.factorize(f, nthreads=threads)
    ilu = factorize(f)
    assert rel_err(ilu.values(), lu_ref, floor=1e-300) <= 1e-12
    x_true, b = g.random_rhs(a, seed=0)
    assert rel_err(ilu.substitute(b), port.substitute(f, lu_ref, b)) <= 1e-12
    tol = 1e-8 * float(np.linalg.norm(b))
    ok, its, _, _ = port.gmres(a, f, lu_ref, b, tol, m, 1000, nthreads=threads)
    assert ok
    gm = api.Gmres(tol, m, 1000)
    gm.set_preconditioner(ilu)
    res = gm.solve(a, b)
    assert res.ok and abs(res.iterations - its) <= 1, (res.iterations, its)
    assert true_residual(a, b, res.x) <= tol * 1.0001
    mixed = api.Gmres(tol, m, 1000)
    mixed.set_preconditioner(ilu)
    mixed.set_option(api.GMRES_OPT_MODE, 1)
    rm = mixed.solve(a, b)
    assert rm.ok and true_residual(a, b, rm.x) <= tol * 1.0001
    print(f"{name}: iterations plain {res.iterations} (oracle {its}), mixed {rm.iterations}; forward error "
          f"plain {np.max(np.abs(res.x - x_true)):.2e}, mixed {np.max(np.abs(rm.x - x_true)):.2e}")


def test_modes_are_deterministic():
    a = g.convdiff3d(24)
    x_true, b = g.random_rhs(a, seed=2)
    tol = 1e-8 * float(np.linalg.norm(b))
    f, _ = api.iluk_symbolic(a, 0)
    ilu = factorize(f)
    xs = []
    for graph, profile in ((1, 0), (0, 0), (0, 1)):
        gm = api.Gmres(tol, 50, 1000)
        gm.set_preconditioner(ilu)
        gm.set_option(api.GMRES_OPT_USE_GRAPH, graph)
        gm.set_option(api.GMRES_OPT_PROFILE, profile)
        res = gm.solve(a, b)
        assert res.ok
        xs.append((res.iterations, res.x))
    assert xs[0][0] == xs[1][0] == xs[2][0]
    assert np.array_equal(xs[0][1], xs[1][1]) and np.array_equal(xs[0][1], xs[2][1])


@pytest.mark.parametrize("make", [lambda: g.laplace2d(128), lambda: g.convdiff3d(32),
                                  lambda: g.lognormal27(16, seed=4)])
def test_mixed_precision_reaches_fp64_tolerance(make):
    a = make()
    x_true, b = g.random_rhs(a, seed=9)
    res, ilu, gm = api.ilu_gmres(a, b, tol=1e-8, restart=40, maxit=1000, mode=1)
    r = true_residual(a, b, res.x)
    assert res.ok and res.report.converged == 1
    assert r <= 1e-8 * np.linalg.norm(b) * 1.0001
    assert res.report.residual <= 1e-8 * np.linalg.norm(b) * 1.0001
    fwd = np.max(np.abs(res.x - x_true)) / np.max(np.abs(x_true))
    assert fwd < 1e-4  # forward error stated for the record; bounded by conditioning


def test_unpreconditioned_gmres():
    a = g.laplace2d(16)
    x_true, b = g.random_rhs(a, seed=1)
    tol = 1e-8 * float(np.linalg.norm(b))
    gm = api.Gmres(tol, 60, 1000)
    res = gm.solve(a, b)
    assert res.ok
    assert true_residual(a, b, res.x) <= tol * 1.0001


def test_missing_diagonal_setup_code():
    ilu = api.IluSolver()
    ilu.set_matrix(g.Csr(2, [0, 1, 2], [1, 1], [1.0, 2.0]))
    assert ilu.setup() == -2


def test_zero_pivot_reported():
    a = g.Csr(2, [0, 2, 4], [0, 1, 0, 1], [0.0, 1.0, 1.0, 1.0])
    ilu = api.IluSolver()
    ilu.set_matrix(a)
    assert ilu.setup() == 0
    assert ilu.factorize() == 0  # the reference returns success on a zero pivot too
    info = ilu.info()
    assert info.breakdowns >= 1 and info.first_breakdown == 0


def test_nan_input_fails_cleanly():
    a = g.laplace2d(8)
    vals = a.values.copy()
    vals[5] = np.nan
    an = g.Csr(a.n, a.row_ptr, a.col_idx, vals)
    b = np.ones(a.n)
    res, ilu, gm = api.ilu_gmres(an, b, tol=1e-8, restart=10, maxit=50)
    assert not res.ok


def test_device_resident_entry_points_match_host_path():
    torch = pytest.importorskip("torch")
    a = g.convdiff3d(20)
    x_true, b = g.random_rhs(a, seed=3)
    tol = 1e-8 * float(np.linalg.norm(b))
    f, _ = api.iluk_symbolic(a, 0)
    for mode in (0, 1):
        ilu = api.IluSolver()
        ilu.set_matrix(f)
        assert ilu.setup() == 0
        ilu.set_option(api.ILU_OPT_COPY_BACK, 0)
        gm = api.Gmres(tol, 30, 1000)
        gm.set_preconditioner(ilu)
        gm.set_option(api.GMRES_OPT_MODE, mode)
        d = {k: torch.from_numpy(v).cuda() for k, v in
             (("rp", a.row_ptr), ("ci", a.col_idx), ("av", a.values), ("fv", f.values), ("b", b))}
        dx = torch.zeros(a.n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        assert ilu.factorize_device(d["fv"].data_ptr()) == 0
        ok, its = gm.solve_device(a.n, d["rp"].data_ptr(), d["ci"].data_ptr(), d["av"].data_ptr(), d["b"].data_ptr(),
                                  dx.data_ptr())
        assert ok
        x_dev = dx.cpu().numpy()
        res_host, _, _ = api.ilu_gmres(a, b, tol=tol, restart=30, maxit=1000, mode=mode, relative=False)
        assert its == res_host.iterations
        assert np.array_equal(x_dev, res_host.x)


@pytest.mark.parametrize("block_rows", [1, 7, 64, 1000])
def test_block_partition_does_not_change_results(golden, block_rows):
    """Any block size gives the same operations in the same order: identical results."""
    ref = factorize(golden.f_csr())
    x_ref = ref.substitute(golden.b)
    ilu = api.IluSolver()
    ilu.set_option(api.ILU_OPT_GRID, -1)  # the block-local kernel, also on stencil matrices
    ilu.set_option(api.ILU_OPT_BLOCK_ROWS, block_rows)
    ilu.set_matrix(golden.f_csr())
    assert ilu.setup() == 0
    assert ilu.factorize() == 0
    x = ilu.substitute(golden.b)
    assert np.array_equal(x, x_ref)
    gm = api.Gmres(golden.tol, golden.restart, 1000)
    gm.set_preconditioner(ilu)
    res = gm.solve(golden.a, golden.b)
    assert res.ok and abs(res.iterations - golden.gmres_iters) <= 1


ROW_LANE_CASES = [
    # (name, matrix, fill level, automatic lanes per row of L)
    ("lognormal27_12_k0", lambda: g.lognormal27(12, seed=3), 0, 2),
    ("lognormal27_12_k1", lambda: g.lognormal27(12, seed=3), 1, 4),
    ("lognormal27_12_k2", lambda: g.lognormal27(12, seed=3), 2, 8),
    ("banded_100", lambda: banded(1500, 100, 4), 0, 16),
    ("banded_200", lambda: banded(1200, 200, 5), 0, 32),
    ("banded_300", lambda: banded(900, 300, 6), 0, 1),
]


def _setup_lanes(f, lanes):
    ilu = api.IluSolver()
    ilu.set_option(api.ILU_OPT_ROW_LANES, lanes)
    ilu.set_matrix(f)
    assert ilu.setup() == 0, api.last_error()
    assert ilu.factorize() == 0, api.last_error()
    return ilu


@pytest.mark.parametrize("name,make,lof,lanes", ROW_LANE_CASES, ids=[c[0] for c in ROW_LANE_CASES])
def test_row_lanes_do_not_change_results(port, name, make, lof, lanes):
    """Rows spread over a group of lanes are consumed in the same entry order as with one
    lane per row: identical results in FP64 and in the mixed-precision solve."""
    a = make()
    f, _ = port.iluk_symbolic(a, lof) if lof else (a, None)
    _, b = g.random_rhs(a, seed=7)
    tol = 1e-8 * float(np.linalg.norm(b))
    auto = _setup_lanes(f, 0)
    assert auto.info().row_lanes_lower == lanes and auto.info().row_lanes_upper == lanes
    x_auto = auto.substitute(b)
    lu_ref, _ = port.factorize(f)
    assert rel_err(x_auto, port.substitute(f, lu_ref, b)) <= 1e-12
    results = {}
    for req in (1, 0, 2, 4, 8, 16, 32):
        ilu = auto if req == 0 else _setup_lanes(f, req)
        if req > 1:
            assert ilu.info().row_lanes_lower == (1 if lanes == 1 else max(lanes, req))
        assert np.array_equal(ilu.substitute(b), x_auto), req
        gm = api.Gmres(tol, 30, 1000)
        gm.set_preconditioner(ilu)
        gm.set_option(api.GMRES_OPT_MODE, 1)
        res = gm.solve(a, b)
        assert res.ok and true_residual(a, b, res.x) <= tol * 1.0001
        results[req] = (res.iterations, res.x)
    for req, (its, x) in results.items():
        assert its == results[1][0] and np.array_equal(x, results[1][1]), req


def test_row_lanes_option_checked():
    ilu = api.IluSolver()
    for bad in (3, 64, -1, 2.5):
        with pytest.raises(RuntimeError):
            ilu.set_option(api.ILU_OPT_ROW_LANES, bad)


def test_wait_limit_gives_up_and_solver_recovers(port):
    """A device wait that reaches its limit gives up without faulting: the call reports
    the timeout, and with the default limit back the same solver factorises and solves
    correctly (a 1 us limit cuts short the real waits of a long dependency chain; the
    sweeps get a warp per task, so tasks far down the 1,500-level chain wait long)."""
    a = banded(1500, 100, 4)
    _, b = g.random_rhs(a, seed=8)
    lu_ref, _ = port.factorize(a)
    x_ref = port.substitute(a, lu_ref, b)
    ilu = api.IluSolver()
    ilu.set_option(api.ILU_OPT_SOLVE_WARPS, 1024)
    ilu.set_matrix(a)
    assert ilu.setup() == 0, api.last_error()
    ilu.set_option(api.ILU_OPT_WAIT_LIMIT_US, 1)
    assert ilu.factorize() == -1
    assert "timed out" in api.last_error()
    ilu.set_option(api.ILU_OPT_WAIT_LIMIT_US, 0)
    assert ilu.factorize() == 0, api.last_error()
    assert rel_err(ilu.values(), lu_ref, floor=1e-300) <= 1e-12
    x = ilu.substitute(b)
    assert rel_err(x, x_ref) <= 1e-12
    ilu.set_option(api.ILU_OPT_WAIT_LIMIT_US, 1)
    with pytest.raises(RuntimeError, match="timed out"):
        ilu.substitute(b)
    ilu.set_option(api.ILU_OPT_WAIT_LIMIT_US, 0)
    assert np.array_equal(ilu.substitute(b), x)
    with pytest.raises(RuntimeError):
        ilu.set_option(api.ILU_OPT_WAIT_LIMIT_US, -5)


@pytest.mark.parametrize("planes", [0.5, 1, 2])
def test_cluster_halos_two_positions_back(planes):
    """Half-plane blocks read the block two positions back (the k-1 neighbours) and the
    one before (the j-1 row): with clusters both are pushed into the consumer's halo.
    Every block size gives the level-ordered kernel's results bit for bit, in FP64
    substitution and in the mixed-precision solve."""
    nx = 24
    a = g.convdiff3d(nx)
    f, _ = api.iluk_symbolic(a, 0)
    _, b = g.random_rhs(a, seed=11)
    tol = 1e-8 * float(np.linalg.norm(b))

    def run(block_rows):
        ilu = api.IluSolver()
        ilu.set_option(api.ILU_OPT_GRID, -1)  # block-local / level-ordered kernels
        ilu.set_option(api.ILU_OPT_BLOCK_ROWS, block_rows)
        ilu.set_matrix(f)
        assert ilu.setup() == 0, api.last_error()
        assert ilu.factorize() == 0, api.last_error()
        x = ilu.substitute(b)
        gm = api.Gmres(tol, 30, 1000)
        gm.set_preconditioner(ilu)
        gm.set_option(api.GMRES_OPT_MODE, 1)
        res = gm.solve(a, b)
        assert res.ok
        return ilu.info(), x, res

    _, x_ref, res_ref = run(-1)
    info, x, res = run(int(planes * nx * nx))
    assert info.block_rows_fp64 == int(planes * nx * nx) and info.block_cluster_fp64 in (8, 16)
    assert np.array_equal(x, x_ref)
    assert res.iterations == res_ref.iterations and np.array_equal(res.x, res_ref.x)


def test_single_row_and_diagonal_only():
    one = csr_from_rows(1, [[0]], [[4.0]])
    ilu = factorize(one)
    assert ilu.values()[0] == 4.0
    assert ilu.substitute(np.array([2.0]))[0] == 0.5
    res, _, _ = api.ilu_gmres(one, np.array([2.0]), tol=1e-12, restart=5, maxit=10)
    assert res.ok and abs(res.x[0] - 0.5) <= 1e-15
    n = 1000
    d = np.linspace(1.0, 3.0, n)
    diag = csr_from_rows(n, [[i] for i in range(n)], [[d[i]] for i in range(n)])
    ilu = factorize(diag)
    assert np.array_equal(ilu.values(), d)
    b = np.arange(n, dtype=np.float64) + 1.0
    assert np.array_equal(ilu.substitute(b), b / d)
    res, _, _ = api.ilu_gmres(diag, b, tol=1e-10, restart=10, maxit=50)
    assert res.ok and res.iterations <= 1
    assert np.max(np.abs(res.x - b / d)) <= 1e-12 * np.max(np.abs(b / d))


def test_empty_matrix():
    empty = g.Csr(0, np.zeros(1, np.int64), np.zeros(0, np.int64), np.zeros(0))
    ilu = api.IluSolver()
    ilu.set_matrix(empty)
    assert ilu.setup() == 0, api.last_error()
    assert ilu.factorize() == 0, api.last_error()
    assert ilu.substitute(np.zeros(0)).size == 0


@pytest.mark.parametrize("lof", [0, 1])
def test_ragged_rows_against_oracle(port, lof):
    """Rows of 0 .. 40 off-diagonal entries at random columns: factors and substitution
    against the oracle, the level-ordered and block-local schedules (with clusters) and
    one lane per row against lane groups bit for bit, and the mixed-precision solve."""
    a = ragged(3000, 40, seed=12 + lof)
    f, _ = port.iluk_symbolic(a, lof)
    lu_ref, _ = port.factorize(f)
    _, b = g.random_rhs(a, seed=13)
    x_ref = port.substitute(f, lu_ref, b)
    results = []
    for opts in ({}, {api.ILU_OPT_ROW_LANES: 1}, {api.ILU_OPT_BLOCK_ROWS: 256}, {api.ILU_OPT_BLOCK_ROWS: 1000}):
        ilu = api.IluSolver()
        for k, v in opts.items():
            ilu.set_option(k, v)
        ilu.set_matrix(f)
        assert ilu.setup() == 0, api.last_error()
        assert ilu.factorize() == 0, api.last_error()
        assert rel_err(ilu.values(), lu_ref, floor=1e-300) <= 1e-12
        x = ilu.substitute(b)
        assert rel_err(x, x_ref) <= 1e-12
        results.append(x)
    for x in results[1:]:
        assert np.array_equal(x, results[0])
    tol = 1e-8 * float(np.linalg.norm(b))
    res, _, _ = api.ilu_gmres(a, b, lof=lof, tol=tol, restart=30, maxit=1000, mode=1, relative=False)
    assert res.ok and true_residual(a, b, res.x) <= tol * 1.0001


LEVELSYNC_CASES = [
    ("convdiff3d_24", lambda: g.convdiff3d(24), 0),
    ("lognormal27_12_k2", lambda: g.lognormal27(12, seed=3), 2),
    ("ragged_3000", lambda: ragged(3000, 40, seed=17), 0),
    ("banded_150", lambda: banded(1200, 150, 6), 0),
]


@pytest.mark.parametrize("name,make,lof", LEVELSYNC_CASES, ids=[c[0] for c in LEVELSYNC_CASES])
def test_level_synchronous_schedule(port, name, make, lof):
    """The level-synchronous sweeps (LLJBASH_ILU_OPT_BLOCK_ROWS = -2: one grid barrier
    per level, no waits) give the level-ordered kernel's results bit for bit, in FP64
    substitution and in the mixed-precision solve, and 1e-12 against the oracle."""
    a = make()
    f, _ = port.iluk_symbolic(a, lof) if lof else (a, None)
    _, b = g.random_rhs(a, seed=21)
    tol = 1e-8 * float(np.linalg.norm(b))
    out = {}
    for sched in (-1, -2):
        ilu = api.IluSolver()
        ilu.set_option(api.ILU_OPT_BLOCK_ROWS, sched)
        ilu.set_matrix(f)
        assert ilu.setup() == 0, api.last_error()
        assert ilu.factorize() == 0, api.last_error()
        x = ilu.substitute(b)
        gm = api.Gmres(tol, 30, 1000)
        gm.set_preconditioner(ilu)
        gm.set_option(api.GMRES_OPT_MODE, 1)
        res = gm.solve(a, b)
        assert res.ok
        out[sched] = (x, res.iterations, res.x)
    assert np.array_equal(out[-2][0], out[-1][0])
    assert out[-2][1] == out[-1][1] and np.array_equal(out[-2][2], out[-1][2])
    lu_ref, _ = port.factorize(f)
    assert rel_err(out[-2][0], port.substitute(f, lu_ref, b)) <= 1e-12


def test_level_synchronous_barrier_recovers_after_give_up():
    """A grid-barrier wait that reaches a 1 us limit gives up and reports the timeout
    (the barrier words are then reset); with the default limit the next solve is right."""
    a = banded(1500, 60, 9)
    _, b = g.random_rhs(a, seed=3)
    ilu = api.IluSolver()
    ilu.set_option(api.ILU_OPT_BLOCK_ROWS, -2)
    ilu.set_matrix(a)
    assert ilu.setup() == 0, api.last_error()
    assert ilu.factorize() == 0, api.last_error()
    x_ref = ilu.substitute(b)
    ilu.set_option(api.ILU_OPT_WAIT_LIMIT_US, 1)
    try:
        ilu.substitute(b)
    except RuntimeError as e:
        assert "timed out" in str(e)
    ilu.set_option(api.ILU_OPT_WAIT_LIMIT_US, 0)
    for _ in range(2):
        assert np.array_equal(ilu.substitute(b), x_ref)


LANE_FACTOR_CASES = [
    ("convdiff3d_32", lambda: g.convdiff3d(32), 0),
    ("laplace2d_128_ilu2", lambda: g.laplace2d(128), 2),
    ("ragged_4000", lambda: ragged(4000, 6, seed=31), 0),
    ("ragged_2000_ilu1", lambda: ragged(2000, 3, seed=32), 1),
    ("banded_5", lambda: banded(3000, 5, 7), 0),
]


@pytest.mark.parametrize("name,make,lof", LANE_FACTOR_CASES, ids=[c[0] for c in LANE_FACTOR_CASES])
def test_lane_factorisation_matches_warp_kernel(port, name, make, lof):
    """The lane-per-row factorisation (LLJBASH_ILU_OPT_FACTOR_KERNEL = 2) gives the
    warp-per-row kernel's factors bit for bit, with and without a diagonal shift, and the
    oracle's to 1e-12."""
    a = make()
    f, _ = port.iluk_symbolic(a, lof) if lof else (a, None)
    shift = np.random.default_rng(5).uniform(0.0, 0.5, a.n)
    vals = {}
    for kern in (1, 2):
        ilu = api.IluSolver()
        ilu.set_option(api.ILU_OPT_FACTOR_KERNEL, kern)
        ilu.set_matrix(f)
        assert ilu.setup() == 0, api.last_error()
        assert ilu.info().factor_lane == (1 if kern == 2 else 0)
        assert ilu.factorize() == 0, api.last_error()
        plain = ilu.values()
        ilu.set_values(f.values)
        ilu.set_shift(shift)
        assert ilu.factorize() == 0, api.last_error()
        vals[kern] = (plain, ilu.values())
    assert np.array_equal(vals[1][0], vals[2][0]) and np.array_equal(vals[1][1], vals[2][1])
    lu_ref, _ = port.factorize(f)
    assert rel_err(vals[2][0], lu_ref, floor=1e-300) <= 1e-12


def test_lane_factorisation_zero_pivot_and_recovery():
    """A zero pivot is reported as with the warp kernel; a wait cut short by a 1 us limit
    reports the timeout and the next factorisation is right."""
    z = g.Csr(2, [0, 2, 4], [0, 1, 0, 1], [0.0, 1.0, 1.0, 1.0])
    ilu = api.IluSolver()
    ilu.set_option(api.ILU_OPT_FACTOR_KERNEL, 2)
    ilu.set_matrix(z)
    assert ilu.setup() == 0 and ilu.info().factor_lane == 1
    assert ilu.factorize() == 0
    assert ilu.info().breakdowns >= 1 and ilu.info().first_breakdown == 0
    a = banded(4000, 6, 3)
    ilu = api.IluSolver()
    ilu.set_option(api.ILU_OPT_FACTOR_KERNEL, 2)
    ilu.set_matrix(a)
    assert ilu.setup() == 0, api.last_error()
    assert ilu.factorize() == 0
    ref = ilu.values()
    ilu.set_values(a.values)
    ilu.set_option(api.ILU_OPT_WAIT_LIMIT_US, 1)
    rc = ilu.factorize()
    assert rc in (0, -1)
    if rc == -1:
        assert "timed out" in api.last_error()
    ilu.set_option(api.ILU_OPT_WAIT_LIMIT_US, 0)
    ilu.set_values(a.values)
    assert ilu.factorize() == 0, api.last_error()
    assert np.array_equal(ilu.values(), ref)
