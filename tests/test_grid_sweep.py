"""Structured-grid line-pipeline sweeps (LLJBASH_ILU_OPT_GRID): the kernels for 7-point
(3-D) and 5-point (2-D) factors in natural order, a lane per grid line.

Every row performs the reference's operations in the reference's order, so the line
schedule must give results bit-identical to the block-local and level-ordered kernels
(FP64 substitution, and the FP32 path through identical mixed-precision GMRES runs), and
1e-12 against the CPU oracle.  Covered: grid shapes whose extents are and are not
multiples of the warp's lanes, 2-D grids, every warp shape (1, 4 or 8 lanes along y),
CTA shapes from one warp to eight, more blocks than resident CTAs (persistent CTAs taking
several blocks), and matrices the detection must reject (27-point stencils, ILU(1) fill,
a permuted 7-point matrix)."""
import numpy as np
import pytest

import oracle
from conftest import rel_err
from par_ilu0_cpp_gb300 import api
from par_ilu0_cpp_gb300 import generators as g
from par_ilu0_cpp_gb300 import sweep_timeline

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def port():
    oracle.build_port()
    return oracle.Port()


def solver(f, grid=1, wy=0, by=0, bz=0, block_rows=0, cluster=1):
    ilu = api.IluSolver()
    ilu.set_option(api.ILU_OPT_GRID, grid)
    ilu.set_option(api.ILU_OPT_GRID_CLUSTER, cluster)
    ilu.set_option(api.ILU_OPT_GRID_WARP_Y, wy)
    ilu.set_option(api.ILU_OPT_GRID_CTA_Y, by)
    ilu.set_option(api.ILU_OPT_GRID_CTA_Z, bz)
    ilu.set_option(api.ILU_OPT_BLOCK_ROWS, block_rows)
    ilu.set_matrix(f)
    assert ilu.setup() == 0, api.last_error()
    assert ilu.factorize() == 0, api.last_error()
    return ilu


SHAPES = [
    ("convdiff3d_32", lambda: g.convdiff3d(32)),
    ("convdiff3d_20x7x9", lambda: g.convdiff3d(20, 7, 9)),
    ("convdiff3d_70x5x6", lambda: g.convdiff3d(70, 5, 6)),
    ("convdiff3d_128x3x4", lambda: g.convdiff3d(128, 3, 4)),
    ("laplace2d_64", lambda: g.laplace2d(64)),
    ("laplace2d_45x80", lambda: g.laplace2d(45, 80)),
    ("laplace2d_256", lambda: g.laplace2d(256)),
]


@pytest.mark.parametrize("name,make", SHAPES, ids=[c[0] for c in SHAPES])
def test_grid_sweep_matches_other_schedules_and_oracle(port, name, make):
    a = make()
    f, _ = api.iluk_symbolic(a, 0)
    ilu = solver(f)
    info = ilu.info()
    assert info.grid_fp64 == 3 and info.grid_fp32 == 3, name  # forward and backward sweeps
    lu_ref, _ = port.factorize(f)
    assert rel_err(ilu.values(), lu_ref, floor=1e-300) <= 1e-12
    _, b = g.random_rhs(a, seed=3)
    x = ilu.substitute(b)
    assert rel_err(x, port.substitute(f, lu_ref, b)) <= 1e-12
    for kw in ({"grid": -1, "block_rows": -1}, {"grid": -1, "block_rows": 0}):
        other = solver(f, **kw)
        assert other.info().grid_fp64 == 0
        assert np.array_equal(other.substitute(b), x), kw
    assert np.array_equal(ilu.substitute(b), x)  # repeatable: faces and counters are reset


TUNINGS = [dict(wy=1, by=1, bz=1), dict(wy=4, by=3, bz=2), dict(wy=4), dict(wy=8, by=2, bz=4),
           dict(wy=1, by=8, bz=1), dict(wy=8, by=4, bz=2), dict(wy=8, by=1, bz=1), dict(wy=1, by=2, bz=4)]


TUNINGS = TUNINGS + [dict(k, cluster=0) for k in TUNINGS[:4]]


@pytest.mark.parametrize("kw", TUNINGS, ids=[str(k) for k in TUNINGS])
@pytest.mark.parametrize("make", [lambda: g.convdiff3d(40, 9, 11), lambda: g.laplace2d(100, 37),
                                  lambda: g.convdiff3d(9, 40, 33)],
                         ids=["convdiff3d_40x9x11", "laplace2d_100x37", "convdiff3d_9x40x33"])
def test_grid_warp_and_cta_shapes(make, kw):
    a = make()
    f, _ = api.iluk_symbolic(a, 0)
    ref = solver(f, grid=-1, block_rows=-1)
    ilu = solver(f, **kw)
    info = ilu.info()
    assert info.grid_fp64 == 3
    assert info.grid_warp_y * info.grid_warp_z == 32 and info.grid_cta_y * info.grid_cta_z <= 8
    _, b = g.random_rhs(a, seed=5)
    xr = ref.substitute(b)
    assert np.array_equal(ilu.substitute(b), xr)
    assert np.array_equal(ilu.substitute(b), xr)


def test_grid_more_blocks_than_resident_ctas():
    """One-warp CTAs over a grid of 64 x 70 lines: 192 blocks, more than the GPU's SMs, so
    persistent CTAs take several blocks each."""
    a = g.convdiff3d(5, 64, 70)
    f, _ = api.iluk_symbolic(a, 0)
    ref = solver(f, grid=-1, block_rows=-1)
    ilu = solver(f, wy=1, by=1, bz=1)
    assert ilu.info().grid_blocks == 192 and ilu.info().grid_fp64 == 3
    _, b = g.random_rhs(a, seed=9)
    assert np.array_equal(ilu.substitute(b), ref.substitute(b))


@pytest.mark.parametrize("make", [lambda: g.convdiff3d(48), lambda: g.laplace2d(160)],
                         ids=["convdiff3d_48", "laplace2d_160"])
def test_grid_gmres_identical_to_block_schedule(make):
    """Plain FP64 and mixed-precision GMRES with the grid sweeps take the same iterations
    and return the same solution as with the block-local / level-ordered sweeps."""
    a = make()
    f, _ = api.iluk_symbolic(a, 0)
    _, b = g.random_rhs(a, seed=7)
    tol = 1e-8 * float(np.linalg.norm(b))
    out = {}
    for grid in (1, -1, 0):
        ilu = solver(f, grid=grid)
        for mode in (0, 1):
            gm = api.Gmres(tol, 40, 1000)
            gm.set_preconditioner(ilu)
            gm.set_option(api.GMRES_OPT_MODE, mode)
            res = gm.solve(a, b)
            assert res.ok
            out[(grid, mode)] = (res.iterations, res.x)
    for mode in (0, 1):
        for grid in (1, 0):
            assert out[(grid, mode)][0] == out[(-1, mode)][0]
            assert np.array_equal(out[(grid, mode)][1], out[(-1, mode)][1])


@pytest.mark.parametrize("make", [lambda: g.convdiff3d(64), lambda: g.laplace2d(200)],
                         ids=["convdiff3d_64", "laplace2d_200"])
def test_grid_automatic_choice(make):
    """Automatic mode times each sweep of each precision against the block-local kernel at
    the first factorisation and keeps the faster: whatever it picks, the substitution is
    bit-identical to the block-local one, and the choice is reported per sweep."""
    a = make()
    f, _ = api.iluk_symbolic(a, 0)
    ref = solver(f, grid=-1)
    ilu = solver(f, grid=0)
    info = ilu.info()
    assert 0 <= info.grid_fp64 <= 3 and 0 <= info.grid_fp32 <= 3
    assert info.grid_nx > 0  # the pattern qualified
    _, b = g.random_rhs(a, seed=13)
    assert np.array_equal(ilu.substitute(b), ref.substitute(b))


def test_grid_detection_rejects_other_patterns():
    permuted = g.convdiff3d(12)
    n = permuted.n
    perm = np.random.default_rng(0).permutation(n)
    sp = permuted.to_scipy()[perm][:, perm].tocsr()
    sp.sort_indices()
    cases = {
        "lognormal27": api.iluk_symbolic(g.lognormal27(8, seed=1), 0)[0],
        "convdiff3d_ilu1": api.iluk_symbolic(g.convdiff3d(12), 1)[0],
        "permuted": g.Csr(n, sp.indptr, sp.indices, sp.data),
    }
    for name, f in cases.items():
        ilu = solver(f)
        assert ilu.info().grid_fp64 == 0, name


@pytest.mark.parametrize("make", [lambda: g.convdiff3d(40, 24, 70), lambda: g.laplace2d(90, 300)],
                         ids=["convdiff3d_40x24x70", "laplace2d_90x300"])
@pytest.mark.parametrize("cluster", [1, 3, 8])
def test_grid_clusters_match_plain_line_kernel(make, cluster):
    """Thread-block clusters along z (handoffs in distributed shared memory, the cluster's
    first CTA and the y-direction through L2) give the results of the plain line kernel and
    of the block-local kernel, including a last cluster that is only partly filled."""
    a = make()
    f, _ = api.iluk_symbolic(a, 0)
    ref = solver(f, grid=-1)
    plain = solver(f, cluster=0)
    clus = solver(f, cluster=cluster, bz=1)
    assert plain.info().grid_cluster == 0 and clus.info().grid_cluster > 1
    if cluster > 1:
        assert clus.info().grid_cluster <= cluster
        assert clus.info().grid_blocks > clus.info().grid_cluster
    _, b = g.random_rhs(a, seed=21)
    x = ref.substitute(b)
    assert np.array_equal(plain.substitute(b), x)
    assert np.array_equal(clus.substitute(b), x)
    assert np.array_equal(clus.substitute(b), x)


def test_sweep_timeline_records_every_block_without_changing_results():
    """LLJBASH_ILU_OPT_SWEEP_TIMELINE: every block of the last sweep of each kind has its
    start, SM and warp end stamps, in order, and the results stay bit-identical."""
    a = g.convdiff3d(40, 24, 70)
    f, _ = api.iluk_symbolic(a, 0)
    plain = solver(f)
    ilu = api.IluSolver()
    ilu.set_option(api.ILU_OPT_GRID, 1)
    ilu.set_option(api.ILU_OPT_SWEEP_TIMELINE, 1)
    ilu.set_matrix(f)
    assert ilu.setup() == 0 and ilu.factorize() == 0, api.last_error()
    _, b = g.random_rhs(a, seed=5)
    assert np.array_equal(ilu.substitute(b), plain.substitute(b))
    info = ilu.info()
    nw = info.grid_cta_y * info.grid_cta_z
    for upper in (False, True):
        tl = ilu.sweep_timeline(upper, False).astype(np.int64)
        assert tl.shape == (info.grid_blocks, api.LINE_TIMELINE_WORDS)
        start, ends = tl[:, 0], tl[:, 2:3 + nw]
        assert (start > 0).all() and (ends >= start[:, None]).all()
        assert (tl[:, 3 + nw:] == 0).all()
        assert (tl[:, 1] < 1024).all()
        s = sweep_timeline.summarize(tl.astype(np.uint64), info)
        assert s["blocks"] == info.grid_blocks and s["span_us"] > 0
    # timelines off: nothing to read
    with pytest.raises(RuntimeError):
        plain.sweep_timeline(False, False)


def test_one_cta_per_sm_gives_the_same_results():
    """LLJBASH_ILU_OPT_GRID_ONE_CTA_PER_SM pads the line kernels' shared memory so that
    no two CTAs share an SM (fewer clusters resident at once): same results."""
    a = g.convdiff3d(40, 24, 70)
    f, _ = api.iluk_symbolic(a, 0)
    base = solver(f)
    ilu = api.IluSolver()
    ilu.set_option(api.ILU_OPT_GRID, 1)
    ilu.set_option(api.ILU_OPT_GRID_ONE_CTA_PER_SM, 1)
    ilu.set_matrix(f)
    assert ilu.setup() == 0 and ilu.factorize() == 0, api.last_error()
    assert ilu.info().grid_fp64 == 3
    _, b = g.random_rhs(a, seed=8)
    assert np.array_equal(ilu.substitute(b), base.substitute(b))
    x1 = api.Gmres(1e-8, 30, 500)
    x1.set_preconditioner(ilu)
    x1.set_option(api.GMRES_OPT_MODE, 1)
    x2 = api.Gmres(1e-8, 30, 500)
    x2.set_preconditioner(base)
    x2.set_option(api.GMRES_OPT_MODE, 1)
    r1, r2 = x1.solve(a, b), x2.solve(a, b)
    assert r1.iterations == r2.iterations and np.array_equal(r1.x, r2.x)
