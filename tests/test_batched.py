"""Batched persistent solver: many uneven systems x right-hand sides in one launch.
Every answer is judged by its FP64 true residual (recomputed here) against the
relative tolerance, and by its forward error against the seeded x_true."""
import numpy as np
import pytest

from par_ilu0_cpp_gb300 import api
from par_ilu0_cpp_gb300 import generators as g

pytestmark = pytest.mark.gpu


def _batch(sides, seed, nrhs):
    rng = np.random.default_rng(seed)
    systems = [g.variable_poisson2d(int(s), int(s), sigma=1.0, seed=int(rng.integers(1 << 30))) for s in sides]
    xs, bs = [], []
    for k, a in enumerate(systems):
        x, b = g.random_rhs(a, seed=seed * 1000 + k, nrhs=nrhs)
        x = np.atleast_2d(x)
        b = np.atleast_2d(b)
        xs.append(x)
        bs.append(b)
    return systems, xs, bs


def _check(systems, xs, bs, out, nrhs, rtol=1e-8):
    x = out["x"]
    pos = 0
    for k, a in enumerate(systems):
        for r in range(nrhs):
            xr = x[pos:pos + a.n]
            b = bs[k][r]
            res = np.linalg.norm(b - g.spmv(a, xr)) / np.linalg.norm(b)
            assert res <= rtol * 1.0001, (k, r, res)
            assert np.max(np.abs(xr - xs[k][r])) < 1e-4
            pos += a.n
    assert out["converged"].all()


def test_batched_uneven_systems_converge():
    sides = [1, 2, 5, 17, 33, 8, 40, 23]
    systems, xs, bs = _batch(sides, 3, nrhs=3)
    bsol = api.BatchSolver(systems, nrhs=3, restart=30)
    out = bsol.solve(np.concatenate([b.ravel() for b in bs]))
    _check(systems, xs, bs, out, 3)
    assert (out["iterations"][3:] > 0).all()


def test_batched_autotune_and_repeat_are_consistent():
    sides = list(range(20, 60, 3))
    systems, xs, bs = _batch(sides, 5, nrhs=4)
    bsol = api.BatchSolver(systems, nrhs=4, restart=30)
    cps, lf = bsol.autotune()
    assert cps in (1, 2)
    trials = bsol.trials()
    assert {t["rhs_per_cta"] for t in trials} == {1, 4}  # 16 is wider than 4 right-hand sides need
    assert all(t["ms"] > 0 for t in trials)
    # the trials iterate on right-hand sides of their own (the caller's come with solve())
    assert all(t["ms"] > 0.05 for t in trials)
    best = min(trials, key=lambda t: t["ms"])
    assert bsol.shape() == (best["ctas_per_sm"], best["largest_first"], best["rhs_per_cta"])
    rhs = np.concatenate([b.ravel() for b in bs])
    out1 = bsol.solve(rhs)
    out2 = bsol.solve(rhs)
    _check(systems, xs, bs, out1, 4)
    assert np.array_equal(out1["iterations"], out2["iterations"])
    assert np.array_equal(out1["x"], out2["x"])


def test_batched_with_learned_shift_model():
    sides = [24, 31, 45]
    systems, xs, bs = _batch(sides, 7, nrhs=2)
    bsol = api.BatchSolver(systems, nrhs=2, restart=30)
    p = np.zeros(369, dtype=np.float32)
    p[368] = np.log(np.expm1(0.02))  # constant relative shift 0.02
    bsol.set_shift_model(p)
    out = bsol.solve(np.concatenate([b.ravel() for b in bs]))
    _check(systems, xs, bs, out, 2)


def test_batched_matches_single_solver_iterations_roughly():
    """Same preconditioner and Krylov method as the single-system mixed solver: the
    iteration counts agree within a few (different reduction orders)."""
    a = g.variable_poisson2d(48, 48, seed=11)
    x, b = g.random_rhs(a, seed=2)
    bsol = api.BatchSolver([a], nrhs=1, restart=30)
    out = bsol.solve(b)
    res, _, _ = api.ilu_gmres(a, b, restart=30, mode=1)
    assert abs(int(out["iterations"][0]) - res.iterations) <= 3


@pytest.mark.parametrize("rhs_per_cta", [1, 4, 16])
def test_batched_rhs_groups(rhs_per_cta):
    """Right-hand sides solved in lockstep groups of 1, 4 or 16 per CTA (7 per system: the
    last group of a system is partly empty): every answer meets the FP64 tolerance, and
    each right-hand side takes nearly the iterations it takes alone (the reductions
    differ in order only)."""
    sides = [9, 30, 47, 16, 52, 3]
    systems, xs, bs = _batch(sides, 17, nrhs=7)
    rhs = np.concatenate([b.ravel() for b in bs])
    ref = api.BatchSolver(systems, nrhs=7, restart=20)
    ref.set_shape(1, True, 1)
    out_ref = ref.solve(rhs)
    bsol = api.BatchSolver(systems, nrhs=7, restart=20)
    bsol.set_shape(2, True, rhs_per_cta)
    assert bsol.shape() == (2, True, rhs_per_cta)
    out = bsol.solve(rhs)
    _check(systems, xs, bs, out, 7)
    assert np.max(np.abs(out["iterations"].astype(int) - out_ref["iterations"].astype(int))) <= 3


def test_batched_shape_is_checked():
    systems, _, _ = _batch([10, 12], 19, nrhs=2)
    bsol = api.BatchSolver(systems, nrhs=2)
    for bad in ((3, True, 1), (1, True, 2), (0, False, 4)):
        with pytest.raises(RuntimeError):
            bsol.set_shape(*bad)
