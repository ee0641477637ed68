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
