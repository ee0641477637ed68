"""Learned per-row diagonal shift for ILU(0): data generation, labels, GPU training,
evaluation and the model file.

Labels are found by the method itself: for every training matrix the solver is run
(ILU(0) with FP32 factors + GMRES(40) in FP32 cycles with FP64 refinement, tol 1e-8,
at most 400 iterations) for each member of a two-parameter family of per-row shifts

    y_i(alpha, beta) = alpha * max(0, 1 - r_i) + beta,      shift_i = sign(a_ii) y_i s_i

(r_i = |a_ii| / s_i the diagonal dominance ratio, s_i = sum_j!=i |a_ij|), and the best
member gives every row its target y_i: among members that converge, the fewest GMRES
iterations; if none converges, the smallest final FP64 relative residual (so that the
matrices on which restarted GMRES stagnates, most of the stress set, still give a
signal); ties go to the smaller shift, plain ILU first.  The MLP (4 features -> 16 -> 16 -> 1, csrc/mlp.cuh) is then fitted
to (features, y) by the library's own GPU kernels (forward, backward, Adam).  At run
time the model's inference runs in the factorisation pre-pass; plain ILU is the
fallback on a pivot breakdown (inside the library) and when the shifted solve does not
converge (``solve``).  ``evaluate`` compares iteration counts with and without the
model on held-out matrices; the min_shift gate stored with the model is chosen on the
training matrices so that the model is never applied where it did not beat plain ILU
there.

    python -m par_ilu0_cpp_gb300.learned_shift train --n-train 2000 --out <model.json>
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

from . import api
from . import generators as g

PKG = os.path.dirname(os.path.abspath(__file__))
DEFAULT_MODEL = os.path.join(PKG, "shift_model.json")
ALPHAS = (0.0, 1.0, 2.0)
BETAS = (0.0, 0.05, 0.1, 0.3, 1.0)
RESTART = 40
LABEL_MAXIT = 400


def dominance(a: g.Csr):
    rows = np.repeat(np.arange(a.n), np.diff(a.row_ptr))
    isdiag = a.col_idx == rows
    d = np.zeros(a.n)
    d[rows[isdiag]] = a.values[isdiag]
    s = np.bincount(rows[~isdiag], weights=np.abs(a.values[~isdiag]), minlength=a.n)
    r = np.where(s > 0, np.abs(d) / np.where(s > 0, s, 1.0), 4.0)
    return d, s, np.minimum(r, 4.0)


def family(a: g.Csr, alpha: float, beta: float):
    """Relative shifts y and absolute diagonal shifts of the (alpha, beta) member."""
    d, s, r = dominance(a)
    y = alpha * np.maximum(0.0, 1.0 - r) + beta
    return y, np.where(d < 0, -1.0, 1.0) * y * s


class Solver:
    """ILU(0) (FP32 factors) + GMRES(m) (mixed precision) on one pattern, reusable."""

    def __init__(self, a: g.Csr, restart: int = RESTART, maxit: int = 1000, rtol: float = 1e-8):
        self.a = a
        self.f, _ = api.iluk_symbolic(a, 0)
        self.ilu = api.IluSolver()
        self.ilu.set_option(api.ILU_OPT_COPY_BACK, 0)
        if a.n <= 24576:
            # small systems: one CTA solves the whole system level by level in shared memory
            self.ilu.set_option(api.ILU_OPT_BLOCK_ROWS, a.n)
        self.ilu.set_matrix(self.f)
        if self.ilu.setup() != 0:
            raise RuntimeError(api.last_error())
        self.analysis = self.ilu.analysis()
        self.nlev = self.ilu.info().levels_lower
        self.rtol = rtol
        self.gm = api.Gmres(1.0, restart, maxit)
        self.gm.set_preconditioner(self.ilu)
        self.gm.set_option(api.GMRES_OPT_MODE, 1)
        self.gm.set_option(api.GMRES_OPT_KEEP_MATRIX, 1)

    def solve(self, b, shift=None, model=None, min_shift=0.0, maxit=None, fallback=True):
        """Returns dict(iterations, converged, residual, shift_applied, fell_back, x)."""
        self.ilu.set_shift_model(model, min_shift) if model is not None else self.ilu.set_shift_model(None)
        self.ilu.set_shift(shift)
        self.ilu.set_values(self.f.values)
        rc = self.ilu.factorize()
        applied = bool(self.ilu.info().shift_applied)
        if rc != 0:
            raise RuntimeError(api.last_error())
        p = self.gm.params
        p.tolerance = self.rtol * float(np.linalg.norm(b))
        p.max_iterations = maxit if maxit is not None else 1000
        res = self.gm.solve(self.a, b)
        out = dict(iterations=res.iterations, converged=bool(res.ok and res.report.converged),
                   residual=res.report.residual, shift_applied=applied, fell_back=False, x=res.x)
        if fallback and applied and not out["converged"]:
            plain = self.solve(b, None, None, maxit=maxit, fallback=False)
            plain["fell_back"] = True
            plain["iterations_shifted"] = out["iterations"]
            return plain
        return out


class PolicySolver(Solver):
    """Learned shift with the per-matrix decision rule: the first solve runs the shifted
    and the plain factors and keeps the one with fewer iterations (plain on ties, on
    breakdown and on non-convergence); later solves of the same matrix reuse it."""

    def __init__(self, a: g.Csr, params, min_shift: float = 0.0, **kw):
        super().__init__(a, **kw)
        self.params = params
        self.min_shift = min_shift
        self.use_shift = None
        self.first = None

    def solve_policy(self, b, maxit=None):
        if self.use_shift is None:
            learned = self.solve(b, model=self.params, min_shift=self.min_shift, maxit=maxit, fallback=False)
            plain = self.solve(b, maxit=maxit)
            self.use_shift = bool(learned["shift_applied"] and learned["converged"]
                                  and learned["iterations"] < plain["iterations"])
            self.first = dict(learned=learned["iterations"], plain=plain["iterations"],
                              learned_converged=learned["converged"], plain_converged=plain["converged"])
            return learned if self.use_shift else plain
        if self.use_shift:
            return self.solve(b, model=self.params, min_shift=self.min_shift, maxit=maxit)
        return self.solve(b, maxit=maxit)


def make_training_set(n_train: int, seed: int, lo: int = 32, hi: int = 128):
    rng = np.random.default_rng(seed)
    sides = rng.integers(lo, hi + 1, size=n_train)
    seeds = rng.integers(0, 1 << 31, size=n_train)
    return [(int(s), int(sd)) for s, sd in zip(sides, seeds)]


def label_matrix(a: g.Csr, b, solver: Solver | None = None):
    """Best (alpha, beta) by GMRES iterations; returns (y_targets, record)."""
    solver = solver or Solver(a)
    best = None
    trials = []
    for alpha in ALPHAS:
        for beta in BETAS:
            if alpha == 0.0 and beta == 0.0:
                y, shift = np.zeros(a.n), None
            else:
                y, shift = family(a, alpha, beta)
            r = solver.solve(b, shift=shift, maxit=LABEL_MAXIT, fallback=False)
            its = r["iterations"] if r["converged"] else LABEL_MAXIT + 1
            trials.append((alpha, beta, its))
            key = (its, float(np.mean(y)))
            if best is None or key < best[0]:
                best = (key, alpha, beta, y)
    return best[3].astype(np.float32), dict(alpha=best[1], beta=best[2], its=best[0][0], trials=trials)


def combos():
    return [(al, be) for al in ALPHAS for be in BETAS]


def build_dataset(specs, log=None, chunk: int = 200):
    """Features and labels for the matrices of `specs`.  The label search runs every
    (matrix, shift-family member) pair as one system of the batched persistent solver
    (GMRES iterates on A, the factorisation sees A + diag(shift)), `chunk` matrices per
    launch."""
    Xs, Ys, recs = [], [], []
    cmb = combos()
    t0 = time.time()
    for c0 in range(0, len(specs), chunk):
        part = specs[c0:c0 + chunk]
        mats, rhs, fvals, systems, ys = [], [], [], [], []
        for side, seed in part:
            a = g.cdr2d(side, seed=seed)
            _, b = g.random_rhs(a, seed=seed + 1)
            mats.append(a)
            rows = np.repeat(np.arange(a.n), np.diff(a.row_ptr))
            isdiag = a.col_idx == rows
            yk = []
            for alpha, beta in cmb:
                y, shift = family(a, alpha, beta)
                fv = a.values.copy()
                fv[isdiag] += shift[rows[isdiag]]
                systems.append(a)
                fvals.append(fv)
                rhs.append(b)
                yk.append(y)
            ys.append(yk)
        bs = api.BatchSolver(systems, nrhs=1, restart=RESTART, maxit=LABEL_MAXIT, factor_values=fvals)
        out = bs.solve(np.concatenate(rhs))
        bs.close()
        for k, (side, seed) in enumerate(part):
            a = mats[k]
            its, keys = [], []
            nb = float(np.linalg.norm(rhs[k * len(cmb)]))
            for j in range(len(cmb)):
                q = k * len(cmb) + j
                conv = bool(out["converged"][q])
                it = int(out["iterations"][q]) if conv else LABEL_MAXIT + 1
                rel = float(out["residual"][q]) / nb if nb > 0 else 0.0
                rel = rel if np.isfinite(rel) and rel >= 0 else np.inf
                its.append(it)
                keys.append((0, it, 0.0) if conv else (1, 0, rel))
            best = min(range(len(cmb)), key=lambda j: (keys[j], float(np.mean(ys[k][j]))))
            f, _ = api.iluk_symbolic(a, 0)
            an = api.analyze_pattern(f)
            Xs.append(api.shift_features(f, an["depth_l"], int(an["nlev"][0])))
            Ys.append(ys[k][best].astype(np.float32))
            recs.append(dict(side=side, seed=seed, alpha=cmb[best][0], beta=cmb[best][1], its=its[best],
                             plain_its=its[0], trials=its, key=keys[best], plain_key=keys[0]))
        if log:
            log(f"labelled {min(c0 + chunk, len(specs))}/{len(specs)} matrices in {time.time() - t0:.1f}s")
    return np.concatenate(Xs), np.concatenate(Ys), recs


def train(X, Y, epochs: int = 30, batch: int = 65536, lr: float = 3e-3, seed: int = 0, log=None):
    tr = api.ShiftTrainer(seed)
    tr.set_data(X, Y)
    rng = np.random.default_rng(seed)
    hist = []
    n = Y.size
    for ep in range(epochs):
        perm = rng.permutation(n).astype(np.int32)
        losses = []
        for s in range(0, n, batch):
            losses.append(tr.step(perm[s:s + batch], lr))
        hist.append(float(np.mean(losses)))
        if log:
            log(f"epoch {ep + 1}/{epochs} loss {hist[-1]:.6f}")
    return tr.params, hist


def save_model(path, params, meta):
    with open(path, "w") as fh:
        json.dump(dict(params=[float(v) for v in params], **meta), fh, indent=1)


def load_model(path=DEFAULT_MODEL):
    with open(path) as fh:
        d = json.load(fh)
    return np.asarray(d["params"], dtype=np.float32), d


def evaluate_batched(params, specs, min_shift=0.0, maxit=1000, chunk=200, log=None):
    """Plain ILU(0) and the learned shift on the matrices of `specs`, each solved by the
    batched persistent solver (the learned shift inferred in its factorisation pre-pass),
    GMRES(40), rtol 1e-8, at most `maxit` iterations: iterations, convergence and final
    FP64 relative residual per matrix."""
    out = []
    for c0 in range(0, len(specs), chunk):
        part = specs[c0:c0 + chunk]
        mats, rhs = [], []
        for side, seed in part:
            a = g.cdr2d(side, seed=seed)
            _, b = g.random_rhs(a, seed=seed + 1)
            mats.append(a)
            rhs.append(b)
        flat = np.concatenate(rhs)
        res = {}
        for label, model in (("plain", None), ("learned", params)):
            bs = api.BatchSolver(mats, nrhs=1, restart=RESTART, maxit=maxit)
            if model is not None:
                bs.set_shift_model(model, min_shift)
            res[label] = bs.solve(flat)
            bs.close()
        for k, (side, seed) in enumerate(part):
            nb = float(np.linalg.norm(rhs[k]))
            rec = dict(side=side, seed=seed)
            for label in ("plain", "learned"):
                o = res[label]
                rel = float(o["residual"][k]) / nb
                rec[label] = int(o["iterations"][k])
                rec[label + "_converged"] = bool(o["converged"][k])
                rec[label + "_residual"] = rel if np.isfinite(rel) and rel >= 0 else float("inf")
            out.append(rec)
        if log:
            log(f"evaluated {min(c0 + chunk, len(specs))}/{len(specs)}")
    return out


def summarize(res):
    """Held-out summary: convergence counts, iterations where both converge, and the
    final relative residual ratio (learned / plain) where neither converges."""
    both = [r for r in res if r["plain_converged"] and r["learned_converged"]]
    neither = [r for r in res if not r["plain_converged"] and not r["learned_converged"]]
    ratios = [r["learned_residual"] / r["plain_residual"] for r in neither
              if np.isfinite(r["plain_residual"]) and r["plain_residual"] > 0]
    broken = [r for r in res if not np.isfinite(r["plain_residual"])]
    return dict(
        matrices=len(res),
        plain_converged=int(sum(bool(r["plain_converged"]) for r in res)),
        learned_converged=int(sum(bool(r["learned_converged"]) for r in res)),
        both_converged=len(both),
        iterations_both=dict(plain=int(sum(r["plain"] for r in both)), learned=int(sum(r["learned"] for r in both)),
                             learned_fewer=int(sum(r["learned"] < r["plain"] for r in both)),
                             learned_more=int(sum(r["learned"] > r["plain"] for r in both))),
        neither_converged=len(neither),
        residual_ratio_median=float(np.median(ratios)) if ratios else None,
        residual_lower=int(sum(x < 1.0 for x in ratios)), residual_higher=int(sum(x > 1.0 for x in ratios)),
        plain_breakdowns=len(broken),
        breakdowns_repaired=int(sum(bool(np.isfinite(r["learned_residual"])) for r in broken)))


def evaluate(params, specs, min_shift=0.0, log=None):
    """Iterations with and without the model on the matrices of `specs`."""
    out = []
    for side, seed in specs:
        a = g.cdr2d(side, seed=seed)
        _, b = g.random_rhs(a, seed=seed + 1)
        s = Solver(a)
        plain = s.solve(b)
        learned = s.solve(b, model=params, min_shift=min_shift)
        out.append(dict(side=side, seed=seed, plain=plain["iterations"], plain_converged=plain["converged"],
                        learned=learned["iterations"], learned_converged=learned["converged"],
                        applied=learned["shift_applied"], fell_back=learned["fell_back"]))
        if log:
            log(f"eval {side}^2 seed {seed}: plain {plain['iterations']} learned {learned['iterations']}")
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train", "eval"])
    ap.add_argument("--n-train", type=int, default=2000)
    ap.add_argument("--n-eval", type=int, default=200)
    ap.add_argument("--eval-lo", type=int, default=256)
    ap.add_argument("--eval-hi", type=int, default=512)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--out", default=DEFAULT_MODEL)
    ap.add_argument("--log", default=None)
    ap.add_argument("--eval-out", default=None, help="held-out results (JSON)")
    args = ap.parse_args(argv)
    logf = open(args.log, "w") if args.log else None

    def log(msg):
        print(msg, file=sys.stderr, flush=True)
        if logf:
            logf.write(msg + "\n")
            logf.flush()

    if args.cmd == "train":
        t0 = time.time()
        specs = make_training_set(args.n_train, args.seed)
        X, Y, recs = build_dataset(specs, log)
        log(f"dataset: {Y.size} rows from {len(specs)} matrices, labels in {time.time() - t0:.1f}s")
        params, hist = train(X, Y, epochs=args.epochs, seed=args.seed, log=log)
        better = sum(1 for r in recs if tuple(r["key"]) < tuple(r["plain_key"]))
        meta = dict(features=["log(|a_ii|/mean|a_jj|)", "log(||a_i,off||_2/mean|a_jj|)", "min(dominance,4)",
                              "depth/(levels-1)"],
                    family="y = alpha*max(0,1-r) + beta", alphas=list(ALPHAS), betas=list(BETAS),
                    label_score="fewest iterations among converging members, else smallest final residual",
                    n_train=args.n_train, train_sides=[32, 128], seed=args.seed, rows=int(Y.size), loss=hist,
                    train_better_than_plain=better, min_shift=0.0, train_seconds=time.time() - t0)
        save_model(args.out, params, meta)
        log(f"saved {args.out}")
    else:
        params, meta = load_model(args.out)
        rng = np.random.default_rng(args.seed + 7)
        sides = rng.integers(args.eval_lo, args.eval_hi + 1, size=args.n_eval)
        seeds = rng.integers(0, 1 << 31, size=args.n_eval)
        res = evaluate_batched(params, list(zip(map(int, sides), map(int, seeds))), meta.get("min_shift", 0.0),
                               log=log)
        summ = summarize(res)
        log("eval: " + json.dumps(summ))
        if args.eval_out:
            with open(args.eval_out, "w") as fh:
                json.dump(dict(summary=summ, matrices=res), fh, indent=1)
    if logf:
        logf.close()


if __name__ == "__main__":
    main()
