"""Benchmark: time to ||b - A x||_2 / ||b||_2 <= 1e-8 on one GB300.

Workload (the single-GPU configuration the metric is quoted on): 3D 7-point upwind
convection-diffusion on a 128^3 grid (n = 2,097,152, nnz = 14,581,760), diffusion 1,
wind (1, 0.5, 0.25) at cell Peclet 0.5, natural ordering, ILU(0) + GMRES(50),
relative tolerance 1e-8 (absolute 1e-8 ||b||_2 passed to the solver), max 1000
iterations, x_true ~ U[-1, 1] (seed 0), b = A x_true, x0 = 0.  Seeded synthetic data.

One step = numeric factorisation (+ learned-shift pre-pass when enabled) + GMRES to the
tolerance, on inputs resident in HBM (device-resident entry points).  ``value`` is the
headline solver (FP32 cycles in FP64 refinement, learned shift when a model is
available); the plain FP64 solver is timed the same way beside it.  ``e2e`` repeats the
headline solve through the reference-facing C ABI with host buffers (IluSolverFactorize +
GmresSolve, every copy inside the timed region).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times the reference's own code on the host cores instead (its
sources compiled against the oracle shim with the threaded-BLAS stand-ins, built into
oracle/_ref by build(); the oracle port where that build is absent), on the same
workload and metric: the test/benchmark.cpp repetition loop (Factorize + GMRES timed,
symbolic and setup once), after a thread-count sweep.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms to ‖r‖/‖b‖≤1e-8: mixed+learned vs plain FP64 ILU-GMRES, same GB300; HBM GB/s"
RESTART = 50
MAXIT = 1000
RTOL = 1e-8
SEED = 0


def workload(size: int):
    from par_ilu0_cpp_gb300 import generators as g

    a = g.convdiff3d(size)
    x_true, b = g.random_rhs(a, SEED)
    return a, x_true, b


def config_of(a, size, solver):
    return {
        "workload": f"convdiff3d 7-pt upwind {size}^3 (Pe 0.5, wind (1,0.5,0.25)), ILU(0)+GMRES({RESTART}), "
                    f"rtol {RTOL:g}, natural order",
        "n": a.n,
        "nnz": a.nnz,
        "restart": RESTART,
        "max_iterations": MAXIT,
        "solver": solver,
        "l2_policy": "inputs larger than L2 (A = 175 MB FP64, Krylov basis 0.4-0.9 GB) - no flush",
        "parallelism": "replicas",
    }


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int = 0):
        self.proc = None
        self.lines = []
        self.device_index = device_index

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device_index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(kind, a, nnz_l, nnz_u, tsize, steps_hist):
    """Algorithmic bytes of all launches of one kernel kind during a profiled solve.
    tsize: bytes per vector / factor value (8 FP64, 4 FP32); indices are int32.
    steps_hist: list of Arnoldi step indices s that ran (one launch each)."""
    n, nnz = a.n, a.nnz
    S = len(steps_hist)
    if kind == "sptrsv_lower":
        # packed L entries (col + value), row ids, rhs read, normalised rhs written back, y written
        return S * ((4 + tsize) * nnz_l + 4 * n + 3 * tsize * n)
    if kind == "sptrsv_upper":
        # packed U entries (col + value), row ids, diagonal, y read, z written
        return S * ((4 + tsize) * nnz_u + 4 * n + 3 * tsize * n)
    if kind == "spmv":
        # CSR (col + value, row pointers), x read, w written, forward-sweep vector reset
        return S * ((4 + tsize) * nnz + 4 * (n + 1) + 3 * tsize * n)
    if kind == "cgs_dot":
        return sum(tsize * n * (s + 2) for s in steps_hist)
    if kind in ("cgs_axpy_dot", "cgs_axpy_norm"):
        return sum(tsize * n * (s + 3) for s in steps_hist)
    return None


def measured_traffic(kernel, size, block_rows, cluster, line=False):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of `kernel`
    for this workload and substitution schedule, from the ncu captures recorded in
    profiles/dram_traffic.json (entries: kernel, size, schedule "line" with the CTAs per
    cluster of the line-pipeline kernel (0: none), or block_rows / cluster of the
    block-local kernel, bytes, source); None when no capture matches the kernel and
    schedule that ran."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if not os.path.isfile(path):
        return None
    with open(path) as fh:
        entries = json.load(fh).get("captures", [])
    for e in entries:
        if e.get("kernel") != kernel or e.get("size") != size:
            continue
        if line and e.get("schedule") == "line" and e.get("cluster", 0) == cluster:
            return int(e["bytes"])
        if not line and e.get("schedule", "block") == "block" and e.get("block_rows") == block_rows \
                and e.get("cluster") == cluster:
            return int(e["bytes"])
    return None


def kernel_profile(gm, ilu, dev, a, f_nnz_l, f_nnz_u, tsize):
    """One extra solve with every kernel timed by CUDA events on its stream."""
    from par_ilu0_cpp_gb300 import api

    gm.reset_kernel_times()
    gm.set_option(api.GMRES_OPT_PROFILE, 1)
    dev["x"].zero_()
    import torch

    torch.cuda.synchronize()
    ilu.factorize_device(dev["fv"].data_ptr())
    ok, its = gm.solve_device(a.n, dev["rp"].data_ptr(), dev["ci"].data_ptr(), dev["av"].data_ptr(),
                              dev["b"].data_ptr(), dev["x"].data_ptr())
    gm.set_option(api.GMRES_OPT_PROFILE, 0)
    kt = gm.kernel_times()
    rep = gm.report()
    # reconstruct the Arnoldi step indices: cycles of up to RESTART steps
    steps = []
    left = kt["spmv"][1]
    while left > 0:
        c = min(RESTART, left)
        steps.extend(range(c))
        left -= c
    out = {}
    for kind, (ms, cnt) in kt.items():
        if cnt == 0:
            continue
        byt = algorithmic_bytes(kind, a, f_nnz_l, f_nnz_u, tsize, steps[:cnt] if kind != "residual" else [])
        out[kind] = {"ms_total": ms, "launches": cnt, "avg_us": 1e3 * ms / cnt,
                     "alg_bytes_total": byt, "gbs": (byt / (ms * 1e-3) / 1e9) if byt else None}
    return out, rep


def batched_section(nsys: int, nrhs: int, learned, seed: int = 5, with_cpu: bool = True):
    """Batched configuration: nsys variable-coefficient 5-point systems (lognormal field
    sigma 1, sides ~ U[32, 224]), nrhs right-hand sides each, x_true ~ U[-1, 1], ILU(0)
    FP32 factors (+ learned shift) + GMRES(30) in one persistent launch, FP64 residuals to
    1e-8 relative.  Returns the JSON section."""
    from par_ilu0_cpp_gb300 import api
    from par_ilu0_cpp_gb300 import generators as g

    t0 = time.perf_counter()
    systems = g.batched_systems(nsys, seed)
    rhs, xt = [], []
    for k, a in enumerate(systems):
        x, b = g.random_rhs(a, seed=seed * 100000 + k, nrhs=nrhs)
        xt.append(np.atleast_2d(x))
        rhs.append(np.atleast_2d(b))
    gen_s = time.perf_counter() - t0
    bs = api.BatchSolver(systems, nrhs=nrhs, restart=30, rtol=RTOL, maxit=MAXIT)
    if learned.get("params") is not None:
        bs.set_shift_model(learned["params"], learned.get("min_shift", 0.0))
    bs.autotune()
    cps, lf, rpc = bs.shape()
    trials = bs.trials()
    flat = np.concatenate([b.ravel() for b in rhs])
    bs.solve(flat)  # warm-up
    out = bs.solve(flat)
    # FP64 true residuals and forward errors, recomputed on the host
    worst, fwd, pos = 0.0, 0.0, 0
    for k, a in enumerate(systems):
        for r in range(nrhs):
            xr = out["x"][pos:pos + a.n]
            worst = max(worst, float(np.linalg.norm(rhs[k][r] - g.spmv(a, xr)) / np.linalg.norm(rhs[k][r])))
            fwd = max(fwd, float(np.max(np.abs(xr - xt[k][r]))))
            pos += a.n
    unknowns = int(sum(a.n for a in systems)) * nrhs
    roof = batched_roofline(systems, nrhs, rpc, out["iterations"], out["ms"])
    cpu = batched_cpu_baseline(systems, rhs, seed) if with_cpu else None
    return {"workload": f"{nsys} variable-coefficient 5-pt systems (sides U[32,224], lognormal sigma 1) x {nrhs} RHS, "
                        "ILU(0) FP32 + GMRES(30), FP64 refinement to rtol 1e-8, one persistent launch",
            "systems": nsys, "rhs_per_system": nrhs, "unknowns": unknowns, "ms": round(out["ms"], 3),
            "solves_per_s": round(nsys * nrhs / (out["ms"] * 1e-3), 1),
            "converged_fraction": float(np.mean(out["converged"])), "max_rel_residual": worst,
            "max_forward_error": fwd, "iterations_mean": float(np.mean(out["iterations"])),
            "iterations_max": int(np.max(out["iterations"])),
            "autotune": {"ctas_per_sm": cps, "largest_first": lf, "rhs_per_cta": rpc,
                         "rows_per_cta_round": 512 // rpc, "trials": trials},
            "roofline": roof,
            "learned_shift": learned.get("params") is not None, "generation_s": round(gen_s, 2),
            "cpu_baseline": cpu}


def batched_roofline(systems, nrhs, rpc, iterations, ms):
    """Algorithmic bytes of the batched launch over its device time, against the measured
    HBM copy bandwidth.  Per right-hand side and Krylov step (GMRES(30), step i of a cycle
    touching i + 1 basis vectors, i = 14.5 on average): the two sweeps (read v, write z,
    read and write z), the SpMV (read z, write w) and CGS2 (two passes reading i + 1 basis
    vectors and w, two axpy passes, a norm) on FP32 vectors, 4 n (9 + 4 (i + 1)) bytes;
    per group of rpc right-hand sides and step, the FP32 factor and matrix values with
    their column indices once, 16 nnz bytes.  Factorisation and FP64 residuals (once per
    cycle) are left out: the figure is a lower bound of the traffic."""
    peak, kind = measured_peaks()
    it = np.asarray(iterations).reshape(len(systems), nrhs)
    vec = coef = 0.0
    for k, a in enumerate(systems):
        vec += float(np.sum(it[k])) * 4.0 * a.n * (9 + 4 * 15.5)
        for r0 in range(0, nrhs, rpc):
            coef += float(np.max(it[k, r0:r0 + rpc])) * 16.0 * a.nnz
    total = vec + coef
    achieved = total / (ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_source": kind, "alg_bytes": total}


BATCH_CPU_SAMPLE = 96


def batched_cpu_baseline(systems, rhs, seed, sample=BATCH_CPU_SAMPLE):
    """The batched workload on the host cores: a random sample of the systems, each
    solved as the reference would (symbolic + setup, one factorisation, GMRES(30) from
    x0 = 0 per right-hand side to 1e-8 relative, plain FP64), systems side by side on all
    cores (one thread each, largest first), the wall time scaled to all systems.  The
    reference's own code when its timing build is present, else the oracle port."""
    import concurrent.futures

    import oracle

    cores = os.cpu_count() or 1
    rng = np.random.default_rng(seed)
    pick = rng.choice(len(systems), size=min(sample, len(systems)), replace=False)
    pick = sorted(pick, key=lambda k: -systems[k].n)
    kind = "port"
    if os.path.isfile(oracle.REF_OMP_SO):
        try:
            ref = oracle.Ref(oracle.REF_OMP_SO)
            kind = "reference"
        except OSError:
            pass
    if kind == "reference":
        def job(k):
            r = ref.solve_system(systems[k], rhs[k], 0, RTOL, 30, MAXIT, 1)
            return r["converged"], int(np.sum(r["iters"]))
    else:
        port = oracle.Port()

        def job(k):
            a = systems[k]
            lu, _ = port.factorize(a)
            conv, its = 0, 0
            for b in rhs[k]:
                ok, it, _, _ = port.gmres(a, a, lu, b, RTOL * float(np.linalg.norm(b)), 30, MAXIT)
                conv += int(ok)
                its += it
            return conv, its
    with oracle.c_stdout_to_stderr():
        t0 = time.perf_counter()
        with concurrent.futures.ThreadPoolExecutor(max_workers=cores) as ex:
            res = list(ex.map(job, pick))
        wall = time.perf_counter() - t0
    nrhs = len(rhs[0])
    conv = sum(c for c, _ in res)
    its = sum(i for _, i in res)
    return {"value": round(1e3 * wall * len(systems) / len(pick), 1), "unit": "ms", "cores": cores, "kind": kind,
            "sample": f"{len(pick)} of {len(systems)} systems x {nrhs} RHS ({sum(systems[k].n for k in pick)} "
                      f"unknowns), plain FP64 ILU(0) once per system + GMRES(30) per RHS, systems side by side "
                      f"on {cores} threads, wall time {wall:.2f} s scaled by {len(systems)}/{len(pick)}",
            "converged_fraction": conv / (len(pick) * nrhs), "iterations_mean": its / (len(pick) * nrhs)}


def other_configs(api, g):
    """Secondary configurations, one solve each (plain FP64 and mixed): the 2D 256^2
    Laplacian with ILU(0)+GMRES(30) and the 64^3 27-point lognormal operator with
    ILU(1) / ILU(2)+GMRES(30) (symbolic ILU(k) on the host included in its own timer)."""
    out = {}
    cases = [("laplace2d_256_ilu0", lambda: g.laplace2d(256), 0),
             ("lognormal27_64_ilu1", lambda: g.lognormal27(64, seed=0), 1),
             ("lognormal27_64_ilu2", lambda: g.lognormal27(64, seed=0), 2)]
    for name, make, lof in cases:
        a = make()
        x_true, b = g.random_rhs(a, SEED)
        t0 = time.perf_counter()
        f, _ = api.iluk_symbolic(a, lof)
        sym_ms = 1e3 * (time.perf_counter() - t0)
        rec = {"n": a.n, "nnz": a.nnz, "nnz_factor": f.nnz, "symbolic_ms": round(sym_ms, 1)}
        for mode, label in ((0, "plain"), (1, "mixed")):
            ilu = api.IluSolver()
            ilu.set_option(api.ILU_OPT_COPY_BACK, 0)
            ilu.set_matrix(f)
            ilu.setup()
            gm = api.Gmres(RTOL * float(np.linalg.norm(b)), 30, MAXIT)
            gm.set_preconditioner(ilu)
            gm.set_option(api.GMRES_OPT_MODE, mode)
            gm.set_option(api.GMRES_OPT_KEEP_MATRIX, 1)
            for rep in range(2):
                ilu.set_values(f.values)
                t0 = time.perf_counter()
                ilu.factorize()
                res = gm.solve(a, b)
                ms = 1e3 * (time.perf_counter() - t0)
            rec[label] = {"ms": round(ms, 2), "iterations": res.iterations,
                          "rel_residual": float(np.linalg.norm(b - g.spmv(a, res.x)) / np.linalg.norm(b))}
        out[name] = rec
    return out


def _reference_solver(a, tol):
    """The reference's own code when oracle/_ref holds its timing build for this machine
    (kind "reference"), else the oracle port (kind "port").  Returns (kind, session),
    session offering set_threads(t) and step(b) -> (ok, iters, x, fact_s, gmres_s)."""
    import oracle

    if os.path.isfile(oracle.REF_OMP_SO):
        try:
            ref = oracle.Ref(oracle.REF_OMP_SO)
            return "reference", ref.session(a, 0, tol, RESTART, MAXIT, os.cpu_count() or 1)
        except OSError:
            pass
    return "port", _PortSession(oracle.Port(), a, tol)


class _PortSession:
    """The oracle port behind the same interface as oracle.RefSession (ILU(0): the
    pattern of A is the pattern of the factors)."""

    def __init__(self, port, a, tol):
        self.port, self.a, self.tol = port, a, tol
        self.threads = os.cpu_count() or 1

    def set_threads(self, t):
        self.threads = int(t)
        return 0.0

    def step(self, b):
        lu, fact_s = self.port.factorize(self.a, nthreads=self.threads)
        t0 = time.perf_counter()
        ok, its, x, _ = self.port.gmres(self.a, self.a, lu, b, self.tol, RESTART, MAXIT, nthreads=self.threads)
        return ok, its, x, fact_s, time.perf_counter() - t0


def _thread_counts(cores, with_one=True):
    return sorted({t for t in ((1, 8, cores) if with_one else (8, cores)) if 1 <= t <= cores})


def cpu_baseline(a, b, tol, cores):
    """The reference on the host cores, as its benchmark runs it: factorisation + a full
    GMRES solve (x0 = 0) per repetition, symbolic ILU and setup once, timed with
    steady_clock; the best of 8 threads and all cores (one repetition each, OpenMP bound
    to cores).  About 10 s of CPU work on the 128^3 workload."""
    os.environ.setdefault("OMP_PROC_BIND", "close")
    os.environ.setdefault("OMP_PLACES", "cores")
    kind, sess = _reference_solver(a, tol)
    best = None
    sweep = {}
    for t in _thread_counts(cores, with_one=False):
        sess.set_threads(t)
        ok, its, x, fs, gs = sess.step(b)
        ms = 1e3 * (fs + gs)
        sweep[str(t)] = round(ms, 1)
        if best is None or ms < best[0]:
            best = (ms, t, its, fs, gs, ok)
    ms, t, its, fs, gs, ok = best
    return {"value": round(ms, 3), "unit": "ms", "cores": t, "kind": kind,
            "sample": f"one full solve per thread count (factorise + GMRES({RESTART}) to the tolerance, "
                      f"{its} iterations), best of {sorted(int(k) for k in sweep)} threads",
            "thread_sweep_ms": sweep, "factorize_ms": round(1e3 * fs, 3), "gmres_ms": round(1e3 * gs, 3),
            "iterations": its, "converged": bool(ok)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    os.environ.setdefault("OMP_PROC_BIND", "close")
    os.environ.setdefault("OMP_PLACES", "cores")
    a, x_true, b = workload(args.size)
    tol = RTOL * float(np.linalg.norm(b))
    cores = os.cpu_count() or 1
    kind, sess = _reference_solver(a, tol)
    # thread sweep (one repetition each), then the timed repetitions at the best count
    sweep = {}
    for t in _thread_counts(cores):
        sess.set_threads(t)
        ok, its, x, fs, gs = sess.step(b)
        sweep[t] = 1e3 * (fs + gs)
    best_t = min(sweep, key=sweep.get)
    sess.set_threads(best_t)
    vals, facts, gms = [], [], []
    ok, its = True, 0
    for i in range(args.warmup + args.steps):
        ok, its, x, fs, gs = sess.step(b)
        if i >= args.warmup:
            vals.append(1e3 * (fs + gs))
            facts.append(1e3 * fs)
            gms.append(1e3 * gs)
    v = float(np.mean(vals))
    res = float(np.linalg.norm(b - _spmv(a, x)) / np.linalg.norm(b))
    sample = (f"test/benchmark.cpp repetition loop: Factorize + GMRES({RESTART}) from x0 = 0 to the tolerance "
              f"({its} iterations), symbolic + setup once; {best_t} threads (sweep "
              f"{ {k: round(w, 1) for k, w in sweep.items()} } ms), mean of {args.steps} repetitions")
    line = {"metric": METRIC, "value": round(v, 3), "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(v, 3), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
            "config": config_of(a, args.size, "reference ILU(0)+GMRES, plain FP64, host cores"),
            "iterations": its, "converged": bool(ok), "relative_residual": res,
            "factorize_ms": round(float(np.mean(facts)), 3), "gmres_ms": round(float(np.mean(gms)), 3),
            "cpu_baseline": {"value": round(v, 3), "unit": "ms", "cores": best_t, "kind": kind, "sample": sample},
            "e2e": {"value": round(v, 3), "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _spmv(a, x):
    from par_ilu0_cpp_gb300 import generators as g

    return g.spmv(a, x)


def max_over_ranks(values, dist, device):
    """Each value's maximum over the ranks (the slowest replica sets every timing); the
    values unchanged without a process group."""
    if dist is None:
        return [float(v) for v in values]
    import torch

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def run_ours(args):
    import torch

    from par_ilu0_cpp_gb300 import api

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    api.load()
    a, x_true, b = workload(args.size)
    bnorm = float(np.linalg.norm(b))
    tol = RTOL * bnorm
    f, nzmap = api.iluk_symbolic(a, 0)
    an = api.analyze_pattern(f)
    diag = an["diag"]
    nnz_l = int(np.sum(diag - f.row_ptr[:-1]))
    nnz_u = int(np.sum(f.row_ptr[1:] - diag - 1))
    dev = {"rp": torch.from_numpy(a.row_ptr).cuda(), "ci": torch.from_numpy(a.col_idx).cuda(),
           "av": torch.from_numpy(a.values).cuda(), "fv": torch.from_numpy(f.values).cuda(),
           "b": torch.from_numpy(b).cuda(), "x": torch.zeros(a.n, dtype=torch.float64, device="cuda")}
    torch.cuda.synchronize()

    def make(mode):
        ilu = api.IluSolver()
        ilu.set_option(api.ILU_OPT_GRID_CLUSTER, args.line_cluster)
        ilu.set_option(api.ILU_OPT_GRID_CTA_Y, args.line_cta[0])
        ilu.set_option(api.ILU_OPT_GRID_CTA_Z, args.line_cta[1])
        ilu.set_matrix(f)
        assert ilu.setup() == 0, api.last_error()
        ilu.set_option(api.ILU_OPT_COPY_BACK, 0)
        gm = api.Gmres(tol, RESTART, MAXIT)
        gm.set_preconditioner(ilu)
        gm.set_option(api.GMRES_OPT_MODE, mode)
        return ilu, gm

    solvers = {"plain": make(0), "mixed": make(1)}

    # Learned shift for the headline solver: the committed model's pre-pass runs in the
    # factorisation; its decision rule (plain ILU when the shifted factors do not beat
    # the plain iteration count on this matrix) is taken once, on the first warm-up
    # solve, and kept for the timed solves.
    learned = {"model": None, "applied": False}
    model_path = os.path.join(ROOT, "par_ilu0_cpp_gb300", "shift_model.json")
    if os.path.isfile(model_path):
        from par_ilu0_cpp_gb300 import learned_shift as ls

        params, meta = ls.load_model(model_path)
        learned["model"] = os.path.relpath(model_path, ROOT)
        learned["params"] = params
        learned["min_shift"] = float(meta.get("min_shift", 0.0))

    def step(name):
        ilu, gm = solvers[name]
        dev["x"].zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        rc = ilu.factorize_device(dev["fv"].data_ptr())
        if rc != 0:
            raise RuntimeError(f"{name} factorisation failed: rc={rc} {api.last_error()}")
        ok, its = gm.solve_device(a.n, dev["rp"].data_ptr(), dev["ci"].data_ptr(), dev["av"].data_ptr(),
                                  dev["b"].data_ptr(), dev["x"].data_ptr())
        e1.record()
        torch.cuda.synchronize()
        if rc != 0 or not ok:
            raise RuntimeError(f"{name} solve failed: rc={rc} ok={ok} its={its} {api.last_error()}")
        return e0.elapsed_time(e1), its

    if learned["model"] is not None:
        ilu_m = solvers["mixed"][0]
        _, its_plain_f = step("mixed")
        ilu_m.set_shift_model(learned["params"], learned["min_shift"])
        _, its_learned = step("mixed")
        applied = bool(ilu_m.info().shift_applied) and its_learned < its_plain_f
        learned.update(iterations_with_shift=its_learned, iterations_plain_factors=its_plain_f, applied=applied,
                       decision="learned shift kept" if applied else "plain ILU kept (shift did not beat plain)")
        if not applied:
            ilu_m.set_shift_model(None)
    for _ in range(args.warmup):
        step("plain")
        step("mixed")
    launches0 = sum(s[0].info().kernel_launches + s[1].report().kernel_launches for s in solvers.values())
    clocks = ClockSampler(local)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    times = {"plain": [], "mixed": []}
    its = {}
    for _ in range(args.steps):
        for name in ("mixed", "plain"):
            ms, it = step(name)
            times[name].append(ms)
            its[name] = it
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clk = clocks.stop()
    launches1 = sum(s[0].info().kernel_launches + s[1].report().kernel_launches for s in solvers.values())
    ms = {k: float(np.mean(v)) for k, v in times.items()}
    ms["mixed"], ms["plain"] = max_over_ranks([ms["mixed"], ms["plain"]], dist, "cuda")

    # accuracy of the headline answer (FP64 true residual, forward error vs x_true)
    step("mixed")
    x = dev["x"].cpu().numpy()
    from par_ilu0_cpp_gb300 import generators as g

    res_m = float(np.linalg.norm(b - g.spmv(a, x))) / bnorm
    fwd_m = float(np.max(np.abs(x - x_true)))
    step("plain")
    xp = dev["x"].cpu().numpy()
    res_p = float(np.linalg.norm(b - g.spmv(a, xp))) / bnorm

    # e2e through the reference-facing C ABI with host buffers (headline mode).  The
    # caller's buffers are page-locked: A in a library-owned CsrMatrix (SetupCsrMatrix
    # allocates page-locked arrays), b and x in pinned host tensors; the factor values
    # live in the solver's own (page-locked) GetMatrix() storage.
    e2e_ms = []
    ilu_h = api.IluSolver()
    ilu_h.set_option(api.ILU_OPT_GRID_CLUSTER, args.line_cluster)
    ilu_h.set_option(api.ILU_OPT_GRID_CTA_Y, args.line_cta[0])
    ilu_h.set_option(api.ILU_OPT_GRID_CTA_Z, args.line_cta[1])
    ilu_h.set_matrix(f)
    assert ilu_h.setup() == 0
    gm_h = api.Gmres(tol, RESTART, MAXIT)
    gm_h.set_preconditioner(ilu_h)
    gm_h.set_option(api.GMRES_OPT_MODE, 1)
    if learned.get("applied"):
        ilu_h.set_shift_model(learned["params"], learned["min_shift"])
    a_pin = api.OwnedCsr(a)
    b_pin = torch.from_numpy(b).pin_memory().numpy()
    x_pin = torch.zeros(a.n, dtype=torch.float64).pin_memory().numpy()
    for i in range(args.warmup + args.steps):
        ilu_h.set_values(f.values)  # the factors of the previous step were copied back in place
        x_pin[:] = 0.0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc = ilu_h.factorize()
        ok_h, _ = gm_h.solve_buffers(a_pin, b_pin, x_pin)
        t1 = time.perf_counter()
        if rc != 0 or not ok_h:
            raise RuntimeError("e2e solve failed")
        if i >= args.warmup:
            e2e_ms.append(1e3 * (t1 - t0))
    e2e_res = float(np.linalg.norm(b - g.spmv(a, x_pin))) / bnorm
    if not e2e_res <= RTOL * 1.0001:
        raise RuntimeError(f"e2e solution misses the tolerance ({e2e_res:.3e})")
    h2d = 8 * f.nnz + 4 * (a.n + 1) + 4 * a.nnz + 8 * a.nnz + 8 * a.n + 8 * a.n
    d2h = 8 * f.nnz + 8 * a.n

    # per-kernel profile of the headline solve (events on the launching stream)
    prof, _ = kernel_profile(solvers["mixed"][1], solvers["mixed"][0], dev, a, nnz_l, nnz_u, 4)
    prof_plain, _ = kernel_profile(solvers["plain"][1], solvers["plain"][0], dev, a, nnz_l, nnz_u, 8)
    dom = max((k for k in prof if prof[k]["gbs"] is not None), key=lambda k: prof[k]["ms_total"])
    peak, peak_kind = measured_peaks()
    achieved = prof[dom]["gbs"]
    info_m = solvers["mixed"][0].info()
    schedule = {"fp64_block_rows": int(info_m.block_rows_fp64), "fp32_block_rows": int(info_m.block_rows_fp32),
                "fp64_cluster": int(info_m.block_cluster_fp64), "fp32_cluster": int(info_m.block_cluster_fp32),
                # line-pipeline sweeps (bit 0 forward, bit 1 backward), chosen by timing at setup
                "fp64_line": int(info_m.grid_fp64), "fp32_line": int(info_m.grid_fp32),
                "line_shape": [int(info_m.grid_warp_y), int(info_m.grid_warp_z), int(info_m.grid_cta_y),
                               int(info_m.grid_cta_z), int(info_m.grid_blocks)],
                "line_cluster": int(info_m.grid_cluster)}
    dom_line = bool(schedule["fp32_line"] & (1 if dom == "sptrsv_lower" else 2 if dom == "sptrsv_upper" else 0))
    traffic = measured_traffic(dom, args.size, schedule["fp32_block_rows"],
                               schedule["line_cluster"] if dom_line else schedule["fp32_cluster"], dom_line)

    batched = None
    others = None
    if rank == 0 and not args.quick:
        batched = batched_section(args.batch_systems, args.batch_rhs, learned, with_cpu=not args.no_cpu)
        from par_ilu0_cpp_gb300 import generators as gg

        others = other_configs(api, gg)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(a, b, tol, os.cpu_count() or 1)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(ms["mixed"], 3), "unit": "ms", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms["mixed"], 3), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 Krylov/ILU + f64 refinement", "data": "synthetic (seeded generator)",
            "config": dict(config_of(a, args.size, "mixed (FP32 cycles in FP64 refinement) + learned shift policy"),
                           substitution_schedule=schedule),
            "learned_shift": {k: v for k, v in learned.items() if k != "params"},
            "plain_fp64_ms": round(ms["plain"], 3),
            "speedup_vs_plain": round(ms["plain"] / ms["mixed"], 3),
            "iterations": {"mixed": its["mixed"], "plain": its["plain"]},
            "relative_residual": {"mixed": res_m, "plain": res_p}, "forward_error_inf": fwd_m,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "peak_source": peak_kind, "traffic": traffic},
            "kernels_mixed": {k: {kk: (round(vv, 4) if isinstance(vv, float) else vv) for kk, vv in d.items()}
                              for k, d in prof.items()},
            "kernels_plain": {k: {kk: (round(vv, 4) if isinstance(vv, float) else vv) for kk, vv in d.items()}
                              for k, d in prof_plain.items()},
            "cpu_baseline": cpu,
            "e2e": {"value": round(float(np.mean(e2e_ms)), 3), "unit": "ms", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "path": "LLJBASH_IluSolverFactorize + LLJBASH_GmresSolve",
                    "host_buffers": "page-locked", "relative_residual": e2e_res},
            "gpu_launches": int(launches1 - launches0),
            "batched": batched,
            "other_configs": others,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=128)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--quick", action="store_true", help="skip the batched and secondary configurations")
    ap.add_argument("--batch-systems", type=int, default=512)
    ap.add_argument("--batch-rhs", type=int, default=16)
    ap.add_argument("--line-cluster", type=int, default=1,
                    help="CTAs per thread-block cluster of the line-pipeline sweeps: 1 automatic (16, else 8), "
                         "2-16 at most that many, 0 none")
    ap.add_argument("--line-cta", type=lambda v: [int(t) for t in v.split(",")], default=[0, 0],
                    help="warps of a line-pipeline CTA along y,z (0,0: automatic)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
