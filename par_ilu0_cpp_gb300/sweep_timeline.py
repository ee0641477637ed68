"""Per-block timeline of the line-pipeline substitution sweeps (diagnostic).

Runs one mixed-precision ILU(0)-GMRES solve of the 7-point convection-diffusion matrix
with LLJBASH_ILU_OPT_SWEEP_TIMELINE on, reads the last sweep of each kind
(LLJBASH_IluSolverGetSweepTimeline: per block its compute start, its SM and the end of
each warp) and splits the sweep's duration into

* the block's own work: the first block (no predecessor) runs its `steps` =
  nx + wy + wz - 2 steps alone, so its duration / steps is the time of one step;
* the pipeline: a block whose first line sits at y0 + z0 in sweep coordinates ends
  about (y0 + z0) step-times after the first block if every handoff cost one step; a
  least-squares fit of the block end times against y0 + z0 gives the measured cost per
  unit of depth, split into handoffs along y (L2, halo warp) and along z (distributed
  shared memory inside a cluster, L2 between clusters).

    python -m par_ilu0_cpp_gb300.sweep_timeline --size 128 [--cta 2,2] [--out timeline.json]
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import api
from . import generators as gen


def summarize(tl: np.ndarray, info: api.IluInfo) -> dict:
    """Splits one sweep's per-block timeline (LLJBASH_IluSolverGetSweepTimeline) into
    per-step and per-handoff costs.  Block index b = iy + nby iz in sweep coordinates."""
    wy, wz, by, bz = info.grid_warp_y, info.grid_warp_z, info.grid_cta_y, info.grid_cta_z
    nx, ny, nz = info.grid_nx, info.grid_ny, info.grid_nz
    nw = by * bz
    nby = -(-ny // (by * wy))
    nblk = tl.shape[0]
    steps = nx + wy + wz - 2
    start = tl[:, 0].astype(np.int64)
    ends = tl[:, 2:2 + nw].astype(np.int64)
    t0 = int(start.min())
    end = ends.max(axis=1) - t0
    st = start - t0
    b = np.arange(nblk)
    iy, iz = b % nby, b // nby
    depth = iy * by * wy + iz * bz * wz
    span = int(end.max())
    dur0 = int(end[0] - st[0])
    step_ns = dur0 / steps
    slope, icpt = np.polyfit(depth.astype(float), end.astype(float), 1)
    # handoff costs: end of block (iy, iz) minus end of its predecessor along y / z, per
    # line of depth the block adds, against one step per line
    dy = [(end[i] - end[i - 1]) / (by * wy) for i in range(nblk) if iy[i] > 0]
    cl = info.grid_cluster
    dz_in, dz_l2 = [], []
    for i in range(nblk):
        if iz[i] == 0:
            continue
        d = (end[i] - end[i - nby]) / (bz * wz)
        (dz_in if cl > 1 and iz[i] % cl != 0 else dz_l2).append(d)
    med = lambda v: float(np.median(v)) if len(v) else None  # noqa: E731
    return {
        "blocks": int(nblk),
        "sms_used": int(len(np.unique(tl[:, 1]))),
        "steps_per_block": int(steps),
        "critical_path_steps": int(nx + ny + nz - 2),
        "span_us": span / 1e3,
        "start_spread_us": float(st.max()) / 1e3,
        "first_block_us": dur0 / 1e3,
        "step_ns": step_ns,
        "ideal_span_us": (nx + ny + nz - 2) * step_ns / 1e3,
        "depth_fit_ns_per_line": float(slope),
        "depth_fit_intercept_us": float(icpt) / 1e3,
        "handoff_y_ns_per_line": med(dy),
        "handoff_z_in_cluster_ns_per_line": med(dz_in),
        "handoff_z_l2_ns_per_line": med(dz_l2),
        "warp_end_skew_first_block_us": [float(e - ends[0, 0]) / 1e3 for e in ends[0]],
    }


def run(size: int, cta=(0, 0), cluster: int = 1, one_cta_per_sm: bool = False) -> dict:
    a = gen.convdiff3d(size)
    f, _ = api.iluk_symbolic(a, 0)
    _, b = gen.random_rhs(a, seed=1)
    ilu = api.IluSolver()
    ilu.set_option(api.ILU_OPT_SWEEP_TIMELINE, 1)
    ilu.set_option(api.ILU_OPT_GRID_CTA_Y, cta[0])
    ilu.set_option(api.ILU_OPT_GRID_CTA_Z, cta[1])
    ilu.set_option(api.ILU_OPT_GRID_CLUSTER, cluster)
    ilu.set_option(api.ILU_OPT_GRID_ONE_CTA_PER_SM, int(one_cta_per_sm))
    ilu.set_matrix(f)
    if ilu.setup() != 0 or ilu.factorize() != 0:
        raise RuntimeError(api.last_error())
    gm = api.Gmres(1e-8, 50, 1000)
    gm.set_preconditioner(ilu)
    gm.set_option(api.GMRES_OPT_MODE, 1)
    res = gm.solve(a, b)
    info = ilu.info()
    out = {"workload": f"convdiff3d {size}^3 ILU(0), mixed GMRES(50)", "iterations": int(res.iterations),
           "line_shape": [info.grid_warp_y, info.grid_warp_z, info.grid_cta_y, info.grid_cta_z, info.grid_blocks],
           "cluster": int(info.grid_cluster), "one_cta_per_sm": bool(one_cta_per_sm),
           "fp64_line": int(info.grid_fp64), "fp32_line": int(info.grid_fp32),
           "sweeps": {}}
    for fp32 in (True, False):
        for upper in (False, True):
            try:
                tl = ilu.sweep_timeline(upper, fp32)
            except RuntimeError:
                continue
            if not tl[:, 0].any():
                continue  # no line-pipeline sweep of this kind ran
            name = f"{'fp32' if fp32 else 'fp64'}_{'backward' if upper else 'forward'}"
            out["sweeps"][name] = summarize(tl, info)
    return out


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--size", type=int, default=128)
    ap.add_argument("--out", default=None)
    ap.add_argument("--cta", type=lambda v: [int(t) for t in v.split(",")], default=[0, 0],
                    help="warps of a CTA along y,z (0,0: automatic)")
    ap.add_argument("--cluster", type=int, default=1, help="LLJBASH_ILU_OPT_GRID_CLUSTER")
    ap.add_argument("--one-cta-per-sm", action="store_true", help="LLJBASH_ILU_OPT_GRID_ONE_CTA_PER_SM")
    args = ap.parse_args()
    r = run(args.size, args.cta, args.cluster, args.one_cta_per_sm)
    text = json.dumps(r, indent=1)
    print(text)
    if args.out:
        with open(args.out, "w") as fh:
            fh.write(text + "\n")


if __name__ == "__main__":
    main()
