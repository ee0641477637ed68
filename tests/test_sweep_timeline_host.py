"""Host-side analysis of a line-pipeline sweep timeline (no GPU): a synthetic timeline
of a perfect pipeline, in which every line of depth costs one step, gives back its step
time through every estimate of `sweep_timeline.summarize`."""
from types import SimpleNamespace

import numpy as np

from par_ilu0_cpp_gb300 import api
from par_ilu0_cpp_gb300 import sweep_timeline


def synthetic(tau=100, t0=5_000, nx=32, ny=32, nz=32, wy=8, wz=4, by=2, bz=2, cluster=2):
    info = SimpleNamespace(grid_nx=nx, grid_ny=ny, grid_nz=nz, grid_warp_y=wy, grid_warp_z=wz, grid_cta_y=by,
                           grid_cta_z=bz, grid_cluster=cluster)
    nby, nbz = -(-ny // (by * wy)), -(-nz // (bz * wz))
    nw = by * bz
    steps = nx + wy + wz - 2
    tl = np.zeros((nby * nbz, api.LINE_TIMELINE_WORDS), dtype=np.uint64)
    for b in range(nby * nbz):
        iy, iz = b % nby, b // nby
        depth = iy * by * wy + iz * bz * wz
        end = t0 + (depth + steps) * tau
        tl[b, 0] = t0
        tl[b, 1] = b % 7
        for w in range(nw):
            tl[b, 2 + w] = end - (nw - 1 - w) * 3
        tl[b, 2 + nw] = end
    return tl, info, steps


def test_summary_of_a_perfect_pipeline():
    tau = 100
    tl, info, steps = synthetic(tau)
    s = sweep_timeline.summarize(tl, info)
    assert s["blocks"] == 8 and s["steps_per_block"] == steps and s["sms_used"] == 7
    assert s["step_ns"] == tau
    assert abs(s["depth_fit_ns_per_line"] - tau) < 1e-6
    assert s["handoff_y_ns_per_line"] == tau
    assert s["handoff_z_in_cluster_ns_per_line"] == tau
    assert s["handoff_z_l2_ns_per_line"] == tau
    assert s["start_spread_us"] == 0.0
    assert abs(s["span_us"] - (16 + 24 + steps) * tau / 1e3) < 1e-9
    assert s["warp_end_skew_first_block_us"][0] == 0.0


def test_slow_l2_handoffs_show_up_per_line():
    """Blocks behind an L2 handoff along z end later: the in-cluster and L2 estimates
    separate."""
    tau, extra = 100, 4_000
    tl, info, _ = synthetic(tau)
    nby = 2
    for b in range(tl.shape[0]):
        iz = b // nby
        late = (iz // 2) * extra  # every cluster boundary crossed adds `extra` ns
        tl[b, 2:] = np.where(tl[b, 2:] > 0, tl[b, 2:] + np.uint64(late), 0)
    s = sweep_timeline.summarize(tl, info)
    assert s["handoff_z_in_cluster_ns_per_line"] == tau
    assert s["handoff_z_l2_ns_per_line"] == tau + extra / (2 * 4)
