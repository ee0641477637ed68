"""Host helpers of the benchmark (no GPU): the roofline's DRAM traffic is looked up in
profiles/dram_traffic.json by kernel, workload size and the substitution schedule that
ran (line-pipeline kernel and its cluster size, or block rows and cluster size of the
block-local kernel), and nothing is reported for a schedule no capture covers."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _captures():
    with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as fh:
        return json.load(fh)["captures"]


def test_every_capture_is_found_by_its_own_schedule():
    caps = _captures()
    assert caps
    for e in caps:
        line = e.get("schedule") == "line"
        cluster = e.get("cluster", 0)
        got = bench.measured_traffic(e["kernel"], e["size"], e.get("block_rows"), cluster, line)
        assert got == int(e["bytes"]), e


def test_schedules_without_a_capture_report_none():
    assert bench.measured_traffic("sptrsv_lower", 64, 32768, 16, False) is None
    assert bench.measured_traffic("sptrsv_lower", 128, 32768, 8, True) is None  # clusters of 8: no capture
    assert bench.measured_traffic("spmv", 128, 32768, 16, False) is None


def test_line_and_block_captures_are_told_apart():
    line16 = bench.measured_traffic("sptrsv_lower", 128, 32768, 16, True)
    block16 = bench.measured_traffic("sptrsv_lower", 128, 32768, 16, False)
    assert line16 is not None and block16 is not None and line16 != block16
