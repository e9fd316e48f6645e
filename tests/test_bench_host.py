"""Host logic of bench.py that needs no GPU: the committed ncu capture index, the rule that a
capture is reported only for the configuration it was taken with, and the roofline arithmetic."""
import json
import re
from pathlib import Path
from types import SimpleNamespace

import pytest

import bench

ROOT = Path(__file__).resolve().parents[1]
KEYS = ("workload", "tile", "order", "bins", "exact", "table_min_log2")


def _captures():
    return json.loads(bench.CAPTURES.read_text())


def test_capture_index_is_well_formed():
    caps = _captures()
    assert caps, "no ncu captures committed"
    seen = set()
    for c in caps:
        for k in KEYS + ("kernel", "dram_bytes_per_launch", "fma_pipe_active_pct", "issue_active_pct",
                         "warp_inst", "registers", "duration_us_ncu", "summary", "command"):
            assert k in c, (k, c.get("workload"))
        assert len(c["tile"]) == 3 and all(isinstance(v, int) for v in c["tile"])
        assert c["dram_bytes_per_launch"] > 0 and c["duration_us_ncu"] > 0 and c["warp_inst"] > 0
        assert 0 < c["fma_pipe_active_pct"] < 100 and 0 < c["issue_active_pct"] < 100
        # every capture names a committed summary and a command that leaves the clocks alone
        assert (ROOT / c["summary"]).is_file(), c["summary"]
        assert "--clock-control none" in c["command"] and c["command"].startswith("ncu ")
        # the figures of one configuration appear once
        key = tuple(json.dumps(c[k]) for k in KEYS)
        assert key not in seen, key
        seen.add(key)


def test_capture_commands_name_their_summary_workload():
    for c in _captures():
        wl = re.search(r"--workload (\S+)", c["command"])
        assert (wl.group(1) if wl else "ljc92k") == c["workload"]
        tile = re.search(r"--tile (\d+),(\d+),(\d+)", c["command"])
        assert tile and [int(v) for v in tile.groups()] == c["tile"]


def test_capture_reported_only_for_its_configuration():
    c = _captures()[0]
    got = bench.ncu_capture(c["workload"], c["tile"], c["order"], c["bins"], c["exact"], c["table_min_log2"])
    assert got["matched"] and got["dram_bytes_per_launch"] == c["dram_bytes_per_launch"]
    other = list(c["tile"])
    other[1] += 7
    miss = bench.ncu_capture(c["workload"], other, c["order"], c["bins"], c["exact"], c["table_min_log2"])
    assert not miss["matched"] and "dram_bytes_per_launch" not in miss
    assert miss["wanted"]["tile"] == other
    miss = bench.ncu_capture(c["workload"], c["tile"], c["order"], c["bins"] * 2, c["exact"], c["table_min_log2"])
    assert not miss["matched"]


def test_roofline_arithmetic():
    props = SimpleNamespace(multi_processor_count=152)
    peak = bench.fp32_peak_tflops(props, 2070.0)
    assert peak == pytest.approx(152 * 128 * 2 * 2.07e9 / 1e12)
    cap = {"matched": True, "dram_bytes_per_launch": 1234}
    r = bench.roofline(1.0e6, 2.0, 1000, props, 2070.0, cap, kernel="k")
    assert r["achieved"] == pytest.approx(1.0e6 * bench.FLOPS_PER_PAIR / 2.0e-3 / 1e12)
    assert r["frac"] == pytest.approx(r["achieved"] / peak)
    assert r["traffic"] == 1234
    assert r["algorithmic_bytes_per_launch"] == 1000 * bench.BYTES_PER_PARTICLE
    # an unmatched capture reports no traffic
    r = bench.roofline(1.0e6, 2.0, 1000, props, 2070.0, {"matched": False}, kernel="k")
    assert r["traffic"] is None


def test_tile_names():
    assert bench.tile_str((1, 2, 1)).startswith("1x2x1 ")
    assert bench.force_kernel_name((1, 1, 1)).startswith("k_force_warp")
    assert bench.force_kernel_name((4, 6, 0)).startswith("k_force ")
    assert "small ones" in bench.force_kernel_name((1, 1, 1), batch=True)
