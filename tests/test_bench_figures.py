"""The bench line's figures that come from the sweep's recorded ncu profile, on the CPU.

bench.py reads two numbers from profiles/k_batch_sweep_water256.md: the DRAM bytes of one full
sweep (the `traffic` of the roofline) and the warp instructions per move (the `issue` roofline).
Checked: both lines parse to plausible values, and the issue-rate arithmetic (instructions per
move x trial rate against 4 issue slots per SM per cycle) is the one the line reports.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_profile_figures_parse():
    import bench
    traffic = bench.traffic_from_profiles()
    per_move = bench.profile_figure("warp_instructions_per_move")
    assert traffic is not None and 1e8 < traffic < 1e10, traffic
    assert per_move is not None and 1e3 < per_move < 1e5, per_move


def test_issue_rate_arithmetic():
    import bench
    per_move = bench.profile_figure("warp_instructions_per_move")
    r = bench.issue_rate(50e6, 2000.0, 152)
    assert r["peak"] == pytest.approx(4 * 152 * 2000e6 / 1e9)
    assert r["achieved"] == pytest.approx(per_move * 50e6 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert bench.issue_rate(50e6, None, 152) is None
