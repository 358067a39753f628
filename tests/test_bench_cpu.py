"""CPU: the bench's clock record — the median SM clock, the maximum and the
throttle reasons seen while the timed region ran, from nvidia-smi's
per-20-ms samples (bench.py Clocks.summary)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

ROWS = """0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active
1, 1200, 2070, 300.0, 0x0, Active, Not Active, Not Active, Not Active
0, 1980, 2070, 1390.5, 0x4, Not Active, Not Active, Not Active, Active
0, [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A]
0, 2055, 2070, 1200.0, 0x0, Not Active, Not Active, Not Active, Not Active
"""


def test_clock_summary(tmp_path):
    path = tmp_path / "clocks.csv"
    path.write_text(ROWS)
    c = bench.Clocks(str(path))
    s = c.summary(0)
    assert s == {"sm_mhz": 2055.0, "sm_max_mhz": 2070.0,
                 "reasons": ["sw_power_cap"], "samples": 3,
                 "samples_in_region": 3}
    s1 = c.summary(1)
    assert s1["sm_mhz"] == 1200.0 and s1["reasons"] == ["hw_slowdown"]
    # the first two lines written before the timed region began
    c.skip = 2
    s2 = c.summary(0)
    assert s2["samples"] == 2 and s2["samples_in_region"] == 2
    assert s2["sm_mhz"] == (1980.0 + 2055.0) / 2
    # none inside the region: the earlier samples, flagged as such
    c.skip = 5
    s3 = c.summary(0)
    assert s3["samples"] == 3 and s3["samples_in_region"] == 0


def test_clock_summary_without_samples(tmp_path):
    assert bench.Clocks(str(tmp_path / "missing.csv")).summary() is None
    path = tmp_path / "na.csv"
    path.write_text("0, [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A]\n")
    assert bench.Clocks(str(path)).summary() is None


def test_rank_seeds_are_disjoint():
    seen = set()
    for rank in range(4):
        s = bench.rank_seeds(2100, rank, 8)
        assert len(s) == 8 and not (seen & set(s))
        seen |= set(s)
