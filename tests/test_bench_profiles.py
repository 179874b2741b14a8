"""bench.py takes the walk's per-launch DRAM traffic from the committed ncu
summary (profiles/k_walk_ncu.md), scaled by piled bases: every benchmarked
workload must find its figures there."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_walk_traffic_for_every_workload():
    for name in ("bacterial-5Mb-100x", "draft-3000-contigs-40x", "eukaryotic-120Mb-repeats", "small-50kb"):
        per_base = bench.roofline_traffic(name, 1_000_000) / 1_000_000
        # DRAM bytes per piled base: above the reads' own bytes (~1.5 B), below a re-read of everything
        assert 1.5 < per_base < 6.0, (name, per_base)


def test_workload_tags_take_precedence_and_scale_linearly():
    a = bench.roofline_traffic("draft-3000-contigs-40x", 10_000)
    b = bench.roofline_traffic("draft-3000-contigs-40x", 20_000)
    assert abs(b - 2 * a) < 1e-6 * b
    assert a != bench.roofline_traffic("bacterial-5Mb-100x", 10_000)  # its own 5% capture, not the untagged one
