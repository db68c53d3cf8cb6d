"""Host-side helpers of bench.py: the kernel launches a frame makes (the library's bin-size
choice mirrored), the bin size of a batch scene, and the committed ncu figures."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_launches_per_frame_follows_the_bin_size(bench):
    # 7 kernels with 16-pixel bins, 8 with 32-pixel bins (the quadrant split)
    assert bench.launches_per_frame(800, 600, 12) == 7            # cube: few triangles, 16-pixel
    assert bench.launches_per_frame(1920, 1080, 100_000) == 8     # soup: 32-pixel from 8192 tris
    assert bench.launches_per_frame(1920, 1080, 8191) == 7
    assert bench.launches_per_frame(3840, 2160, 12) == 8          # 16-pixel bins would exceed 16384
    assert bench.launches_per_frame(1920, 1080, 100_000, tile=16) == 7
    assert bench.launches_per_frame(3840, 2160, 100, tile=16) == 7  # asked for: two counting bands
    assert bench.launches_per_frame(16384, 16384, 100) == 8        # beyond one band either way: 32
    assert bench.launches_per_frame(256, 256, 100, tile=32) == 8


def test_batch_tile(bench):
    s4 = {"width": 512, "height": 512, "msaa": 4, "draws": [{"idx": [[0, 1, 2]] * 10}]}
    s1 = dict(s4, msaa=1)
    tuned = {"msaa1_tile": 8, "msaa4_tile": 32}
    assert bench.batch_tile(s4, tuned) == 32
    assert bench.batch_tile(s1, tuned) == 8
    assert bench.batch_tile(s4, {}) == 16  # untuned: the automatic choice for 10 triangles


def test_committed_profile(bench):
    assert bench.committed_profile(1) > 0 and bench.committed_profile(2) > 0
    assert 0.0 < bench.committed_profile(1, "issue_active") <= 1.0
    assert bench.committed_profile(0) is None and bench.committed_profile(0, "issue_active") is None


def test_sustained_rate_is_the_passing_prefix(bench):
    sweep = [{"offered_rate": r, "p99_ms": p} for r, p in
             [(1000, 1.0), (2000, 2.0), (4000, 40.0), (6000, 137.0), (8000, 8.0)]]
    assert bench.sustained_point(sweep, 50.0)["offered_rate"] == 4000  # 8000 passed by luck
    assert bench.sustained_point(sweep, 1.5)["offered_rate"] == 1000
    assert bench.sustained_point(sweep, 0.5) is None
    assert bench.sustained_point([], 50.0) is None
