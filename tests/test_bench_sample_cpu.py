"""The benchmark's CPU sample (bench.cpu_sample): the pixels the CPU baseline
traces and whose oracle counters give the algorithmic bytes per ray of the
roofline.  The sample must spread over every view evenly at any size -- a
whole-number stride cut to k pixels keeps only the top rows, and the counters
then drift with the sample's size -- and be every pixel when it is complete."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

VIEWS = [(1000, 700, None, None), (333, 257, None, None), (1, 1, None, None)]
TOTAL = sum(w * h for w, h, _, _ in VIEWS)


def test_sample_spreads_over_every_row():
    for n in (100, 5000, TOTAL // 2, int(TOTAL * 0.9), TOTAL - 1):
        sample = bench.cpu_sample(VIEWS, n)
        assert [vi for vi, _ in sample] == [0, 1, 2]
        assert abs(sum(p.size for _, p in sample) - n) <= len(VIEWS)
        for vi, pix in sample:
            w, h = VIEWS[vi][:2]
            assert pix.dtype == np.uint32 and pix.max() < w * h
            assert np.unique(pix).size == pix.size
            if h > 100 and pix.size > 1000:
                rows = pix // w
                assert rows.max() >= h - 2                      # reaches the bottom rows
                assert abs(rows.mean() / (h - 1) - 0.5) < 0.01  # centred


def test_full_sample_is_every_pixel():
    for vi, pix in bench.cpu_sample(VIEWS, TOTAL):
        w, h = VIEWS[vi][:2]
        assert np.array_equal(pix, np.arange(w * h, dtype=np.uint32))
