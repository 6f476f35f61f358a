"""Calibration table post-processing (util/centroid.py:1206-1250) on the host."""
import numpy as np

from dasp_gb300.calibration import bounds_and_force, calibration_steps


def test_calibration_steps_match_the_reference_formula():
    s = calibration_steps(8, 0.5)
    ref = (np.arange(8) - 4 + 0.5) / (4 - 0.5) * np.pi * 0.5
    np.testing.assert_allclose(s, ref.astype(np.float32))
    assert s.dtype == np.float32 and s[0] == -s[-1]


def test_bounds_and_forcing():
    d = np.zeros((2, 1, 2, 6), np.float32)
    d[0, 0, 0] = [0.0, 1.0, 3.0, 2.5, 4.0, 5.0]   # one dip inside the range
    d[0, 0, 1] = [2.0, 0.0, 1.0, 2.0, 3.0, 1.0]   # range 1..4, wraps after
    d[1, 0, 0] = [5.0, 4.0, 3.0, 2.0, 1.0, 0.0]   # decreasing: empty range
    d[1, 0, 1] = [0.0, 1.0, 2.0, 3.0, 4.0, 5.0]
    b, forced = bounds_and_force(d)
    assert b[0, 0, 0].tolist() == [0, 5] and b[0, 0, 1].tolist() == [1, 4]
    assert b[1, 0, 0].tolist() == [5, 0] and b[1, 0, 1].tolist() == [0, 5]
    # k = 2 > k + 1: replaced by the mean of its neighbours 1.0 and 2.5
    assert d[0, 0, 0, 2] == np.float32(1.75) and forced == 1
    assert d[0, 0, 1].tolist() == [2.0, 0.0, 1.0, 2.0, 3.0, 1.0]
