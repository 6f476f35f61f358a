"""Centroid calibration and reference capture on the GPU against the oracle
running the same tilt ramps one frame at a time."""
import numpy as np
import pytest

from dasp_gb300.calibration import calibrate_shs_unique, calibration_steps, take_reference
from oracle.shwfs_oracle import CALDATA
from tests.wfs_cases import Case

pytestmark = pytest.mark.gpu


def _oracle_table(c, steps, frac):
    orc = c.oracle("f32")
    s = calibration_steps(steps, frac)
    W = c.W
    data = np.zeros((2, c.nsubx, c.nsubx, steps), np.float32)
    for k in range(steps):
        for ax in range(2):
            ramp = -np.arange(W) * s[k]
            ph = np.ascontiguousarray(np.broadcast_to(ramp if ax == 0 else ramp[:, None], (W, W)), np.float32)
            cents, _ = c.oracle_run(orc, phs=ph)
            data[ax, :, :, k] = cents.reshape(c.nsubx, c.nsubx, 2)[..., ax]
    return data, s


def test_calibration_table_matches_oracle_and_applies():
    c = Case(nsubx=8, p=8, N=16, psf="gauss")
    eng = c.engine()
    res = calibrate_shs_unique(eng, 12, 0.8, apply=False)
    ref, s = _oracle_table(c, 12, 0.8)
    lit = c.lit().reshape(8, 8)
    np.testing.assert_array_equal(res["steps"], s)
    assert np.abs(res["data"][:, lit] - ref[:, lit]).max() < 1e-5
    # apply: a tilted frame through the engine and the oracle with the table
    eng2 = c.engine()
    calibrate_shs_unique(eng2, 12, 0.8, apply=True)
    orc = c.oracle("f32")
    orc.update(CALDATA, (res["data"], res["bounds"], res["steps"]))
    ph = np.ascontiguousarray(np.broadcast_to(-np.arange(c.W) * np.float32(0.3), (c.W, c.W)), np.float32)
    c.phs[...] = ph
    eng2.run(0)
    oc, _ = c.oracle_run(orc, phs=ph)
    got = c.cents.reshape(-1, 2)[c.lit()]
    assert np.abs(got - oc.reshape(-1, 2)[c.lit()]).max() < 1e-4
    eng.free()
    eng2.free()


def test_take_reference_zeroes_flat_centroids():
    c = Case(nsubx=8, p=8, N=16, psf="gauss")
    eng = c.engine()
    ref = take_reference(eng)
    assert np.abs(ref).max() > 0  # the spot is not centred on the window by itself
    eng.run(1)
    assert np.abs(c.cents).max() < 1e-6
    eng.free()
