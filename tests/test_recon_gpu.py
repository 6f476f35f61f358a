"""Reconstructor step (tomoRecon's decay + MVM) on the device against numpy."""
import numpy as np
import pytest
import torch

from dasp_gb300.recon import Reconstructor

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ncents,vec_gain", [(1000, True), (1001, False)])
def test_mvm_update_matches_numpy(ncents, vec_gain):
    rng = np.random.default_rng(ncents)
    nacts = 300
    R = rng.standard_normal((nacts, ncents)).astype(np.float32)
    gains = rng.uniform(0.2, 0.6, nacts).astype(np.float32) if vec_gain else 0.4
    decay = 0.99 if vec_gain else rng.uniform(0.9, 1.0, nacts).astype(np.float32)
    rec = Reconstructor(R, gains, decay)
    act = np.zeros(nacts)
    for k in range(3):
        x = rng.standard_normal(ncents).astype(np.float32)
        got = rec.step(torch.from_numpy(x).cuda()).cpu().numpy()
        act = np.asarray(decay, np.float64) * act - np.asarray(gains, np.float64) * (R.astype(np.float64) @ x)
        np.testing.assert_allclose(got, act, rtol=1e-4, atol=1e-4 * np.abs(act).max())


def test_engine_centroids_feed_the_reconstructor():
    from tests.wfs_cases import Case
    c = Case(nsubx=8, p=8, N=16)
    eng = c.engine()
    dc = torch.zeros(c.nsubaps * 2, device="cuda")
    db = torch.zeros((c.nsubaps, c.m, c.m), device="cuda")
    ph = torch.from_numpy(c.phs).cuda()
    eng.set_io(phs=ph, cents=dc, bimg=db)
    eng.run(0)
    R = np.random.default_rng(1).standard_normal((40, c.nsubaps * 2)).astype(np.float32)
    rec = Reconstructor(R, 0.5, 1.0)
    got = rec.step(dc).cpu().numpy()
    ref = -0.5 * (R.astype(np.float64) @ dc.cpu().numpy().astype(np.float64))
    np.testing.assert_allclose(got, ref, rtol=1e-4, atol=1e-5 * np.abs(ref).max())
    eng.free()
