"""interpolatePhase on the GPU (a phase array that is not nsubx*phasesize
square) against the oracle's float32 restatement."""
import numpy as np
import pytest
import torch

from dasp_gb300.screens import von_karman_screen
from oracle.shwfs_oracle import OUTPUTPHASEARR, interpolate_phase
from tests.wfs_cases import Case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nin", [50, 90, 64 + 13])
def test_interpolated_phase_matches_oracle(nin):
    c = Case(nsubx=8, p=8, N=16, psf="gauss")
    inp = np.ascontiguousarray(von_karman_screen(nin, 4.2, 0.15, 30.0, nin, 640.0))
    out = np.full((64, 64), -7.0, np.float32)
    eng = c.engine(phs=inp)
    eng.update(OUTPUTPHASEARR, out)
    eng.run(0)
    orc = c.oracle("f32")
    oout = np.full((64, 64), -7.0, np.float32)
    orc.update(OUTPUTPHASEARR, oout)
    oc, ob = c.oracle_run(orc, phs=inp)
    lit = c.lit()
    # the resampled phase is bit-identical (same float operations, same order)
    np.testing.assert_array_equal(out, oout)
    assert np.abs(c.cents.reshape(-1, 2)[lit] - oc.reshape(-1, 2)[lit]).max() < 1e-5
    eb = c.bimg.reshape(64, -1)[lit]
    obl = ob.reshape(64, -1)[lit]
    assert np.abs(eb - obl).max() / np.abs(obl).max() < 1e-4
    eng.free()


def test_interpolated_phase_device_output_and_batch():
    c = Case(nsubx=8, p=8, N=16)
    frames = [np.ascontiguousarray(von_karman_screen(50, 4.2, 0.15, 30.0, 20 + f, 640.0)) for f in range(3)]
    eng = c.engine(phs=frames[0].copy())
    dout = torch.full((64, 64), -7.0, device="cuda")
    eng.update(OUTPUTPHASEARR, dout)
    singles = []
    for fr in frames:
        eng.set_io(phs=fr.copy())
        eng.run(0)
        singles.append(c.cents.copy())
    ref = interpolate_phase(frames[-1], 8, 8)
    lit = c.lit().reshape(8, 8)
    got = dout.cpu().numpy()
    for sy in range(8):
        for sx in range(8):
            blk = (slice(sy * 8, sy * 8 + 8), slice(sx * 8, sx * 8 + 8))
            if lit[sy, sx]:
                np.testing.assert_array_equal(got[blk], ref[blk])
            else:
                assert (got[blk] == -7.0).all()
    # three interpolated frames in one launch equal the three single runs
    ph = torch.from_numpy(np.stack(frames)).cuda()
    dc = torch.zeros((3, 128), device="cuda")
    db = torch.zeros((3, 64, 8, 8), device="cuda")
    eng2 = c.engine(phs=frames[0].copy())
    eng2.run_batch(ph, dc, db)
    torch.cuda.synchronize()
    for f in range(3):
        np.testing.assert_array_equal(dc[f].cpu().numpy(), singles[f])
    eng.free()
    eng2.free()


def test_interpolated_phase_tensor_core_form():
    c = Case(nsubx=8, p=8, N=16)
    inp = np.ascontiguousarray(von_karman_screen(70, 4.2, 0.15, 30.0, 5, 640.0))
    eng = c.engine(phs=inp)
    eng.set_form("bf16x3")
    assert eng.info()["form_active"] == 2
    eng.run(0)
    oc, _ = c.oracle_run(c.oracle("f64"), phs=inp)
    lit = c.lit()
    assert np.abs(c.cents.reshape(-1, 2)[lit] - oc.reshape(-1, 2)[lit]).max() < 1e-4
    eng.free()
