"""Physical integration (SHWFS_INTEG_PHYSICAL, centcmod.set_integration_mode):
sub-exposures averaged on the device, noise and centroiding once per readout.

The reference zeroes its image accumulator on every sub-exposure
(cmod/src/centmodule.c:478; the engine's default "compat" mode keeps that).
The physical mode is checked against the oracle's restatement of the same
rule (every exposed frame of cmod/src/centmodule.c:1774-1788 contributes; the
readout image is the mean), noiseless, within 1e-5 px and 1e-4 of the peak
pixel for the FP32 form and 1e-3 px for the FP16 tensor-core form.
"""
import numpy as np
import pytest

from tests.wfs_cases import Case

pytestmark = pytest.mark.gpu


def _run(c, form, nframes, cent_tol, img_rtol, mode="f32"):
    eng = c.engine()
    eng.set_form(form)
    eng.set_integration_mode("physical")
    orc = c.oracle(mode)
    orc.update(104, 1)
    c.cents[...] = 3.0
    oc = np.full(c.nsubaps * 2, 3.0, np.float32)
    ob = np.zeros((c.nsubaps, c.m, c.m), np.float32)
    readouts = 0
    for f in range(nframes):
        ph = c.new_phase(20 + f)
        c.phs[...] = ph
        ro = orc.additive() in (2, -1)
        eng.run(0)
        c.oracle_run(orc, ph, oc, ob)
        lit = c.lit()
        ec, rc = c.cents.reshape(-1, 2)[lit], oc.reshape(-1, 2)[lit]
        assert np.abs(ec - rc).max() <= cent_tol, (f, np.abs(ec - rc).max())
        if ro:
            readouts += 1
            eb, rb = c.bimg.reshape(c.nsubaps, -1)[lit], ob.reshape(c.nsubaps, -1)[lit]
            assert np.abs(eb - rb).max() <= img_rtol * np.abs(rb).max()
    eng.free()
    return readouts


@pytest.mark.parametrize("nint,nlat", [(3, 0), (3, 1), (2, 2)])
def test_physical_fp32_matches_oracle(nint, nlat):
    c = Case(nsubx=8, p=8, N=16, psf="gauss", sig=2e3, skybrightness=3.0, noiseFloor=1.0, nintegrations=nint,
             nlatency=nlat)
    assert _run(c, "fp32", 2 * (nint + nlat), 1e-5, 1e-4) == 2


def test_physical_fp16_vs_float64():
    c = Case(nsubx=16, p=10, N=20, C=20, m=10, psf="gauss", sig=500.0, skybrightness=10.0, nintegrations=4)
    assert _run(c, "fp16", 8, 1e-3, 5e-3, mode="f64") == 2


def test_physical_mean_differs_from_compat_and_equals_single_exposure():
    # nintegrations 1: physical and compat give the same noisy images (same
    # pre-noise images, same streams); the centroids agree to the rounding of
    # the two centroid kernels' summation orders
    c = Case(nsubx=8, p=8, N=16, sig=1e4, addPoisson=1, readnoise=2.0, noiseFloor=2.0, seed=4)
    e1 = c.engine()
    e1.run(0)
    a, ab = c.cents.copy(), c.bimg.copy()
    e1.free()
    e2 = c.engine()
    e2.set_integration_mode("physical")
    e2.run(0)
    lit = c.lit()
    np.testing.assert_array_equal(c.bimg.reshape(64, -1)[lit], ab.reshape(64, -1)[lit])
    assert np.abs(c.cents - a).max() <= 1e-5
    e2.free()
    # nintegrations 2: the image is the mean of the two sub-exposures
    c2 = Case(nsubx=8, p=8, N=16, sig=1e4, nintegrations=2)
    eng = c2.engine()
    eng.set_integration_mode("physical")
    p0, p1 = c2.new_phase(1), c2.new_phase(2)
    c2.phs[...] = p0
    eng.run(0)
    c2.phs[...] = p1
    eng.run(0)
    phys = c2.bimg.copy()
    eng.free()
    imgs = []
    for ph in (p0, p1):
        e = c2.engine()
        c2.phs[...] = ph
        e.update(21, 1)  # INTEGSTEPS 1: a single-exposure readout
        e.run(0)
        imgs.append(c2.bimg.copy())
        e.free()
    lit = c2.lit()
    mean = 0.5 * (imgs[0] + imgs[1])
    pb, mb = phys.reshape(64, -1)[lit], mean.reshape(64, -1)[lit]
    assert np.abs(pb - mb).max() <= 1e-5 * np.abs(mb).max()


def test_physical_serving_matches_engine():
    torch = pytest.importorskip("torch")
    from dasp_gb300.serving import WfsServer
    from tests.test_serving_gpu import _kw
    c = Case(nsubx=12, p=8, N=16, sig=2e3, addPoisson=1, readnoise=2.0, skybrightness=3.0, noiseFloor=1.0, seed=6,
             nintegrations=3)
    phases = [torch.from_numpy(np.ascontiguousarray(c.new_phase(40 + k), np.float32)).cuda() for k in range(6)]
    srv = WfsServer(4 << 30, max_inflight=4, integration="physical")
    sid = srv.add_system(form="fp16", **_kw(c))
    outs = [np.zeros(c.nsubaps * 2, np.float32) for _ in phases]
    for k, p in enumerate(phases):
        srv.submit(sid, p, out=outs[k])
    done = srv.drain(60)
    assert all(d["status"] == 0 for d in done)
    assert sum(d["readout"] for d in done) == 2
    srv.close()
    dphs = torch.zeros_like(phases[0])
    dc = torch.zeros(c.nsubaps * 2, device="cuda")
    db = torch.zeros((c.nsubaps, c.m, c.m), device="cuda")
    eng = c.engine(phs=dphs, cents=dc, bimg=db)
    eng.set_form("fp16")
    eng.set_integration_mode("physical")
    for k, p in enumerate(phases):
        dphs.copy_(p)
        eng.run(0)
        torch.cuda.synchronize()
        if k % 3 == 2:
            np.testing.assert_array_equal(dc.cpu().numpy(), outs[k])
    eng.free()
