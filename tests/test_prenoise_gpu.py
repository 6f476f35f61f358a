"""Noise injection through shwfs_run_prenoise (C ABI, dasp_gb300.centcmod):
one readout from caller-supplied pre-noise images, with the engine's noise
generators or with caller-drawn noise.

* Reference-stream noise on the reference module's own pre-noise images
  reproduces the reference module's noisy frames (oracle/_ref: the
  unmodified cmod/src/centmodule.c), pixel for pixel, centroids within
  1e-5 px.
* Injected draws: the engine's images equal the oracle's bit for bit for the
  same images and draws; centroids within 1e-5 px.
* Counter-stream noise on constant images has Poisson + read-noise moments.
"""
import numpy as np
import pytest

from oracle import ref_cent
from tests.wfs_cases import Case

pytestmark = pytest.mark.gpu

needs_ref = pytest.mark.skipif(not ref_cent.available(), reason="reference sources not available")


def _ref_lambda(c):
    quiet = dict(addPoisson=0, readnoise=0.0, readbg=0.0, noiseFloor=0.0, useBrightest=0, pxlPower=1.0)
    lam_c = np.zeros(c.nsubaps * 2, np.float32)
    lam_b = np.zeros((c.nsubx, c.nsubx, c.m, c.m), np.float32)
    keep = (getattr(c, "ref_cents", None), getattr(c, "ref_bimg", None))
    ref = c.reference(cents=lam_c, bimg=lam_b, **quiet)
    ref.run(0)
    ref.free()
    c.ref_cents, c.ref_bimg = keep
    return lam_b.reshape(c.nsubaps, c.m, c.m).copy()


@needs_ref
@pytest.mark.parametrize("kw", [dict(), dict(useBrightest=-20, threshType=1, noiseFloor=3.0),
                                dict(imageOnly=1, readbg=2.0)])
def test_reference_streams_reproduce_reference_module(kw):
    p = dict(nsubx=16, p=8, N=16, sig=3e3, addPoisson=1, readnoise=3.0, skybrightness=10.0, noiseFloor=6.0,
             nthreads=5, seed=17)
    p.update(kw)
    c = Case(**p)
    eng = c.engine()
    eng.set_noise_mode("reference")
    ref = c.reference()
    for f in range(3):
        if f:
            c.ref_phs[...] = c.new_phase(f)
        lam = _ref_lambda(c)
        ref.run(0)
        eng.run_prenoise(lam)
        if c.params.get("imageOnly"):
            np.testing.assert_array_equal(c.bimg, c.ref_bimg)
        else:
            lit = c.lit()
            np.testing.assert_array_equal(c.bimg.reshape(c.nsubaps, -1)[lit], c.ref_bimg.reshape(c.nsubaps, -1)[lit])
            assert np.abs(c.cents - c.ref_cents).max() <= 1e-5
    eng.free()
    ref.free()


@pytest.mark.parametrize("form", ["fp32", "fp16"])
def test_injected_draws_match_oracle_bit_for_bit(form):
    c = Case(nsubx=74, p=10, N=20, C=20, m=10, obs=0.28, Dtel=39.0, r0=0.157, L0=25.0, wavelength=589.0,
             psf="gauss", sig=500.0, addPoisson=1, readnoise=3.0, skybrightness=10.0, noiseFloor=6.0)
    orc = c.oracle()
    lit = np.nonzero(c.lit())[0]
    img, _, _ = orc.pre_noise_images(c.phs, lit)
    lam = np.zeros((c.nsubaps, c.m, c.m), np.float32)
    lam[lit] = img
    rng = np.random.default_rng(11)
    shot = rng.poisson(lam).astype(np.float32)
    readn = (3.0 * rng.standard_normal(lam.shape)).astype(np.float32)
    eng = c.engine()
    eng.set_form(form)
    oc = np.zeros(c.nsubaps * 2, np.float32)
    ob = np.zeros((c.nsubaps, c.m, c.m), np.float32)
    for f in range(2):
        eng.run_prenoise(lam, shot, readn)
        orc.run_prenoise(lam, oc, ob, shot=shot, readn=readn)
        np.testing.assert_array_equal(c.bimg.reshape(c.nsubaps, -1)[lit], ob.reshape(c.nsubaps, -1)[lit])
        assert np.abs(c.cents - oc).max() <= 1e-5
        shot = rng.poisson(lam).astype(np.float32)
        readn = (3.0 * rng.standard_normal(lam.shape)).astype(np.float32)
    eng.free()


def test_injected_draws_device_arrays_and_image_only():
    torch = pytest.importorskip("torch")
    c = Case(nsubx=8, p=8, N=16, sig=2e3, addPoisson=1, readnoise=2.0, readbg=4.0, noiseFloor=1.0, imageOnly=1)
    rng = np.random.default_rng(3)
    lam = (20 * rng.random((64, 8, 8))).astype(np.float32)
    shot = rng.poisson(lam).astype(np.float32)
    readn = (2.0 * rng.standard_normal(lam.shape)).astype(np.float32)
    eng = c.engine()
    eng.run_prenoise(torch.from_numpy(lam).cuda(), torch.from_numpy(shot).cuda(), torch.from_numpy(readn).cuda())
    oc = np.zeros(128, np.float32)
    ob = np.zeros((64, 8, 8), np.float32)
    c.oracle().run_prenoise(lam, oc, ob, shot=shot, readn=readn)
    np.testing.assert_array_equal(c.bimg.reshape(64, 8, 8), ob)
    eng.free()


def test_counter_streams_on_given_images_have_poisson_moments():
    c = Case(nsubx=8, p=8, N=16, sig=2e3, addPoisson=1, readnoise=2.0, noiseFloor=-1e9, threshType=1, seed=9)
    lam = np.full((64, 8, 8), 7.5, np.float32)
    eng = c.engine()
    frames = []
    for _ in range(300):
        eng.run_prenoise(lam)
        frames.append(c.bimg.reshape(64, -1)[c.lit()].copy())
    x = np.stack(frames)
    assert abs(x.mean() - 7.5) < 0.05
    assert abs(x.var() / (7.5 + 4.0) - 1) < 0.03
    eng.free()


def test_argument_checks():
    c = Case(nsubx=8, p=8, N=16, sig=2e3, addPoisson=1, readnoise=2.0)
    eng = c.engine()
    lam = np.ones((64, 8, 8), np.float32)
    with pytest.raises(ValueError):
        eng.run_prenoise(lam[:32])
    with pytest.raises(ValueError):
        eng.run_prenoise(lam, shot=lam)  # read noise is drawn: readn is required too
    eng.free()
    c2 = Case(nsubx=8, p=8, N=16, sig=2e3, opticalBinning=1)
    eng2 = c2.engine()
    with pytest.raises(NotImplementedError):
        eng2.run_prenoise(lam)
    eng2.free()


@pytest.mark.parametrize("geom", [dict(nsubx=8, p=8, N=16), dict(nsubx=8, p=8, N=16, C=16, m=5),
                                  dict(nsubx=6, p=8, N=24, C=24, m=6)])
@pytest.mark.parametrize("sig", [2e3, 1e6])
@pytest.mark.parametrize("extra", [dict(), dict(parabolicFit=1)])
def test_counter_draws_identical_in_every_noise_kernel(sig, extra, geom):
    """The fused FP32 kernel (noise drawn on its own images), the warp noise
    kernel (run_prenoise, window CoG) and the general noise kernel
    (run_prenoise with a parabolic fit) draw each quad of pixels from one
    stream: on equal pre-noise images their noisy images are equal bit for
    bit.  sig 1e6 puts most pixels above lambda 64, so the rejection
    sampler's queue fills and drains inside a chunk; nimg 5 (25 pixels)
    ends every image on a partial quad, nimg 6 (36) on whole quads that
    straddle image rows."""
    kw = dict(sig=sig, addPoisson=1, readnoise=2.0, readbg=1.5, noiseFloor=-1e9, threshType=1, seed=9)
    kw.update(geom)
    kw.update(extra)
    quiet = Case(**dict(kw, addPoisson=0, readnoise=0.0, readbg=0.0))
    n, m = quiet.nsubaps, quiet.m
    qe = quiet.engine()
    qe.set_form("fp32")
    qe.run(0)
    lam = quiet.bimg.reshape(n, m, m).copy()
    qe.free()
    lit = quiet.lit()
    if sig > 1e5:
        assert np.mean(lam[lit] >= 64) > 0.5
    fused = Case(**kw)
    fe = fused.engine()
    fe.set_form("fp32")
    post = Case(**kw)
    pe = post.engine()
    for f in range(3):
        fe.run(0)
        pe.run_prenoise(lam)
        a = fused.bimg.reshape(n, -1)[lit]
        b = post.bimg.reshape(n, -1)[lit]
        np.testing.assert_array_equal(a, b, err_msg="frame %d" % f)
        assert np.abs(fused.cents - post.cents).max() <= 1e-4
    fe.free()
    pe.free()
