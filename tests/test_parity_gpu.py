"""CUDA engine vs the oracle on identical seeded inputs, through the C ABI
(dasp_gb300.centcmod -> libshwfs.so).

Tolerances: noiseless centroids within 1e-5 px of the float32 oracle (the
reference's own arithmetic) and within 1e-3 px of the float64 oracle; images
within 1e-4 of the frame's peak pixel.  Noisy frames: reference-stream mode
agrees pixel for pixel except where a float transcendental differs in the
last bit; counter mode by moments.
"""
import numpy as np
import pytest

from tests.wfs_cases import Case

pytestmark = pytest.mark.gpu

CENT_TOL = 1e-5
IMG_RTOL = 1e-4


def compare(c, eng_cents, eng_bimg, orc_cents, orc_bimg, cent_tol=CENT_TOL, img_rtol=IMG_RTOL, lit_only=False):
    ec = eng_cents.reshape(-1, 2)
    oc = orc_cents.reshape(-1, 2)
    eb = eng_bimg.reshape(c.nsubaps, -1)
    ob = orc_bimg.reshape(c.nsubaps, -1)
    if lit_only:
        sel = c.lit()
        ec, oc, eb, ob = ec[sel], oc[sel], eb[sel], ob[sel]
    peak = max(float(np.abs(ob).max()), 1e-30)
    assert np.abs(eb - ob).max() <= img_rtol * peak, "image mismatch %g (peak %g)" % (np.abs(eb - ob).max(), peak)
    assert np.abs(ec - oc).max() <= cent_tol, "centroid mismatch %g px" % np.abs(ec - oc).max()


def run_both(c, nframes=1, mode="f32", cent_tol=CENT_TOL, img_rtol=IMG_RTOL, phases=None):
    eng = c.engine()
    orc = c.oracle(mode)
    oc = np.zeros(c.nsubaps * 2, np.float32)
    ob = np.zeros((c.nsubaps, c.m, c.m), np.float32)
    for f in range(nframes):
        ph = c.phs if phases is None else phases[f]
        if phases is not None:
            c.phs[...] = ph
        eng.run(c.params["calsource"])
        c.oracle_run(orc, ph, oc, ob)
        compare(c, c.cents, c.bimg, oc, ob, cent_tol, img_rtol)
    eng.free()
    return oc, ob


def test_scao_8x8_noiseless():
    c = Case(nsubx=8, p=8, N=16, C=16, m=8, sig=1e4)
    phases = [c.new_phase(s) for s in range(5)]
    run_both(c, 5, phases=phases)


def test_scao_8x8_vs_fp64_oracle():
    c = Case(nsubx=8, p=8, N=16, C=16, m=8, sig=1e4)
    run_both(c, mode="f64", cent_tol=1e-4)


def test_elt_74x74_psf_sky_floor_noiseless():
    c = Case(nsubx=74, p=10, N=20, C=20, m=10, obs=0.28, Dtel=39.0, r0=0.157, L0=25.0, wavelength=589.0,
             psf="gauss", sig=500.0, skybrightness=10.0, noiseFloor=6.0)
    run_both(c)
    c2 = Case(nsubx=74, p=10, N=20, C=20, m=10, obs=0.28, Dtel=39.0, r0=0.157, L0=25.0, wavelength=589.0,
              psf="gauss", sig=500.0)
    run_both(c2, mode="f64", cent_tol=1e-3)


@pytest.mark.parametrize("N,C,m", [(20, 20, 8), (20, 16, 8), (16, 16, 6), (24, 24, 12), (32, 32, 16)])
def test_binning_and_crop_variants(N, C, m):
    c = Case(nsubx=10, p=N // 2, N=N, C=C, m=m, sig=3e3)
    run_both(c)


@pytest.mark.parametrize("N,psf,P,preBin", [(16, "gauss", 32, 1), (20, "gauss", 40, 1), (32, "gauss", 16, 2),
                                             (20, "gauss", 20, 1), (16, "gauss", 16, 1)])
def test_psf_pad_and_prebin(N, psf, P, preBin):
    C = min(P, N) if preBin == 1 else P
    c = Case(nsubx=8, p=N // 2, N=N, C=C, m=C // 2, psf=psf, psfsize=P, sig=2e3, preBinningFactor=preBin)
    run_both(c)


def test_per_subap_psfs():
    c = Case(nsubx=12, p=8, N=16, C=16, m=8, psf="gauss4d", sig=1e3)
    run_both(c)


@pytest.mark.parametrize("N", [8, 10, 12, 15, 25, 30, 40, 48, 50, 60, 64])
def test_fft_sizes(N):
    # With large windows the reference's own sequential float32 sums drift from
    # exact arithmetic by more than 1e-5 px; the engine must agree with the
    # float32 oracle to 1e-5 px beyond that drift (measured against float64).
    c = Case(nsubx=6, p=N // 2, N=N, C=N, m=N // 2 if N % 2 == 0 else N, sig=1e3)
    eng = c.engine()
    eng.run(0)
    oc32, ob32 = c.oracle_run(c.oracle("f32"))
    oc64, _ = c.oracle_run(c.oracle("f64"))
    compare(c, c.cents, c.bimg, oc32, ob32, cent_tol=1.0)
    drift = np.abs(oc32 - oc64)
    assert np.all(np.abs(c.cents - oc32) <= CENT_TOL + drift)
    assert np.abs(c.cents - oc64).max() <= 1e-4
    eng.free()


def test_phase_plus_amplitude():
    c = Case(nsubx=8, p=8, N=16, sig=1e4, amp=True)
    run_both(c)


def test_sig_and_sky_arrays():
    rng = np.random.default_rng(3)
    sig = (1e3 * (1 + rng.random(64))).astype(np.float32)
    sky = (5 * rng.random((64, 8, 8))).astype(np.float32)
    c = Case(nsubx=8, p=8, N=16, sig=sig, skybrightness=sky, noiseFloor=2.0)
    run_both(c)


def test_threshold_type1_and_readbg():
    c = Case(nsubx=8, p=8, N=16, sig=1e4, readbg=3.0, noiseFloor=25.0, threshType=1)
    run_both(c, cent_tol=1e-4)


@pytest.mark.parametrize("ub", [5, -5, 40])
def test_brightest_pixels(ub):
    c = Case(nsubx=8, p=8, N=16, sig=1e4, useBrightest=ub)
    run_both(c)


def test_brightest_pixels_array():
    ub = np.arange(64, dtype=np.int32) % 7 - 3
    c = Case(nsubx=8, p=8, N=16, sig=1e4, useBrightest=ub)
    run_both(c)


@pytest.mark.parametrize("pw", [2.0, 1.5, 0.0])
def test_pixel_power(pw):
    c = Case(nsubx=8, p=8, N=16, sig=1e3, pxlPower=pw)
    run_both(c, img_rtol=3e-4)


def test_centroid_weights():
    w2 = np.exp(-((np.arange(8) - 3.5) ** 2)[:, None] / 8 - ((np.arange(8) - 3.5) ** 2)[None, :] / 8).astype(np.float32)
    run_both(Case(nsubx=8, p=8, N=16, sig=1e4, centWeight=w2))
    w4 = np.ascontiguousarray(np.broadcast_to(w2, (8, 8, 8, 8)) * np.linspace(0.5, 1.5, 64).reshape(8, 8, 1, 1),
                              dtype=np.float32)
    run_both(Case(nsubx=8, p=8, N=16, sig=1e4, centWeight=w4))


def test_smaller_centroid_window():
    run_both(Case(nsubx=8, p=8, N=16, sig=1e4, ncen=4))


@pytest.mark.parametrize("fit", [3, 5, -1])
def test_parabolic_fit(fit):
    run_both(Case(nsubx=8, p=8, N=16, sig=1e4, parabolicFit=fit), cent_tol=1e-4)


def test_gaussian_fit():
    run_both(Case(nsubx=8, p=8, N=16, sig=1e4, gaussianFitVals=(1.0, 0.0)), cent_tol=1e-4)


def test_optical_binning():
    run_both(Case(nsubx=8, p=8, N=16, sig=1e4, opticalBinning=1), cent_tol=1e-4)


def test_reference_and_calibration_flow():
    # takeReference (util/centroid.py:1536-1570): flat phase, cal source,
    # copy the centroids back in as REFCENTS; then polynomial and
    # interpolation calibration (CALCOEFF / CALDATA)
    c = Case(nsubx=8, p=8, N=16, sig=1e4, readbg=1.0, noiseFloor=1.0)
    eng = c.engine()
    orc = c.oracle()
    flat = np.zeros_like(c.phs)
    saved = c.phs.copy()
    c.phs[...] = flat
    eng.run(1)
    orc.update(1, 1)
    oc, ob = c.oracle_run(orc, flat)
    compare(c, c.cents, c.bimg, oc, ob)
    ref = c.cents.copy()
    eng.update(18, ref)
    orc.update(18, ref)
    c.phs[...] = saved
    eng.run(0)
    orc.update(1, 0)
    oc, ob = c.oracle_run(orc)
    compare(c, c.cents, c.bimg, oc, ob)
    coeff = np.zeros((8, 8, 2, 3), np.float32)
    coeff[..., 1] = 1.1
    coeff[..., 2] = 0.05
    eng.update(19, coeff)
    orc.update(19, coeff)
    eng.run(0)
    oc, ob = c.oracle_run(orc)
    compare(c, c.cents, c.bimg, oc, ob)
    eng.update(19, None)
    orc.update(19, None)
    steps = np.linspace(-2, 2, 9).astype(np.float32)
    cal = np.ascontiguousarray(np.broadcast_to(steps * 0.9, (2, 8, 8, 9)), dtype=np.float32)
    bounds = np.zeros((2, 8, 8, 2), np.int32)
    bounds[..., 1] = 8
    eng.update(17, (cal, bounds, steps))
    orc.update(17, (cal, bounds, steps))
    eng.run(0)
    oc, ob = c.oracle_run(orc)
    compare(c, c.cents, c.bimg, oc, ob)
    eng.free()


def test_integration_and_latency():
    c = Case(nsubx=8, p=8, N=16, sig=1e4, nintegrations=3, nlatency=1)
    eng = c.engine()
    orc = c.oracle()
    oc = np.full(128, 5.0, np.float32)
    ob = np.zeros((64, 8, 8), np.float32)
    c.cents[...] = 5.0
    for f in range(8):
        ph = c.new_phase(f)
        c.phs[...] = ph
        eng.run(0)
        c.oracle_run(orc, ph, oc, ob)
        compare(c, c.cents, c.bimg, oc, ob)
        assert eng.info()["cur_integ"] == orc.curInteg


def test_update_codes_follow_oracle():
    c = Case(nsubx=8, p=8, N=16, sig=1e4)
    eng = c.engine()
    orc = c.oracle()
    for code, val in ((2, 5e3), (8, 3.0), (7, 2.0), (6, 1.0), (4, 6), (9, 2.0), (20, 10),
                      (10, np.ascontiguousarray(np.pad(np.ones((4, 4), np.float32), 6)))):
        eng.update(code, val)
        orc.update(code, val)
        eng.run(0)
        oc, ob = c.oracle_run(orc)
        compare(c, c.cents, c.bimg, oc, ob, cent_tol=2e-5)
    eng.free()


def test_unlit_image_only_gets_noise_and_no_cents():
    c = Case(nsubx=8, p=8, N=16, sig=1e4, imageOnly=1, readnoise=2.0, readbg=5.0)
    eng = c.engine()
    c.cents[...] = 7.0
    eng.run(0)
    assert np.all(c.cents == 7.0)
    unlit = ~c.lit()
    b = c.bimg.reshape(64, -1)
    assert b[unlit].std() > 1.0 and abs(b[unlit].mean() - 5.0) < 0.5
    eng.free()


def test_reference_stream_noise_matches_oracle():
    """Reference-stream noise on images the engine forms itself: its
    pre-noise means differ from the oracle's float restatement in the last
    bits, and a mean that moves across a step of the Poisson inversion (or
    the PTRS acceptance test) changes that pixel's draw and, through the
    shared PCG32 stream, the later draws of its worker thread.  So a small
    share of pixels may differ here; the exact reproduction -- every pixel,
    centroids within 1e-5 px -- is tested on the reference module's own
    pre-noise images (test_prenoise_gpu.py)."""
    c = Case(nsubx=16, p=8, N=16, sig=3e3, addPoisson=1, readnoise=3.0, skybrightness=10.0, noiseFloor=6.0,
             nthreads=5, seed=17)
    eng = c.engine()
    eng.set_noise_mode("reference")
    orc = c.oracle()
    oc = np.zeros(c.nsubaps * 2, np.float32)
    ob = np.zeros((c.nsubaps, c.m, c.m), np.float32)
    for f in range(3):
        eng.run(0)
        c.oracle_run(orc, None, oc, ob)
        eb = c.bimg.reshape(c.nsubaps, -1)
        same = np.mean(np.abs(eb - ob.reshape(c.nsubaps, -1)) <= 1e-3 * np.abs(ob.reshape(c.nsubaps, -1)) + 1e-3)
        assert same > 0.995, "only %.4f of pixels match the reference streams" % same
    eng.free()


def test_counter_noise_moments():
    # constant image: many frames of Poisson + read noise, no threshold
    c = Case(nsubx=8, p=8, N=16, sig=2e3, addPoisson=1, readnoise=2.0, readbg=0.0, noiseFloor=-1e9,
             threshType=1, seed=5)
    quiet = Case(nsubx=8, p=8, N=16, sig=2e3, noiseFloor=-1e9, threshType=1)
    clean = quiet.oracle_run(quiet.oracle())[1].reshape(64, -1)
    eng = c.engine()
    frames = []
    for _ in range(400):
        eng.run(0)
        frames.append(c.bimg.reshape(64, -1).copy())
    x = np.stack(frames)[:, c.lit()]
    lam = clean[c.lit()]
    sel = lam > 2
    mean_err = (x.mean(0) - lam)[sel] / np.sqrt((lam[sel] + 4.0) / x.shape[0])
    assert np.abs(mean_err).mean() < 1.2
    var_ratio = x.var(0)[sel] / (lam[sel] + 4.0)
    assert abs(np.median(var_ratio) - 1) < 0.05
    eng.free()


def test_calsource_disables_shot_and_read_noise():
    c = Case(nsubx=8, p=8, N=16, sig=2e3, addPoisson=1, readnoise=2.0, readbg=1.0, noiseFloor=1.0, calsource=1)
    run_both(c)


def test_batch_matches_single_frames():
    torch = pytest.importorskip("torch")
    c = Case(nsubx=16, p=8, N=16, psf="gauss", sig=2e3, skybrightness=2.0, noiseFloor=1.0)
    eng = c.engine()
    phases = np.stack([c.new_phase(s) for s in range(4)])
    singles = []
    for f in range(4):
        c.phs[...] = phases[f]
        eng.run(0)
        singles.append((c.cents.copy(), c.bimg.copy()))
    dp = torch.from_numpy(phases).cuda()
    dc = torch.zeros((4, c.nsubaps * 2), device="cuda")
    db = torch.zeros((4, c.nsubaps, c.m, c.m), device="cuda")
    eng.run_batch(dp, dc, db)
    torch.cuda.synchronize()
    for f in range(4):
        np.testing.assert_array_equal(dc[f].cpu().numpy(), singles[f][0])
        np.testing.assert_array_equal(db[f].cpu().numpy().reshape(c.bimg.shape), singles[f][1])
    eng.free()


def test_torch_device_arrays_in_place():
    torch = pytest.importorskip("torch")
    c = Case(nsubx=8, p=8, N=16, sig=1e4)
    oc, ob = c.oracle_run(c.oracle())
    dphs = torch.from_numpy(c.phs).cuda()
    dc = torch.zeros(128, device="cuda")
    db = torch.zeros((8, 8, 8, 8), device="cuda")
    eng = c.engine(phs=dphs, cents=dc, bimg=db)
    eng.run(0)
    torch.cuda.synchronize()
    compare(c, dc.cpu().numpy(), db.cpu().numpy(), oc, ob)
    eng.free()


# ---------------------------------------------------------------- image input (runSlope)

def _detector_image(c, rng, scale=50.0):
    img = (scale * rng.random((c.nsubx * c.m, c.nsubx * c.m)) ** 4).astype(np.float32)
    return np.ascontiguousarray(img)


@pytest.mark.parametrize("kw", [dict(), dict(useBrightest=6), dict(pxlPower=2.0), dict(calsource=1),
                                dict(ncen=6, threshType=1)])
def test_run_slope_2d_image(kw):
    rng = np.random.default_rng(21)
    c = Case(nsubx=8, p=8, N=16, sig=1e4, noiseFloor=5.0, **kw)
    img = _detector_image(c, rng)
    eng = c.engine(inputImage=img)
    orc = c.oracle()
    oc = np.zeros(128, np.float32)
    ob = np.zeros((64, 8, 8), np.float32)
    for f in range(2):
        img[...] = _detector_image(c, rng)
        eng.runSlope(c.params["calsource"])
        orc.run_slope(img, oc, ob)
        compare(c, c.cents, c.bimg, oc, ob)
    eng.free()


def test_run_slope_4d_image_without_phase():
    rng = np.random.default_rng(5)
    c = Case(nsubx=8, p=8, N=16, sig=1e4, noiseFloor=2.0)
    img4 = np.ascontiguousarray((30 * rng.random((8, 8, 8, 8)) ** 3).astype(np.float32))
    eng = c.engine(inputImage=img4, no_phase=True)
    eng.runSlope(0)
    oc = np.zeros(128, np.float32)
    ob = np.zeros((64, 8, 8), np.float32)
    c.oracle().run_slope(img4, oc, ob)
    compare(c, c.cents, c.bimg, oc, ob)
    with pytest.raises(Exception):
        eng.run(0)  # no phase bound
    eng.free()


def test_run_slope_subap_locations_smaller_windows():
    # 6x6 windows inside 8x8 images: pixels outside the window keep their old
    # bimg values and the threshold covers the first 36 pixels in storage order
    rng = np.random.default_rng(8)
    c = Case(nsubx=8, p=8, N=16, sig=1e4, noiseFloor=3.0)
    img = _detector_image(c, rng)
    loc = np.zeros((64, 4), np.int32)
    for i in range(64):
        r0, c0 = (i // 8) * 8 + 1, (i % 8) * 8 + 1
        loc[i] = (r0, r0 + 6, c0, c0 + 6)
    bimg0 = np.full((8, 8, 8, 8), 2.5, np.float32)
    eng = c.engine(bimg=bimg0.copy(), inputImage=img, subapLocation=loc)
    eng.runSlope(0)
    oc = np.zeros(128, np.float32)
    ob = bimg0.reshape(64, 8, 8).copy()
    c.oracle().run_slope(img, oc, ob, subapLocation=loc)
    compare(c, c.cents, c.bimg, oc, ob)
    eng.free()


def test_run_slope_image_only_noise_reference_streams():
    rng = np.random.default_rng(9)
    c = Case(nsubx=8, p=8, N=16, sig=1e4, imageOnly=1, readnoise=2.0, readbg=4.0, noiseFloor=1.0, nthreads=3)
    img = _detector_image(c, rng)
    eng = c.engine(inputImage=img)
    eng.set_noise_mode("reference")
    eng.runSlope(0)
    oc = np.zeros(128, np.float32)
    ob = np.zeros((64, 8, 8), np.float32)
    c.oracle().run_slope(img, oc, ob)
    eb = c.bimg.reshape(64, -1)
    same = np.mean(np.abs(eb - ob.reshape(64, -1)) <= 1e-5 * np.abs(ob.reshape(64, -1)) + 1e-5)
    assert same > 0.995
    eng.free()


# ---------------------------------------------------------------- borrowed-output semantics

def test_host_outputs_only_written_where_the_reference_writes():
    c = Case(nsubx=8, p=8, N=16, sig=1e4)
    eng = c.engine()
    unlit = ~c.lit()
    c.bimg.reshape(64, -1)[unlit] = 4.0   # caller data in subapertures the engine never images
    eng.run(0)
    assert np.all(c.bimg.reshape(64, -1)[unlit] == 4.0)
    assert np.all(c.cents.reshape(-1, 2)[unlit] == 0.0)
    eng.free()
    c2 = Case(nsubx=8, p=8, N=16, sig=1e4, nintegrations=2)
    eng2 = c2.engine()
    c2.cents[...] = 1.5
    eng2.run(0)  # first sub-exposure: nothing is read out
    assert np.all(c2.cents == 1.5)
    eng2.free()
