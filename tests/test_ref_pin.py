"""Pin the oracle to the reference itself: the unmodified cmod/src/centmodule.c,
built by oracle/build_ref.py against FFT/GSL shims, run beside
oracle/shwfs_oracle.py (float32 mode) on the same inputs.

Tolerances: centroids within 1e-5 px and images within 1e-4 of the frame's
peak pixel (the two differ only by the rounding of their transforms, which
evaluate the same DFTs in a different order).  Noisy frames use the
reference's own PCG32 / rk_poisson code and the shim's MT19937 gaussian; on
inputs whose pre-noise images agree bit for bit the noisy images must too.
These tests need no GPU; they are skipped where neither the reference tree
nor a staged copy of its sources is present.
"""
import numpy as np
import pytest

from oracle import ref_cent
from tests.wfs_cases import Case

pytestmark = pytest.mark.skipif(not ref_cent.available(), reason="reference sources not available")

CENT_TOL = 1e-5
IMG_RTOL = 1e-4


def compare(c, rc, rb, oc, ob, cent_tol=CENT_TOL, img_rtol=IMG_RTOL):
    rb = rb.reshape(c.nsubaps, -1)
    ob = ob.reshape(c.nsubaps, -1)
    peak = max(float(np.abs(ob).max()), 1e-30)
    di = float(np.abs(rb - ob).max())
    dc = float(np.abs(rc - oc).max())
    assert di <= img_rtol * peak, "image mismatch %g (peak %g)" % (di, peak)
    assert dc <= cent_tol, "centroid mismatch %g px" % dc
    return dc, di


def pin(c, nframes=1, cent_tol=CENT_TOL, img_rtol=IMG_RTOL, phases=None):
    ref = c.reference()
    orc = c.oracle("f32")
    oc = np.zeros(c.nsubaps * 2, np.float32)
    ob = np.zeros((c.nsubaps, c.m, c.m), np.float32)
    for f in range(nframes):
        if phases is not None:
            c.ref_phs[...] = phases[f]
        ref.run(c.params["calsource"])
        c.oracle_run(orc, c.ref_phs, oc, ob)
        compare(c, c.ref_cents, c.ref_bimg, oc, ob, cent_tol, img_rtol)
    ref.free()
    return oc, ob


def test_scao_8x8_noiseless_bit_identical():
    c = Case(nsubx=8, p=8, N=16, C=16, m=8, sig=1e4)
    phases = [c.new_phase(s) for s in range(4)]
    ref = c.reference()
    orc = c.oracle("f32")
    oc = np.zeros(128, np.float32)
    ob = np.zeros((64, 8, 8), np.float32)
    for ph in phases:
        c.ref_phs[...] = ph
        ref.run(0)
        c.oracle_run(orc, c.ref_phs, oc, ob)
        np.testing.assert_array_equal(c.ref_cents, oc)
        np.testing.assert_array_equal(c.ref_bimg.reshape(ob.shape), ob)
    ref.free()


def test_elt_74x74_psf_sky_floor_noiseless():
    c = Case(nsubx=74, p=10, N=20, C=20, m=10, obs=0.28, Dtel=39.0, r0=0.157, L0=25.0, wavelength=589.0,
             psf="gauss", sig=500.0, skybrightness=10.0, noiseFloor=6.0, nthreads=8)
    pin(c)


@pytest.mark.parametrize("N,C,m", [(20, 20, 8), (20, 16, 8), (24, 24, 12), (32, 32, 16)])
def test_binning_and_crop_variants(N, C, m):
    pin(Case(nsubx=10, p=N // 2, N=N, C=C, m=m, sig=3e3))


@pytest.mark.parametrize("N,P,preBin", [(16, 32, 1), (20, 40, 1), (32, 16, 2), (20, 20, 1)])
def test_psf_pad_and_prebin(N, P, preBin):
    C = min(P, N) if preBin == 1 else P
    pin(Case(nsubx=8, p=N // 2, N=N, C=C, m=C // 2, psf="gauss", psfsize=P, sig=2e3, preBinningFactor=preBin))


def test_per_subap_psfs():
    pin(Case(nsubx=12, p=8, N=16, C=16, m=8, psf="gauss4d", sig=1e3))


@pytest.mark.parametrize("N", [8, 12, 15, 30, 64])
def test_fft_sizes(N):
    # large windows: the two float32 CoG sums may differ by their own rounding
    pin(Case(nsubx=6, p=N // 2, N=N, C=N, m=N // 2 if N % 2 == 0 else N, sig=1e3), cent_tol=2e-5)


def test_phase_plus_amplitude():
    pin(Case(nsubx=8, p=8, N=16, sig=1e4, amp=True))


def test_sig_and_sky_arrays():
    rng = np.random.default_rng(3)
    sig = (1e3 * (1 + rng.random(64))).astype(np.float32)
    sky = (5 * rng.random((64, 8, 8))).astype(np.float32)
    pin(Case(nsubx=8, p=8, N=16, sig=sig, skybrightness=sky, noiseFloor=2.0))


def test_threshold_type1_and_readbg():
    pin(Case(nsubx=8, p=8, N=16, sig=1e4, readbg=3.0, noiseFloor=25.0, threshType=1), cent_tol=1e-4)


@pytest.mark.parametrize("ub", [5, -5, 40])
def test_brightest_pixels(ub):
    pin(Case(nsubx=8, p=8, N=16, sig=1e4, useBrightest=ub))


def test_brightest_pixels_array():
    pin(Case(nsubx=8, p=8, N=16, sig=1e4, useBrightest=np.arange(64, dtype=np.int32) % 7 - 3))


@pytest.mark.parametrize("pw", [2.0, 1.5])
def test_pixel_power(pw):
    pin(Case(nsubx=8, p=8, N=16, sig=1e3, pxlPower=pw), img_rtol=3e-4)


def test_centroid_weights_and_window():
    w2 = np.exp(-((np.arange(8) - 3.5) ** 2)[:, None] / 8 - ((np.arange(8) - 3.5) ** 2)[None, :] / 8).astype(np.float32)
    pin(Case(nsubx=8, p=8, N=16, sig=1e4, centWeight=w2))
    w4 = np.ascontiguousarray(np.broadcast_to(w2, (8, 8, 8, 8)) * np.linspace(0.5, 1.5, 64).reshape(8, 8, 1, 1),
                              dtype=np.float32)
    pin(Case(nsubx=8, p=8, N=16, sig=1e4, centWeight=w4))
    pin(Case(nsubx=8, p=8, N=16, sig=1e4, ncen=4))


@pytest.mark.parametrize("fit", [3, 5, -1])
def test_parabolic_fit(fit):
    pin(Case(nsubx=8, p=8, N=16, sig=1e4, parabolicFit=fit), cent_tol=1e-4)


def test_gaussian_fit():
    pin(Case(nsubx=8, p=8, N=16, sig=1e4, gaussianFitVals=(1.0, 0.0)), cent_tol=1e-4)


def test_optical_binning():
    pin(Case(nsubx=8, p=8, N=16, sig=1e4, opticalBinning=1), cent_tol=1e-4)


def test_image_only_and_calsource():
    pin(Case(nsubx=8, p=8, N=16, sig=1e4, imageOnly=1))
    pin(Case(nsubx=8, p=8, N=16, sig=2e3, addPoisson=1, readnoise=2.0, readbg=1.0, noiseFloor=1.0, calsource=1))


def test_reference_and_calibration_flow():
    # takeReference (util/centroid.py:1536-1570), then CALCOEFF and CALDATA
    c = Case(nsubx=8, p=8, N=16, sig=1e4, readbg=1.0, noiseFloor=1.0)
    ref = c.reference()
    orc = c.oracle()
    saved = c.ref_phs.copy()
    c.ref_phs[...] = 0.0
    ref.run(1)
    orc.update(1, 1)
    oc, ob = c.oracle_run(orc, c.ref_phs)
    compare(c, c.ref_cents, c.ref_bimg, oc, ob)
    refc = c.ref_cents.copy()
    ref.update(18, refc)
    orc.update(18, refc)
    c.ref_phs[...] = saved
    ref.run(0)
    orc.update(1, 0)
    oc, ob = c.oracle_run(orc, c.ref_phs)
    compare(c, c.ref_cents, c.ref_bimg, oc, ob)
    coeff = np.zeros((8, 8, 2, 3), np.float32)
    coeff[..., 1] = 1.1
    coeff[..., 2] = 0.05
    ref.update(19, coeff)
    orc.update(19, coeff)
    ref.run(0)
    oc, ob = c.oracle_run(orc, c.ref_phs)
    compare(c, c.ref_cents, c.ref_bimg, oc, ob)
    ref.update(19, None)
    orc.update(19, None)
    steps = np.linspace(-2, 2, 9).astype(np.float32)
    cal = np.ascontiguousarray(np.broadcast_to(steps * 0.9, (2, 8, 8, 9)), dtype=np.float32)
    bounds = np.zeros((2, 8, 8, 2), np.int32)
    bounds[..., 1] = 8
    ref.update(17, (cal, bounds, steps))
    orc.update(17, (cal, bounds, steps))
    ref.run(0)
    oc, ob = c.oracle_run(orc, c.ref_phs)
    compare(c, c.ref_cents, c.ref_bimg, oc, ob)
    ref.free()


def test_integration_and_latency():
    c = Case(nsubx=8, p=8, N=16, sig=1e4, nintegrations=3, nlatency=1)
    ref = c.reference()
    orc = c.oracle()
    c.ref_cents[...] = 5.0
    oc = np.full(128, 5.0, np.float32)
    ob = np.zeros((64, 8, 8), np.float32)
    for f in range(8):
        c.ref_phs[...] = c.new_phase(f)
        ref.run(0)
        c.oracle_run(orc, c.ref_phs, oc, ob)
        compare(c, c.ref_cents, c.ref_bimg, oc, ob)
    ref.free()


def test_update_codes():
    c = Case(nsubx=8, p=8, N=16, sig=1e4)
    ref = c.reference()
    orc = c.oracle()
    for code, val in ((2, 5e3), (8, 3.0), (7, 2.0), (6, 1.0), (4, 6), (9, 2.0), (20, 10),
                      (10, np.ascontiguousarray(np.pad(np.ones((4, 4), np.float32), 6)))):
        ref.update(code, val)
        orc.update(code, val)
        ref.run(0)
        oc, ob = c.oracle_run(orc, c.ref_phs)
        compare(c, c.ref_cents, c.ref_bimg, oc, ob, cent_tol=2e-5)
    ref.free()


def _corr_pattern(nsubx, cs, mode):
    """A centred Gaussian reference spot per subaperture; for mode 1 its
    half-complex spectrum after a 180-degree rotation (a cross-correlation)."""
    from oracle.shwfs_oracle import r2hc_2d
    y, x = np.mgrid[0:cs, 0:cs] - (cs - 1) / 2.0
    spot = 50.0 * np.exp(-(x * x + y * y) / (2 * 1.3 ** 2))
    ref = np.broadcast_to(spot, (nsubx, nsubx, cs, cs))
    if mode == 1:
        rot = np.roll(spot[::-1, ::-1], (1, 1), (0, 1))
        ref = np.broadcast_to(r2hc_2d(rot), (nsubx, nsubx, cs, cs))
    return np.ascontiguousarray(ref, dtype=np.float32)


@pytest.mark.parametrize("mode,cs", [(1, 8), (1, 12), (2, 8), (2, 12), (3, 8), (4, 12), (5, 8), (5, 12)])
def test_correlation_modes(mode, cs):
    corrimg = np.zeros((8, 8, cs, cs), np.float32)
    c = Case(nsubx=8, p=8, N=16, C=16, m=8, ncen=6, sig=2e3, correlationCentroiding=mode, corrThresh=0.1,
             corrPattern=_corr_pattern(8, cs, mode), corrimg=corrimg, phase_seed=4)
    orc = c.oracle()
    oc, ob = pin(c, cent_tol=2e-5)
    lit = c.lit()
    ci = corrimg.reshape(64, -1)[lit]
    oi = orc.corrimg.reshape(64, -1)[lit] if orc.corrimg is not None else None
    orc2 = c.oracle()
    c.oracle_run(orc2, c.ref_phs)
    oi = orc2.corrimg.reshape(64, -1)[lit]
    assert np.abs(ci).max() > 0
    assert np.abs(ci - oi).max() <= 1e-4 * np.abs(oi).max()


def test_gaussian_fit_on_correlation_logs_corrimg():
    corrimg = np.zeros((8, 8, 8, 8), np.float32)
    c = Case(nsubx=8, p=8, N=16, C=16, m=8, ncen=6, sig=2e3, correlationCentroiding=5, corrThresh=0.0,
             corrPattern=_corr_pattern(8, 8, 5), corrimg=corrimg, gaussianFitVals=(1.0, 0.0), phase_seed=4)
    pin(c, cent_tol=1e-4)
    orc = c.oracle()
    c.oracle_run(orc, c.ref_phs)
    lit = c.lit()
    np.testing.assert_allclose(corrimg.reshape(64, -1)[lit], orc.corrimg.reshape(64, -1)[lit], atol=1e-4)


def test_noisy_streams_bit_identical():
    # pre-noise images agree bit for bit here, so the reference's own
    # PCG32/rk_poisson draws and the shim's MT19937 gaussian must give the
    # oracle's noisy images exactly
    c = Case(nsubx=8, p=8, N=16, sig=3e3, addPoisson=1, readnoise=2.0, skybrightness=5.0, noiseFloor=2.0,
             nthreads=3, seed=11)
    ref = c.reference()
    orc = c.oracle()
    oc = np.zeros(128, np.float32)
    ob = np.zeros((64, 8, 8), np.float32)
    for f in range(3):
        ref.run(0)
        c.oracle_run(orc, c.ref_phs, oc, ob)
        np.testing.assert_array_equal(c.ref_bimg.reshape(ob.shape), ob)
        np.testing.assert_allclose(c.ref_cents, oc, atol=1e-5, rtol=0)
    ref.free()


def test_run_slope_image_input():
    rng = np.random.default_rng(21)
    c = Case(nsubx=8, p=8, N=16, sig=1e4, noiseFloor=5.0, useBrightest=6)
    img = np.ascontiguousarray((50.0 * rng.random((64, 64)) ** 4).astype(np.float32))
    ref = c.reference(inputImage=img)
    ref.runSlope(0)
    oc = np.zeros(128, np.float32)
    ob = np.zeros((64, 8, 8), np.float32)
    c.oracle().run_slope(img, oc, ob)
    compare(c, c.ref_cents, c.ref_bimg, oc, ob)
    ref.free()
    img4 = np.ascontiguousarray((30 * rng.random((8, 8, 8, 8)) ** 3).astype(np.float32))
    c = Case(nsubx=8, p=8, N=16, sig=1e4, noiseFloor=2.0)
    ref = c.reference(inputImage=img4)
    ref.runSlope(0)
    oc[...] = 0
    ob[...] = 0
    c.oracle().run_slope(img4, oc, ob)
    compare(c, c.ref_cents, c.ref_bimg, oc, ob)
    ref.free()


def test_run_slope_subap_locations():
    rng = np.random.default_rng(8)
    c = Case(nsubx=8, p=8, N=16, sig=1e4, noiseFloor=3.0)
    img = np.ascontiguousarray((50.0 * rng.random((64, 64)) ** 4).astype(np.float32))
    loc = np.zeros((64, 4), np.int32)
    for i in range(64):
        r0, c0 = (i // 8) * 8 + 1, (i % 8) * 8 + 1
        loc[i] = (r0, r0 + 6, c0, c0 + 6)
    bimg0 = np.full((8, 8, 8, 8), 2.5, np.float32)
    ref = c.reference(bimg=bimg0.copy(), inputImage=img, subapLocation=loc)
    ref.runSlope(0)
    oc = np.zeros(128, np.float32)
    ob = bimg0.reshape(64, 8, 8).copy()
    c.oracle().run_slope(img, oc, ob, subapLocation=loc)
    compare(c, c.ref_cents, c.ref_bimg, oc, ob)
    ref.free()


def test_phase_interpolation():
    # phase array larger than nsubx*phasesize: the reference resamples it
    c = Case(nsubx=8, p=8, N=16, sig=1e4)
    big = np.ascontiguousarray(
        np.kron(c.phs, np.ones((1, 1), np.float32))[:60, :60].repeat(2, 0).repeat(2, 1)[:100, :100])
    ref = c.reference(phs=big)
    ref.run(0)
    oc = np.zeros(128, np.float32)
    ob = np.zeros((64, 8, 8), np.float32)
    c.oracle_run(c.oracle(), big, oc, ob)
    compare(c, c.ref_cents, c.ref_bimg, oc, ob)
    ref.free()


@pytest.mark.parametrize("n", [8, 9, 12])
def test_testcorrelation(n):
    """cent.testcorrelation of the reference against the oracle's
    calc_correlation with corrsize = nimg = n."""
    from dasp_gb300.correlation import transform_psf
    from oracle.shwfs_oracle import calc_correlation
    rng = np.random.default_rng(n)
    img = (rng.random((n, n)) ** 2).astype(np.float32)
    y, x = np.mgrid[0:n, 0:n] - (n - 1) / 2.0
    pat = transform_psf((np.exp(-(x * x + y * y) / 4.0) * (1 + 0.2 * rng.random((n, n)))).astype(np.float32))
    want = calc_correlation(n, n, pat.copy(), img, np.float32)
    got = pat.copy()
    ref_cent.testcorrelation(img, got)
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()


def _ref_lambda(c, **over):
    """Pre-noise images of the reference module: the same handle settings with
    shot and read noise, background and threshold off, so bimg holds the
    normalised, sky-added images the noisy run poissonises."""
    quiet = dict(addPoisson=0, readnoise=0.0, readbg=0.0, noiseFloor=0.0, useBrightest=0, pxlPower=1.0)
    quiet.update(over)
    lam_c = np.zeros(c.nsubaps * 2, np.float32)
    lam_b = np.zeros((c.nsubx, c.nsubx, c.m, c.m), np.float32)
    ref = c.reference(cents=lam_c, bimg=lam_b, **quiet)
    ref.run(0)
    ref.free()
    return lam_b.reshape(c.nsubaps, c.m, c.m).copy()


def test_prenoise_oracle_equals_reference_noisy_frames():
    # the oracle's run_prenoise on the reference's own pre-noise images, with
    # the reference's streams, reproduces the reference's noisy frames
    c = Case(nsubx=16, p=8, N=16, sig=3e3, addPoisson=1, readnoise=3.0, skybrightness=10.0, noiseFloor=6.0,
             nthreads=5, seed=17, useBrightest=-20)
    lam = _ref_lambda(c)
    ref = c.reference()
    orc = c.oracle()
    oc = np.zeros(c.nsubaps * 2, np.float32)
    ob = np.zeros((c.nsubaps, c.m, c.m), np.float32)
    for f in range(3):
        ref.run(0)
        orc.run_prenoise(lam, oc, ob)
        np.testing.assert_array_equal(c.ref_bimg.reshape(ob.shape)[c.lit()], ob[c.lit()])
        np.testing.assert_allclose(c.ref_cents, oc, atol=1e-5, rtol=0)
    ref.free()


def test_prenoise_oracle_injected_draws():
    # injected draws equal to the streams' own draws give the same frame
    c = Case(nsubx=8, p=8, N=16, sig=3e3, addPoisson=1, readnoise=2.0, skybrightness=5.0, noiseFloor=2.0,
             nthreads=1, seed=5, imageOnly=0)
    lam = _ref_lambda(c)
    ref = c.reference()
    ref.run(0)
    # the streams' draws, recovered from an oracle run without threshold
    # and background: Poisson counts from a run with read noise off, read
    # noise values as the difference of the two runs
    o1 = c.oracle()
    o1.update(7, -1e30)  # NOISEFLOOR far below: threshold keeps every pixel
    o1.threshType = 1
    o1.update(5, 0.0)
    b1 = np.zeros((64, 8, 8), np.float32)
    o1.run_prenoise(lam, np.zeros(128, np.float32), b1)
    o2 = c.oracle()
    o2.update(7, -1e30)
    o2.threshType = 1
    b2 = np.zeros((64, 8, 8), np.float32)
    o2.run_prenoise(lam, np.zeros(128, np.float32), b2)
    shot = b1.copy()
    readn = (b2 - b1).astype(np.float32)
    o3 = c.oracle()
    oc = np.zeros(128, np.float32)
    ob = np.zeros((64, 8, 8), np.float32)
    o3.run_prenoise(lam, oc, ob, shot=shot, readn=readn)
    lit = c.lit()
    # equal up to the float rounding of recovering readn by subtraction
    assert np.abs(ob[lit] - c.ref_bimg.reshape(64, 8, 8)[lit]).max() <= 1e-3
    ref.free()
