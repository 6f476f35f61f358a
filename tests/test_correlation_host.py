"""The correlation helpers of util/correlation.py (transformPSF, r2hc, hc2r)
restated in dasp_gb300.correlation, on the CPU: the half-complex layout
against the oracle's independent FFTW-convention transform, the normalised
round trip, and the property that makes transformPSF's output a correlation
pattern -- its unnormalised inverse is n^2 times the circularly reversed,
fftshift-ed spot, so correlation mode 1 (the oracle's calcCorrelation,
cmod/src/centmodule.c:1403-1486) with it is the circular cross-correlation
of the padded image with the shifted spot."""
import numpy as np
import pytest

from dasp_gb300.correlation import hc2r, hc2r1d, r2hc, r2hc1d, transform_psf, transformPSF
from oracle.shwfs_oracle import calc_correlation, hc2r_2d, r2hc_2d


def _reversed(x):
    """x[-i mod n, -j mod n]"""
    return np.roll(x[::-1, ::-1], (1, 1), (0, 1))


@pytest.mark.parametrize("n", [7, 8, 9, 10, 16, 17])
def test_half_complex_layout_and_round_trip(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal((n, n))
    np.testing.assert_array_equal(r2hc(x), r2hc_2d(x))
    np.testing.assert_allclose(hc2r(r2hc(x)), x, atol=1e-12)
    v = rng.standard_normal(n)
    np.testing.assert_allclose(hc2r1d(r2hc1d(v)), v, atol=1e-12)
    # the 1-D layout: Re F_k at k (k <= n/2), Im F_k at n - k
    F = np.fft.fft(v)
    h = r2hc1d(v)
    for k in range(n // 2 + 1):
        assert h[k] == pytest.approx(F[k].real, abs=1e-12)
    for k in range(1, (n + 1) // 2):
        assert h[n - k] == pytest.approx(F[k].imag, abs=1e-12)


@pytest.mark.parametrize("n", [8, 9, 10, 12])
def test_transform_psf_is_a_correlation_pattern(n):
    rng = np.random.default_rng(100 + n)
    psf = rng.random((n, n)).astype(np.float32)
    pat = transform_psf(psf)
    assert pat.dtype == np.float32 and pat.shape == (n, n) and pat.flags.c_contiguous
    want = n * n * _reversed(np.fft.fftshift(psf).astype(np.float64))
    got = hc2r_2d(pat)
    assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()


def test_transform_psf_per_subaperture_and_alias():
    rng = np.random.default_rng(3)
    psfs = rng.random((3, 4, 10, 10)).astype(np.float32)
    pats = transformPSF(psfs)
    assert pats.shape == psfs.shape and pats.flags.c_contiguous
    for i in range(3):
        for j in range(4):
            np.testing.assert_array_equal(pats[i, j], transform_psf(psfs[i, j]))
    assert transform_psf(None) is None
    with pytest.raises(ValueError):
        transform_psf(np.zeros((2, 3, 4)))


@pytest.mark.parametrize("nimg,corrsize", [(8, 8), (8, 12), (10, 16)])
def test_mode1_with_transformed_spot_is_cross_correlation(nimg, corrsize):
    rng = np.random.default_rng(nimg + corrsize)
    img = rng.random((nimg, nimg))
    y, x = np.mgrid[0:corrsize, 0:corrsize] - (corrsize - 1) / 2.0
    spot = np.exp(-(x * x + y * y) / 3.0) * (1 + 0.3 * rng.random((corrsize, corrsize)))
    pat = transform_psf(spot.astype(np.float32))
    got = calc_correlation(nimg, corrsize, pat, img, np.float64)
    # direct circular cross-correlation of the padded image with the
    # shifted spot: out[k] = n^2 sum_j pad[j] s[j - k]
    pad = np.zeros((corrsize, corrsize))
    o = (corrsize - nimg) // 2
    pad[o:o + nimg, o:o + nimg] = img
    s = np.fft.fftshift(spot.astype(np.float32).astype(np.float64))
    want = np.zeros((corrsize, corrsize))
    for ky in range(corrsize):
        for kx in range(corrsize):
            want[ky, kx] = (pad * np.roll(s, (ky, kx), (0, 1))).sum()
    want *= corrsize * corrsize
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()


def test_testcorrelation_argument_checks():
    """testcorrelation rejects what py_testcorrelation rejects
    (cmod/src/centmodule.c:3287-3299) before touching the device."""
    from dasp_gb300.centcmod import testcorrelation
    ok = np.zeros((8, 8), np.float32)
    with pytest.raises(ValueError):
        testcorrelation(ok.astype(np.float64), ok.copy())
    with pytest.raises(ValueError):
        testcorrelation(ok, np.zeros((8, 9), np.float32))
    with pytest.raises(ValueError):
        testcorrelation(np.zeros((8, 9), np.float32), np.zeros((8, 9), np.float32))
    with pytest.raises(ValueError):
        testcorrelation(np.asfortranarray(np.zeros((8, 8), np.float32))[:, ::-1], ok.copy())
