"""Correlation centroiding (correlationCentroiding 1-5) against the oracle's
restatement of calcCorrelation / diffCorrelation / bruteCorrelation /
thresholdCorrelation (cmod/src/centmodule.c:1203-1505): the thresholded
correlation images written to corrimg and the centroids computed from them
(centred on the brightest pixel for modes 1 and 5, on the faintest for the
difference modes)."""
import numpy as np
import pytest

from tests.wfs_cases import Case
from oracle.shwfs_oracle import r2hc_2d

pytestmark = pytest.mark.gpu


def _reference_spots(c: Case, cs):
    """A reference spot per subaperture, cs x cs, centred (the flat-phase
    image of a Gaussian spot)."""
    y, x = np.mgrid[0:cs, 0:cs] - (cs - 1) / 2.0
    spot = np.exp(-(x * x + y * y) / (2 * 1.3 ** 2)).astype(np.float32)
    return np.broadcast_to(spot, (c.nsubx, c.nsubx, cs, cs)).copy()


def _pattern(c: Case, cs, mode):
    ref = _reference_spots(c, cs) * 50.0
    if mode == 1:
        # half-complex spectrum of the 180-degree rotated reference: the
        # convolution with it is the cross-correlation with the reference
        rot = ref[:, :, ::-1, ::-1]
        out = np.stack([r2hc_2d(np.roll(rot[i, j], (1, 1), (0, 1))) for i in range(c.nsubx) for j in range(c.nsubx)])
        return np.ascontiguousarray(out.reshape(c.nsubx, c.nsubx, cs, cs).astype(np.float32))
    return np.ascontiguousarray(ref.astype(np.float32))


def _run(mode, cs, form="fp32", thresh=0.0, **kw):
    c = Case(nsubx=8, p=8, N=16, C=16, m=8, ncen=6, sig=2e3, correlationCentroiding=mode, corrThresh=thresh,
             phase_seed=4, **kw)
    c.params["corrPattern"] = _pattern(c, cs, mode)
    corrimg = np.zeros((c.nsubx, c.nsubx, cs, cs), np.float32)
    c.params["corrimg"] = corrimg
    eng = c.engine()
    if form != "fp32":
        eng.set_form(form)
    eng.run(0)
    orc = c.oracle("f64")
    oc, ob = c.oracle_run(orc)
    lit = c.lit()
    ec = np.abs(c.cents.reshape(-1, 2)[lit] - oc.reshape(-1, 2)[lit]).max()
    ci = corrimg.reshape(c.nsubaps, -1)[lit]
    oi = orc.corrimg.reshape(c.nsubaps, -1)[lit]
    ei = np.abs(ci - oi).max() / max(np.abs(oi).max(), 1e-30)
    eng.free()
    return ec, ei, ci, oc.reshape(-1, 2)[lit]


@pytest.mark.parametrize("mode,cs", [(1, 8), (1, 12), (2, 8), (2, 12), (4, 8), (4, 12), (5, 8), (5, 12), (3, 8)])
def test_correlation_modes_match_oracle(mode, cs):
    ec, ei, ci, _ = _run(mode, cs)
    assert np.abs(ci).max() > 0
    assert ei < 1e-4, "corrimg error %g" % ei
    assert ec < 1e-3, "centroid error %g px" % ec


@pytest.mark.parametrize("thresh", [0.3, 5.0])
def test_correlation_threshold(thresh):
    ec, ei, _, _ = _run(5, 8, thresh=thresh)
    assert ei < 1e-4 and ec < 1e-3, (ei, ec)


def test_correlation_with_tensor_core_form():
    ec, ei, _, _ = _run(1, 12, form="fp16")
    assert ei < 5e-3 and ec < 5e-3, (ei, ec)


def test_correlation_update_codes():
    from dasp_gb300.centcmod import CORRELATIONCENTROIDING, CORRPATTERN, CORRTHRESH
    c = Case(nsubx=8, p=8, N=16, C=16, m=8, ncen=6, sig=2e3, phase_seed=5)
    eng = c.engine()
    eng.run(0)
    plain = c.cents.copy()
    corrimg = np.zeros((8, 8, 8, 8), np.float32)
    # switch on with a brute-force pattern via update codes; the corrimg
    # array of the constructor is None, so results go to cents only
    eng.update(CORRPATTERN, _pattern(c, 8, 5))
    eng.update(CORRTHRESH, 0.0)
    eng.update(CORRELATIONCENTROIDING, 5)
    eng.run(0)
    c2 = Case(nsubx=8, p=8, N=16, C=16, m=8, ncen=6, sig=2e3, phase_seed=5, correlationCentroiding=5)
    c2.params["corrPattern"] = _pattern(c2, 8, 5)
    oc, _ = c2.oracle_run(c2.oracle("f64"))
    lit = c.lit()
    assert np.abs(c.cents.reshape(-1, 2)[lit] - oc.reshape(-1, 2)[lit]).max() < 1e-3
    eng.update(CORRELATIONCENTROIDING, 0)
    eng.run(0)
    np.testing.assert_allclose(c.cents, plain, atol=1e-6)
    eng.free()


@pytest.mark.parametrize("cs", [8, 12])
def test_mode1_pattern_from_transform_psf(cs):
    """util/centroid.py builds mode 1's pattern from the user's reference
    spot with transformPSF (util/correlation.py:20-51); the engine on the
    pattern dasp_gb300.correlation.transform_psf makes matches the oracle,
    and its correlation peak sits where a cross-correlation puts it."""
    from dasp_gb300.correlation import transform_psf
    c = Case(nsubx=8, p=8, N=16, C=16, m=8, ncen=6, sig=2e3, correlationCentroiding=1, phase_seed=4)
    c.params["corrPattern"] = transform_psf(_reference_spots(c, cs) * 50.0)
    corrimg = np.zeros((c.nsubx, c.nsubx, cs, cs), np.float32)
    c.params["corrimg"] = corrimg
    eng = c.engine()
    eng.run(0)
    orc = c.oracle("f64")
    oc, _ = c.oracle_run(orc)
    lit = c.lit()
    ec = np.abs(c.cents.reshape(-1, 2)[lit] - oc.reshape(-1, 2)[lit]).max()
    ci = corrimg.reshape(c.nsubaps, -1)[lit]
    oi = orc.corrimg.reshape(c.nsubaps, -1)[lit]
    assert np.abs(ci - oi).max() / max(np.abs(oi).max(), 1e-30) < 1e-4
    assert ec < 1e-3, "centroid error %g px" % ec
    eng.free()


@pytest.mark.parametrize("n", [8, 9, 12, 16])
def test_testcorrelation_module_function(n):
    """cmod.cent.testcorrelation (cmod/src/centmodule.c:3275-3309): the
    pattern array is replaced by calcCorrelation of the image with it
    (corrsize = nimg), as the oracle's calc_correlation computes."""
    from dasp_gb300.centcmod import testcorrelation
    from dasp_gb300.correlation import transform_psf
    from oracle.shwfs_oracle import calc_correlation
    rng = np.random.default_rng(n)
    img = (rng.random((n, n)) ** 2).astype(np.float32)
    y, x = np.mgrid[0:n, 0:n] - (n - 1) / 2.0
    corr = transform_psf((np.exp(-(x * x + y * y) / 4.0) * (1 + 0.2 * rng.random((n, n)))).astype(np.float32))
    want = calc_correlation(n, n, corr.copy(), img, np.float64)
    got = corr.copy()
    testcorrelation(img, got)
    assert np.abs(got - want).max() <= 1e-4 * np.abs(want).max()
