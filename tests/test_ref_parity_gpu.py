"""The CUDA engine against the reference's own module (oracle/_ref: the
unmodified cmod/src/centmodule.c with FFT/GSL shims) on identical inputs,
through the C ABI (dasp_gb300.centcmod -> libshwfs.so).

Tolerances: FP32 form noiseless centroids within 1e-5 px and images within
1e-4 of the frame's peak pixel; the tensor-core forms within their stated
accuracy (FP16 and TF32 1e-3 px, BF16x3 1e-4 px).
"""
import numpy as np
import pytest

from oracle import ref_cent
from tests.wfs_cases import Case

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_cent.available(), reason="reference sources not available")]

CENT_TOL = 1e-5
IMG_RTOL = 1e-4


def _elt(**kw):
    return Case(nsubx=74, p=10, N=20, C=20, m=10, obs=0.28, Dtel=39.0, r0=0.157, L0=25.0, wavelength=589.0,
                psf="gauss", nthreads=8, **kw)


def compare(c, cents, bimg, cent_tol=CENT_TOL, img_rtol=IMG_RTOL, lit_only=False):
    ec, rc = cents.reshape(-1, 2), c.ref_cents.reshape(-1, 2)
    eb, rb = bimg.reshape(c.nsubaps, -1), c.ref_bimg.reshape(c.nsubaps, -1)
    if lit_only:
        sel = c.lit()
        ec, rc, eb, rb = ec[sel], rc[sel], eb[sel], rb[sel]
    peak = max(float(np.abs(rb).max()), 1e-30)
    di, dc = float(np.abs(eb - rb).max()), float(np.abs(ec - rc).max())
    assert di <= img_rtol * peak, "image mismatch %g (peak %g)" % (di, peak)
    assert dc <= cent_tol, "centroid mismatch %g px" % dc
    return dc, di


def run_pair(c, nframes=1, form=None, cent_tol=CENT_TOL, img_rtol=IMG_RTOL, lit_only=False):
    eng = c.engine()
    if form:
        eng.set_form(form)
        assert eng.info()["form_active"] != 0, "tensor-core form did not engage"
    ref = c.reference(phs=c.phs)
    for f in range(nframes):
        if f:
            c.phs[...] = c.new_phase(f)
        eng.run(c.params["calsource"])
        ref.run(c.params["calsource"])
        compare(c, c.cents, c.bimg, cent_tol, img_rtol, lit_only)
    eng.free()
    ref.free()


def test_scao_8x8_noiseless():
    run_pair(Case(nsubx=8, p=8, N=16, C=16, m=8, sig=1e4), nframes=5)


def test_elt_74x74_noiseless_psf_sky_floor():
    run_pair(_elt(sig=500.0, skybrightness=10.0, noiseFloor=6.0))


@pytest.mark.parametrize("form,tol", [("fp16", 1e-3), ("tf32", 1e-3), ("bf16x3", 1e-4)])
def test_elt_74x74_tensor_core_forms(form, tol):
    run_pair(_elt(sig=500.0), form=form, cent_tol=tol, img_rtol=5e-3, lit_only=True)


def test_gaussian_fit_log_image():
    run_pair(Case(nsubx=8, p=8, N=16, sig=1e4, gaussianFitVals=(1.0, 0.0)), cent_tol=1e-4)


def test_prebin_and_lgs_psfs():
    run_pair(Case(nsubx=8, p=16, N=32, C=16, m=8, psf="gauss", psfsize=16, sig=2e3, preBinningFactor=2))
    run_pair(Case(nsubx=12, p=8, N=16, C=16, m=8, psf="gauss4d", sig=1e3))


def test_run_slope_image_input():
    rng = np.random.default_rng(21)
    c = Case(nsubx=8, p=8, N=16, sig=1e4, noiseFloor=5.0, useBrightest=6)
    img = np.ascontiguousarray((50.0 * rng.random((64, 64)) ** 4).astype(np.float32))
    eng = c.engine(inputImage=img)
    ref = c.reference(inputImage=img)
    eng.runSlope(0)
    ref.runSlope(0)
    compare(c, c.cents, c.bimg)
    eng.free()
    ref.free()
