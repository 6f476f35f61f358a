"""Zero-copy host I/O of ``run`` (update code 103): the kernels write the
centroids and the final images straight into the caller's pinned host arrays
and may read the phase from the host array.  Every switch setting must give
bit-identical outputs to the copying path, leave the images of unlit
subapertures untouched (the reference writes only lit ones unless imageOnly,
cmod/src/centmodule.c:1964-1981) and zero their centroids."""
import numpy as np
import pytest

from dasp_gb300.centcmod import HOSTIO, HOSTIO_OUTPUTS, HOSTIO_PHASE
from tests.wfs_cases import Case

pytestmark = pytest.mark.gpu


_KEEP = []


def _pinned(shape, fill=0.0):
    """A numpy view of page-locked host memory (whole pages of its own), so
    that the zero-copy path is certain to apply."""
    torch = pytest.importorskip("torch")
    t = torch.full(tuple(shape), float(fill), dtype=torch.float32).pin_memory()
    _KEEP.append(t)
    return t.numpy()


def _expected_direct(hostio, image_only):
    d = 0
    if hostio & HOSTIO_OUTPUTS:
        d |= 2 | (0 if image_only else 1)
    if hostio & HOSTIO_PHASE:
        d |= 4
    return d


def _frames(c, form, hostio, nframes=3):
    cents = _pinned((c.nsubaps * 2,), 7.0)
    bimg = _pinned((c.nsubx, c.nsubx, c.m, c.m), -3.0)
    phs = _pinned(c.phs.shape)
    phs[...] = c.phs
    eng = c.engine(phs=phs, cents=cents, bimg=bimg)
    eng.set_form(form)
    eng.update(HOSTIO, hostio)
    out = []
    for f in range(nframes):
        phs[...] = c.new_phase(200 + f)
        eng.run(0)
        out.append((cents.copy(), bimg.copy()))
    info = eng.info()
    eng.free()
    return info, out


@pytest.mark.parametrize("image_only", [0, 1])
@pytest.mark.parametrize("form,code", [("fp32", 0), ("fp16", 3)])
def test_zero_copy_matches_copies(form, code, image_only):
    c = Case(nsubx=12, p=8, N=16, C=16, m=8, sig=2e3, readnoise=3.0, addPoisson=1, skybrightness=5.0,
             noiseFloor=1.0, imageOnly=image_only)
    info, ref = _frames(c, form, 0)
    assert info["form_active"] == code
    lit = c.lit()
    for cents, bimg in ref:
        b = bimg.reshape(c.nsubaps, -1)
        if image_only:
            assert (b[~lit] != -3.0).any(), "imageOnly writes the unlit images"
            assert (cents == 7.0).all(), "imageOnly writes no centroids"
        else:
            assert (b[~lit] == -3.0).all(), "unlit images are left as they were"
            assert (cents.reshape(-1, 2)[~lit] == 0.0).all(), "unlit centroids are zero"
        assert np.isfinite(b[lit]).all() and (b[lit] != -3.0).any()
    assert info["host_io_direct"] == 0
    for hostio in (HOSTIO_OUTPUTS, HOSTIO_PHASE, HOSTIO_OUTPUTS | HOSTIO_PHASE):
        ginfo, got = _frames(c, form, hostio)
        # the tensor-core form writes the unlit noise images of imageOnly
        # through the device mirror (then copied): images direct only without
        expect = _expected_direct(hostio, image_only)
        if form != "fp32" and image_only:
            expect &= ~2
        assert ginfo["host_io_direct"] == expect, (hostio, ginfo["host_io_direct"])
        for f, ((rc, rb), (gc, gb)) in enumerate(zip(ref, got)):
            assert np.array_equal(rc, gc), (hostio, f, "cents")
            assert np.array_equal(rb, gb), (hostio, f, "bimg")


def test_zero_copy_with_calibration_and_refs():
    # reference centroids are subtracted inside the kernels, so the direct
    # host writes must carry them too
    c = Case(nsubx=10, p=8, N=16, C=16, m=8, sig=2e3)
    _, ref = _frames(c, "fp16", 0, nframes=1)
    refc = (0.01 * np.arange(c.nsubaps * 2, dtype=np.float32)).astype(np.float32)
    outs = []
    for hostio in (0, HOSTIO_OUTPUTS):
        cents = np.zeros(c.nsubaps * 2, np.float32)
        bimg = np.zeros((c.nsubx, c.nsubx, c.m, c.m), np.float32)
        eng = c.engine(phs=np.ascontiguousarray(c.new_phase(200)), cents=cents, bimg=bimg)
        eng.set_form("fp16")
        eng.update(HOSTIO, hostio)
        eng.update(18, refc)  # REFCENTS
        eng.run(0)
        outs.append((cents.copy(), bimg.copy()))
        eng.free()
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    lit = c.lit()
    np.testing.assert_allclose(outs[0][0].reshape(-1, 2)[lit] + refc.reshape(-1, 2)[lit],
                               ref[0][0].reshape(-1, 2)[lit], atol=1e-5)


@pytest.mark.parametrize("image_only", [0, 1])
def test_zero_copy_run_slope_matches_copies(image_only):
    """runSlope (image input): the image kernel reading the pinned detector
    frame and writing into the pinned outputs gives the copying path's
    results bit for bit."""
    c = Case(nsubx=12, p=8, N=16, C=16, m=8, sig=2e3, noiseFloor=2.0, readnoise=1.0, imageOnly=image_only)
    outs = {}
    for hostio in (0, HOSTIO_OUTPUTS | HOSTIO_PHASE):
        img = _pinned((c.nsubx * c.m, c.nsubx * c.m))
        cents = _pinned((c.nsubaps * 2,), 7.0)
        bimg = _pinned((c.nsubx, c.nsubx, c.m, c.m), -3.0)
        eng = c.engine(cents=cents, bimg=bimg, inputImage=img)
        eng.update(HOSTIO, hostio)
        res = []
        for f in range(2):
            img[...] = (50 * np.random.default_rng(30 + f).random(img.shape) ** 4).astype(np.float32)
            eng.runSlope(0)
            res.append((cents.copy(), bimg.copy()))
        assert eng.info()["host_io_direct"] == _expected_direct(hostio, image_only)
        eng.free()
        outs[hostio] = res
    for (rc, rb), (gc, gb) in zip(outs[0], outs[HOSTIO_OUTPUTS | HOSTIO_PHASE]):
        assert np.array_equal(rc, gc) and np.array_equal(rb, gb)


def test_bad_switches_rejected():
    c = Case(nsubx=8, p=8, N=16)
    eng = c.engine()
    with pytest.raises(ValueError):
        eng.update(HOSTIO, 4)
    eng.free()
