"""The allocation-free image-centroiding entry point against the handle-based
image path.

shwfs_image_centroids_noalloc exists for callers that may not allocate GPU
memory: a real-time control thread that must never call cudaMalloc/cudaFree
(an allocation can stall the whole device) or an application whose device
memory belongs to its own allocator.  It takes only caller-owned device
buffers and keeps its working lists in a static device array.  This file is
collected last so that a run stopping at its first failure has already run
every other test.
"""
import ctypes

import numpy as np
import pytest

from tests.wfs_cases import Case

pytestmark = pytest.mark.gpu

CENT_TOL = 1e-5
IMG_RTOL = 1e-4


def _image(rng, n):
    return np.ascontiguousarray((60.0 * rng.random((n, n)) ** 4).astype(np.float32))


def _job(_lib, c, img_dev, subflag_dev, cents_dev, bimg_dev):
    p = c.params
    j = _lib.ShwfsImageJob()
    j.nsubx, j.nimg, j.ncen = c.nsubx, c.m, c.ncen
    j.image_ndim = 2
    j.image_rows, j.image_cols = img_dev.shape[-2], img_dev.shape[-1]
    j.image = img_dev.data_ptr()
    j.subflag = subflag_dev.data_ptr()
    j.refCents = None
    j.noiseFloor = p["noiseFloor"]
    j.threshType = p["threshType"]
    j.calsource = p["calsource"]
    j.useBrightest = p["useBrightest"]
    j.pxlPower = p["pxlPower"]
    j.imageOnly = p["imageOnly"]
    j.readNoise, j.readBg = p["readnoise"], p["readbg"]
    j.seed, j.frame = 0, 0
    j.cents = cents_dev.data_ptr()
    j.bimg = bimg_dev.data_ptr()
    return j


def test_noalloc_matches_run_slope_on_two_calls(engine_lib):
    torch = pytest.importorskip("torch")
    from dasp_gb300 import _lib
    rng = np.random.default_rng(2024)
    c = Case(nsubx=8, p=8, N=16, sig=1e4, noiseFloor=4.0, useBrightest=30, pxlPower=1.0)
    img = _image(rng, c.nsubx * c.m)
    eng = c.engine(inputImage=img)  # existing entry point: handle + shwfs_run_slope
    subflag = torch.from_numpy(c.pup.getSubapFlag(c.nsubx, 0.5).astype(np.int32).ravel()).cuda()
    cents_dev = torch.zeros(c.nsubaps * 2, device="cuda")
    bimg_dev = torch.zeros(c.nsubaps * c.m * c.m, device="cuda")
    err = ctypes.create_string_buffer(256)
    for _ in range(2):
        img[...] = _image(rng, c.nsubx * c.m)
        eng.runSlope(0)
        img_dev = torch.from_numpy(img).cuda()
        job = _job(_lib, c, img_dev, subflag, cents_dev, bimg_dev)
        torch.cuda.synchronize()
        st = engine_lib.shwfs_image_centroids_noalloc(ctypes.byref(job), None, err, len(err))
        assert st == 0, err.value
        torch.cuda.synchronize()
        got_c = cents_dev.cpu().numpy()
        got_b = bimg_dev.cpu().numpy().reshape(c.nsubaps, -1)
        ref_b = c.bimg.reshape(c.nsubaps, -1)
        assert np.abs(got_c - c.cents).max() <= CENT_TOL
        assert np.abs(got_b - ref_b).max() <= IMG_RTOL * float(np.abs(ref_b).max())
    eng.free()


@pytest.mark.parametrize("variant", ["image4d", "image_only_read_noise", "ref_cents"])
def test_noalloc_variants_match_run_slope(engine_lib, variant):
    """A 4-D image, images only with read noise on the unused subapertures
    (the counter stream of the same seed and frame), and reference centroids:
    each against shwfs_run_slope on a handle with the same settings, twice."""
    torch = pytest.importorskip("torch")
    from dasp_gb300 import _lib
    from dasp_gb300.centcmod import REFCENTS
    rng = np.random.default_rng(77)
    kw = dict(sig=1e4, noiseFloor=3.0, seed=19)
    if variant == "image_only_read_noise":
        kw.update(imageOnly=1, readnoise=2.5, readbg=4.0)
    c = Case(nsubx=8, p=8, N=16, **kw)
    shape4 = (c.nsubx, c.nsubx, c.m, c.m)
    img = (np.ascontiguousarray((40.0 * rng.random(shape4) ** 3).astype(np.float32)) if variant == "image4d"
           else _image(rng, c.nsubx * c.m))
    eng = c.engine(inputImage=img)
    refc = None
    if variant == "ref_cents":
        refc = (0.1 * rng.standard_normal(c.nsubaps * 2)).astype(np.float32)
        eng.update(REFCENTS, refc)
    subflag = torch.from_numpy(c.pup.getSubapFlag(c.nsubx, 0.5).astype(np.int32).ravel()).cuda()
    cents_dev = torch.zeros(c.nsubaps * 2, device="cuda")
    bimg_dev = torch.zeros(c.nsubaps * c.m * c.m, device="cuda")
    refc_dev = None if refc is None else torch.from_numpy(refc).cuda()
    err = ctypes.create_string_buffer(256)
    for _ in range(2):
        img[...] = (40.0 * rng.random(img.shape) ** 3).astype(np.float32)
        frame = eng.info()["frames_read"]
        eng.runSlope(0)
        img_dev = torch.from_numpy(img).cuda()
        job = _job(_lib, c, img_dev, subflag, cents_dev, bimg_dev)
        if variant == "image4d":
            job.image_ndim = 4
            job.image_rows, job.image_cols = c.nsubaps * c.m, c.m
        job.seed, job.frame = c.params["seed"], frame
        if refc_dev is not None:
            job.refCents = refc_dev.data_ptr()
        torch.cuda.synchronize()
        st = engine_lib.shwfs_image_centroids_noalloc(ctypes.byref(job), None, err, len(err))
        assert st == 0, err.value
        torch.cuda.synchronize()
        got_b = bimg_dev.cpu().numpy().reshape(c.nsubaps, -1)
        ref_b = c.bimg.reshape(c.nsubaps, -1)
        assert np.abs(got_b - ref_b).max() <= IMG_RTOL * float(np.abs(ref_b).max())
        if not c.params["imageOnly"]:
            assert np.abs(cents_dev.cpu().numpy() - c.cents).max() <= CENT_TOL
    eng.free()


def test_noalloc_rejects_sensors_beyond_its_fixed_scratch(engine_lib):
    torch = pytest.importorskip("torch")
    from dasp_gb300 import _lib
    c = Case(nsubx=8, p=8, N=16)
    t = torch.zeros(16, device="cuda")
    job = _job(_lib, c, torch.zeros((8, 8), device="cuda"), t.int(), t, t)
    job.nsubx = 257  # 66049 subapertures > 65536
    err = ctypes.create_string_buffer(256)
    st = engine_lib.shwfs_image_centroids_noalloc(ctypes.byref(job), None, err, len(err))
    assert st == _lib.SHWFS_ERR_INVALID
    assert b"65536" in err.value
