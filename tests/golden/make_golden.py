"""Make the golden fixtures in this folder from the reference's own module.

Each ``<name>.npz`` holds one configuration's exact inputs and the outputs of
the reference's ``cent`` module -- cmod/src/centmodule.c, unmodified, built by
oracle/build_ref.py against its FFT/GSL shims -- on them:

* ``spec``: JSON: the ``tests.wfs_cases.Case`` arguments, the number of
  calls, the input kind (``phase``: ``run`` per frame, util/centcmod.py:147;
  ``image``: ``runSlope``, :158), the initial centroid value, the
  tolerances, which engine tests use the case, and the machine it was made on;
* ``phs``: the phase of every call (float32), ``psf``: the spot PSF, when
  there is one; ``image``: the detector image of an image-input case;
  ``param_<name>``: array-valued parameters (useBrightest, sig, centWeight);
* ``cents`` / ``bimg``: the reference's centroids and images after every call.

The fixtures let the tests pin the oracle (tests/test_golden.py) and the
engine (tests/test_golden_gpu.py) to the reference where its sources are not
at hand.  Regenerate with ``python tests/golden/make_golden.py`` where the
reference tree (or oracle/_ref's staged copy of it) is present.
"""
from __future__ import annotations

import json
import os
import platform
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# centroid tolerance (px) and image tolerance (fraction of the frame's peak);
# "gpu": the FP32-form engine test compares the case, "tc": the FP16
# tensor-core form too (lit subapertures, 1e-3 px)
CASES = {
    # SCAO 8x8, two frames of independent phase
    "scao_8x8": dict(case=dict(nsubx=8, p=8, N=16, C=16, m=8, sig=1e4), frames=2),
    # the 74x74 ELT sensor's subaperture geometry on 10x10 subapertures
    # (0.53 m subapertures, r0 0.157 m at 589 nm): Gaussian spot PSF, sky,
    # noise floor
    "elt_subaps_psf_sky_floor": dict(
        case=dict(nsubx=10, p=10, N=20, C=20, m=10, obs=0.28, Dtel=5.27, r0=0.157, L0=25.0, wavelength=589.0,
                  psf="gauss", sig=500.0, skybrightness=10.0, noiseFloor=6.0), tc=True),
    # clip narrower than the FFT; fractional binning (2.5 pixels per image pixel)
    "crop_20_16_bin_8": dict(case=dict(nsubx=10, p=10, N=20, C=16, m=8, sig=3e3)),
    "bin_fractional_20_8": dict(case=dict(nsubx=10, p=10, N=20, C=20, m=8, sig=3e3)),
    # PSF wider than the FFT (zero padding), and pre-binning of a 32-point FFT
    "psf_pad_16_32": dict(case=dict(nsubx=8, p=8, N=16, C=16, m=8, psf="gauss", psfsize=32, sig=2e3)),
    "prebin_32_psf16": dict(case=dict(nsubx=8, p=16, N=32, C=16, m=8, psf="gauss", psfsize=16, sig=2e3,
                                      preBinningFactor=2)),
    # per-subaperture (LGS) PSFs
    "lgs_psf4d": dict(case=dict(nsubx=8, p=8, N=16, C=16, m=8, psf="gauss4d", sig=1e3)),
    # phase + amplitude input
    "phase_amplitude": dict(case=dict(nsubx=8, p=8, N=16, sig=1e4, amp=True)),
    # per-subaperture signal and sky arrays
    "sig_sky_arrays": dict(case=dict(nsubx=8, p=8, N=16, noiseFloor=2.0), arrays="sig_sky"),
    # threshold type 1 with a read background
    "threshold1_readbg": dict(case=dict(nsubx=8, p=8, N=16, sig=1e4, readbg=3.0, noiseFloor=25.0, threshType=1),
                              cent_tol=1e-4),
    # brightest pixels: a count, and a per-subaperture array
    "brightest_5": dict(case=dict(nsubx=8, p=8, N=16, sig=1e4, useBrightest=5)),
    "brightest_array": dict(case=dict(nsubx=8, p=8, N=16, sig=1e4), arrays="brightest"),
    # pixel power, centroid weights and a smaller centroid window
    "pixel_power_2": dict(case=dict(nsubx=8, p=8, N=16, sig=1e3, pxlPower=2.0), img_rtol=3e-4),
    "centroid_weights": dict(case=dict(nsubx=8, p=8, N=16, sig=1e4), arrays="centweight"),
    "centroid_window_4": dict(case=dict(nsubx=8, p=8, N=16, sig=1e4, ncen=4)),
    # parabolic and Gaussian fits
    "parabolic_fit": dict(case=dict(nsubx=8, p=8, N=16, sig=1e4, parabolicFit=1), cent_tol=1e-4),
    "gaussian_fit": dict(case=dict(nsubx=8, p=8, N=16, sig=1e4, gaussianFitVals=[1.0, 0.0]), cent_tol=1e-4),
    # image only (no centroids written)
    "image_only": dict(case=dict(nsubx=8, p=8, N=16, sig=1e4, imageOnly=1)),
    # integration and latency: outputs only on readout calls, centroids
    # start at 5 to show which calls write them
    "integration_3_latency_1": dict(case=dict(nsubx=8, p=8, N=16, sig=1e4, nintegrations=3, nlatency=1),
                                    frames=6, init_cents=5.0),
    # noisy frames from the reference's own PCG32 / rk_poisson draws and the
    # shim's MT19937 gaussian (the oracle must give the images bit for bit)
    "noisy_reference_streams": dict(
        case=dict(nsubx=8, p=8, N=16, sig=3e3, addPoisson=1, readnoise=2.0, skybrightness=5.0, noiseFloor=2.0,
                  nthreads=3, seed=11), frames=2, gpu=False, exact_images=True),
    # image input (runSlope): a 2-D detector frame with brightest pixels and
    # a noise floor, and a 4-D one
    "run_slope_2d": dict(case=dict(nsubx=8, p=8, N=16, sig=1e4, noiseFloor=5.0, useBrightest=6), input="image2d"),
    "run_slope_4d": dict(case=dict(nsubx=8, p=8, N=16, sig=1e4, noiseFloor=2.0), input="image4d"),
}


def _arrays(kind):
    """Array-valued parameters of a case (seeded)."""
    if kind == "sig_sky":
        rng = np.random.default_rng(3)
        return dict(sig=(1e3 * (1 + rng.random(64))).astype(np.float32),
                    skybrightness=(5 * rng.random((64, 8, 8))).astype(np.float32))
    if kind == "brightest":
        return dict(useBrightest=(np.arange(64, dtype=np.int32) % 7 - 3).astype(np.int32))
    if kind == "centweight":
        r = (np.arange(8) - 3.5) ** 2
        return dict(centWeight=np.exp(-r[:, None] / 8 - r[None, :] / 8).astype(np.float32))
    return {}


def _image(kind):
    rng = np.random.default_rng(21)
    if kind == "image2d":
        return np.ascontiguousarray((50.0 * rng.random((64, 64)) ** 4).astype(np.float32))
    return np.ascontiguousarray((30 * rng.random((8, 8, 8, 8)) ** 3).astype(np.float32))


def build(spec):
    """The fixture's arrays for one entry of CASES: inputs, the reference's
    outputs and the JSON spec."""
    from tests.wfs_cases import Case
    arrays = _arrays(spec.get("arrays"))
    c = Case(**spec["case"], **arrays)
    frames = spec.get("frames", 1)
    inp = spec.get("input", "phase")
    out = {}
    if inp == "phase":
        ref = c.reference()
        c.ref_cents[...] = spec.get("init_cents", 0.0)
        phs, cents, bimg = [], [], []
        for f in range(frames):
            if f:
                c.ref_phs[...] = c.new_phase(f)
            phs.append(c.ref_phs.copy())
            ref.run(c.params["calsource"])
            cents.append(c.ref_cents.copy())
            bimg.append(c.ref_bimg.reshape(c.nsubaps, c.m, c.m).copy())
        ref.free()
        out["phs"] = np.stack(phs)
    else:
        img = _image(inp)
        ref = c.reference(inputImage=img)
        ref.runSlope(0)
        cents, bimg = [c.ref_cents.copy()], [c.ref_bimg.reshape(c.nsubaps, c.m, c.m).copy()]
        ref.free()
        out["image"] = img
    out["cents"] = np.stack(cents)
    out["bimg"] = np.stack(bimg)
    if c.psf is not None:
        out["psf"] = np.ascontiguousarray(c.psf, dtype=np.float32)
    for k, v in arrays.items():
        out["param_" + k] = v
    case = dict(spec["case"])
    case.pop("psfsize", None)  # the stored PSF carries its size
    meta = dict(case=case, frames=frames, input=inp, init_cents=spec.get("init_cents", 0.0),
                cent_tol=spec.get("cent_tol", 1e-5), img_rtol=spec.get("img_rtol", 1e-4),
                gpu=spec.get("gpu", True), tc=spec.get("tc", False), exact_images=spec.get("exact_images", False),
                arrays=sorted(arrays), machine=platform.machine(),
                reference="cmod/src/centmodule.c (unmodified) via oracle/build_ref.py")
    out["spec"] = np.array(json.dumps(meta, sort_keys=True))
    return out


def make(name, spec):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **build(spec))
    return path


def main():
    from oracle import ref_cent
    if not ref_cent.available():
        raise SystemExit("the reference's sources are not available here")
    total = 0
    for name, spec in CASES.items():
        path = make(name, spec)
        total += os.path.getsize(path)
        print("%-28s %7d bytes" % (name, os.path.getsize(path)))
    print("total %d bytes" % total)


if __name__ == "__main__":
    main()
