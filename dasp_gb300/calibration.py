"""Centroid linearisation and reference capture on the engine.

DASP's centroid object calibrates each subaperture's centroid response by
running noiseless frames with phase tilt ramps (util/centroid.py:1162-1254,
``calibrateSHSUnique``), keeps the range where the response is single
valued, forces it monotonic, and hands the table to the module
(``update(CALDATA, (data, bounds, steps))``, :1526) or fits polynomials
(``makeCalibrationCoeffs`` :1497-1509, ``update(CALCOEFF, ...)``).  Reference
centroids come from a flat phase with the calibration source on
(``takeReference`` :1536-1570).

Here the 2*steps ramp frames run as one batch on the GPU (``run_batch``), so
calibrating a 74x74 sensor costs a few milliseconds instead of 2*steps
sequential module calls; the table post-processing follows the reference
step by step.
"""
from __future__ import annotations

import numpy as np

from .centcmod import ADDPOISSON, CALCOEFF, CALDATA, CALSOURCE, READNOISE, REFCENTS


def calibration_steps(steps: int, step_range_frac: float = 1.0) -> np.ndarray:
    """Tilt per pixel of each calibration step (util/centroid.py:1173)."""
    return ((np.arange(steps) - steps / 2. + 0.5) / (steps / 2. - 0.5) * np.pi * step_range_frac).astype(np.float32)


def bounds_and_force(cal_data: np.ndarray, force: bool = True):
    """Single-valued range of each subaperture's response and the forcing of
    non-increasing points inside it (util/centroid.py:1206-1250).

    ``cal_data`` (2, nsubx, nsubx, steps) float32 is modified in place;
    returns (bounds (2, nsubx, nsubx, 2) int32, points forced)."""
    _, nsx, nsy, _ = cal_data.shape
    bounds = np.zeros((2, nsx, nsy, 2), np.int32)
    bounds[..., 0] = np.argmin(cal_data, axis=-1)
    bounds[..., 1] = np.argmax(cal_data, axis=-1)
    forced = 0
    if force:
        for ax in range(2):
            for i in range(nsx):
                for j in range(nsy):
                    d = cal_data[ax, i, j]
                    for k in range(bounds[ax, i, j, 0], bounds[ax, i, j, 1]):
                        if d[k] > d[k + 1]:
                            # the reference averages the neighbours k-1 and k+1
                            d[k] = (d[k - 1] + d[k + 1]) / 2.
                            forced += 1
    return bounds, forced


def calibrate_shs_unique(eng, steps: int, step_range_frac: float = 1.0, cal_ncoeff: int = 0,
                         apply: bool = True) -> dict:
    """Calibrate ``eng`` (a ``centcmod``) as calibrateSHSUnique does, with the
    2*steps ramp frames in one GPU batch.

    Noise is switched off for the ramps and restored from the engine's
    construction values afterwards, as the reference does (:1179-1182,
    :1199-1201); the calibration source is off (:1178).  The handle's
    current reference centroids and calibration apply to the ramp frames as
    they would in the reference, so calibrate before taking references.
    Returns ``{"data", "bounds", "steps", "forced"}`` and, with
    ``cal_ncoeff`` > 0, the polynomial coefficients ``"coeff"``.
    """
    import torch

    if getattr(eng, "nintegrations", 1) != 1:
        raise ValueError("calibration frames are single readouts: nintegrations must be 1")
    if eng.phs is None or len(eng.phs.shape) != 2:
        raise ValueError("calibration ramps need a phase-only (2-D) phase array")
    nsx = eng.nsubx
    width = int(eng.phs.shape[-1])
    step_list = calibration_steps(steps, step_range_frac)
    dev = torch.device("cuda")
    ramp = -torch.arange(width, device=dev, dtype=torch.float32)
    s = torch.from_numpy(step_list).to(dev)
    frames = torch.empty((2 * steps, width, width), device=dev, dtype=torch.float32)
    frames[0::2] = (ramp[None, None, :] * s[:, None, None]).expand(steps, width, width)  # x: along columns
    frames[1::2] = (ramp[None, :, None] * s[:, None, None]).expand(steps, width, width)  # y: along rows
    nsub = nsx * nsx
    cents = torch.zeros((2 * steps, nsub * 2), device=dev, dtype=torch.float32)
    bimg = torch.zeros((2 * steps, nsub, eng.nimg, eng.nimg), device=dev, dtype=torch.float32)
    eng.update(ADDPOISSON, 0)
    eng.update(READNOISE, 0)
    if eng.calsource != 0:
        eng.update(CALSOURCE, 0)
        eng.calsource = 0
    try:
        eng.run_batch(frames, cents, bimg)
        torch.cuda.synchronize()
    finally:
        eng.update(ADDPOISSON, eng.addPoisson)
        eng.update(READNOISE, eng.readnoise)
    c = cents.cpu().numpy().reshape(steps, 2, nsx, nsx, 2)
    data = np.empty((2, nsx, nsx, steps), np.float32)
    data[0] = np.moveaxis(c[:, 0, :, :, 0], 0, -1)  # x centroids of the x ramps
    data[1] = np.moveaxis(c[:, 1, :, :, 1], 0, -1)  # y centroids of the y ramps
    bounds, forced = bounds_and_force(data, force=cal_ncoeff == 0)
    out = {"data": data, "bounds": bounds, "steps": step_list, "forced": forced}
    if cal_ncoeff > 0:
        # makeCalibrationCoeffs (util/centroid.py:1497-1509): polynomial in
        # the measured centroid giving the applied tilt, lowest order first
        coeff = np.zeros((nsx, nsx, 2, cal_ncoeff), np.float32)
        flag = np.asarray(eng.subflag).reshape(nsx, nsx)
        for i in range(nsx):
            for j in range(nsx):
                if flag[i, j]:
                    for ax in range(2):
                        f, t = bounds[ax, i, j]
                        coeff[i, j, ax] = np.polyfit(data[ax, i, j, f:t], step_list[f:t], cal_ncoeff - 1)[::-1]
        out["coeff"] = coeff
        if apply:
            eng.update(CALCOEFF, coeff)
    elif apply:
        eng.update(CALDATA, (data, bounds, step_list))
    return out


def take_reference(eng) -> np.ndarray:
    """Reference centroids from a flat phase with the calibration source on
    (util/centroid.py:1536-1570), handed to the engine (REFCENTS).  The
    engine's bound phase array is zeroed, as the reference does."""
    eng.update(REFCENTS, None)
    phs = eng.phs
    phs[...] = 0
    eng.run(1)
    cents = eng.cents
    ref = (cents.cpu().numpy() if hasattr(cents, "cpu") else np.asarray(cents)).astype(np.float32).copy()
    eng.update(REFCENTS, ref.reshape(-1))
    return ref
