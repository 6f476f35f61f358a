"""The reference's own ``cent`` module (built by ``oracle/build_ref.py``) behind
the ``util.centcmod`` constructor -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs may
use this, as the checker and as the timed CPU baseline; the product never
loads it.  ``RefCent`` takes the arguments of util/centcmod.py:42-45, derives
``pupfn``/``subflag``/``fracSubArea`` from the pupil object as
util/centcmod.py:76-78 does, and calls ``cent.initialise`` with the 41
positional arguments in the order of cmod/src/centmodule.c:2876-2883; ``run``,
``runSlope``, ``update`` and ``free`` call the module's own functions
(:3188-3229, :3230-3272, :2573-2856, :3163-3186).  The module borrows every
array by pointer (phs, pupfn, cents, bimg, subflag, fracSubArea, and the
arrays handed to ``update``), so this object keeps them referenced.
"""
from __future__ import annotations

import importlib.machinery
import importlib.util
import os

import numpy as np

from . import build_ref

_mod = None

CALSOURCE = 1


def available() -> bool:
    """True when the reference module is built or can be built here."""
    try:
        return build_ref.available()
    except Exception:
        return False


def module():
    """Build (if needed) and import oracle/_ref/cent.so as module ``cent``."""
    global _mod
    if _mod is None:
        path = build_ref.build()
        loader = importlib.machinery.ExtensionFileLoader("cent", path)
        spec = importlib.util.spec_from_file_location("cent", path, loader=loader)
        m = importlib.util.module_from_spec(spec)
        loader.exec_module(m)
        _mod = m
    return _mod


def _f32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


class RefCent:
    """cmod.cent through the util.centcmod constructor (numpy arrays only)."""

    def __init__(self, nthreads, nsubx, ncen, fftsize, clipsize, nimg, phasesize, readnoise, readbg,
                 addPoisson, noiseFloor, sig, skybrightness, calsource, pxlPower, nintegrations, nlatency, seed,
                 phs, pup, spotpsf, cents, bimg, minarea, opticalBinning, centWeight, correlationCentroiding,
                 corrThresh, corrPattern, corrimg, threshType, imageOnly, useBrightest, preBinningFactor,
                 parabolicFit, gaussianFitVals, inputImage=None, subapLocation=None):
        m = module()
        self.nsubx = nsubx
        self.calsource = calsource
        self.pupfn = np.ascontiguousarray(pup.perSubap(nsubx, vectorAlign=0), dtype=np.float32)
        self.subflag = np.ascontiguousarray(pup.getSubapFlag(nsubx, minarea), dtype=np.int32)
        self.fracSubArea = np.ascontiguousarray(pup.getSubarea(nsubx) / (phasesize * phasesize), dtype=np.float32)
        if isinstance(sig, np.ndarray):
            sig = np.ascontiguousarray(sig, dtype=np.float32)
        elif sig is not None:
            sig = float(sig)
        if isinstance(skybrightness, np.ndarray):
            skybrightness = np.ascontiguousarray(skybrightness, dtype=np.float32)
        else:
            skybrightness = float(skybrightness)
        if gaussianFitVals is None:
            gfit, gmin, grep = 0, 0.0, 0.0
        else:
            gfit, gmin, grep = 1, float(gaussianFitVals[0]), float(gaussianFitVals[1])
        self._keep = [phs, spotpsf, cents, bimg, centWeight, corrPattern, corrimg, useBrightest, inputImage,
                      subapLocation, sig, skybrightness]
        self.phs, self.cents, self.bimg = phs, cents, bimg
        self.ptr = m.initialise(
            int(nthreads), int(nsubx * nsubx), int(ncen), int(fftsize), int(clipsize), int(nimg), int(phasesize),
            float(readnoise), float(readbg), int(addPoisson), float(noiseFloor), sig, skybrightness,
            int(calsource), float(1.0 if pxlPower is None else pxlPower), int(nintegrations), int(nlatency),
            int(seed), phs, self.pupfn, spotpsf, cents, self.subflag, bimg, self.fracSubArea,
            int(opticalBinning), centWeight, int(correlationCentroiding), float(corrThresh), corrPattern, corrimg,
            int(threshType), int(imageOnly), useBrightest, int(preBinningFactor), int(parabolicFit), gfit, gmin,
            grep, inputImage, subapLocation)
        if self.ptr is None:
            raise RuntimeError("cent.initialise failed (see the module's printed message)")

    def run(self, calsource=None):
        """One frame (the reference's py_run); returns its elapsed seconds."""
        if calsource is not None and calsource != self.calsource:
            self.update(CALSOURCE, calsource)
            self.calsource = calsource
        return module().run(self.ptr)

    def runSlope(self, calsource=None):
        if calsource is not None and calsource != self.calsource:
            self.update(CALSOURCE, calsource)
            self.calsource = calsource
        return module().runSlope(self.ptr)

    def update(self, code, val):
        self._keep.append(val)
        module().update(self.ptr, int(code), val)

    def free(self):
        if self.ptr is not None:
            module().free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def testcorrelation(img, corr):
    module().testcorrelation(img, corr)


def nthreads_default() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
