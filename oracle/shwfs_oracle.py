"""CPU oracle for the Shack-Hartmann WFS step -- TEST INFRASTRUCTURE ONLY.

This module restates, in numpy, the reference's per-frame phase -> image ->
centroid pipeline (``cmod/src/centmodule.c`` ``centroidsFromPhase`` :1760-1984
and the init-time helpers it relies on).  It is the checker for the CUDA path:
only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s ``cpu_baseline``
leg may import it, and never as the thing measured or shipped.

Two arithmetic modes:

* ``mode="f32"`` mirrors the reference's float32 roundings at every stage the C
  code stores a ``float`` (tilt table, ``phs - tilt``, the complex64 field, the
  power spectrum, PSF spectra, the binned image, the normalisation factor);
  transforms are evaluated in float64 and rounded to float32 where the C code
  keeps single precision.
* ``mode="f64"`` evaluates the same algorithm in float64 throughout.  This is
  the FP64 accuracy reference for centroid-error statements.

The noise streams (PCG32 Poisson, GSL-style MT19937 read noise) are restated
in ``oracle/noise_ref.c`` and driven here subaperture by subaperture in the
reference's per-thread order, so noisy frames are reproducible given
``nthreads`` and ``seed`` (cmod/src/centmodule.c:2535-2563).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import time

import numpy as np

# update codes: util/centcmod.py:19-40, cmod/src/centmodule.c:109-130
CALSOURCE, SIG, ADDPOISSON, NCEN, READNOISE, READBG, NOISEFLOOR = 1, 2, 3, 4, 5, 6, 7
SKYBRIGHTNESS, PXLPOWER, SPOTPSF, NTHREADS, OPTICALBINNING, CENTWEIGHT = 8, 9, 10, 11, 12, 13
CORRELATIONCENTROIDING, CORRTHRESH, CORRPATTERN, CALDATA, REFCENTS = 14, 15, 16, 17, 18
CALCOEFF, USEBRIGHTEST, INTEGSTEPS, OUTPUTPHASEARR = 19, 20, 21, 22

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_NOISE_SO = os.path.join(_BUILD, "libnoise_ref.so")


def build_noise_lib(force: bool = False) -> str:
    """Compile oracle/noise_ref.c (no FMA contraction) into oracle/_build."""
    src = os.path.join(_HERE, "noise_ref.c")
    if force or not os.path.exists(_NOISE_SO) or os.path.getmtime(_NOISE_SO) < os.path.getmtime(src):
        os.makedirs(_BUILD, exist_ok=True)
        tmp = _NOISE_SO + ".%d.tmp" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                               "-o", tmp, src, "-lm"])
        os.replace(tmp, _NOISE_SO)
    return _NOISE_SO


_noise_lib = None


def noise_lib():
    global _noise_lib
    if _noise_lib is None:
        lib = ctypes.CDLL(build_noise_lib())
        lib.orc_pcg32_next.restype = ctypes.c_uint32
        lib.orc_pcg32_seed.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64]
        lib.orc_pcg32_next.argtypes = [ctypes.c_void_p]
        lib.orc_poisson.restype = ctypes.c_long
        lib.orc_poisson.argtypes = [ctypes.c_void_p, ctypes.c_float]
        lib.orc_poissonise.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        lib.orc_mt_seed.argtypes = [ctypes.c_void_p, ctypes.c_ulong]
        lib.orc_mt_next.restype = ctypes.c_uint32
        lib.orc_mt_next.argtypes = [ctypes.c_void_p]
        lib.orc_gaussian.restype = ctypes.c_double
        lib.orc_gaussian.argtypes = [ctypes.c_void_p, ctypes.c_double]
        lib.orc_readccd.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_float,
                                    ctypes.c_float, ctypes.c_float, ctypes.c_int]
        _noise_lib = lib
    return _noise_lib


class PCG32:
    """Handle on one oracle PCG32 state (cmod/src/centmodule.c:70-98)."""

    def __init__(self, initstate: int, initseq: int):
        lib = noise_lib()
        self.buf = ctypes.create_string_buffer(lib.orc_sizeof_pcg32())
        lib.orc_pcg32_seed(self.buf, initstate & (2**64 - 1), initseq & (2**64 - 1))

    def next(self) -> int:
        return noise_lib().orc_pcg32_next(self.buf)


class MT19937:
    """Handle on one oracle MT19937 state seeded the way gsl_rng_set does."""

    def __init__(self, seed: int):
        lib = noise_lib()
        self.buf = ctypes.create_string_buffer(lib.orc_sizeof_mt())
        lib.orc_mt_seed(self.buf, seed & (2**64 - 1))

    def next(self) -> int:
        return noise_lib().orc_mt_next(self.buf)


# ----------------------------------------------------------------------------
# init-time helpers
# ----------------------------------------------------------------------------

def tilt_fn(p: int, N: int, mode: str = "f32") -> np.ndarray:
    """tiltfn[i,j] = pi(N+1)/N * (i+j+1-p): cmod/src/centmodule.c:3074-3081."""
    k = np.arange(p)[:, None] + np.arange(p)[None, :] + 1 - p
    if mode == "f32":
        tmp = np.float32(np.pi / N * (N + 1.0))
        return (tmp * k.astype(np.float32)).astype(np.float32)
    return np.pi / N * (N + 1.0) * k.astype(np.float64)


def flip_array(a: np.ndarray, mirror: int) -> np.ndarray:
    """flipQuad/flipArray: cmod/src/centmodule.c:253-349 (returns a copy)."""
    a = np.array(a, copy=True)
    n = a.shape[-1]

    def flip_quad(r0, c0, h, w):
        a[..., r0:r0 + h, c0:c0 + w] = a[..., r0:r0 + h, c0:c0 + w][..., ::-1, ::-1]

    if mirror == 0:
        w1 = n // 2
        w3 = (n + 1) // 2
        flip_quad(0, 0, w1, w1)
        flip_quad(w1, 0, w3, w1)
        flip_quad(0, w1, w1, w3)
        flip_quad(w1, w1, w3, w3)
        return a
    if n % 2 == 0:
        f2 = n // 2
        out = np.empty_like(a)
        out[..., :f2, :f2] = a[..., f2:, f2:]
        out[..., f2:, f2:] = a[..., :f2, :f2]
        out[..., :f2, f2:] = a[..., f2:, :f2]
        out[..., f2:, :f2] = a[..., :f2, f2:]
        return out
    a = flip_array(a, 0)
    return a[..., ::-1, ::-1].copy()


def bin_weights(C: int, m: int):
    """prepareBinImage: cmod/src/centmodule.c:565-608 (float32 weights)."""
    this = np.zeros(C, np.float32)
    nxt = np.zeros(C, np.float32)
    indx = np.zeros(C, np.int32)
    cnt = 0
    for i in range(C):
        cnt += m
        if cnt >= C:
            excess = cnt - C
            this[i] = np.float32((m - excess) / np.float32(m))
            nxt[i] = np.float32(excess / np.float32(m))
            indx[i] = 1
            cnt = excess
        else:
            this[i] = 1.0
            nxt[i] = 0.0
            indx[i] = 0
    return this, nxt, indx


def bin_image(img: np.ndarray, m: int, weights, dtype) -> np.ndarray:
    """binImage: cmod/src/centmodule.c:609-651, vectorised over the leading axis.

    Reproduces the reference's accumulation pattern literally, including that
    the 'next pixel' share of column j is taken from input column j+1.
    """
    S, C, _ = img.shape
    if C == m:
        return img.astype(dtype, copy=True)
    t, n, idx = weights
    t = t.astype(dtype)
    n = n.astype(dtype)
    out = np.zeros((S, m, m), dtype)
    ii = 0
    for i in range(C):
        jj = 0
        last_i = i == C - 1
        for j in range(C):
            last_j = j == C - 1
            out[:, ii, jj] += t[i] * t[j] * img[:, i, j]
            if not last_j and jj + 1 < m:
                out[:, ii, jj + 1] += t[i] * n[j] * img[:, i, j + 1]
            if not last_i and ii + 1 < m:
                out[:, ii + 1, jj] += n[i] * t[j] * img[:, i + 1, j]
                if not last_j and jj + 1 < m:
                    out[:, ii + 1, jj + 1] += n[i] * n[j] * img[:, i + 1, j + 1]
            if not last_j:
                jj += idx[j]
        if not last_i:
            ii += idx[i]
    return out


def fit_matrix(fitsize: int) -> np.ndarray:
    """makeFitMx: cmod/src/centmodule.c:997-1056 (5x6 rows of the 6x6 inverse)."""
    mx = np.zeros((6, 6))
    for y in range(fitsize):
        for x in range(fitsize):
            v = np.array([x * x, x * y, y * y, x, y, 1.0])
            mx += np.outer(v, v)
    inv = np.linalg.inv(mx)
    return inv[:5].astype(np.float32).ravel()


# ----------------------------------------------------------------------------
# the per-frame pipeline
# ----------------------------------------------------------------------------

# Catmull-Rom basis rows (cmod/src/centmodule.c:1642), times 1/2 through t[0..3]
_MX = ((0.0, 2.0, 0.0, 0.0), (-1.0, 0.0, 1.0, 0.0), (2.0, -5.0, 4.0, -1.0), (-1.0, 3.0, -3.0, 1.0))


def _dot4_f32(c, v):
    """c[0]*v[0] + c[1]*v[1] + c[2]*v[2] + c[3]*v[3], left to right, each
    product and sum rounded to float32 (the C code's float arithmetic)."""
    s = (np.float32(c[0]) * v[0]).astype(np.float32)
    for k in range(1, 4):
        s = (s + (np.float32(c[k]) * v[k]).astype(np.float32)).astype(np.float32)
    return s


def _dot4_f32v(w, v):
    """Like _dot4_f32 with per-sample float32 weights w[0..3]."""
    s = (w[0] * v[0]).astype(np.float32)
    for k in range(1, 4):
        s = (s + (w[k] * v[k]).astype(np.float32)).astype(np.float32)
    return s


def _cubic_axis(nin, nout):
    """Per output sample: first of the four input samples (before clamping)
    and the weights 0.5 (1, t, t^2, t^3) (cmod/src/centmodule.c:1645-1680)."""
    scale = np.float32((nin - 1.0) / (nout - 1))
    t = (scale * np.arange(nout).astype(np.float32)).astype(np.float32)
    i0 = np.floor(t).astype(np.int64)
    t = (t - i0.astype(np.float32)).astype(np.float32)
    i0 = i0 - 1
    t[nout - 1] = 1.0  # the last output sample: the special case of :1663-1666
    i0[nout - 1] = nin - 3
    w1 = (np.float32(0.5) * t).astype(np.float32)
    w2 = (w1 * t).astype(np.float32)
    w3 = (w2 * t).astype(np.float32)
    return i0, [np.full(nout, 0.5, np.float32), w1, w2, w3]


def interpolate_phase(inp, nsubx, p):
    """interpolatePhase (cmod/src/centmodule.c:1628-1758): bicubic
    (Catmull-Rom) resample of a square input phase to (nsubx p)^2 samples
    spanning the same extent, in float32 with the C code's operation order:
    four column sums of the basis rows over four input rows, weighted in y,
    then the basis rows over those four values, weighted in x.  Samples
    outside the input repeat the edge row/column (:1685-1728)."""
    inp = np.asarray(inp, np.float32)
    nin = inp.shape[0]
    nout = nsubx * p
    iy, wy = _cubic_axis(nin, nout)
    ix, wx = _cubic_axis(nin, nout)
    rows = np.clip(iy[:, None] + np.arange(4)[None, :], 0, nin - 1)  # (nout, 4)
    cols = np.clip(ix[:, None] + np.arange(4)[None, :], 0, nin - 1)
    wyb = [w[:, None] for w in wy]
    pcol = []
    for i in range(4):  # column inx+i: interpolate in y
        f = [inp[rows[:, j][:, None], cols[:, i][None, :]] for j in range(4)]
        tmp = [_dot4_f32(_MX[k], f) for k in range(4)]
        pcol.append(_dot4_f32v(wyb, tmp))
    tmp2 = [_dot4_f32(_MX[i], pcol) for i in range(4)]
    return _dot4_f32v([w[None, :] for w in wx], tmp2)


class CentOracle:
    """State and per-frame step of one WFS, following ``centstruct``.

    Constructor arguments are the already-derived arrays that
    ``cmod.cent.initialise`` receives (cmod/src/centmodule.c:2858-3161):
    ``pupfn`` (nsubaps,p,p), ``subflag`` (nsubaps,), ``fracSubArea``
    (nsubaps,), and an optional ``spotpsf`` of shape (P,P) or
    (nsubx,nsubx,P,P).
    """

    def __init__(self, *, nsubx, phasesize, fftsize, clipsize, nimg, ncen, pupfn, subflag,
                 fracSubArea, sig=1.0, readnoise=0.0, readbg=0.0, addPoisson=0, noiseFloor=0.0,
                 skybrightness=0.0, calsource=0, pxlPower=1.0, nintegrations=1, nlatency=0,
                 seed=1, nthreads=1, spotpsf=None, opticalBinning=0, centWeight=None,
                 threshType=0, imageOnly=0, useBrightest=0, preBinningFactor=1,
                 parabolicFit=0, gaussianFit=0, gaussianMinVal=0.0, gaussianReplaceVal=0.0,
                 correlationCentroiding=0, corrThresh=0.0, corrPattern=None, mode="f32"):
        self.mode = mode
        self.dt = np.float32 if mode == "f32" else np.float64
        self.nsubx = nsubx
        self.nsubaps = nsubx * nsubx
        self.p = phasesize
        self.N = fftsize
        self.C = clipsize
        self.m = nimg
        self.ncen = ncen
        self.pupfn = np.asarray(pupfn, np.float32).reshape(self.nsubaps, self.p, self.p)
        self.subflag = np.asarray(subflag).reshape(self.nsubaps).astype(np.int32)
        self.frac = np.asarray(fracSubArea, np.float32).reshape(self.nsubaps)
        self.readNoise = np.float32(readnoise)
        self.readBg = np.float32(readbg)
        self.addPoisson = int(addPoisson)
        self.noiseFloor = np.float32(noiseFloor)
        self.calsource = int(calsource)
        self.pxlPower = np.float32(1.0 if pxlPower is None else pxlPower)
        self.nintegrations = int(nintegrations)
        self.nlatency = int(nlatency)
        self.curInteg = 0
        self.seed = int(seed)
        self.opticalBinning = int(opticalBinning)
        self.threshType = int(threshType)
        self.imageOnly = int(imageOnly)
        self.preBinningFactorOrig = int(preBinningFactor)
        self.parabolicFit = int(parabolicFit)
        self.gaussianFit = int(gaussianFit)
        self.gaussianMinVal = np.float32(gaussianMinVal)
        self.gaussianReplaceVal = np.float32(gaussianReplaceVal)
        self.correlationCentroiding = int(correlationCentroiding)
        self.corrThresh = np.float32(corrThresh)
        self.corrPattern = None
        self.corrPatternSize = 0
        if corrPattern is not None:
            cp = np.asarray(corrPattern, np.float32)
            self.corrPattern = cp.reshape(self.nsubaps, cp.shape[-2], cp.shape[-1]).copy()
            self.corrPatternSize = cp.shape[-1]
        self.corrsize = self.corrPatternSize if (self.correlationCentroiding and self.corrPattern is not None) \
            else self.m
        self.corrimg = None
        self.interpOut = None  # OUTPUTPHASEARR: interpolated phase of the lit subapertures
        self.fitMx = None
        self.fitMxParam = 0
        self.refCents = None
        self.calData = None
        self.calCoeff = None
        self.skyArr = None
        self.sky = np.float32(0)
        self.set_sky(skybrightness)
        self.sigArr = None
        self.sig = np.float32(0)
        self.set_sig(sig, init=True)
        self.useBrightestArr = None
        self.useBrightest = 0
        self.set_use_brightest(useBrightest)
        self.centWeight = None
        self.centWeightDim = 0
        self.set_cent_weight(centWeight)
        self.tilt = tilt_fn(self.p, self.N, mode)
        self.binw = bin_weights(self.C, self.m)
        self.set_spot_psf(spotpsf)
        self.setup_threads(nthreads)

    # -- parameter setters (py_update: cmod/src/centmodule.c:2573-2856) --
    def set_sky(self, sky):
        if isinstance(sky, np.ndarray):
            sky = np.asarray(sky, np.float32)
            if sky.shape != (self.nsubaps, self.m, self.m):
                raise ValueError("skybrightness should be 3D array shape nsubaps,nimg,nimg")
            self.sky = np.float32(0)
            self.skyArr = sky
        else:
            self.sky = np.float32(sky)
            self.skyArr = None

    def set_sig(self, sig, init=False):
        if isinstance(sig, np.ndarray):
            sig = np.asarray(sig, np.float32)
            if sig.ndim != 1 or sig.shape[0] != self.nsubaps:
                raise ValueError("sig arr dimensions must be 1D (nsubx^2)")
            self.sigArr = sig.copy()
        else:
            self.sig = np.float32(sig)
            if not init:
                self.update_totsig()

    def set_use_brightest(self, ub):
        if isinstance(ub, np.ndarray):
            self.useBrightest = 0
            self.useBrightestArr = np.asarray(ub, np.int32).reshape(self.nsubaps)
        else:
            self.useBrightest = int(ub)
            self.useBrightestArr = None

    def set_cent_weight(self, cw):
        self.centWeight = None
        self.centWeightDim = 0
        if cw is None:
            return
        cw = np.asarray(cw, np.float32)
        if cw.ndim not in (2, 4):
            raise ValueError("centWeight not 2d or 4d")
        if cw.shape[-1] != self.corrsize or cw.shape[-2] != self.corrsize:
            raise ValueError("centweight array not correct dimensions")
        self.centWeightDim = cw.ndim
        self.centWeight = cw.reshape(-1, self.corrsize, self.corrsize) if cw.ndim == 4 else cw

    def set_spot_psf(self, psf):
        """setSpotPsf + prepareSpotPsf + updateTotSigArr (:2255-2427)."""
        self.spotpsfDim = 0
        self.spotpsf = None
        self.P = self.C
        self.preBin = 1
        self.padded = self.C
        if psf is not None:
            psf = np.asarray(psf, np.float32)
            if psf.ndim == 2:
                self.spotpsfDim = 2
                self.P = psf.shape[0]
            elif psf.ndim == 4:
                self.spotpsfDim = 4
                self.P = psf.shape[2]
                psf = psf.reshape(self.nsubaps, self.P, self.P)
            else:
                raise ValueError("spotpsf not 2d or 4d")
            self.preBin = self.preBinningFactorOrig
            self.padded = self.P if self.preBin <= 1 else self.N
            if self.padded % self.preBin != 0:
                raise ValueError("paddedsize modulo preBinningFactor should be zero")
            if self.preBin > 1 and self.P > self.padded:
                raise ValueError("spotpsf dimensions should be <= paddedsize")
            if self.P < self.C:
                raise ValueError("spotpsf dimensions should be at least clipsize")
            self.spotpsf = psf
            flipped = flip_array(psf, 1)
            spec = np.fft.rfft2(flipped.astype(np.float64))
            self.fftPsf = spec.astype(np.complex64) if self.mode == "f32" else spec
        self.update_totsig()

    def update_totsig(self):
        """updateTotSigArr: cmod/src/centmodule.c:2403-2427 (float accumulation)."""
        if self.mode == "f32":
            tot = np.zeros(self.nsubaps, np.float32)
            for j in range(self.p * self.p):
                tot = (tot + self.pupfn.reshape(self.nsubaps, -1)[:, j]).astype(np.float32)
            tot = (tot * np.float32(self.N * self.N)).astype(np.float32)
            if self.spotpsfDim:
                ps = self.spotpsf.reshape(-1, self.P * self.P)
                s = np.zeros(ps.shape[0], np.float32)
                for j in range(self.P * self.P):
                    s = (s + ps[:, j]).astype(np.float32)
                scale = (s * np.float32(self.P) * np.float32(self.P)).astype(np.float32)
                tot = (tot * scale).astype(np.float32)
        else:
            tot = self.pupfn.reshape(self.nsubaps, -1).astype(np.float64).sum(1) * self.N * self.N
            if self.spotpsfDim:
                s = self.spotpsf.reshape(-1, self.P * self.P).astype(np.float64).sum(1)
                tot = tot * s * self.P * self.P
        self.totsig = tot

    def setup_threads(self, nthreads):
        """setupThreads: partition + per-thread RNG seeding (:2457-2571)."""
        self.nthreads = int(nthreads)
        starts = [0]
        cnt, left = 0, self.nsubaps
        for i in range(self.nthreads):
            cnt += left // (self.nthreads - i)
            left -= left // (self.nthreads - i)
            starts.append(cnt)
        starts[-1] = self.nsubaps
        self.subapStart = starts
        base = int(time.time()) if self.seed == 0 else self.seed
        self.pcg = [PCG32(base + i, 1) for i in range(self.nthreads)]
        self.mt = [MT19937(base + i) for i in range(self.nthreads)]

    def update(self, code, val):
        if code == 104:  # the engine's integration-mode extension
            self.integMode = int(val)
            self.curInteg = 0
        elif code == CALSOURCE:
            self.calsource = int(val)
        elif code == SIG:
            self.set_sig(val)
        elif code == ADDPOISSON:
            self.addPoisson = int(val)
        elif code == NCEN:
            self.ncen = int(val)
        elif code == READNOISE:
            self.readNoise = np.float32(val)
        elif code == READBG:
            self.readBg = np.float32(val)
        elif code == NOISEFLOOR:
            self.noiseFloor = np.float32(val)
        elif code == SKYBRIGHTNESS:
            self.set_sky(val)
        elif code == PXLPOWER:
            self.pxlPower = np.float32(val)
        elif code == SPOTPSF:
            self.set_spot_psf(val)
        elif code == NTHREADS:
            self.setup_threads(int(val))
        elif code == OPTICALBINNING:
            self.opticalBinning = int(val)
        elif code == CENTWEIGHT:
            self.set_cent_weight(val)
        elif code == REFCENTS:
            self.refCents = None if val is None else np.asarray(val, np.float32).reshape(-1).copy()
        elif code == CALDATA:
            if val is None:
                self.calData = None
            else:
                calData, calBounds, calSteps = val
                self.calData = (np.asarray(calData, np.float32).reshape(2, self.nsubaps, -1),
                                np.asarray(calBounds, np.int32).reshape(2, self.nsubaps, 2),
                                np.asarray(calSteps, np.float32).reshape(-1))
        elif code == CALCOEFF:
            self.calCoeff = None if val is None else np.asarray(val, np.float32).reshape(self.nsubaps, 2, -1)
        elif code == USEBRIGHTEST:
            self.set_use_brightest(val)
        elif code == INTEGSTEPS:
            self.nintegrations = int(val)
        elif code == OUTPUTPHASEARR:
            self.interpOut = None if val is None else val
        elif code == CORRELATIONCENTROIDING:
            self.correlationCentroiding = int(val)
            self.corrsize = self.corrPatternSize if self.correlationCentroiding else self.m
        elif code == CORRTHRESH:
            self.corrThresh = np.float32(val)
        elif code == CORRPATTERN:
            if val is None:
                self.corrPattern = None
            else:
                cp = np.asarray(val, np.float32)
                self.corrPattern = cp.reshape(self.nsubaps, cp.shape[-2], cp.shape[-1]).copy()
        else:
            raise ValueError("code %d not handled by the oracle" % code)

    # -- stages --
    def _field(self, phs, lit, amp=None):
        """computeHll field: pup * exp(i (phs - tilt)) (:473-497)."""
        p, W = self.p, self.nsubx * self.p
        sy, sx = np.divmod(lit, self.nsubx)
        rows = (sy * p)[:, None, None] + np.arange(p)[None, :, None]
        cols = (sx * p)[:, None, None] + np.arange(p)[None, None, :]
        ph = phs[rows, cols]
        pup = self.pupfn[lit]
        if self.mode == "f32":
            t = (ph.astype(np.float32) - self.tilt).astype(np.float32)
            a = pup if amp is None else (pup * amp[rows, cols]).astype(np.float32)
            e = a.astype(np.float64) * np.exp(1j * t.astype(np.float64))
            return e.astype(np.complex64), rows, cols
        t = ph.astype(np.float64) - self.tilt
        a = pup.astype(np.float64) if amp is None else pup.astype(np.float64) * amp[rows, cols]
        return a * np.exp(1j * t), rows, cols

    def _hll(self, e):
        """FFT + addPowerSpecCentral (:498-504, :430-471)."""
        S = e.shape[0]
        N, P = self.N, self.padded
        E = np.zeros((S, N, N), np.complex128)
        E[:, :self.p, :self.p] = e
        F = np.fft.fft2(E)
        if self.mode == "f32":
            F = F.astype(np.complex64)
            pw = (F.real * F.real + F.imag * F.imag).astype(np.float32)
        else:
            pw = F.real ** 2 + F.imag ** 2
        if P > N:
            rs, ro, c = (P - N) // 2, 0, N
        else:
            rs, ro, c = 0, (N - P) // 2, P
        hll = np.zeros((S, P, P), self.dt)
        hll[:, rs:rs + c, rs:rs + c] = pw[:, ro:ro + c, ro:ro + c][:, ::-1, ::-1]
        return hll

    def _prebin(self, hll):
        """prebinImage: cmod/src/centmodule.c:1583-1626."""
        f, padded, P = self.preBin, self.padded, self.P
        scaled = padded // f
        S = hll.shape[0]
        if scaled > P:
            off = (scaled - P) // 2
            b = P
        else:
            off = 0
            b = scaled
        sub = hll[:, off * 1:, off * 1:]
        out = np.zeros((S, b, b), self.dt)
        for i in range(b):
            for j in range(b):
                blk = hll[:, i * f + off:i * f + off + f, j * f + off:j * f + off + f]
                acc = np.zeros(S, self.dt)
                for ii in range(f):
                    for jj in range(f):
                        acc = (acc + blk[:, ii, jj]).astype(self.dt)
                out[:, i, j] = acc
        del sub
        if scaled < P:
            o = (P - scaled) // 2
            full = np.zeros((S, P, P), self.dt)
            full[:, o:o + scaled, o:o + scaled] = out
            return full
        return out

    def _convolve(self, img, lit):
        """doConvolution: r2c * fftPsf -> c2r (unnormalised), centre clip (:524-564)."""
        P, C = self.P, self.C
        spec = np.fft.rfft2(img.astype(np.float64))
        if self.mode == "f32":
            spec = spec.astype(np.complex64)
        psf = self.fftPsf if self.spotpsfDim == 2 else self.fftPsf[lit]
        prod = spec * psf
        if self.mode == "f32":
            prod = prod.astype(np.complex64)
        out = np.fft.irfft2(prod.astype(np.complex128), s=(P, P)) * (P * P)
        out = out.astype(self.dt)
        if C < P:
            off = (P - C) // 2
            out = out[:, off:off + C, off:off + C]
        return out

    def _optically_bin(self, img):
        """opticallyBin: cmod/src/centmodule.c:819-851 (per subap, in place)."""
        m, ncen = self.m, self.ncen
        for a in img:
            flat = a.reshape(-1)
            s = (m - ncen) // 2
            e = m - s
            v0 = self.dt(0)
            for i in range(s, e):
                v0 = self.dt(v0 + flat[m * s + i])
            if s != 0:
                flat[:ncen] = 0
            for i in range(s, e):
                for j in range(1 if s == 0 else s, e):
                    flat[i - s] = self.dt(flat[i - s] + flat[j * m + i])
            for i in range(s + 1, e):
                if s != 0:
                    flat[i - s + ncen] = 0
                for j in range(1 if s == 0 else s, e):
                    flat[i - s + ncen] = self.dt(flat[i - s + ncen] + flat[i * m + j])
            flat[ncen] = v0
            flat[2 * ncen:] = 0

    def _brightest(self, flat, ub):
        """selectBrightestPixels: cmod/src/centmodule.c:1544-1581."""
        npxl = flat.shape[0]
        subtract = False
        if ub < 0:
            ub = -ub
            subtract = True
        if 0 < ub < npxl:
            srt = np.sort(flat)
            thr = srt[npxl - ub]
            if subtract:
                k = npxl - ub - 1
                while k >= 0 and srt[k] == thr:
                    k -= 1
                sub = srt[k] if k >= 0 else self.dt(0)
                flat[:] = np.where(flat < thr, self.dt(0), (flat - sub).astype(self.dt))
            else:
                flat[:] = np.where(flat < thr, self.dt(0), flat)

    def _cog(self, img, weight, centre_on_brightest):
        """computeCoG: cmod/src/centmodule.c:873-971 (sequential float sums)."""
        n, ncen = img.shape[0], self.ncen
        flat = img.reshape(-1)
        dt = self.dt
        if centre_on_brightest == 0:
            sx = (n - ncen) // 2
            ex = n - sx
            sy, ey = sx, ex
        else:
            mx = dt(0)
            pos = 0
            if centre_on_brightest == 1:
                for i in range(n * n):
                    if flat[i] > mx:
                        mx, pos = flat[i], i
            else:
                for i in range(n * n):
                    if flat[i] < mx or mx == 0:
                        mx, pos = flat[i], i
            sx = int(pos % n - ncen / 2.0 + 0.5)
            sy = int(pos // n - ncen / 2.0 + 0.5)
            sx = min(max(sx, 0), n - ncen)
            sy = min(max(sy, 0), n - ncen)
            ex, ey = sx + ncen, sy + ncen
        s = dt(0)
        cx = dt(0)
        cy = dt(0)
        sign = -1 if centre_on_brightest not in (0, 1) and weight is None else 1
        for i in range(sy, ey):
            for j in range(sx, ex):
                v = img[i, j] if weight is None else dt(img[i, j] * weight[i, j])
                s = dt(s + v)
                cx = dt(cx + dt(sign * v * j))
                cy = dt(cy + dt(sign * v * i))
        if s > 0:
            cx = dt(cx / s)
            cy = dt(cy / s)
            if centre_on_brightest != 0:
                cx = dt(cx + sx)
                cy = dt(cy + sy)
            cx = dt(cx - (n - 1) / 2.0)
            cy = dt(cy - (n - 1) / 2.0)
            return cx, cy
        return dt(0), dt(0)

    def _fit(self, img, fitsize, do_gauss, corr_mode):
        """computeFit: cmod/src/centmodule.c:1069-1188."""
        n, ncen = img.shape[0], self.ncen
        a = img.reshape(-1).astype(np.float32).copy()
        nc = (n - ncen) // 2
        quad = 0
        if fitsize < 0:
            quad = 1
            fitsize = 3
        if fitsize < 3:
            fitsize = 3
        s = np.float32(0)
        mx = np.float32(0)
        pos = 0
        if do_gauss:
            for i in range(n * n):
                s = np.float32(s + a[i])
                if a[i] > mx:
                    pos, mx = i, a[i]
                a[i] = self.gaussianReplaceVal if a[i] < self.gaussianMinVal else np.float32(np.log(a[i]))
        elif corr_mode in (0, 1, 5):
            for i in range(n * n):
                s = np.float32(s + a[i])
                if a[i] > mx:
                    pos, mx = i, a[i]
        else:
            mx = a[nc * n + nc]
            pos = nc * n + nc
            for i in range(nc, nc + ncen):
                for j in range(nc, nc + ncen):
                    s = np.float32(s + a[i * n + j])
                    if a[i * n + j] < mx:
                        pos, mx = i * n + j, a[i * n + j]
        if do_gauss:
            # computeFit logs the caller's image in place (:1087-1096)
            img.reshape(-1)[:] = a
        if not s >= 0:
            return np.float32(0), np.float32(0)
        startx = int(pos % n - fitsize // 2)
        starty = int(pos // n - fitsize // 2)
        startx = max(startx, nc)
        starty = max(starty, nc)
        startx = min(startx, nc + ncen - fitsize)
        starty = min(starty, nc + ncen - fitsize)
        if quad == 0:
            vec = np.zeros(6, np.float32)
            for y in range(fitsize):
                for x in range(fitsize):
                    v = a[(y + starty) * n + x + startx]
                    vec += np.array([v * x * x, v * x * y, v * y * y, v * x, v * y, v], np.float32)
            if self.fitMxParam != fitsize:
                self.fitMx = fit_matrix(fitsize)
                self.fitMxParam = fitsize
            res = (self.fitMx.reshape(5, 6).astype(np.float64) @ vec.astype(np.float64)).astype(np.float32)
            if do_gauss:
                cx = np.float32(-res[3] / (2 * res[0]))
                cy = np.float32(-res[4] / (2 * res[2]))
            else:
                cx = np.float32((res[1] * res[4] / (2 * res[2]) - res[3]) / (2. * res[0] - res[1] * res[1] / (2. * res[2])))
                cy = np.float32(-(res[4] + res[1] * cx) / (2. * res[2]))
        else:
            b = a[starty * n + startx:]
            a2 = (b[2 * n + 1] - b[1]) / 2.
            a3 = (b[2 * n + 1] - 2 * b[n + 1] + b[1]) / 2.
            a4 = (b[n + 2] - b[n]) / 2.
            a5 = (b[n + 2] - 2 * b[n + 1] + b[n]) / 2.
            a6 = (b[2 * n + 2] - b[2] - b[2 * n] + b[0]) / 4.
            cy = np.float32((2 * a2 * a5 - a4 * a6) / (a6 * a6 - 4 * a3 * a5) + 1)
            cx = np.float32((2 * a3 * a4 - a2 * a6) / (a6 * a6 - 4 * a3 * a5) + 1)
        if cx < 0 or cy < 0 or cx >= fitsize or cy >= fitsize:
            cx = np.float32(pos % n - startx)
            cy = np.float32(pos // n - starty)
        cy = np.float32(cy - (ncen / 2. - 0.5))
        cx = np.float32(cx - (ncen / 2. - 0.5))
        cx = np.float32(cx + (startx + ncen / 2. - n / 2.))
        cy = np.float32(cy + (starty + ncen / 2. - n / 2.))
        return cx, cy

    @staticmethod
    def _interp(x, n, xp, fp):
        """interp: cmod/src/centmodule.c:1506-1518."""
        if x <= xp[0]:
            return fp[0]
        if x >= xp[n]:
            return fp[n]
        i = 1
        while x > xp[i]:
            i += 1
        return np.float32((x - xp[i - 1]) * (fp[i] - fp[i - 1]) / (xp[i] - xp[i - 1]) + fp[i - 1])

    def _calibrate(self, i, cx, cy):
        """calibration + refCents (:1943-1961)."""
        if self.calData is not None:
            cal, bounds, steps = self.calData
            out = []
            for axis, v in ((0, cx), (1, cy)):
                lo = bounds[axis, i, 0]
                n = bounds[axis, i, 1] - lo
                out.append(self._interp(v, n, cal[axis, i, lo:], steps[lo:]))
            cx, cy = out
        elif self.calCoeff is not None:
            out = []
            for axis, v in ((0, cx), (1, cy)):
                res = np.float32(0)
                xc = np.float32(1)
                for k in range(self.calCoeff.shape[2]):
                    res = np.float32(res + xc * self.calCoeff[i, axis, k])
                    xc = np.float32(xc * v)
                out.append(res)
            cx, cy = out
        if self.refCents is not None:
            cx = np.float32(cx - self.refCents[2 * i])
            cy = np.float32(cy - self.refCents[2 * i + 1])
        return cx, cy

    def additive(self):
        """Integration state for the current frame (:1774-1788); None = skip."""
        if self.curInteg == 0:
            return -1 if self.nintegrations + self.nlatency == 1 else 0
        if self.curInteg + 1 < self.nintegrations:
            return 1
        if self.curInteg + 1 < self.nintegrations + self.nlatency:
            return None
        return 2

    def pre_noise_images(self, phs, lit, amp=None):
        """Stages a3-a9: field, FFT, power, prebin, convolve, bin, normalise, sky."""
        e, rows, cols = self._field(phs, lit, amp)
        hll = self._hll(e)
        if self.spotpsfDim and self.preBin > 1:
            hll = self._prebin(hll)
        if self.spotpsfDim:
            hll = self._convolve(hll, lit)
        img = bin_image(hll, self.m, self.binw, self.dt)
        if amp is None:
            totsig = self.totsig[lit]
        else:
            pup = self.pupfn[lit].astype(self.dt)
            a = amp[rows, cols].astype(self.dt)
            tot = (pup * a).reshape(len(lit), -1).sum(1).astype(self.dt)
            totpup = pup.reshape(len(lit), -1).sum(1).astype(self.dt)
            with np.errstate(divide="ignore", invalid="ignore"):
                totsig = np.where(totpup != 0, tot * (self.totsig[lit] / totpup), 0).astype(self.dt)
        frac = self.frac[lit].astype(self.dt)
        if self.sigArr is None:
            with np.errstate(divide="ignore", invalid="ignore"):
                scale = (self.dt(self.sig) * frac / totsig).astype(self.dt)
        else:
            with np.errstate(divide="ignore", invalid="ignore"):
                scale = (self.sigArr[lit].astype(self.dt) / totsig).astype(self.dt)
        pos = totsig > 0
        img[pos] = (img[pos] * scale[pos, None, None]).astype(self.dt)
        skyv = (self.dt(self.sky) * frac).astype(self.dt)
        addsky = skyv > 0
        img[addsky] = (img[addsky] + skyv[addsky, None, None]).astype(self.dt)
        if self.skyArr is not None:
            img = (img + self.skyArr[lit].astype(self.dt)).astype(self.dt)
        return img, totsig, skyv

    def run(self, phs, cents, bimg, amp=None):
        """One frame: py_run -> centroidsFromPhase for every thread partition."""
        add = self.additive()
        if getattr(self, "integMode", 0) == 1:
            # physical integration (the engine's SHWFS_INTEG_PHYSICAL): every
            # exposed frame's normalised, sky-added images are summed in
            # float; the readout frame's image is the sum times 1/count
            if add is not None:
                lit = np.nonzero(self.subflag == 1)[0]
                img, totsig, skyv = self.pre_noise_images(np.asarray(phs), lit, amp)
                img = img.astype(np.float32)
                first = add in (0, -1)
                self._acc = img.copy() if first else (self._acc + img).astype(np.float32)
                self._accn = 1 if first else self._accn + 1
                if add in (2, -1):
                    mean = (self._acc * np.float32(np.float32(1.0) / np.float32(self._accn))).astype(np.float32)
                    self._readout(None, cents.reshape(-1), bimg.reshape(self.nsubaps, self.m, self.m), None,
                                  pre=(mean.astype(self.dt), totsig, skyv))
            self.curInteg += 1
            if self.curInteg >= self.nintegrations + self.nlatency:
                self.curInteg = 0
            return
        if add is not None and add in (2, -1):
            phs = np.asarray(phs)
            W = self.nsubx * self.p
            if phs.shape != (W, W):
                # phase of another (square) size: interpolatePhase per lit
                # subaperture (:1795-1804), here the whole array at once
                full = interpolate_phase(phs, self.nsubx, self.p)
                if self.interpOut is not None:
                    out = self.interpOut.reshape(W, W)
                    for i in np.nonzero(self.subflag == 1)[0]:
                        sy, sx = divmod(int(i), self.nsubx)
                        blk = (slice(sy * self.p, (sy + 1) * self.p), slice(sx * self.p, (sx + 1) * self.p))
                        out[blk] = full[blk]
                phs = full
            self._readout(phs, cents.reshape(-1), bimg.reshape(self.nsubaps, self.m, self.m), amp)
        self.curInteg += 1
        if self.curInteg >= self.nintegrations + self.nlatency:
            self.curInteg = 0

    def run_prenoise(self, images, cents, bimg, shot=None, readn=None):
        """A readout from pre-noise images (the engine's shwfs_run_prenoise):
        ``images`` (nsubaps, m, m) replace stages a3-a9 for the lit
        subapertures; the noise comes from the reference's streams, or from
        ``shot`` (the Poisson draws) / ``readn`` (the (float)gsl_ran_gaussian
        values) per pixel where the reference would draw them.  The
        integration state is not advanced."""
        lit = np.nonzero(self.subflag == 1)[0]
        img = np.asarray(images, np.float32).reshape(self.nsubaps, self.m, self.m)[lit].astype(self.dt)
        frac = self.frac[lit].astype(self.dt)
        pre = (img, self.totsig[lit], (self.dt(self.sky) * frac).astype(self.dt))
        inj = None
        if shot is not None or readn is not None:
            inj = (None if shot is None else np.asarray(shot, np.float32).reshape(self.nsubaps, -1),
                   None if readn is None else np.asarray(readn, np.float32).reshape(self.nsubaps, -1))
        self._readout(None, cents.reshape(-1), bimg.reshape(self.nsubaps, self.m, self.m), None, pre=pre,
                      inject=inj)

    @staticmethod
    def _readccd_injected(buf, readn, readBg, readNoise, floor_, threshType):
        """readCCD (:785-817) with the gaussian draws given: float adds in the
        reference's order, data += (g + noiseMean)."""
        f32 = np.float32
        if readNoise == 0:
            v = (buf + f32(readBg)).astype(f32)
        else:
            v = (buf + (readn.astype(f32) + f32(readBg)).astype(f32)).astype(f32)
        if threshType == 0:
            v = np.where(v < f32(floor_), f32(0), (v - f32(floor_)).astype(f32))
        elif threshType == 1:
            v = np.where(v < f32(floor_), f32(0), v)
        buf[:] = v.astype(f32)

    def _readout(self, phs, cents, bimg, amp, pre=None, inject=None):
        m, npxl = self.m, self.m * self.m
        lit = np.nonzero(self.subflag == 1)[0]
        if len(lit):
            img, totsig, skyv = self.pre_noise_images(phs, lit, amp) if pre is None else pre
            if self.opticalBinning == 1:
                self._optically_bin(img)
                nexp = 2 * self.ncen
            else:
                nexp = npxl
            litpos = {int(s): k for k, s in enumerate(lit)}
        else:
            img = np.zeros((0, m, m), self.dt)
            litpos = {}
            nexp = npxl
        do_noise = self.addPoisson == 1 and self.calsource == 0
        lib = noise_lib()
        readNoise = np.float32(self.readNoise * (self.calsource == 0))
        for t in range(self.nthreads):
            for i in range(self.subapStart[t], self.subapStart[t + 1]):
                k = litpos.get(i)
                if k is not None:
                    buf = np.ascontiguousarray(img[k].reshape(-1).astype(np.float32))
                    if do_noise and (totsig[k] > 0 or skyv[k] > 0 or self.skyArr is not None):
                        if inject is None:
                            lib.orc_poissonise(self.pcg[t].buf, buf.ctypes.data, nexp)
                        else:
                            buf[:nexp] = inject[0][i, :nexp]
                    if inject is None:
                        lib.orc_readccd(self.mt[t].buf, buf.ctypes.data, nexp, self.readBg, readNoise,
                                        self.noiseFloor, self.threshType)
                    else:
                        self._readccd_injected(buf[:nexp], None if inject[1] is None else inject[1][i, :nexp],
                                               self.readBg, readNoise, self.noiseFloor, self.threshType)
                    img[k] = buf.reshape(m, m).astype(self.dt)
                elif self.imageOnly != 0:
                    buf = np.zeros(npxl, np.float32)
                    if inject is None:
                        lib.orc_readccd(self.mt[t].buf, buf.ctypes.data, npxl, self.readBg, readNoise,
                                        self.noiseFloor, self.threshType)
                    else:
                        self._readccd_injected(buf, None if inject[1] is None else inject[1][i],
                                               self.readBg, readNoise, self.noiseFloor, self.threshType)
                    bimg[i] = buf.reshape(m, m)
                else:
                    cents[2 * i] = 0
                    cents[2 * i + 1] = 0
        vec_cog = (self.imageOnly == 0 and self.opticalBinning != 1 and self.parabolicFit == 0
                   and self.gaussianFit <= 0 and self.correlationCentroiding == 0)
        if self.corrimg is None or self.corrimg.shape[-1] != self.corrsize:
            self.corrimg = np.zeros((self.nsubaps, self.corrsize, self.corrsize), np.float32)
        for k, i in enumerate(lit):
            flat = img[k].reshape(-1)
            if self.calsource == 0:
                ub = self.useBrightest if self.useBrightestArr is None else int(self.useBrightestArr[i])
                sub = flat[:nexp].copy()
                self._brightest(sub, ub)
                flat[:nexp] = sub
            if self.pxlPower == 2:
                flat[:nexp] = (flat[:nexp] * flat[:nexp]).astype(self.dt)
            elif self.pxlPower != 1 and self.pxlPower != 0:
                flat[:nexp] = np.power(flat[:nexp], self.dt(self.pxlPower)).astype(self.dt)
            bimg[i] = img[k].astype(np.float32)
            if self.imageOnly == 0 and not vec_cog:
                cx, cy = self._centroid(i, img[k])
                cents[2 * i] = cx
                cents[2 * i + 1] = cy
                if self.gaussianFit > 0:
                    # a Gaussian fit leaves the log image in bimg (:1087-1096)
                    bimg[i] = img[k].astype(np.float32)

        if vec_cog and len(lit):
            if self.centWeightDim == 2:
                w = np.broadcast_to(self.centWeight, img.shape)
            elif self.centWeightDim == 4:
                w = self.centWeight[lit]
            else:
                w = None
            cx, cy = self._cog_vec(img, w)
            for k, i in enumerate(lit):
                cxk, cyk = self._calibrate(i, cx[k], cy[k])
                cents[2 * i] = cxk
                cents[2 * i + 1] = cyk

    def _correlate(self, i, img):
        """The correlation image of subap i (centroidsFromPhase :1898-1925):
        written to corrimg and returned, or the image itself when off."""
        cc = self.correlationCentroiding
        if cc == 0 or self.corrPattern is None:
            return img
        n, cs, dt = self.m, self.corrsize, self.dt
        pat = self.corrPattern[i]
        if cc == 1:
            out = calc_correlation(n, cs, pat, img, dt)
        elif 1 < cc < 5:
            out = diff_correlation(n, cs, self.ncen, img, pat, cc - 1, dt)
        else:
            out = brute_correlation(n, cs, self.ncen, img, pat, dt)
        threshold_correlation(out, self.corrThresh, dt)
        self.corrimg[i] = out.astype(np.float32)
        return out

    def _centroid(self, i, img):
        """correlation (optional), then optical-binning/fit/CoG, calibration
        and references for one lit subap (:1898-1961)."""
        flat = img.reshape(-1)
        if self.opticalBinning == 1:
            cx, cy = self._ob_cents(flat)
        else:
            cimg = self._correlate(i, img)
            if self.parabolicFit != 0 or self.gaussianFit > 0:
                cx, cy = self._fit(cimg, self.parabolicFit + self.gaussianFit, self.gaussianFit,
                                   self.correlationCentroiding)
                if self.gaussianFit > 0 and cimg is not img:
                    # the logged image is the correlation output (:1925)
                    self.corrimg[i] = cimg.astype(np.float32)
            else:
                if self.centWeightDim == 2:
                    w = self.centWeight
                elif self.centWeightDim == 4:
                    w = self.centWeight[i]
                else:
                    w = None
                cob = self.correlationCentroiding
                if cob == 5:
                    cob = 1
                cx, cy = self._cog(cimg, w, cob)
        return self._calibrate(i, cx, cy)

    def _cog_vec(self, img, weight):
        """computeCoG with a centred window, vectorised over subaps.

        Sums run in the reference's row-major order for every subap.
        """
        dt = self.dt
        S, n, _ = img.shape
        sx = (n - self.ncen) // 2
        ex = n - sx
        s = np.zeros(S, dt)
        cx = np.zeros(S, dt)
        cy = np.zeros(S, dt)
        for i in range(sx, ex):
            for j in range(sx, ex):
                v = img[:, i, j] if weight is None else (img[:, i, j] * weight[:, i, j]).astype(dt)
                s = (s + v).astype(dt)
                cx = (cx + (v * dt(j)).astype(dt)).astype(dt)
                cy = (cy + (v * dt(i)).astype(dt)).astype(dt)
        pos = s > 0
        with np.errstate(divide="ignore", invalid="ignore"):
            rx = (cx / s).astype(dt)
            ry = (cy / s).astype(dt)
        rx = (rx - dt((n - 1) / 2.0)).astype(dt)
        ry = (ry - dt((n - 1) / 2.0)).astype(dt)
        return np.where(pos, rx, dt(0)), np.where(pos, ry, dt(0))

    def run_slope(self, image, cents, bimg, subapLocation=None):
        """py_runSlope -> centroidsFromImage (cmod/src/centmodule.c:1987-2127).

        ``image`` is the 2-D detector image or a (nsubx,nsubx,nimg,nimg)
        array; bimg/cents are updated in place as the reference does
        (including keeping old bimg pixels outside a smaller window).
        """
        m, npxl = self.m, self.m * self.m
        cents = cents.reshape(-1)
        bimg = bimg.reshape(self.nsubaps, m, m)
        lib = noise_lib()
        readNoise = np.float32(self.readNoise * (self.calsource == 0))
        loc = None if subapLocation is None else np.asarray(subapLocation, np.int32).reshape(-1)
        for t in range(self.nthreads):
            for i in range(self.subapStart[t], self.subapStart[t + 1]):
                if self.subflag[i] == 1:
                    b = np.ascontiguousarray(bimg[i].reshape(-1).astype(np.float32))
                    if image.ndim == 2:
                        if loc is None:
                            r0 = (i // self.nsubx) * m
                            r1 = r0 + m
                            c0 = (i % self.nsubx) * m
                            c1 = c0 + m
                        else:
                            r0, r1, c0, c1 = (int(x) for x in loc[i * 4:i * 4 + 4])
                        for j in range(r1 - r0):
                            b[j * m:j * m + (c1 - c0)] = image[r0 + j, c0:c1]
                        nexp = (r1 - r0) * (c1 - c0)
                    else:
                        b[:] = image.reshape(self.nsubaps, npxl)[i]
                        nexp = npxl
                    if self.calsource == 0:
                        lib.orc_readccd(self.mt[t].buf, b.ctypes.data, nexp, np.float32(0), np.float32(0),
                                        self.noiseFloor, self.threshType)
                        ub = self.useBrightest if self.useBrightestArr is None else int(self.useBrightestArr[i])
                        sub = b[:nexp].astype(self.dt)
                        self._brightest(sub, ub)
                        b[:nexp] = sub
                    if self.pxlPower == 2:
                        b[:nexp] = b[:nexp] * b[:nexp]
                    elif self.pxlPower != 1 and self.pxlPower != 0:
                        b[:nexp] = np.power(b[:nexp], np.float32(self.pxlPower))
                    bimg[i] = b.reshape(m, m)
                    if self.imageOnly == 0:
                        if self.corrimg is None or self.corrimg.shape[-1] != self.corrsize:
                            self.corrimg = np.zeros((self.nsubaps, self.corrsize, self.corrsize), np.float32)
                        work = b.reshape(m, m).astype(self.dt)
                        cx, cy = self._centroid(i, work)
                        cents[2 * i] = cx
                        cents[2 * i + 1] = cy
                        if self.gaussianFit > 0 and self.opticalBinning != 1:
                            bimg[i] = work.astype(np.float32)
                else:
                    if self.imageOnly == 0:
                        cents[2 * i] = 0
                        cents[2 * i + 1] = 0
                    else:
                        buf = np.zeros(npxl, np.float32)
                        lib.orc_readccd(self.mt[t].buf, buf.ctypes.data, npxl, self.readBg, readNoise,
                                        self.noiseFloor, self.threshType)
                        bimg[i] = buf.reshape(m, m)

    def _ob_cents(self, flat):
        """computeOBCents: cmod/src/centmodule.c:853-872."""
        ncen = self.ncen
        dt = self.dt
        sx = sy = cx = cy = dt(0)
        for i in range(ncen):
            sx = dt(sx + flat[i])
            cx = dt(cx + flat[i] * i)
            sy = dt(sy + flat[i + ncen])
            cy = dt(cy + flat[i + ncen] * i)
        if sx > 0:
            cx = dt(dt(cx / sx) - (ncen - 1) / 2.0)
        if sy > 0:
            cy = dt(dt(cy / sy) - (ncen - 1) / 2.0)
        return cx, cy


# ----------------------------------------------------------------------------
# correlation centroiding (cmod/src/centmodule.c:1203-1505)

def r2hc_2d(x: np.ndarray) -> np.ndarray:
    """FFTW's 2-D r2r transform with kinds (R2HC, R2HC): the unnormalised
    1-D real-to-halfcomplex transform along each axis (r_k at k, i_k at n-k)."""
    def r2hc(a, axis):
        n = a.shape[axis]
        X = np.fft.fft(a, axis=axis)
        out = np.real(X).copy()
        idx = np.arange(n)
        im = np.imag(X)
        # i_k goes to position n-k for 0 < k < (n+1)/2
        ks = np.arange(1, (n + 1) // 2)
        take = np.take(im, ks, axis=axis)
        put = [slice(None)] * a.ndim
        put[axis] = n - ks
        out[tuple(put)] = take
        return out
    return r2hc(r2hc(np.asarray(x, np.float64), 1), 0)


def hc2r_2d(h: np.ndarray) -> np.ndarray:
    """FFTW's 2-D r2r transform with kinds (HC2R, HC2R): the unnormalised
    inverse of r2hc_2d along each axis (hc2r_2d(r2hc_2d(x)) = n^2 x)."""
    def hc2r(a, axis):
        n = a.shape[axis]
        a = np.moveaxis(np.asarray(a, np.float64), axis, 0)
        j = np.arange(n)[:, None]
        out = np.repeat(a[0:1], n, axis=0).astype(np.float64)
        for k in range(1, (n + 1) // 2):
            ang = 2 * np.pi * j * k / n
            out = out + 2 * (np.cos(ang).reshape((n,) + (1,) * (a.ndim - 1)) * a[k]
                             - np.sin(ang).reshape((n,) + (1,) * (a.ndim - 1)) * a[n - k])
        if n % 2 == 0:
            out = out + ((-1.0) ** np.arange(n)).reshape((n,) + (1,) * (a.ndim - 1)) * a[n // 2]
        return np.moveaxis(out, 0, axis)
    return hc2r(hc2r(h, 1), 0)


def calc_correlation(nimg, corrsize, pattern, img, dt):
    """calcCorrelation (:1403-1486): zero-pad the image to corrsize, r2hc,
    multiply by the half-complex pattern, hc2r (all unnormalised).  The
    half-complex product is the product of the complex spectra, so this is
    the circular convolution of the padded image with hc2r_2d(pattern)."""
    tmp = np.zeros((corrsize, corrsize), np.float64)
    o = (corrsize - nimg) // 2
    tmp[o:o + nimg, o:o + nimg] = img
    n = corrsize
    a = r2hc_2d(tmp)
    B = np.asarray(pattern, np.float64)
    out = a.copy()
    m = n
    neven, meven = n % 2 == 0, m % 2 == 0
    out[0, 0] = a[0, 0] * B[0, 0]
    if neven:
        out[0, n // 2] = a[0, n // 2] * B[0, n // 2]
    if meven:
        out[m // 2, 0] = a[m // 2, 0] * B[m // 2, 0]
        if neven:
            out[m // 2, n // 2] = a[m // 2, n // 2] * B[m // 2, n // 2]
    for i in range(1, (n + 1) // 2):
        out[0, i] = a[0, i] * B[0, i] - a[0, n - i] * B[0, n - i]
        out[0, n - i] = a[0, i] * B[0, n - i] + a[0, n - i] * B[0, i]
        if meven:
            r = m // 2
            out[r, i] = a[r, i] * B[r, i] - a[r, n - i] * B[r, n - i]
            out[r, n - i] = a[r, i] * B[r, n - i] + a[r, n - i] * B[r, i]
    for i in range(1, (m + 1) // 2):
        out[i, 0] = a[i, 0] * B[i, 0] - a[m - i, 0] * B[m - i, 0]
        out[m - i, 0] = a[i, 0] * B[m - i, 0] + a[m - i, 0] * B[i, 0]
        if neven:
            c = n // 2
            out[i, c] = a[i, c] * B[i, c] - a[m - i, c] * B[m - i, c]
            out[m - i, c] = a[i, c] * B[m - i, c] + a[m - i, c] * B[i, c]
        for j in range(1, (n + 1) // 2):
            out[i, j] = (a[i, j] * B[i, j] + a[m - i, n - j] * B[m - i, n - j] - a[i, n - j] * B[i, n - j]
                         - a[m - i, j] * B[m - i, j])
            out[m - i, n - j] = (a[i, j] * B[m - i, n - j] + a[m - i, n - j] * B[i, j] + a[m - i, j] * B[i, n - j]
                                 + a[i, n - j] * B[m - i, j])
            out[i, n - j] = (a[i, j] * B[i, n - j] - a[m - i, n - j] * B[m - i, j] + a[i, n - j] * B[i, j]
                             - a[m - i, j] * B[m - i, n - j])
            out[m - i, j] = (a[i, j] * B[m - i, j] - a[m - i, n - j] * B[i, n - j] + a[m - i, j] * B[i, j]
                             - a[i, n - j] * B[m - i, n - j])
    return hc2r_2d(out).astype(dt)


def _overlap(i, nimg, corrsize, ncen):
    """offsets/extent of the reference/image overlap for output offset i
    (diffCorrelation/bruteCorrelation, :1228-1240)."""
    off = i - ncen // 2
    mm = min(corrsize, nimg)
    sref = max(0, -off - (nimg - corrsize) // 2)
    sin_ = max(0, (nimg - corrsize) // 2 + off)
    if sin_ + mm > nimg:
        mm = nimg - sin_
    if sref + mm > corrsize:
        mm = corrsize - sref
    return sref, sin_, mm


def diff_correlation(nimg, corrsize, ncen, img, pattern, mode, dt):
    """diffCorrelation (:1203-1338); mode 1: mean squared difference, 3:
    squared difference over the product of the fluxes, 2: the reference's
    abs-difference branch (with its own indexing)."""
    out = np.zeros((corrsize, corrsize), dt)
    c0 = (corrsize - ncen) // 2
    if mode in (1, 3):
        for i in range(ncen):
            srefy, siny, my = _overlap(i, nimg, corrsize, ncen)
            for j in range(ncen):
                srefx, sinx, mx = _overlap(j, nimg, corrsize, ncen)
                s = dt(0)
                tot = dt(0)
                tot2 = dt(0)
                for y in range(my):
                    for x in range(mx):
                        b = dt(img[siny + y, sinx + x])
                        c = dt(pattern[srefy + y, srefx + x])
                        d = dt(c - b)
                        s = dt(s + d * d)
                        tot = dt(tot + b)
                        tot2 = dt(tot2 + c)
                if mode == 1:
                    if mx != 0 and my != 0:
                        out[i + c0, j + c0] = dt(s / (mx * my))
                elif tot != 0 and tot2 != 0:
                    out[i + c0, j + c0] = dt(s / (tot * tot2))
    else:
        flat_out = out.reshape(-1)
        for i in range(ncen):
            my = corrsize - abs(ncen // 2 - i)
            for j in range(ncen):
                mx = corrsize - abs(ncen // 2 - j)
                s = dt(0)
                for y in range(my):
                    for x in range(mx):
                        if i < ncen // 2:
                            if j < ncen // 2:
                                d = pattern.flat[y * corrsize + x] - img.flat[(ncen // 2 - i + y) * nimg + ncen // 2 - j + x]
                            else:
                                d = pattern.flat[y * corrsize + j - ncen // 2 + x] - img.flat[(ncen // 2 - i + y) * nimg + x]
                        else:
                            if j < ncen // 2:
                                d = pattern.flat[(i - ncen // 2 + y) * corrsize + x] - img.flat[y * nimg + ncen // 2 - j + x]
                            else:
                                d = pattern.flat[(i - ncen // 2 + y) * corrsize + j - ncen // 2 + x] - img.flat[y * nimg + x]
                        s = dt(s + abs(dt(d)))
                flat_out[(i + (nimg - ncen) // 2) * corrsize + j + (nimg - ncen) // 2] = dt(s * s / (my * mx))
    return out


def brute_correlation(nimg, corrsize, ncen, img, pattern, dt):
    """bruteCorrelation (:1339-1398): overlap sums of the product."""
    out = np.zeros((corrsize, corrsize), dt)
    c0 = (corrsize - ncen) // 2
    for i in range(ncen):
        srefy, siny, my = _overlap(i, nimg, corrsize, ncen)
        for j in range(ncen):
            srefx, sinx, mx = _overlap(j, nimg, corrsize, ncen)
            s = dt(0)
            for y in range(my):
                for x in range(mx):
                    s = dt(s + dt(pattern[srefy + y, srefx + x] * img[siny + y, sinx + x]))
            if mx != 0 and my != 0:
                out[i + c0, j + c0] = s
    return out


def threshold_correlation(img, thresh, dt):
    """thresholdCorrelation (:1488-1505), in place on the flat image."""
    flat = img.reshape(-1)
    t = dt(thresh)
    if 0 < thresh <= 1:
        mx = dt(0)
        for v in flat:
            if v > mx:
                mx = v
        t = dt(mx * t)
    flat[:] = np.where(flat < t, dt(0), (flat - t).astype(dt))


# counter-based stream of the engine's default noise mode
# ----------------------------------------------------------------------------

def philox4x32_10(ctr, key):
    """Philox4x32-10 (Salmon et al., SC'11) on one 4-word counter, 2-word key."""
    M0, M1 = 0xD2511F53, 0xCD9E8D57
    W0, W1 = 0x9E3779B9, 0xBB67AE85
    c0, c1, c2, c3 = [int(x) & 0xFFFFFFFF for x in ctr]
    k0, k1 = [int(x) & 0xFFFFFFFF for x in key]
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> 32, p0 & 0xFFFFFFFF
        hi1, lo1 = p1 >> 32, p1 & 0xFFFFFFFF
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        k0 = (k0 + W0) & 0xFFFFFFFF
        k1 = (k1 + W1) & 0xFFFFFFFF
    return c0, c1, c2, c3
