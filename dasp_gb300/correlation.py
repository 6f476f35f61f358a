"""Host-side helpers of correlation centroiding: DASP's util/correlation.py
(transformPSF :20-51, r2hc :55-62, r2hc1d :65-74, hc2r1d :76-85, hc2r
:88-95), as ``util/centroid.py`` uses them (:304, :1626, :1653) to turn the
user's reference spot into the pattern that correlation mode 1 multiplies
with (``corrPattern``).  The transform runs once, at initialise/update, on
the host as in the reference; the correlation itself runs on the GPU.

Half-complex layout (FFTW's R2HC): for a length-n axis, position k holds
Re F_k for 0 <= k <= n/2 and position n-k holds Im F_k for 0 < k < (n+1)/2.
The 2-D form transforms the rows (last axis) first, then the columns, with
the intermediate stored in the array's own dtype (the reference assigns each
transformed row back into its float32 array); each 1-D transform is computed
in float64, as the reference's numpy did.
"""
from __future__ import annotations

import numpy as np


def _r2hc_axis(a: np.ndarray, axis: int) -> np.ndarray:
    n = a.shape[axis]
    spec = np.fft.fft(np.asarray(a, np.float64), axis=axis)
    re = np.moveaxis(spec.real, axis, -1)
    im = np.moveaxis(spec.imag, axis, -1)
    out = np.empty(re.shape, np.float64)
    h = n // 2 + 1
    out[..., :h] = re[..., :h]
    # Im F_k at n - k: positions h .. n-1 hold k = (n+1)//2 - 1 .. 1
    out[..., h:] = im[..., (n + 1) // 2 - 1:0:-1]
    return np.ascontiguousarray(np.moveaxis(out, -1, axis), dtype=a.dtype)


def _hc2r_axis(a: np.ndarray, axis: int) -> np.ndarray:
    """Inverse of _r2hc_axis, normalised (numpy's ifft), as hc2r1d."""
    n = a.shape[axis]
    x = np.moveaxis(np.asarray(a, np.float64), axis, -1)
    spec = np.zeros(x.shape, np.complex128)
    h = n // 2 + 1
    spec.real[..., :h] = x[..., :h]
    spec.real[..., h:] = x[..., (n + 1) // 2 - 1:0:-1]
    spec.imag[..., (n + 1) // 2 - 1:0:-1] = x[..., h:]
    spec.imag[..., h:] = -x[..., h:]
    out = np.fft.ifft(spec, axis=-1).real
    return np.ascontiguousarray(np.moveaxis(out, -1, axis), dtype=a.dtype)


def r2hc1d(a):
    """r2hc1d (util/correlation.py:65-74): 1-D real to half-complex."""
    return _r2hc_axis(np.array(a, copy=True), 0)


def hc2r1d(a):
    """hc2r1d (util/correlation.py:76-85): 1-D half-complex to real, divided
    by n (numpy's inverse)."""
    return _hc2r_axis(np.array(a, copy=True), 0)


def r2hc(a):
    """r2hc (util/correlation.py:55-62): rows, then columns, of a 2-D array."""
    a = np.array(a, copy=True)
    return _r2hc_axis(_r2hc_axis(a, -1), -2)


def hc2r(a):
    """hc2r (util/correlation.py:88-95): the inverse of r2hc (normalised)."""
    a = np.array(a, copy=True)
    return _hc2r_axis(_hc2r_axis(a, -1), -2)


def transform_psf(psf):
    """transformPSF (util/correlation.py:20-51): the correlation pattern of a
    reference spot, (nsubx, nsubx, n, n) or (n, n).  Each spot is
    fftshift-ed, transformed to the 2-D half-complex layout, and the signs of
    the two off-diagonal blocks [:n/2+1, n/2+1:] and [n/2+1:, :n/2+1] are
    flipped (the reference's conjugate), so that convolving with the
    pattern's inverse transform is correlating with the spot.  Returns
    float32; None gives None."""
    if psf is None:
        return None
    psf = np.array(psf, copy=True)
    if psf.ndim not in (2, 4):
        raise ValueError("PSF shape wrong: expected (n, n) or (nsubx, nsubx, n, n)")
    ff = r2hc(np.fft.fftshift(psf, axes=(-2, -1)))
    mm = ff.shape[-2] // 2 + 1
    nn = ff.shape[-1] // 2 + 1
    ff[..., :mm, nn:] *= -1
    ff[..., mm:, :nn] *= -1
    return np.ascontiguousarray(ff, dtype=np.float32)


# the reference's name
transformPSF = transform_psf
