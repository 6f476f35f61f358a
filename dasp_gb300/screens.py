"""Synthetic WFS inputs: von Karman phase screens and spot PSFs.

* ``von_karman_screen`` restates ``makeInitialScreen``
  (science/infScrn.py:244-343): white Gaussian noise from the legacy MT19937
  ``numpy.random.RandomState(seed).randn`` coloured by the von Karman
  spectrum ``(f^2 + f0^2)^(-11/12)`` with the same normalisation constant, on
  an FFT grid of ``max(round(dpix*scrnSize/Dtel), npix)`` pixels.
* ``gaussian_psf`` restates ``util.elong.Gauss.make`` (util/elong.py:22-52).
* ``lgs_psfs`` restates the per-subaperture elongated-spot geometry of
  ``util.elong.make`` (util/elong.py:418-486), parameterised directly in
  detector pixels.

These generate inputs only; nothing here runs in the per-frame path.
"""
from __future__ import annotations

import math

import numpy as np


def von_karman_screen(npix: int, Dtel: float, r0: float, L0: float, seed: int,
                      wavelength_nm: float = 500.0, dpix: int | None = None) -> np.ndarray:
    """float32 ``npix`` x ``npix`` phase screen in radians at ``wavelength_nm``.

    ``r0`` is quoted at 500 nm; the screen is scaled by 500/wavelength, which
    is the same as using r0 * (wavelength/500)^(6/5).
    """
    if dpix is None:
        dpix = npix
    if L0 >= Dtel:
        scrn_size = 2 * L0
    elif Dtel >= 2 * L0:
        scrn_size = Dtel
    else:
        scrn_size = 2 * L0
    nfft = int(np.around(dpix * 1.0 * scrn_size / Dtel))
    nfft = max(nfft, npix)
    rn = np.random.RandomState(seed).randn(nfft, nfft)
    axe = np.arange(nfft) - nfft / 2.0
    f = np.sqrt(axe[:, None] ** 2 + axe[None, :] ** 2)
    ff = np.fft.fftshift(f)
    fact = math.gamma(11.0 / 6.0) ** 2
    fact /= 2 * math.pi ** (11.0 / 3.0)
    fact *= ((24.0 / 5) * math.gamma(6.0 / 5)) ** (5.0 / 6)
    f0 = 1.0 / L0 * scrn_size
    spec = (ff ** 2 + f0 ** 2) ** (-11.0 / 12.0)
    spec *= np.sqrt(fact * ((scrn_size / r0) ** (5.0 / 3.0)) * (nfft * 1.0) ** 2)
    w = np.fft.fft2(rn)
    w.real *= spec
    w.imag *= spec
    phi = np.fft.ifft2(w).real
    return (phi[:npix, :npix] * (500.0 / wavelength_nm)).astype(np.float32)


def gaussian_psf(n: int, fwhmx: float, fwhmy: float | None = None, th: float = 0.0,
                 xoff: float = 0.0, yoff: float = 0.0) -> np.ndarray:
    """2-D Gaussian spot on an ``n`` x ``n`` grid, float32 (peak 1)."""
    if fwhmy is None:
        fwhmy = fwhmx
    sig2x = fwhmx ** 2 / (8.0 * np.log(2.0))
    sig2y = fwhmy ** 2 / (8.0 * np.log(2.0))
    thr = th * np.pi / 180.0
    a = np.cos(thr) ** 2 / (2.0 * sig2x) + np.sin(thr) ** 2 / (2.0 * sig2y)
    b = np.sin(2.0 * thr) / (4.0 * sig2y) - np.sin(2.0 * thr) / (4.0 * sig2x)
    c = np.sin(thr) ** 2 / (2.0 * sig2x) + np.cos(thr) ** 2 / (2.0 * sig2y)
    i, j = np.meshgrid(np.arange(n, dtype=np.float64), np.arange(n, dtype=np.float64), indexing="ij")
    x = i - n // 2 + 0.5 - xoff
    y = j - n // 2 + 0.5 - yoff
    return np.exp(-1.0 * (c * y * y + 2.0 * b * x * y + a * x * x)).astype(np.float32)


def lgs_psfs(nsubx: int, spotsize: int, fwhm_across: float = 1.2, max_elong: float = 6.0,
             launch_dist_frac: float = 1.0, launch_theta_deg: float = 0.0,
             subap_area: np.ndarray | None = None) -> np.ndarray:
    """Per-subaperture elongated Gaussian spots (nsubx, nsubx, spotsize, spotsize).

    Elongation grows with distance from the launch point (a fraction of the
    pupil radius from the centre, at ``launch_theta_deg``), reaching
    ``max_elong`` pixels FWHM at the farthest subaperture; spots point
    radially away from the launch point (util/elong.py:458-477).  Each spot is
    normalised to unit sum times its illuminated area fraction when
    ``subap_area`` (fraction 0..1 per subaperture) is given.
    """
    theta = (launch_theta_deg - 90.0) * np.pi / 180.0
    lx = launch_dist_frac * nsubx / 2.0 * np.cos(theta)
    ly = launch_dist_frac * nsubx / 2.0 * np.sin(theta)
    pos = np.arange(nsubx) - nsubx / 2.0 + 0.5
    xs, ys = np.meshgrid(pos + lx, pos + ly, indexing="ij")
    r = np.sqrt(xs * xs + ys * ys)
    rmax = r.max() if r.max() > 0 else 1.0
    out = np.zeros((nsubx, nsubx, spotsize, spotsize), np.float32)
    for a in range(nsubx):
        for b in range(nsubx):
            phi = np.arctan2(xs[a, b], ys[a, b]) * 180.0 / np.pi
            e = np.sqrt((max_elong * r[a, b] / rmax) ** 2 + fwhm_across ** 2)
            g = gaussian_psf(spotsize, fwhm_across, e, phi).astype(np.float64)
            g /= g.sum()
            if subap_area is not None:
                g *= subap_area[a, b]
            out[a, b] = g
    return out
