"""Infinite phase screen on the device: DASP's infScrn column/row extrusion
(science/infScrn.py) with the screen resident in HBM.

DASP's ``infScrn`` keeps a (scrnYPxls+1) x (scrnXPxls+1) screen and, as the
wind moves it, appends columns (rows) computed from the last two by the
method of Assemat, Wilson and Gendron (Optics Express 14, 2006): with Z the
last two columns and X the new one, X = A Z + B n, n ~ N(0, 1) per pixel,
A = <XZ^T><ZZ^T>^-1 and B B^T = <XX^T> - A <ZX^T>, from the von Karman phase
covariance (computePhaseCovarianceMatrix :549-611, computeAandBmatrices
:672-746, addNewColumnOnEnd :747-791, addNewRowOnEnd :825-855).  The host
builds A and B once, in float64 as the reference does; each step the device
computes the new columns in float64, writes them into a circular buffer (no
shifting of the screen) and cuts the sensor's phase window out of it, so the
per-frame phase never crosses the host link.  Noise comes from the
counter-based Philox stream, or from an array the caller injects (to
reproduce a given sequence of normals exactly).
"""
from __future__ import annotations

import ctypes

import numpy as np


def _distance_map(n, m, dy, dx):
    """distanceMap (science/infScrn.py:158-191): float32 distances of an
    n x m grid from its offset centre."""
    ax = (np.arange(m) - m / 2. - dx) * 1.0
    ay = (np.arange(n) - n / 2. - dy) * 1.0
    return np.sqrt(ay[:, None] ** 2. + ax[None, :] ** 2.).astype(np.float32)


def phase_covariance(dpix, L0, pix_scale, nb_col_to_add=1, nb_col=2):
    """Covariance of the phase at nb_col + nb_col_to_add columns of dpix
    points (points ordered column by column, rows ascending), for L0/r0 = 1
    (science/infScrn.py:549-611)."""
    from scipy.special import gamma, kv
    nc = nb_col + nb_col_to_add
    npts = nc * dpix
    f0 = 1. / L0
    coeff = 2 * gamma(11. / 6) / (2 ** (5. / 6)) / (np.pi ** (8. / 3))
    coeff *= (24. / 5 * gamma(6. / 5)) ** (5. / 6)
    sigma2 = coeff / 2. * gamma(5. / 6) / (2 ** (1. / 6))
    dist = _distance_map(nc * 2 - 1, dpix * 2 - 1, -0.5, -0.5) * np.float32(pix_scale * 2 * np.pi * f0)
    with np.errstate(invalid="ignore"):
        c = dist ** np.float32(5. / 6)
        c *= kv(5. / 6, dist).astype(np.float32)  # the zero distance is the variance, set below
    c *= np.float32(coeff / 2.)
    cov = np.empty((npts, npts), np.float64)
    for i in range(npts):
        ic, jc = i % dpix, i // dpix
        line = np.ravel(c[nc - 1 - jc:nc * 2 - 1 - jc, dpix - 1 - ic:dpix * 2 - 1 - ic]).astype(np.float64)
        line[jc * dpix + ic] = sigma2
        cov[i, i:] = line[i:]
        cov[i:, i] = line[i:]
    return cov


def extrusion_matrices(dpix, cov, nb_col_to_add=1, nb_col=2):
    """A (dpix x nb_col*dpix) and B (dpix x dpix) of one axis
    (science/infScrn.py:672-746); B from the SVD of <XX^T> - A<ZX^T>."""
    import scipy.linalg as la
    n = dpix * (nb_col + nb_col_to_add)
    m = dpix * nb_col_to_add
    zz = cov[:n - m, :n - m]
    xx = cov[n - m:, n - m:]
    xz = cov[n - m:, :n - m]
    zx = cov[:n - m, n - m:]
    try:
        zz_inv = la.cho_solve(la.cho_factor(zz), np.identity(nb_col * dpix))
    except la.LinAlgError:
        zz_inv = la.inv(zz)
    a = xz @ zz_inv
    u, w, _ = la.svd(xx - a @ zx)
    b = u * np.sqrt(w)[None, :]
    return np.ascontiguousarray(a), np.ascontiguousarray(b)


def new_column_host(screen_cols2, a, b, rn, coeff_turb, step=0.0):
    """One extruded column (host restatement, float64): A Z + coeff B n +
    step, Z the two last columns stacked (older first)."""
    z = np.ravel(np.asarray(screen_cols2, np.float64).T)
    return a @ z + (b @ np.asarray(rn, np.float64)) * coeff_turb + step


class DeviceScreen:
    """A (ny x nx) infinite phase screen held on the GPU.

    ``ay, by`` extrude columns (length ny), ``ax, bx`` rows (length nx), as
    built by :func:`extrusion_matrices`; ``init`` is the starting screen.
    ``add_columns(n, r0)`` / ``add_rows(n, r0)`` append at the end with the
    random part scaled by (L0/r0)^(5/6) (science/infScrn.py:764);
    ``window(y0, x0, out)`` writes the phase a sensor sees into a CUDA tensor.
    """

    def __init__(self, init, L0, ay=None, by=None, ax=None, bx=None, seed=0):
        from . import _lib
        self._lib = _lib
        init = np.ascontiguousarray(init, np.float32)
        self.ny, self.nx = init.shape
        self.L0 = float(L0)
        keep = [np.ascontiguousarray(m, np.float64) if m is not None else None for m in (ay, by, ax, bx)]
        for m, shape in zip(keep, ((self.ny, 2 * self.ny), (self.ny, self.ny), (self.nx, 2 * self.nx),
                                   (self.nx, self.nx))):
            if m is not None and m.shape != shape:
                raise ValueError("extrusion matrix of shape %s, expected %s" % (m.shape, shape))
        ptr = [None if m is None else m.ctypes.data for m in keep]
        s = ctypes.c_void_p()
        _lib.check(_lib.lib().shwfs_screen_create(self.ny, self.nx, init.ctypes.data, ptr[0], ptr[1], ptr[2], ptr[3],
                                                  int(seed), ctypes.byref(s)), "screen_create")
        self._s = s

    @classmethod
    def von_karman(cls, ny, nx, pix_scale, r0, L0, seed=0, axes=("columns",)):
        """A screen with the matrices of the requested axes built on the
        host and an FFT-method initial screen (seeded)."""
        from .screens import von_karman_screen
        n = max(ny, nx)
        big = von_karman_screen(n, n * pix_scale, r0, L0, seed, 500.0)
        mats = {}
        if "columns" in axes:
            mats["ay"], mats["by"] = extrusion_matrices(ny, phase_covariance(ny, L0, pix_scale))
        if "rows" in axes:
            mats["ax"], mats["bx"] = extrusion_matrices(nx, phase_covariance(nx, L0, pix_scale))
        return cls(big[:ny, :nx], L0, seed=seed, **mats)

    def _add(self, axis, n, r0, step, noise, stream):
        coeff = (self.L0 / r0) ** (5. / 6)
        if noise is not None:
            noise = np.ascontiguousarray(noise, np.float64)
            if noise.size != n * self._check_noise_axis(axis):
                raise ValueError("noise must hold n * (screen height or width) values")
            if stream is not None:
                # the host-to-device copies of the normals read the array
                # after this call returns
                raise ValueError("injected noise needs stream=None (the call waits for its copies)")
        s = getattr(stream, "cuda_stream", stream)
        self._lib.check(self._lib.lib().shwfs_screen_add(self._s, axis, int(n), coeff, float(step),
                                                         None if noise is None else noise.ctypes.data, s),
                        "screen_add")

    # With ``stream`` (torch stream or raw handle) the extrusions are queued
    # there and not waited for; without, the call waits on the screen's own
    # stream.

    def add_columns(self, n, r0, step=0.0, noise=None, stream=None):
        self._add(0, n, r0, step, noise, stream)

    def add_rows(self, n, r0, step=0.0, noise=None, stream=None):
        self._add(1, n, r0, step, noise, stream)

    def add_columns_start(self, n, r0, step=0.0, noise=None, stream=None):
        """n new columns at the start (the wind blowing the other way;
        addNewColumnOnStart, science/infScrn.py:793-823): the last column is
        dropped for each."""
        self._add(2, n, r0, step, noise, stream)

    def add_rows_start(self, n, r0, step=0.0, noise=None, stream=None):
        """n new rows at the start (addNewRowOnStart, science/infScrn.py:
        857-887)."""
        self._add(3, n, r0, step, noise, stream)

    def window(self, y0, x0, out, stream=None):
        """The out.shape[-2:] window at (y0, x0) into the CUDA tensor out."""
        h, w = out.shape[-2], out.shape[-1]
        if not (out.is_cuda and out.is_contiguous() and str(out.dtype) == "torch.float32"):
            raise ValueError("out must be a contiguous float32 CUDA tensor")
        s = getattr(stream, "cuda_stream", stream)
        self._lib.check(self._lib.lib().shwfs_screen_window(self._s, int(y0), int(x0), h, w, out.data_ptr(), w, s),
                        "screen_window")

    def _check_noise_axis(self, axis):
        return self.ny if axis in (0, 2) else self.nx

    def numpy(self):
        out = np.empty((self.ny, self.nx), np.float32)
        self._lib.check(self._lib.lib().shwfs_screen_read(self._s, out.ctypes.data), "screen_read")
        return out

    def free(self):
        if getattr(self, "_s", None) is not None:
            self._lib.lib().shwfs_screen_free(self._s)
            self._s = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def pupil_phase(layers, pupil, out, pupil_area=None, wavelength=500.0, remove_piston=True, stream=None):
    """Pupil phase of a source at infinity from several device screens
    (util/atmos.py:678-833, createPupilPhs for an NGS): ``layers`` is a list
    of ``(screen, y0, x0, yshift, xshift)`` -- the (npup+1)-square window of
    the screen at logical (y0, x0) and its fractional row / column shifts in
    [0, 1] (linearshift, cmod/src/interpmodule.c:1234-1300) -- added in the
    order given (the reference sorts by height); the piston over ``pupil``
    is removed, the result multiplied by ``pupil`` and by 500/wavelength.
    ``pupil`` and ``out`` are npup x npup float32 CUDA tensors."""
    from . import _lib
    n = len(layers)
    npup = int(out.shape[-1])
    for t in (pupil, out):
        if not (t.is_cuda and t.is_contiguous() and str(t.dtype) == "torch.float32" and tuple(t.shape) == (npup, npup)):
            raise ValueError("pupil and out must be npup x npup contiguous float32 CUDA tensors")
    if pupil_area is None:
        pupil_area = float(pupil.double().sum().item())
    arr_s = (ctypes.c_void_p * n)(*[ly[0]._s.value for ly in layers])
    y0 = (ctypes.c_int * n)(*[int(ly[1]) for ly in layers])
    x0 = (ctypes.c_int * n)(*[int(ly[2]) for ly in layers])
    ys = (ctypes.c_float * n)(*[float(ly[3]) for ly in layers])
    xs = (ctypes.c_float * n)(*[float(ly[4]) for ly in layers])
    s = getattr(stream, "cuda_stream", stream)
    _lib.check(_lib.lib().shwfs_screens_pupil_phase(arr_s, n, y0, x0, ys, xs, npup, pupil.data_ptr(),
                                                    float(pupil_area), 1 if remove_piston else 0,
                                                    float(500.0 / wavelength), out.data_ptr(), s),
               "screens_pupil_phase")
    return out
