"""Host restatements of the reference's phase-screen helpers -- TEST
INFRASTRUCTURE ONLY (tests/ only).

* ``astart_matrix``: the A matrix for extruding at the start of a screen,
  A with its column blocks in reverse order (science/infScrn.py:722-731).
* ``linearshift``: cmod/src/interpmodule.c:1234-1300 (float32 products and
  sums in its order).
* ``pupil_phase``: util/atmos.py:678-833 for a source at infinity: layers
  shifted and added, piston removed over the pupil, times the pupil, times
  500/wavelength.
"""
import numpy as np


def astart_matrix(a, dpix, nb_col=2):
    a = np.asarray(a, np.float64)
    out = np.empty_like(a)
    for col in range(nb_col):
        js, je = col * dpix, (col + 1) * dpix
        # matrixA[:, -(js+1):-(je+1):-1][:, ::-1]
        n = a.shape[1]
        out[:, js:je] = a[:, n - je:n - js]
    return out


def linearshift(inarr, xshift, yshift, ny, nx):
    f32 = np.float32
    x, y = float(np.float32(xshift)), float(np.float32(yshift))
    s1 = f32((1.0 - x) * (1.0 - y))
    s2 = f32((1.0 - x) * y)
    s3 = f32(x * (1.0 - y))
    s4 = f32(np.float32(x) * np.float32(y))
    a = np.asarray(inarr, np.float32)
    o = (a[:ny, :nx] * s1).astype(f32)
    o = (o + (a[1:ny + 1, :nx] * s2).astype(f32)).astype(f32)
    o = (o + (a[:ny, 1:nx + 1] * s3).astype(f32)).astype(f32)
    o = (o + (a[1:ny + 1, 1:nx + 1] * s4).astype(f32)).astype(f32)
    return o


def pupil_phase(screens, layers, pupil, pupil_area=None, wavelength=500.0, remove_piston=True):
    """screens: list of host screens; layers: (index, y0, x0, yshift, xshift)."""
    pupil = np.asarray(pupil, np.float32)
    npup = pupil.shape[0]
    out = np.zeros((npup, npup), np.float32)
    for q, y0, x0, ys, xs in layers:
        win = screens[q][y0:y0 + npup + 1, x0:x0 + npup + 1]
        out = (out + linearshift(win, xs, ys, npup, npup)).astype(np.float32)
    area = float(pupil.astype(np.float64).sum()) if pupil_area is None else pupil_area
    if remove_piston:
        pist = float((out.astype(np.float64) * pupil).sum()) / area
        out = (out - np.float32(pist)).astype(np.float32)
    out = (out * pupil).astype(np.float32)
    return (out * np.float32(500.0 / wavelength)).astype(np.float32)
