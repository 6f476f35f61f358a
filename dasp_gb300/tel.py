"""Telescope pupil geometry for deriving the WFS per-subaperture inputs.

Restates the annular-pupil subset of the reference's ``util/tel.py``:

* ``makeCircularGrid`` (util/tel.py:37-53): pixel-centre distances with the
  grid origin between the two central pixels;
* ``Pupil.__init__`` annulus ``r2 <= grid <= r1`` (util/tel.py:154-165);
* ``getSubapFlag`` / ``getSubarea`` / ``perSubap`` (util/tel.py:564-613), the
  three methods ``centcmod`` calls (util/centcmod.py:76-78).

Hexagonal segments, spiders and pupil maps are out of scope for the WFS step;
any object exposing the same three methods can be passed to ``centcmod``.
"""
from __future__ import annotations

import numpy as np


def circular_grid(npup: int, dtype=np.float64) -> np.ndarray:
    """Distance of each pixel centre from the array centre (util/tel.py:37-53)."""
    tab = np.arange(npup) - npup / 2.0 + 0.5
    grid = np.sqrt(tab[np.newaxis, :] ** 2 + tab[:, np.newaxis] ** 2)
    return grid.astype(dtype)


class Pupil:
    """Annular telescope pupil sampled on an ``npup`` x ``npup`` grid.

    ``r1``/``r2`` are the outer/inner radii in pixels; ``fn`` is the 0/1 map.
    """

    def __init__(self, npup: int, r1: float | None = None, r2: float = 0.0,
                 nsubx: int | None = None, minarea: float = 0.5):
        self.npup = int(npup)
        self.r1 = npup / 2.0 if r1 is None else float(r1)
        self.r2 = float(r2)
        self.nsubx = nsubx
        self.minarea = minarea
        grid = circular_grid(self.npup)
        self.fn = np.logical_and(grid <= self.r1, grid >= self.r2)
        self.area = float(self.fn.sum())

    def _blocks(self, nsubx: int) -> np.ndarray:
        n = self.npup // nsubx
        f = self.fn[: n * nsubx, : n * nsubx]
        return f.reshape(nsubx, n, nsubx, n).transpose(0, 2, 1, 3)

    def getSubarea(self, nsubx: int) -> np.ndarray:
        """Illuminated pixel count per subaperture, float64 (nsubx, nsubx)."""
        return self._blocks(nsubx).sum(axis=(2, 3)).astype(np.float64)

    def getSubapFlag(self, nsubx: int, minarea: float | None = None) -> np.ndarray:
        """1 where the subaperture area is at least ``minarea`` of full."""
        if minarea is None:
            minarea = self.minarea
        n = self.npup // nsubx
        return (self.getSubarea(nsubx) >= minarea * n * n).astype(np.int32)

    def perSubap(self, nsubx: int | None = None, vectorAlign: int = 1) -> np.ndarray:
        """Per-subaperture pupil, float32 (nsubx, nsubx, n, n[_aligned])."""
        if nsubx is None:
            nsubx = self.nsubx
        if nsubx is None:
            raise ValueError("Number of x subaps must be defined")
        n = self.npup // nsubx
        nv = (n + 3) & ~3 if vectorAlign else n
        out = np.zeros((nsubx, nsubx, n, nv), np.float32)
        out[:, :, :, :n] = self._blocks(nsubx).astype(np.float32)
        return out
