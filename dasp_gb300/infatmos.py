"""A layered atmosphere on the device: DASP's atmosphere geometry and
infScrn/infAtmos frame bookkeeping driving the device-resident screens.

In DASP a simulation's atmosphere is described by ``util.atmos.geom`` (layers
with height, wind and Cn2 fraction; sources with direction and height).  Each
layer is an ``infScrn`` that grows its screen as the wind blows, and
``infAtmos`` keeps the layers' screens and, per source, cuts out and sums the
phase the telescope sees (``util.atmos.atmos.createPupilPhs``).  This module
restates the host-side arithmetic of that chain:

* :class:`AtmosGeom` -- the screen sizes and layer offsets
  (util/atmos.py:109-390, ``getScrnSize`` / ``getLayerOffset`` without
  rotated directions), the zenith scaling of layers and r0 (:40-62, :122);
* :func:`wind_steps` -- the fractional columns / rows a layer moves per frame
  (science/infAtmos.py:188-197, science/infScrn.py:386-390);
* :class:`NewCols` -- how many whole lines to add each frame and the
  remaining sub-pixel position (util/getNewCols.py);
* :class:`AtmosFrames` -- per frame, the lines each layer's screen gains
  and, for a source, where each layer's window starts and its sub-pixel
  shift (util/atmos.py:590-640 and :696-720);

and :class:`DeviceAtmosphere` applies it to one :class:`DeviceScreen` per
layer: each frame it extrudes the lines infAtmos adds (at the end of a screen
when the step is negative, at the start otherwise; columns before rows, as
infScrn does), and forms a source's pupil phase from the layers' windows with
``pupil_phase`` -- all on the device.

infAtmos places the lines it receives with ``getNewCols.nextOld`` and takes
its interpolation positions from the same counter (science/infAtmos.py:
366-368), so the pupil sees the wind move the screen by exactly the step per
frame; the device screens follow that counter.  (infScrn's own screen follows
``next``, which adds a line one frame earlier whenever the position is an
integer; infAtmos receives it a frame later.)

For an LGS each layer below it is seen through the cone's width and
expanded to the pupil by the natural cubic spline DASP uses
(gslCubSplineInterp, util/atmos.py:788-799); uplink tip/tilt is not built,
and neither are screens generated along one axis and rotated
(``rotateDirections``).  The reference's elliptical-pupil stretching for
zenith angles is disabled in the reference itself (``zenithOld`` is always
0), so windows are npup wide at every zenith angle.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, replace

import numpy as np

# angle units as util/atmos.py writes them (2 pi / 360 per degree)
_DEG = 2 * np.pi / 360.
_ARCSEC = 2 * np.pi / 360. / 3600.
OVERSIZE = 5  # util/atmos.py:121: screen pixels beyond the sources' footprint


def _next_lines(pos, extra, step, integer_fix):
    """One frame of util/getNewCols.py: the screen has moved to pos + step
    pixels; ``extra`` lines beyond its standard size are held.  Returns
    (lines dropped, lines to add, new sub-pixel position, new extra).
    ``integer_fix`` adds the line an integer position needs at once (``next``,
    :24-34); without it (``nextOld``, :37-47) that line comes a frame later."""
    target = pos + step
    dropped = math.floor(target)
    add = int(math.ceil(target) - extra)
    if integer_fix and target % 1 == 0:
        add += 1
    return dropped, add, target - dropped, extra + add - dropped


class NewCols:
    """Lines to add per frame for a screen moving ``step`` pixels per frame
    (util/getNewCols.py ``getNewCols``)."""

    def __init__(self, step):
        self.step = float(step)
        self.pos = 0.
        self.extra = 0
        self.nadd = 0

    def _frame(self, integer_fix):
        dropped, self.nadd, self.pos, self.extra = _next_lines(self.pos, self.extra, self.step, integer_fix)
        return dropped, self.nadd, self.pos

    def next(self):
        """(lines to remove, lines to add, interpolation position): infScrn's counter."""
        return self._frame(True)

    def next_old(self):
        """The same with the line at integer positions a frame late: infAtmos's counter."""
        return self._frame(False)


@dataclass
class Layer:
    """One turbulent layer (util/atmos.py:25-38): height (m), wind direction
    (degrees), wind speed (m/s), strength (fraction of Cn2), seed."""
    height: float
    direction: float
    speed: float
    strength: float
    seed: int = 0

    def at_zenith(self, zenith, zenith_az):
        """The layer along a line of sight ``zenith`` degrees from the zenith
        towards azimuth ``zenith_az`` (adjustForZenith, util/atmos.py:40-62):
        height stretched by 1/cos(zenith), the wind component along the
        azimuth foreshortened."""
        if zenith == 0.:
            return replace(self)
        rad = np.pi / 180.
        rel = (zenith_az - self.direction) * rad
        vx = self.speed * np.cos(rel) * np.cos(zenith * rad)
        vy = self.speed * np.sin(rel)
        return replace(self, height=self.height / np.cos(zenith * rad), speed=float(np.sqrt(vx * vx + vy * vy)),
                       direction=float(zenith_az - np.arctan(np.tan(rel) / np.cos(zenith * rad)) / rad))


@dataclass
class Source:
    """A line of sight (util/atmos.py:64-93): ``theta`` off axis (arcsec),
    ``phi`` azimuth (degrees), ``alt`` -1 for a star at infinity (else the
    LGS height, m), ``fov`` radius of an extended source (arcsec), ``lam``
    wavelength of the phase (nm)."""
    idstr: str
    theta: float = 0.
    phi: float = 0.
    alt: float = -1.
    fov: float = 0.
    lam: float = 500.


class AtmosGeom:
    """Atmosphere and source geometry (util/atmos.py ``geom``): ``layers``
    maps layer ids to :class:`Layer`, ``sources`` lists :class:`Source`;
    ``ntel`` pixels across the telescope diameter ``tel_diam`` (m), ``npup``
    pixels across the pupil array, ``r0`` (m at 500 nm, at zenith) and
    ``l0`` (m)."""

    def __init__(self, layers, sources, ntel, npup, tel_diam, r0, l0, zenith=0., zenith_az=0.):
        self.zenith, self.zenith_az = float(zenith), float(zenith_az)
        self.r0 = r0 * np.cos(self.zenith * np.pi / 180.) ** 0.6
        self.l0 = float(l0)
        total = sum(ly.strength for ly in layers.values())
        self.layers = {}
        for key, ly in layers.items():
            ly = ly.at_zenith(self.zenith, self.zenith_az)
            if total != 1.:
                ly = replace(ly, strength=ly.strength / total)
            self.layers[key] = ly
        self.sources = {}
        for s in sources:
            if self.zenith != 0 and s.alt > 0:
                s = replace(s, alt=s.alt / np.cos(self.zenith * np.pi / 180.))
            old = self.sources.get(s.idstr)
            if old is not None and (old.alt, old.theta, old.phi, old.lam) != (s.alt, s.theta, s.phi, s.lam):
                raise ValueError("source %r defined twice with different directions" % s.idstr)
            self.sources.setdefault(s.idstr, s)
        self.ntel, self.npup, self.tel_diam = int(ntel), int(npup), float(tel_diam)

    @classmethod
    def from_reference(cls, g, default_lam=500.):
        """The geometry of a reference ``util.atmos.geom`` object (duck-typed:
        ``layerDict``, ``sourceOrder``/``sourceDict``, ``ntel``, ``npup``,
        ``telDiam``, ``r0``, ``l0``, ``zenith``, ``zenithAz``), as a parameter
        file builds it.  That object has already scaled its layers, LGS
        heights and r0 for its zenith angle and normalised the strengths,
        so they are taken as they are.  A source's wavelength is its
        ``sourcelam`` (science/infAtmos.py:245), else ``default_lam``."""
        obj = cls({}, [], g.ntel, g.npup, g.telDiam, 1.0, g.l0)
        obj.zenith, obj.zenith_az = float(g.zenith), float(getattr(g, "zenithAz", 0.))
        obj.r0 = g.r0
        obj.layers = {k: Layer(float(ly.height), float(ly.direction), float(ly.speed), float(ly.strength),
                               int(getattr(ly, "seed", 0) or 0)) for k, ly in g.layerDict.items()}
        order = getattr(g, "sourceOrder", None) or list(g.sourceDict)
        for k in order:
            s = g.sourceDict[k]
            lam = getattr(s, "sourcelam", None)
            obj.sources[s.idstr] = Source(s.idstr, float(s.theta), float(s.phi), float(s.alt),
                                          float(getattr(s, "fov", 0.) or 0.), float(lam if lam else default_lam))
        return obj

    def layer_r0(self, key):
        """r0 of one layer: r0 * strength^(-3/5) (science/infScrn.py:272, :411-420)."""
        return self.r0 * self.layers[key].strength ** (-3. / 5)

    def screen_size(self, key):
        """(scrnXPxls, scrnYPxls) of a layer (getScrnSize, util/atmos.py:273-312):
        the pupil, OVERSIZE pixels, and the spread of the sources' lines of
        sight (with their fields of view) at the layer's height.  The screen
        itself is one pixel larger each way (science/infScrn.py:328)."""
        h = self.layers[key].height
        xs, ys = [], []
        for s in self.sources.values():
            x = h * np.tan(s.theta * _ARCSEC) * np.cos(s.phi * _DEG)
            # the reference widens the y extent by the field of view times
            # sqrt(2) inside the tangent
            y = h * np.tan((s.theta + s.fov * np.sqrt(2)) * _ARCSEC) * np.sin(s.phi * _DEG)
            xf = h * np.tan(s.fov * _ARCSEC)
            yf = h * np.tan(s.fov * _ARCSEC)
            xs += [x + xf, x - xf]
            ys += [y + yf, y - yf]
        # unrotated square pupil: its width is npup pixels
        base = int(np.ceil(self.npup * 1.0)) + int(OVERSIZE)
        return (base + int(np.ceil((max(xs) - min(xs)) * self.ntel / self.tel_diam)),
                base + int(np.ceil((max(ys) - min(ys)) * self.ntel / self.tel_diam)))

    def layer_offsets(self):
        """({layer: x offset}, {layer: y offset}) in pixels (getLayerOffset,
        util/atmos.py:324-379): shifts that put every source's window at
        non-negative indices of its layer."""
        xo, yo = {}, {}
        for key, ly in self.layers.items():
            h = ly.height
            xs, ys = [], []
            for s in self.sources.values():
                t = np.tan(s.theta * _ARCSEC)
                x = t * np.cos(s.phi * _DEG) * h / self.tel_diam * self.ntel - self.npup / 2.
                y = t * np.sin(s.phi * _DEG) * h / self.tel_diam * self.ntel - self.npup / 2.
                f = np.tan(s.fov * _ARCSEC) * h / self.tel_diam * self.ntel
                xs += [x + f, x - f]
                ys += [y + f, y - f]
            xo[key] = _offset(min(xs))
            yo[key] = _offset(min(ys))
        return xo, yo


def _offset(lo):
    return int(np.ceil(np.fabs(lo))) if lo < 0. else -int(np.floor(lo))


def wind_steps(layer, pix_scale, tstep):
    """(colAdd, rowAdd): pixels the layer moves per frame along columns and
    rows (science/infAtmos.py:188-193): negative adds lines at the end of the
    screen, positive (or zero) at the start."""
    col = -layer.speed * np.cos(layer.direction * np.pi / 180) / pix_scale * tstep
    row = -layer.speed * np.sin(layer.direction * np.pi / 180) / pix_scale * tstep
    return (0. if col == 0 else float(col)), (0. if row == 0 else float(row))


@dataclass
class LayerFrame:
    """One layer's frame state: its wind steps, line counters and infAtmos'
    sub-pixel positions (interpPosCol / interpPosRow)."""
    key: str
    height: float
    r0: float
    col_add: float
    row_add: float
    shape: tuple  # the screen's (rows, columns): (scrnYPxls + 1, scrnXPxls + 1)
    cols: NewCols = None
    rows: NewCols = None
    pos_col: float = 0.
    pos_row: float = 0.

    def __post_init__(self):
        self.cols = NewCols(abs(self.col_add))
        self.rows = NewCols(abs(self.row_add))


class AtmosFrames:
    """The frame-by-frame bookkeeping of infAtmos for the layers of an
    :class:`AtmosGeom` (host only): per frame, how many columns and rows each
    layer's screen gains and at which end, and where each layer's window
    lies for a source.  ``tstep`` is the frame time (s)."""

    def __init__(self, geom, tstep):
        self.geom = geom
        self.tstep = float(tstep)
        self.pix_scale = geom.tel_diam / geom.npup      # screens' pixel scale (infScrn, infAtmos)
        self.scrn_scale = geom.tel_diam / geom.ntel     # source positions (util/atmos.py)
        heights = [ly.height for ly in geom.layers.values()]
        if len(set(heights)) != len(heights):
            raise ValueError("layers need distinct heights (the reference sorts them by height)")
        self.xoff, self.yoff = geom.layer_offsets()
        self.layers = []
        for key in sorted(geom.layers, key=lambda k: geom.layers[k].height):
            ly = geom.layers[key]
            xpx, ypx = geom.screen_size(key)
            col_add, row_add = wind_steps(ly, self.pix_scale, self.tstep)
            self.layers.append(LayerFrame(key, ly.height, geom.layer_r0(key), col_add, row_add, (ypx + 1, xpx + 1)))
        self.frames = 0

    def advance(self):
        """One frame (science/infAtmos.py:366-402): per layer, lowest first,
        (columns to add, at the end?, rows to add, at the end?) -- lines go
        at the end of a screen when its step is negative, else at the start;
        columns are extruded before rows."""
        plan = []
        for lf in self.layers:
            _, ncol, lf.pos_col = lf.cols.next_old()
            _, nrow, lf.pos_row = lf.rows.next_old()
            plan.append((ncol, lf.col_add < 0, nrow, lf.row_add < 0))
        self.frames += 1
        return plan

    def windows(self, idstr):
        """The :class:`Window` of every layer the source sees this frame,
        lowest first (util/atmos.py:590-640 for the static position, :696-720
        for the sub-pixel motion).  A star at infinity sees every layer
        through an npup-wide window; an LGS at height H sees only the layers
        below it, each through the cone's width npup (1 - h/H) (rounded),
        centred on its line of sight."""
        src = self.geom.sources[idstr]
        npup = self.geom.npup
        xpos = np.tan(src.theta * _ARCSEC) * np.cos(src.phi * _DEG)
        ypos = np.tan(src.theta * _ARCSEC) * np.sin(src.phi * _DEG)
        out = []
        for i, lf in enumerate(self.layers):
            if not (src.alt < 0 or src.alt >= lf.height):
                continue  # a layer above the LGS
            x = xpos * lf.height / self.scrn_scale - npup / 2 + self.xoff[lf.key]
            y = ypos * lf.height / self.scrn_scale - npup / 2 + self.yoff[lf.key]
            ny, nx = lf.shape
            if x < 0 or y < 0 or x + npup + 1 > nx or y + npup + 1 > ny:
                raise ValueError("layer %r's screen does not contain source %r" % (lf.key, idstr))
            width = npup
            if src.alt > 0:
                cone = npup * (1. - lf.height / src.alt)
                x = x + (npup - cone) / 2
                y = y + (npup - cone) / 2
                width = int(cone + 0.5)
            col = (x - np.floor(x)) + _frame_shift(lf.col_add, lf.pos_col)
            row = (y - np.floor(y)) + _frame_shift(lf.row_add, lf.pos_row)
            dc, dr = int(np.floor(col)), int(np.floor(row))
            out.append(Window(i, int(y) + dr, int(x) + dc, float(row - dr), float(col - dc), width))
        return out


@dataclass(frozen=True)
class Window:
    """What one layer contributes to a source's pupil phase: the
    (width+1)-square window of the layer's screen at row y0, column x0,
    shifted by (yshift, xshift) in [0, 1) (linearshift) to width x width,
    then, for an LGS (width < npup), expanded to npup x npup by a natural
    cubic spline."""
    layer: int     # index into AtmosFrames.layers (lowest first)
    y0: int
    x0: int
    yshift: float
    xshift: float
    width: int


def spline_matrix(width, npup):
    """S (npup x width, float64) with S @ v the natural cubic spline through
    (i, v[i]), i = 0 .. width-1, evaluated at i (width-1)/(npup-1),
    i = 0 .. npup-1: the axes the reference hands to gslCubSplineInterp for
    an LGS's cone (util/atmos.py:619-623, :788-799), whose spline is GSL's
    ``gsl_interp_cspline`` (natural end conditions), applied along both axes
    (cmod/src/interpmodule.c ``gslCubSplineIntrp``).  With unit knot spacing
    the second derivatives m solve m[i-1] + 4 m[i] + m[i+1] = 6 (v[i+1] -
    2 v[i] + v[i-1]) with m[0] = m[width-1] = 0, and on [i, i+1] at offset
    t the spline is v[i] + b t + m[i]/2 t^2 + (m[i+1] - m[i])/6 t^3 with
    b = v[i+1] - v[i] - (2 m[i] + m[i+1])/6 -- all linear in v."""
    if width < 3:
        raise ValueError("a cubic spline needs at least 3 points (cone width %d)" % width)
    n = width
    # m = M @ v: the tridiagonal solve applied to the second differences
    d2 = np.zeros((n - 2, n))
    for i in range(n - 2):
        d2[i, i:i + 3] = (6., -12., 6.)
    tri = np.diag(np.full(n - 2, 4.)) + np.diag(np.ones(n - 3), 1) + np.diag(np.ones(n - 3), -1)
    mm = np.zeros((n, n))
    mm[1:-1] = np.linalg.solve(tri, d2)
    xs = np.arange(npup, dtype=np.float64) * ((width - 1) / float(npup - 1))
    S = np.zeros((npup, n))
    for r, x in enumerate(xs):
        i = min(int(np.floor(x)), n - 2)  # the last point closes the last interval
        t = x - i
        e = np.zeros(n)
        e[i], e[i + 1] = 1. - t, t          # v[i] + (v[i+1] - v[i]) t
        # + m terms: -(2 m[i] + m[i+1])/6 t + m[i]/2 t^2 + (m[i+1] - m[i])/6 t^3
        ci = -t / 3. + t * t / 2. - t ** 3 / 6.
        cj = -t / 6. + t ** 3 / 6.
        S[r] = e + ci * mm[i] + cj * mm[i + 1]
    return S


class DeviceAtmosphere:
    """The layers of an :class:`AtmosGeom` as device screens driven by
    :class:`AtmosFrames`, with the pupil phase of any source (stars, and
    LGSs with the cone effect).

    Each layer gets a (scrnYPxls+1) x (scrnXPxls+1) screen at the pupil pixel
    scale (tel_diam / npup), its initial phase from the FFT method (seeded
    with the layer's seed plus ``seed``) and the extrusion matrices of the
    axes its wind moves along (shared between layers of equal size).
    ``screen_factory(init, l0, ay, by, ax, bx, seed)`` makes a screen (default
    :class:`dasp_gb300.infscreen.DeviceScreen`) and ``pupil_phase_fn`` forms
    the pupil phase (default :func:`dasp_gb300.infscreen.pupil_phase`)."""

    def __init__(self, geom, tstep, seed=0, screen_factory=None, pupil_phase_fn=None):
        from . import infscreen
        self.frames = AtmosFrames(geom, tstep)
        self.geom = geom
        self._pupil_phase = pupil_phase_fn or infscreen.pupil_phase
        self._lgs_cache = {}  # (cone width, device) -> (window, unit pupil, spline matrix)
        factory = screen_factory or (lambda init, l0, ay, by, ax, bx, seed: infscreen.DeviceScreen(
            init, l0, ay=ay, by=by, ax=ax, bx=bx, seed=seed))
        pix = self.frames.pix_scale
        mats = {}

        def matrices(n):
            if n not in mats:
                mats[n] = infscreen.extrusion_matrices(n, infscreen.phase_covariance(n, geom.l0, pix))
            return mats[n]

        self.screens = []
        for lf in self.frames.layers:
            ny, nx = lf.shape
            ay = by = ax = bx = None
            if lf.col_add != 0 or lf.row_add == 0:  # a screen needs one axis even when still
                ay, by = matrices(ny)
            if lf.row_add != 0:
                ax, bx = matrices(nx)
            sd = geom.layers[lf.key].seed + seed
            self.screens.append(factory(_initial_screen(ny, nx, pix, lf.r0, geom.l0, sd), geom.l0, ay, by, ax, bx,
                                        sd))

    def advance(self, stream=None):
        """One frame: each layer's new columns, then rows, extruded on the
        device (queued on ``stream`` if given)."""
        for scr, lf, (ncol, col_end, nrow, row_end) in zip(self.screens, self.frames.layers, self.frames.advance()):
            if ncol:
                (scr.add_columns if col_end else scr.add_columns_start)(ncol, lf.r0, stream=stream)
            if nrow:
                (scr.add_rows if row_end else scr.add_rows_start)(nrow, lf.r0, stream=stream)

    def windows(self, idstr):
        """Per layer the source sees, lowest first: (screen, y0, x0, yshift,
        xshift), the layer tuples of :func:`dasp_gb300.infscreen.pupil_phase`."""
        return [(self.screens[w.layer], w.y0, w.x0, w.yshift, w.xshift) for w in self.frames.windows(idstr)]

    def pupil_phase(self, idstr, pupil, out, pupil_area=None, remove_piston=True, stream=None, intrinsic=None):
        """The source's pupil phase this frame into ``out`` (npup x npup
        float32 tensor on the device): the layers' shifted windows (for an LGS
        each expanded from the cone's width to npup by the natural cubic
        spline) summed lowest first, piston removed over ``pupil``, times
        ``pupil`` and 500 / the source's wavelength (util/atmos.py:678-833).
        A star's layers are summed in one pupil-phase kernel; an LGS's layers
        go one at a time through that kernel (the shift) and two float32
        library GEMMs (S W S^T, S from :func:`spline_matrix`; TF32 off, as
        torch leaves it by default), the sum, piston and scaling in torch,
        all on one stream.  With ``stream`` the work is queued there and not
        waited for (extrude the screens on the same stream); without, it runs
        on torch's current stream and the call waits, as a star's does.
        ``intrinsic`` (npup x npup tensor on the device, radians at 500 nm) is
        a static phase the sum starts from, before the piston removal and the
        scaling (infAtmos' intrinsicPhase, util/atmos.py:685-688); with it a
        star's layers also go one at a time."""
        src = self.geom.sources[idstr]
        if src.alt < 0 and intrinsic is None:
            return self._pupil_phase(self.windows(idstr), pupil, out, pupil_area=pupil_area, wavelength=src.lam,
                                     remove_piston=remove_piston, stream=stream)
        return self._composed_pupil_phase(idstr, pupil, out, pupil_area, remove_piston, stream, intrinsic)

    def _composed_pupil_phase(self, idstr, pupil, out, pupil_area, remove_piston, stream, intrinsic):
        import contextlib

        import torch
        npup = self.geom.npup
        dev = out.device
        ctx, ks = contextlib.nullcontext(), stream
        if dev.type == "cuda":
            # the shift kernels, the GEMMs and the element-wise steps share one
            # stream (the given one, else torch's current stream), so that a
            # kernel never overwrites a window buffer a pending GEMM still reads
            if stream is None:
                ks = torch.cuda.current_stream(dev)
            elif not isinstance(stream, torch.cuda.Stream):
                ks = torch.cuda.ExternalStream(stream)
            ctx = torch.cuda.stream(ks)
        with ctx:
            if intrinsic is None:
                total = torch.zeros((npup, npup), dtype=torch.float32, device=dev)
            else:
                total = intrinsic.to(device=dev, dtype=torch.float32).clone()
            for w in self.frames.windows(idstr):
                tmp, ones, S = self._lgs_buffers(w.width, dev)
                self._pupil_phase([(self.screens[w.layer], w.y0, w.x0, w.yshift, w.xshift)], ones, tmp,
                                  pupil_area=1.0, wavelength=500.0, remove_piston=False, stream=ks)
                # the ground layer spans the whole pupil: the spline through
                # its own knots is the identity
                total += tmp if S is None else torch.matmul(torch.matmul(S, tmp), S.t())
            p = pupil.to(torch.float32)
            scale = np.float32(500.0 / self.geom.sources[idstr].lam)
            if remove_piston:
                area = p.double().sum() if pupil_area is None else float(pupil_area)
                pist = ((total.double() * p.double()).sum() / area).to(torch.float32)
                out.copy_((total - pist) * p * scale)
            else:
                out.copy_(total * p * scale)
        if stream is None and dev.type == "cuda":
            # as every screen call without a stream: the result is ready on
            # return, and the screens may be extruded again at once
            ks.synchronize()
        return out

    def _lgs_buffers(self, width, dev):
        """(shifted window, unit pupil, spline matrix or None) for a cone
        width, kept per width and device."""
        import torch
        cache = self._lgs_cache
        key = (width, str(dev))
        if key not in cache:
            S = None
            if width != self.geom.npup:
                S = torch.from_numpy(spline_matrix(width, self.geom.npup).astype(np.float32)).to(dev)
            cache[key] = (torch.empty((width, width), dtype=torch.float32, device=dev),
                          torch.ones((width, width), dtype=torch.float32, device=dev), S)
        return cache[key]

    def free(self):
        for scr in self.screens:
            free = getattr(scr, "free", None)
            if free:
                free()
        self.screens = []


def _frame_shift(step, pos):
    """The part of a window's position that moves with the wind
    (util/atmos.py:698-705): with lines added at the start the window moves
    back by 1 - pos (none at an integer position), with lines added at the
    end forward by pos (a whole pixel at an integer position)."""
    if step >= 0:
        return 1. - pos if pos > 0 else 0.
    return pos if pos > 0 else 1.


def _initial_screen(ny, nx, pix_scale, r0, l0, seed):
    from .screens import von_karman_screen
    n = max(ny, nx)
    return np.ascontiguousarray(von_karman_screen(n, n * pix_scale, r0, l0, seed, 500.0)[:ny, :nx], np.float32)
