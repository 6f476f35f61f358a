"""The layered-atmosphere bookkeeping (dasp_gb300/infatmos.py) against the
reference's own code, on CPU.

tests/golden/atmos_frames.json holds what DASP's code gives (made by
tests/golden/make_atmos_golden.py from util/getNewCols.py, util/atmos.py and
science/infAtmos.py): the getNewCols counters, the atmosphere geometry, the
wind steps, and 30 frames of lines added and source windows.  Integers must
match exactly and positions to 1e-12.  Beyond the fixture: the window a
source sees moves with the wind by exactly the step per frame; the LGS
spline matrix is the natural cubic spline (scipy); DeviceAtmosphere
applies the frame plan to its screens; and its LGS pupil phase (cone
windows, spline expansion, piston) agrees with a float64 restatement to
2e-5 of the peak (host stand-ins for the screens and the shift kernel,
which have their own GPU tests).
"""
import json
import os

import numpy as np
import pytest

from dasp_gb300.infatmos import (AtmosFrames, AtmosGeom, DeviceAtmosphere, Layer, NewCols, Source, spline_matrix,
                                 wind_steps)

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "atmos_frames.json")
with open(GOLDEN) as _fh:
    DATA = json.load(_fh)
CASES = DATA["cases"]


def _geom(case):
    layers = {k: Layer(*v) for k, v in case["layers"].items()}
    sources = [Source(s[0], s[1], s[2], s[3], s[4]) for s in case["sources"]]
    return AtmosGeom(layers, sources, case["ntel"], case["npup"], case["tel_diam"], case["r0"], case["l0"],
                     zenith=case["zenith"], zenith_az=case["zenith_az"])


def test_newcols_match_reference():
    for step, seqs in DATA["newcols"].items():
        a, b = NewCols(float(step)), NewCols(float(step))
        assert [list(a.next()) for _ in seqs["next"]] == seqs["next"], step
        assert [list(b.next_old()) for _ in seqs["next_old"]] == seqs["next_old"], step


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_geometry_matches_reference(case):
    g = _geom(case)
    res = case["result"]
    assert g.r0 == pytest.approx(res["r0"], rel=1e-14)
    xo, yo = g.layer_offsets()
    pix = case["tel_diam"] / case["npup"]
    for k, want in res["layers"].items():
        ly = g.layers[k]
        assert list(g.screen_size(k)) == want["scrn"], k
        assert [xo[k], yo[k]] == want["offset"], k
        for f in ("height", "speed", "direction", "strength"):
            assert getattr(ly, f) == pytest.approx(want[f], rel=1e-12, abs=1e-12), (k, f)
        assert list(wind_steps(ly, pix, case["tstep"])) == pytest.approx(want["steps"], rel=1e-12, abs=1e-15)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_frames_match_reference(case):
    fr = AtmosFrames(_geom(case), case["tstep"])
    keys = [lf.key for lf in fr.layers]
    for frame in case["result"]["frames"]:
        plan = fr.advance()
        assert [[p[0], p[2]] for p in plan] == [frame["lines"][k] for k in keys]
        for sid, want in frame["windows"].items():
            got = fr.windows(sid)
            used = [i for i, w in enumerate(want) if w is not None]  # layers above an LGS are skipped
            want = [want[i] for i in used]
            assert [w.layer for w in got] == used, sid
            assert [[w.y0, w.x0, w.width, w.width] for w in got] == [[w[0], w[1], w[4], w[5]] for w in want], sid
            assert np.allclose([[w.yshift, w.xshift] for w in got], [w[2:4] for w in want], rtol=0, atol=1e-12), sid


def test_window_moves_with_the_wind():
    # in the screen's content coordinates (lines added at the end shift the
    # content back, at the start forward) a source's window moves by exactly
    # -colAdd columns and -rowAdd rows per frame, for any wind
    rng = np.random.default_rng(5)
    for trial in range(6):
        layers = {"l%d" % i: Layer(2000. * i, float(rng.uniform(0, 360)), float(rng.uniform(0, 60)), 1.) for i in range(3)}
        g = AtmosGeom(layers, [Source("s", 30., 70.), Source("o", 0., 0.)], 32, 32, 2.0, 0.15, 20.)
        fr = AtmosFrames(g, float(rng.uniform(0.001, 0.01)))
        moved = {lf.key: [0, 0] for lf in fr.layers}  # net lines added at the end, per axis

        def content(sid):
            return [(w.x0 + w.xshift + moved[lf.key][0], w.y0 + w.yshift + moved[lf.key][1])
                    for lf, w in zip(fr.layers, fr.windows(sid))]

        start = {sid: content(sid) for sid in ("s", "o")}
        for n in range(1, 60):
            for lf, (nc, cend, nr, rend) in zip(fr.layers, fr.advance()):
                moved[lf.key][0] += nc if cend else -nc
                moved[lf.key][1] += nr if rend else -nr
            for sid in ("s", "o"):
                for lf, (u, v), (u0, v0) in zip(fr.layers, content(sid), start[sid]):
                    assert u - u0 == pytest.approx(-n * lf.col_add, abs=1e-9), (trial, lf.key, n)
                    assert v - v0 == pytest.approx(-n * lf.row_add, abs=1e-9), (trial, lf.key, n)


def test_lgs_cone_widths_and_distinct_heights():
    g = AtmosGeom({"a": Layer(0., 0., 5., .5), "b": Layer(30000., 0., 5., .3), "c": Layer(95000., 0., 5., .2)},
                  [Source("lgs", 10., 0., alt=90000.)], 32, 32, 2.0, 0.15, 20.)
    wins = AtmosFrames(g, 0.002).windows("lgs")
    assert [w.layer for w in wins] == [0, 1]  # the layer above the LGS is not seen
    assert [w.width for w in wins] == [32, int(32 * (1 - 30000. / 90000.) + 0.5)]
    with pytest.raises(ValueError, match="at least 3 points"):
        spline_matrix(2, 32)
    g = AtmosGeom({"a": Layer(0., 0., 5., .5), "b": Layer(0., 90., 5., .5)}, [Source("s")], 32, 32, 2.0, 0.15, 20.)
    with pytest.raises(ValueError, match="distinct heights"):
        AtmosFrames(g, 0.002)


def test_spline_matrix_is_the_natural_cubic_spline():
    from scipy.interpolate import CubicSpline
    rng = np.random.default_rng(0)
    for width, npup in ((3, 10), (5, 8), (59, 64), (100, 740), (683, 740)):
        S = spline_matrix(width, npup)
        v = rng.standard_normal(width)
        xs = np.arange(npup) * ((width - 1) / float(npup - 1))
        want = CubicSpline(np.arange(width, dtype=float), v, bc_type="natural")(xs)
        assert np.abs(S @ v - want).max() <= 1e-13 * max(1.0, np.abs(want).max())


class _FakeScreen:
    def __init__(self, init, l0, ay, by, ax, bx, seed):
        self.shape, self.axes, self.seed, self.calls = init.shape, (ay is not None, ax is not None), seed, []
        for m, n in ((ay, init.shape[0]), (ax, init.shape[1])):
            assert m is None or m.shape == (n, 2 * n)

    def _rec(name):
        def f(self, n, r0, stream=None):
            self.calls.append((name, n, r0, stream))
        return f

    add_columns, add_columns_start = _rec("cols_end"), _rec("cols_start")
    add_rows, add_rows_start = _rec("rows_end"), _rec("rows_start")


def test_device_atmosphere_applies_the_frame_plan():
    layers = {"g": Layer(0., 0., 12., .5, 1), "h": Layer(5000., 135., 20., .3, 2), "s": Layer(9000., 0., 0., .2, 3)}
    g = AtmosGeom(layers, [Source("on"), Source("off", 20., 40., lam=640.)], 16, 16, 1.6, 0.12, 20.)
    got = {}

    def fake_pupil(wins, pupil, out, pupil_area=None, wavelength=500., remove_piston=True, stream=None):
        got["wins"], got["lam"] = wins, wavelength
        return out

    atm = DeviceAtmosphere(g, 0.004, seed=10, screen_factory=_FakeScreen, pupil_phase_fn=fake_pupil)
    ref = AtmosFrames(g, 0.004)
    for scr, lf in zip(atm.screens, ref.layers):
        assert scr.shape == lf.shape and scr.seed == g.layers[lf.key].seed + 10
        assert scr.axes == (lf.col_add != 0 or lf.row_add == 0, lf.row_add != 0)
    for _ in range(25):
        plan = ref.advance()
        before = [len(s.calls) for s in atm.screens]
        atm.advance(stream="st")
        for scr, lf, b, (nc, cend, nr, rend) in zip(atm.screens, ref.layers, before, plan):
            want = ([("cols_end" if cend else "cols_start", nc, lf.r0, "st")] if nc else []) + \
                   ([("rows_end" if rend else "rows_start", nr, lf.r0, "st")] if nr else [])
            assert scr.calls[b:] == want
        atm.pupil_phase("off", None, None)
        assert got["lam"] == 640.
        assert [w[0] for w in got["wins"]] == atm.screens
        assert [w[1:] for w in got["wins"]] == [(w.y0, w.x0, w.yshift, w.xshift) for w in ref.windows("off")]


class _MovingScreen:
    """A host screen that moves as the device screen does: lines added at
    one end push the others along (new lines are seeded normals)."""

    def __init__(self, init, l0, ay, by, ax, bx, seed):
        self.screen = np.array(init, np.float32)
        self.rng = np.random.default_rng(seed)

    def _line(self, n):
        return self.rng.standard_normal(n).astype(np.float32)

    def add_columns(self, n, r0, stream=None):
        for _ in range(n):
            self.screen = np.concatenate([self.screen[:, 1:], self._line(self.screen.shape[0])[:, None]], 1)

    def add_columns_start(self, n, r0, stream=None):
        for _ in range(n):
            self.screen = np.concatenate([self._line(self.screen.shape[0])[:, None], self.screen[:, :-1]], 1)

    def add_rows(self, n, r0, stream=None):
        for _ in range(n):
            self.screen = np.concatenate([self.screen[1:], self._line(self.screen.shape[1])[None]], 0)

    def add_rows_start(self, n, r0, stream=None):
        for _ in range(n):
            self.screen = np.concatenate([self._line(self.screen.shape[1])[None], self.screen[:-1]], 0)


def test_lgs_pupil_phase_composition_matches_a_host_restatement():
    # the LGS path (shift of each layer's cone window, natural-spline
    # expansion, sum, piston, pupil, scale) with host stand-ins for the
    # screens and the shift kernel, torch on the CPU for the rest, against
    # the same chain in float64 with scipy's natural cubic spline
    import torch
    from scipy.interpolate import CubicSpline

    from dasp_gb300.tel import Pupil
    from oracle import atmos_oracle

    def host_pupil_phase(wins, pupil, out, pupil_area=None, wavelength=500., remove_piston=True, stream=None):
        scr = [w[0].screen for w in wins]
        lay = [(q,) + tuple(w[1:]) for q, w in enumerate(wins)]
        res = atmos_oracle.pupil_phase(scr, lay, pupil.numpy(), pupil_area=pupil_area, wavelength=wavelength,
                                       remove_piston=remove_piston)
        out.copy_(torch.from_numpy(res))
        return out

    npup = 32
    layers = {"a": Layer(0., 30., 14., .5, 1), "b": Layer(6000., 200., 22., .3, 2), "c": Layer(12000., 110., 9., .2, 3),
              "d": Layer(95000., 0., 5., .1, 4)}
    g = AtmosGeom(layers, [Source("lgs", 20., 45., alt=90000., lam=589.)], npup, npup, 2.0, 0.15, 20.)
    atm = DeviceAtmosphere(g, 0.003, screen_factory=_MovingScreen, pupil_phase_fn=host_pupil_phase)
    pup = Pupil(npup, npup / 2., npup / 2. * 0.2).fn.astype(np.float32)
    out = torch.zeros((npup, npup))
    for frame in range(6):
        atm.advance()
        atm.pupil_phase("lgs", torch.from_numpy(pup), out)
        total = np.zeros((npup, npup))
        for w in atm.frames.windows("lgs"):
            win = atm.screens[w.layer].screen[w.y0:w.y0 + w.width + 1, w.x0:w.x0 + w.width + 1]
            shifted = atmos_oracle.linearshift(win, w.xshift, w.yshift, w.width, w.width).astype(np.float64)
            if w.width < npup:
                knots, xs = np.arange(w.width, dtype=float), np.arange(npup) * ((w.width - 1) / float(npup - 1))
                shifted = CubicSpline(knots, shifted, axis=0, bc_type="natural")(xs)
                shifted = CubicSpline(knots, shifted, axis=1, bc_type="natural")(xs)
            total += shifted
        want = (total - (total * pup).sum() / pup.sum()) * pup * (500. / 589.)
        got = out.numpy()
        assert np.abs(got - want).max() <= 2e-5 * np.abs(want).max(), frame
        assert len(atm.frames.windows("lgs")) == 3
    # an intrinsic phase is summed first, then piston-removed and scaled
    # with the layers (a star's layers then go one at a time too)
    intr = np.outer(np.linspace(-1, 1, npup), np.ones(npup)).astype(np.float32) * 3.0
    g2 = AtmosGeom({"a": Layer(0., 30., 14., .6, 1), "b": Layer(6000., 200., 22., .4, 2)},
                   [Source("ngs", 10., 20.)], npup, npup, 2.0, 0.15, 20.)
    atm2 = DeviceAtmosphere(g2, 0.003, screen_factory=_MovingScreen, pupil_phase_fn=host_pupil_phase)
    atm2.advance()
    plain = atm2.pupil_phase("ngs", torch.from_numpy(pup), torch.zeros((npup, npup))).numpy().copy()
    with_i = atm2.pupil_phase("ngs", torch.from_numpy(pup), torch.zeros((npup, npup)),
                              intrinsic=torch.from_numpy(intr)).numpy()
    extra = (intr - (intr * pup).sum() / pup.sum()) * pup
    assert np.abs(with_i - plain - extra).max() <= 2e-5 * np.abs(plain).max()


def test_fixture_regenerates_from_the_reference():
    from tests.golden import make_atmos_golden as mk
    if not os.path.exists(os.path.join(mk.REF, "util", "getNewCols.py")):
        pytest.skip("reference sources not available")
    assert json.loads(json.dumps(mk.build(), sort_keys=True)) == DATA


def _reference_geom(case):
    """The reference's own util.atmos.geom object for a fixture case (its
    classes run as the fixture generator runs them)."""
    from tests.golden import make_atmos_golden as mk
    if not os.path.exists(os.path.join(mk.REF, "util", "atmos.py")):
        pytest.skip("reference sources not available")
    ns = mk.reference_code()
    layers = {k: ns["layer"](*v) for k, v in case["layers"].items()}
    sources = [ns["source"](s[0], s[1], s[2], s[3], sourcelam=500. + 50 * i, fov=s[4])
               for i, s in enumerate(case["sources"])]
    return ns["geom"](layers, sources, case["ntel"], case["npup"], case["tel_diam"], case["r0"], case["l0"],
                      zenith=case["zenith"], zenithAz=case["zenith_az"])


@pytest.mark.parametrize("name", ["zenith_fast_wind_fov", "lgs_cone_and_layer_above"])
def test_geometry_from_a_reference_geom_object(name):
    case = next(c for c in CASES if c["name"] == name)
    ref = _reference_geom(case)
    g = AtmosGeom.from_reference(ref)
    mine = _geom(case)
    assert g.r0 == mine.r0 and (g.zenith, g.zenith_az) == (mine.zenith, mine.zenith_az)
    assert g.layer_offsets() == mine.layer_offsets()
    for k in case["layers"]:
        assert g.screen_size(k) == mine.screen_size(k)
        for f in ("height", "speed", "direction", "strength", "seed"):
            assert getattr(g.layers[k], f) == pytest.approx(getattr(mine.layers[k], f), rel=1e-12)
    assert list(g.sources) == [s[0] for s in case["sources"]]
    assert [g.sources[s[0]].lam for s in case["sources"]] == [500. + 50 * i for i in range(len(case["sources"]))]
    for sid in g.sources:
        assert g.sources[sid].alt == mine.sources[sid].alt
    # the same frames follow from either
    a, b = AtmosFrames(g, case["tstep"]), AtmosFrames(mine, case["tstep"])
    for _ in range(5):
        assert a.advance() == b.advance()
        for sid in g.sources:
            assert a.windows(sid) == b.windows(sid)


def test_geometry_from_a_duck_typed_geom():
    import types
    ly = types.SimpleNamespace(height=1000., direction=90., speed=12., strength=1., seed=4)
    src = types.SimpleNamespace(idstr="s", theta=10., phi=20., alt=-1, fov=0., sourcelam=None)
    ref = types.SimpleNamespace(layerDict={"l": ly}, sourceDict={"s": src}, ntel=32, npup=32, telDiam=2.,
                                r0=0.12, l0=20., zenith=0.)
    g = AtmosGeom.from_reference(ref, default_lam=640.)
    assert g.sources["s"].lam == 640. and g.layers["l"].seed == 4 and g.r0 == 0.12 and g.zenith_az == 0.
