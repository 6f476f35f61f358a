"""The layered-atmosphere bookkeeping (dasp_gb300/infatmos.py) against the
reference's own code, on CPU.

tests/golden/atmos_frames.json holds what DASP's code gives (made by
tests/golden/make_atmos_golden.py from util/getNewCols.py, util/atmos.py and
science/infAtmos.py): the getNewCols counters, the atmosphere geometry, the
wind steps, and 30 frames of lines added and source windows.  Integers must
match exactly and positions to 1e-12.  Beyond the fixture: the window a
source sees moves with the wind by exactly the step per frame, and
DeviceAtmosphere applies the frame plan to its screens (fake screens here;
the screen and pupil-phase kernels have their own GPU tests).
"""
import json
import os

import numpy as np
import pytest

from dasp_gb300.infatmos import AtmosFrames, AtmosGeom, DeviceAtmosphere, Layer, NewCols, Source, wind_steps

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
            assert [list(w[:2]) for w in got] == [w[:2] for w in want], sid
            assert np.allclose([w[2:] for w in got], [w[2:] for w in want], rtol=0, atol=1e-12), sid


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
            return [(w[1] + w[3] + moved[lf.key][0], w[0] + w[2] + moved[lf.key][1])
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


def test_only_sources_at_infinity_and_distinct_heights():
    g = AtmosGeom({"a": Layer(0., 0., 5., 1.)}, [Source("lgs", 10., 0., alt=90000.)], 32, 32, 2.0, 0.15, 20.)
    with pytest.raises(ValueError, match="LGS"):
        AtmosFrames(g, 0.002).windows("lgs")
    g = AtmosGeom({"a": Layer(0., 0., 5., .5), "b": Layer(0., 90., 5., .5)}, [Source("s")], 32, 32, 2.0, 0.15, 20.)
    with pytest.raises(ValueError, match="distinct heights"):
        AtmosFrames(g, 0.002)


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
        assert [w[1:] for w in got["wins"]] == ref.windows("off")


def test_fixture_regenerates_from_the_reference():
    from tests.golden import make_atmos_golden as mk
    if not os.path.exists(os.path.join(mk.REF, "util", "getNewCols.py")):
        pytest.skip("reference sources not available")
    assert json.loads(json.dumps(mk.build(), sort_keys=True)) == DATA
