"""Make tests/golden/atmos_frames.json from the reference's own Python code.

The fixture pins dasp_gb300/infatmos.py to DASP's atmosphere bookkeeping:
for a few atmospheres it holds the layer geometry (screen sizes, layer
offsets, zenith-scaled layers and r0), the layers' wind steps, and for 30
frames the lines each layer's screen gains and each source's window per
layer (start row / column, sub-pixel shifts, and the window's size: the
pupil for a star, the cone's width at the layer for an LGS; none for a
layer above the LGS).  They are computed by running
the reference's code itself, read from the reference tree:

* util/getNewCols.py: the ``getNewCols`` class (the file up to its
  ``__main__`` block, which is Python 2 only);
* util/atmos.py: the ``layer``, ``source`` and ``geom`` classes, the
  source-position block of ``atmos.__init__`` (``self.positionDict``) and the
  window lines of ``atmos.createPupilPhs``;
* science/infAtmos.py: the wind-step statements (``self.colAdd[key]=...``).

The reference is Python 2: the extracted code runs under Python 3 after two
mechanical changes -- ``print`` statements become ``pass`` and
``d.has_key(k)`` becomes ``d.__contains__(k)`` -- nothing else is edited.
Run ``python tests/golden/make_atmos_golden.py`` where the reference tree is
present (``DASP_REFERENCE`` overrides its location).
"""
from __future__ import annotations

import json
import os
import re
import textwrap
import types

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("DASP_REFERENCE", "/root/reference")
NFRAMES = 30

# atmospheres: layers (height m, direction deg, speed m/s, strength, seed),
# sources (idstr, theta arcsec, phi deg, alt, fov arcsec), telescope
CASES = [
    dict(name="three_layers_three_stars",
         layers={"ground": (0., 0., 10., 0.6, 1), "mid": (4000., 90., 15., 0.25, 2), "high": (10000., 225., 25., 0.15, 3)},
         sources=[("on", 0., 0., -1, 0.), ("ne", 30., 45., -1, 0.), ("sw", 60., 200., -1, 0.)],
         ntel=64, npup=64, tel_diam=4.2, r0=0.15, l0=25., zenith=0., zenith_az=0., tstep=0.002),
    dict(name="zenith_fast_wind_fov",
         layers={"a": (500., 30., 40., 1., 4), "b": (8000., 300., 8., 2., 5)},
         sources=[("sci", 20., 120., -1, 5.), ("gs", 45., 10., -1, 0.)],
         ntel=80, npup=80, tel_diam=8.0, r0=0.12, l0=30., zenith=30., zenith_az=10., tstep=0.005),
    dict(name="lgs_cone_and_layer_above",
         layers={"low": (0., 20., 12., 0.5, 8), "mid": (7000., 160., 18., 0.3, 9), "top": (95000., 70., 30., 0.2, 10)},
         sources=[("lgs", 15., 60., 90000., 0.), ("lgs2", 0., 0., 90000., 0.), ("ngs", 25., 300., -1, 0.)],
         ntel=64, npup=64, tel_diam=8.0, r0=0.14, l0=25., zenith=0., zenith_az=0., tstep=0.004),
    dict(name="integer_steps_ntel_differs",
         layers={"x": (0., 180., 50., 0.5, 6), "y": (6000., 270., 20., 0.5, 7)},
         sources=[("on", 0., 0., -1, 0.), ("off", 40., 300., -1, 0.)],
         ntel=60, npup=64, tel_diam=4.0, r0=0.2, l0=20., zenith=0., zenith_az=0., tstep=0.0125),
]


def _read(rel):
    with open(os.path.join(REF, rel)) as fh:
        return fh.read()


def _py3(lines):
    out = []
    for ln in lines:
        m = re.match(r"^(\s*)print\b", ln)
        out.append(m.group(1) + "pass" if m else ln.replace(".has_key(", ".__contains__("))
    return out


def _block(text, first, last, start_after=None):
    """The lines of ``text`` from the first line containing ``first`` (after
    the line containing ``start_after``) to the next containing ``last``."""
    lines = text.split("\n")
    i0 = 0
    if start_after:
        i0 = next(i for i, ln in enumerate(lines) if start_after in ln)
    a = next(i for i in range(i0, len(lines)) if first in lines[i])
    b = next(i for i in range(a, len(lines)) if last in lines[i])
    return lines[a:b + 1]


def _function(name, args, lines, ret):
    body = textwrap.indent(textwrap.dedent("\n".join(_py3(lines))), "    ")
    return "def %s(%s):\n%s\n    return %s\n" % (name, args, body, ret)


def reference_code():
    """A namespace with the reference's classes and extracted blocks."""
    ns = {"numpy": numpy, "math": __import__("math")}
    gnc = _read("util/getNewCols.py").split('if __name__=="__main__":')[0]
    exec(compile(gnc, "util/getNewCols.py", "exec"), ns)
    atm = _read("util/atmos.py")
    lines = atm.split("\n")
    a = next(i for i, ln in enumerate(lines) if ln.startswith("class layer"))
    b = next(i for i, ln in enumerate(lines) if ln.startswith("class atmos"))
    exec(compile("\n".join(_py3(lines[a:b])), "util/atmos.py", "exec"), ns)
    pos = _block(atm, "self.positionDict={}", "self.positionDict[key]=()")
    exec(compile(_function("position_dict", "self, arcsecRad, degRad", pos, "self.positionDict"),
                 "util/atmos.py:positionDict", "exec"), ns)
    win = _block(atm, "interpPosCol=posDict[4]", "interpPosRow-=phsShiftX", start_after="def createPupilPhs")
    exec(compile(_function("window", "self, key, posDict, interpPosColDict, interpPosRowDict", win,
                           "(phsShiftX, phsShiftY, interpPosCol, interpPosRow)"),
                 "util/atmos.py:createPupilPhs", "exec"), ns)
    steps = _block(_read("science/infAtmos.py"), "self.colAdd[key]=-self.vWind[key]", "self.colAdd[key]=0.")
    exec(compile(_function("wind_steps", "self, key", steps, "(self.colAdd[key], self.rowAdd[key])"),
                 "science/infAtmos.py:colAdd", "exec"), ns)
    return ns


def run_case(ns, case):
    layers = {k: ns["layer"](*v) for k, v in case["layers"].items()}
    sources = [ns["source"](s[0], s[1], s[2], s[3], sourcelam=500., fov=s[4]) for s in case["sources"]]
    g = ns["geom"](layers, sources, case["ntel"], case["npup"], case["tel_diam"], case["r0"], case["l0"],
                   zenith=case["zenith"], zenithAz=case["zenith_az"])
    xo, yo = g.getLayerXOffset(), g.getLayerYOffset()
    out = {"r0": g.r0, "layers": {}, "frames": []}
    pix = case["tel_diam"] / float(case["npup"])
    st = types.SimpleNamespace(vWind=g.windSpeeds(), windDirection=g.windDirections(), pixScale=pix,
                               tstep=case["tstep"], colAdd={}, rowAdd={})
    keys = sorted(layers, key=lambda k: g.layerHeight(k))
    counters = {}
    for k in keys:
        ca, ra = ns["wind_steps"](st, k)
        ly = g.layerDict[k]
        out["layers"][k] = {"scrn": [g.getScrnXPxls(k), g.getScrnYPxls(k)], "offset": [xo[k], yo[k]],
                            "height": ly.height, "speed": ly.speed, "direction": ly.direction,
                            "strength": ly.strength, "steps": [ca, ra]}
        counters[k] = (ns["getNewCols"](numpy.fabs(ca)), ns["getNewCols"](numpy.fabs(ra)))
    # each source's static positions, from atmos.__init__'s own block
    shapes = {k: types.SimpleNamespace(shape=(g.getScrnYPxls(k) + 1, g.getScrnXPxls(k) + 1)) for k in keys}
    posd = {}
    for s in sources:
        a = types.SimpleNamespace(sourceTheta=s.theta, sourcePhi=s.phi, sourceAlt=s.alt, layerList=keys,
                                  layerAltitude=g.layerAltitudes(), scrnScale=case["tel_diam"] / float(case["ntel"]),
                                  npup=case["npup"], zenithOld=0., layerXOffset=xo, layerYOffset=yo,
                                  phaseScreens=shapes, storePupilLayers=0, computeUplinkTT=0)
        posd[s.idstr] = ns["position_dict"](a, 2 * numpy.pi / 360 / 3600, 2 * numpy.pi / 360)
    wa = types.SimpleNamespace(colAdd=st.colAdd, rowAdd=st.rowAdd)
    for _ in range(NFRAMES):
        frame = {"lines": {}, "windows": {}}
        ipc, ipr = {}, {}
        for k in keys:
            _, nc, ipc[k] = counters[k][0].nextOld()
            _, nr, ipr[k] = counters[k][1].nextOld()
            frame["lines"][k] = [int(nc), int(nr)]
        for s in sources:
            wins = []
            for k in keys:
                pd = posd[s.idstr][k]
                if len(pd) == 0:  # a layer above the source is not used
                    wins.append(None)
                    continue
                sx, sy, pc, pr = ns["window"](wa, k, pd, ipc, ipr)
                # rows start at pd[1] + phsShiftX, columns at pd[0] + phsShiftY;
                # linearshift(phs, interpPosCol, interpPosRow): column then row
                # shift; the window is pd[3] + 1 rows by pd[2] + 1 columns
                wins.append([int(pd[1] + sx), int(pd[0] + sy), float(pr), float(pc), int(pd[3]), int(pd[2])])
            frame["windows"][s.idstr] = wins
        out["frames"].append(frame)
    # the counters themselves for a spread of steps, both methods
    return out


def newcols_sequences(ns):
    seqs = {}
    for step in (0., 0.19, 0.25, 0.5, 0.75, 1.0, 1.3, 2.0, 2.5, 3.7):
        a, b = ns["getNewCols"](step), ns["getNewCols"](step)
        seqs[repr(step)] = {"next": [list(a.next()) for _ in range(NFRAMES)],
                            "next_old": [list(b.nextOld()) for _ in range(NFRAMES)]}
    return seqs


def build():
    ns = reference_code()
    return {"cases": [dict(case, result=run_case(ns, case)) for case in CASES], "newcols": newcols_sequences(ns),
            "reference": ["util/getNewCols.py", "util/atmos.py", "science/infAtmos.py"]}


def main():
    data = build()
    path = os.path.join(HERE, "atmos_frames.json")
    with open(path, "w") as fh:
        json.dump(data, fh, indent=None, separators=(",", ":"), sort_keys=True)
    print("wrote %s (%d bytes)" % (path, os.path.getsize(path)))


if __name__ == "__main__":
    main()
