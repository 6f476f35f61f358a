"""The device atmosphere (dasp_gb300/infatmos.py) on the GPU: device screens
advanced frame by frame with the device's own noise, each frame's screens
read back, and the pupil phase the device forms for a star and for an LGS
compared with the same chain on the host from those screens (the oracle's
linearshift and pupil phase; scipy's natural cubic spline for the LGS
cone), within 2e-5 of the peak.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host_pupil(atm, idstr, pup, screens):
    from scipy.interpolate import CubicSpline

    from oracle import atmos_oracle
    npup = pup.shape[0]
    total = np.zeros((npup, npup))
    for w in atm.frames.windows(idstr):
        win = screens[w.layer][w.y0:w.y0 + w.width + 1, w.x0:w.x0 + w.width + 1]
        sh = atmos_oracle.linearshift(win, w.xshift, w.yshift, w.width, w.width).astype(np.float64)
        if w.width < npup:
            knots, xs = np.arange(w.width, dtype=float), np.arange(npup) * ((w.width - 1) / float(npup - 1))
            sh = CubicSpline(knots, sh, axis=0, bc_type="natural")(xs)
            sh = CubicSpline(knots, sh, axis=1, bc_type="natural")(xs)
        total += sh
    lam = atm.geom.sources[idstr].lam
    return (total - (total * pup).sum() / pup.sum()) * pup * (500. / lam)


def test_device_atmosphere_star_and_lgs_pupil_phase():
    import torch

    from dasp_gb300.infatmos import AtmosGeom, DeviceAtmosphere, Layer, Source
    from dasp_gb300.tel import Pupil
    npup = 32
    layers = {"a": Layer(0., 30., 14., .5, 1), "b": Layer(6000., 200., 22., .3, 2), "c": Layer(12000., 110., 9., .2, 3)}
    g = AtmosGeom(layers, [Source("ngs", 15., 300., lam=640.), Source("lgs", 20., 45., alt=90000., lam=589.)],
                  npup, npup, 2.0, 0.15, 20.)
    atm = DeviceAtmosphere(g, 0.003, seed=3)
    pup = Pupil(npup, npup / 2., npup / 2. * 0.2).fn.astype(np.float32)
    pt = torch.from_numpy(pup).cuda()
    out = torch.zeros((npup, npup), device="cuda")
    try:
        for frame in range(5):
            atm.advance()
            screens = [s.numpy() for s in atm.screens]
            for sid in ("ngs", "lgs"):
                atm.pupil_phase(sid, pt, out)
                if sid == "lgs":
                    # queued again at once (no host wait in between): the
                    # kernels reuse the window buffers the GEMMs read
                    atm.pupil_phase(sid, pt, out)
                got = out.cpu().numpy()
                want = _host_pupil(atm, sid, pup, screens)
                assert np.abs(got - want).max() <= 2e-5 * np.abs(want).max(), (frame, sid)
    finally:
        atm.free()
