"""Infinite phase screen on the device against the host restatement of
infScrn's extrusion (injected normals) and against von Karman statistics."""
import numpy as np
import pytest
import torch

from dasp_gb300.infscreen import DeviceScreen, extrusion_matrices, new_column_host, phase_covariance

pytestmark = pytest.mark.gpu


def test_extrusion_matches_host_restatement():
    ny, nx, L0, pix, r0 = 24, 20, 25.0, 0.05, 0.12
    ay, by = extrusion_matrices(ny, phase_covariance(ny, L0, pix))
    ax, bx = extrusion_matrices(nx, phase_covariance(nx, L0, pix))
    rng = np.random.default_rng(3)
    init = rng.standard_normal((ny, nx)).astype(np.float32)
    scr = DeviceScreen(init, L0, ay, by, ax, bx, seed=1)
    host = init.copy()
    coeff = (L0 / r0) ** (5. / 6)
    for step in range(3):
        nc = rng.standard_normal((2, ny))
        scr.add_columns(2, r0, step=0.25 * step, noise=nc)
        for k in range(2):
            col = new_column_host(host[:, -2:], ay, by, nc[k], coeff, 0.25 * step if k == 0 else 0.0)
            host = np.concatenate([host[:, 1:], col.astype(np.float32)[:, None]], axis=1)
        nr = rng.standard_normal((1, nx))
        scr.add_rows(1, r0, noise=nr)
        row = new_column_host(host[-2:, :].T, ax, bx, nr[0], coeff)
        host = np.concatenate([host[1:, :], row.astype(np.float32)[None, :]], axis=0)
    got = scr.numpy()
    np.testing.assert_allclose(got, host, rtol=1e-5, atol=1e-5 * np.abs(host).max())
    # the window a sensor reads
    out = torch.empty((10, 12), device="cuda")
    scr.window(5, 3, out)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), got[5:15, 3:15])
    scr.free()


def test_extruded_columns_follow_von_karman_structure_function():
    """The extruded screen's structure function follows the covariance model
    the matrices are built from (2 (C(0) - C(r)) (L0/r0)^(5/3)); the
    two-column memory of the method keeps it within ~10 % in steady state."""
    ny, pix, r0, L0 = 48, 0.02, 0.1, 20.0
    cov = phase_covariance(ny, L0, pix)
    scale = (L0 / r0) ** (5. / 3)
    scr = DeviceScreen.von_karman(ny, 40, pix, r0, L0, seed=7)
    cols = []
    for _ in range(60):
        scr.add_columns(40, r0)
        cols.append(scr.numpy())
    s = np.concatenate(cols, axis=1)  # 48 x 2400, all extruded
    ratios = {}
    for r in (1, 2):
        model_x = 2 * (cov[0, 0] - cov[0, ny * r]) * scale
        ratios["x%d" % r] = np.mean((s[:, r:] - s[:, :-r]) ** 2) / model_x
    for r in (1, 2, 4):
        model_y = 2 * (cov[0, 0] - cov[0, r]) * scale
        ratios["y%d" % r] = np.mean((s[r:, :] - s[:-r, :]) ** 2) / model_y
    assert all(0.85 < v < 1.15 for v in ratios.values()), ratios
    scr.free()


def test_extrusion_at_the_start_matches_astart_restatement():
    # addNewColumnOnStart / addNewRowOnStart (science/infScrn.py:793-823,
    # 857-887): AStart (A's column blocks reversed) on the first two lines
    from oracle.atmos_oracle import astart_matrix
    ny, nx, L0, pix, r0 = 20, 18, 25.0, 0.05, 0.12
    ay, by = extrusion_matrices(ny, phase_covariance(ny, L0, pix))
    ax, bx = extrusion_matrices(nx, phase_covariance(nx, L0, pix))
    asy, asx = astart_matrix(ay, ny), astart_matrix(ax, nx)
    rng = np.random.default_rng(5)
    init = rng.standard_normal((ny, nx)).astype(np.float32)
    scr = DeviceScreen(init, L0, ay, by, ax, bx, seed=2)
    host = init.copy()
    coeff = (L0 / r0) ** (5. / 6)
    for step in range(3):
        nc = rng.standard_normal((2, ny))
        scr.add_columns_start(2, r0, step=0.5 * step, noise=nc)
        for k in range(2):
            z = np.ravel(host[:, :2].astype(np.float64).T)
            col = asy @ z + (by @ nc[k]) * coeff + (0.5 * step if k == 0 else 0.0)
            host = np.concatenate([col.astype(np.float32)[:, None], host[:, :-1]], axis=1)
        nr = rng.standard_normal((1, nx))
        scr.add_rows_start(1, r0, noise=nr)
        z = np.ravel(host[:2, :].astype(np.float64))
        row = asx @ z + (bx @ nr[0]) * coeff
        host = np.concatenate([row.astype(np.float32)[None, :], host[:-1, :]], axis=0)
        # and one at the end in between: both directions on one circular buffer
        ne = rng.standard_normal((1, ny))
        scr.add_columns(1, r0, noise=ne)
        col = new_column_host(host[:, -2:], ay, by, ne[0], coeff)
        host = np.concatenate([host[:, 1:], col.astype(np.float32)[:, None]], axis=1)
    np.testing.assert_allclose(scr.numpy(), host, rtol=1e-5, atol=1e-5 * np.abs(host).max())
    scr.free()


def test_pupil_phase_from_layers_matches_restatement():
    # createPupilPhs for an NGS (util/atmos.py:678-833): windows, linearshift,
    # layers added, piston removed over the pupil, pupil, 500/lambda
    from dasp_gb300.infscreen import pupil_phase
    from dasp_gb300.tel import Pupil
    from oracle import atmos_oracle
    npup = 64
    rng = np.random.default_rng(9)
    hosts, scrs = [], []
    for k, (ny, nx) in enumerate(((80, 90), (72, 100), (70, 70))):
        init = (3 * rng.standard_normal((ny, nx))).astype(np.float32)
        ay, by = extrusion_matrices(ny, phase_covariance(ny, 25.0, 0.06))
        s = DeviceScreen(init, 25.0, ay, by, seed=k)
        nc = rng.standard_normal((3, ny))
        s.add_columns(3, 0.15, noise=nc)
        hosts.append(s.numpy())
        scrs.append(s)
    pup = Pupil(npup, npup / 2.0, npup / 2.0 * 0.25).fn.astype(np.float32)
    layers = [(0, 3, 7, 0.25, 0.6), (1, 5, 20, 0.0, 1.0), (2, 2, 1, 0.8, 0.125)]
    want = atmos_oracle.pupil_phase(hosts, layers, pup, wavelength=640.0)
    out = torch.empty((npup, npup), device="cuda")
    pupil_phase([(scrs[q], y0, x0, ys, xs) for q, y0, x0, ys, xs in layers], torch.from_numpy(pup).cuda(), out,
                wavelength=640.0)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    # the piston sum is a float64 reduction in both, in different orders
    np.testing.assert_allclose(got, want, rtol=0, atol=2e-5 * np.abs(want).max())
    # without piston removal the layer arithmetic is exact
    want2 = atmos_oracle.pupil_phase(hosts, layers, pup, remove_piston=False)
    pupil_phase([(scrs[q], y0, x0, ys, xs) for q, y0, x0, ys, xs in layers], torch.from_numpy(pup).cuda(), out,
                remove_piston=False)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), want2)
    for s in scrs:
        s.free()
