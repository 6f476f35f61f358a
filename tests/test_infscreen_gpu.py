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
