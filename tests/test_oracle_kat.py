"""The oracle pinned on CPU: published known-answer vectors for the random
streams, and known-answer properties of the reference's image formation
(flat phase, tilt ramps, gradients, flux, unlit subapertures, Poisson moments)."""
import numpy as np
import pytest

from oracle.shwfs_oracle import (MT19937, PCG32, bin_image, bin_weights, flip_array, noise_lib,
                                 philox4x32_10, tilt_fn)
from tests.wfs_cases import Case

# ---------------------------------------------------------------- RNG vectors


def test_pcg32_published_vector():
    # pcg32-demo (pcg-c-basic): pcg32_srandom_r(&rng, 42u, 54u), first six outputs
    r = PCG32(42, 54)
    got = [r.next() for _ in range(6)]
    assert got == [0xa15c02b7, 0x7b47f409, 0xba1d3330, 0x83d2f293, 0xbfa4784b, 0xcbed606e]


def test_mt19937_published_vector():
    # init_genrand(5489): first output 3499211612, 10000th output 4123659995
    m = MT19937(5489)
    v = [m.next() for _ in range(10000)]
    assert v[0] == 3499211612
    assert v[-1] == 4123659995


@pytest.mark.parametrize("ctr,key,want", [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
])
def test_philox_published_vectors(ctr, key, want):
    # Random123 known-answer vectors for philox4x32-10
    assert list(philox4x32_10(ctr, key)) == want


def test_poisson_sampler_moments(noise_lib):
    import ctypes
    r = PCG32(11, 1)
    for lam in (0.5, 3.0, 9.5, 10.0, 40.0, 900.0):
        buf = np.full(20000, lam, np.float32)
        noise_lib.orc_poissonise(r.buf, buf.ctypes.data_as(ctypes.c_void_p), buf.size)
        assert np.all(buf == np.round(buf))
        assert abs(buf.mean() - lam) < 5 * np.sqrt(lam / buf.size)
        assert abs(buf.var() / lam - 1) < 0.06


def test_gaussian_moments(noise_lib):
    m = MT19937(3)
    v = np.array([noise_lib.orc_gaussian(m.buf, 2.5) for _ in range(20000)])
    assert abs(v.mean()) < 5 * 2.5 / np.sqrt(v.size)
    assert abs(v.std() / 2.5 - 1) < 0.03


# ---------------------------------------------------------------- helpers


def test_flip_array_is_ifftshift():
    rng = np.random.default_rng(0)
    for n in (4, 5, 7, 8, 16, 20, 21):
        a = rng.random((n, n))
        assert np.array_equal(flip_array(a, 1), np.fft.ifftshift(a))


def test_tilt_fn_values():
    t = tilt_fn(8, 16, "f32")
    assert t.dtype == np.float32
    step = np.float32(np.pi / 16 * 17)
    assert t[0, 0] == step * np.float32(1 - 8)
    assert t[7, 7] == step * np.float32(15 - 8 + 1 - 1)


def test_integer_binning_is_block_sum():
    rng = np.random.default_rng(1)
    img = rng.random((3, 20, 20)).astype(np.float32)
    out = bin_image(img, 10, bin_weights(20, 10), np.float64)
    ref = img.astype(np.float64).reshape(3, 10, 2, 10, 2).sum(axis=(2, 4))
    np.testing.assert_allclose(out, ref, rtol=1e-12)


def test_fractional_binning_conserves_interior_flux():
    # non-integer factor: weights sum to 1 per input pixel (the reference's
    # next-share indexing moves flux between neighbours but keeps the total
    # of a constant image except at the last row/column)
    img = np.ones((1, 20, 20), np.float64)
    out = bin_image(img, 8, bin_weights(20, 8), np.float64)
    assert out.shape == (1, 8, 8)
    assert abs(out.sum() - 400) < 20


# ---------------------------------------------------------------- KATs


def test_lit_counts_match_configs():
    assert Case(nsubx=8, p=8, N=16).lit().sum() == 48
    assert Case(nsubx=74, p=10, N=20, obs=0.28, Dtel=39.0, r0=0.157, L0=25.0, wavelength=589.0).lit().sum() == 3972


def test_flat_phase_gives_zero_centroids_after_reference():
    c = Case(nsubx=8, p=8, N=16, sig=1e4)
    orc = c.oracle()
    flat = np.zeros_like(c.phs)
    cents, _ = c.oracle_run(orc, flat)
    lit = c.lit()
    # the symmetric spot sits at the centre (tilt + 180-degree rotation)
    assert np.abs(cents.reshape(-1, 2)[lit]).max() < 1e-5
    orc.update(18, cents.copy())
    cents2, _ = c.oracle_run(orc, flat)
    assert np.abs(cents2).max() == 0.0


def test_tilt_ramp_shifts_spot_linearly():
    c = Case(nsubx=8, p=8, N=16, sig=1e4)
    orc = c.oracle("f64")
    lit = c.lit()
    xs = []
    for s in (0.05, 0.1, 0.2):
        ph = (np.arange(c.W)[None, :] * s * np.ones((c.W, 1))).astype(np.float32)
        cents, _ = c.oracle_run(orc, ph)
        cx = cents.reshape(-1, 2)[lit, 0]
        cy = cents.reshape(-1, 2)[lit, 1]
        assert np.abs(cy).max() < 1e-6
        xs.append(np.median(cx))
    # shift = -s*N/(2 pi) FFT pixels * m/C, sign from the 180-degree rotation
    for s, x in zip((0.05, 0.1, 0.2), xs):
        assert abs(x / (-s * 16 / (2 * np.pi) * 8 / 16) - 1) < 0.08


def test_gradient_orientation():
    # test/standalone/wfsCent.py:105,115 -- x gradient: var(x) < var(y) fails
    # the other way; the transpose swaps them
    c = Case(nsubx=8, p=8, N=16, sig=1e4)
    orc = c.oracle()
    lit = c.lit()
    ph = (np.arange(c.W)[None, :] ** 2 * 0.01 * np.ones((c.W, 1))).astype(np.float32)
    cx = c.oracle_run(orc, ph)[0].reshape(-1, 2)[lit]
    cy = c.oracle_run(orc, np.ascontiguousarray(ph.T))[0].reshape(-1, 2)[lit]
    assert cx[:, 0].var() > cx[:, 1].var()
    assert cy[:, 1].var() > cy[:, 0].var()


def test_flux_normalisation_by_analytic_total():
    # Q2: bimg sums to sig*frac*(power inside the clip)/(total power)
    c = Case(nsubx=8, p=8, N=16, sig=1e4)
    orc = c.oracle("f64")
    _, bimg = c.oracle_run(orc, np.zeros_like(c.phs))
    lit = c.lit()
    frac = (c.pup.getSubarea(8) / 64).reshape(-1)
    tot = bimg.reshape(64, -1).sum(1)
    assert np.all(tot[lit] <= 1e4 * frac[lit] * (1 + 1e-6))
    assert np.all(tot[lit] > 0.5e4 * frac[lit])
    assert np.all(tot[~lit] == 0)


def test_unlit_subaps_zero_centroids():
    c = Case(nsubx=8, p=8, N=16, sig=1e4)
    cents = np.full(128, 3.0, np.float32)
    c.oracle_run(c.oracle(), None, cents)
    assert np.all(cents.reshape(-1, 2)[~c.lit()] == 0)


def test_f32_and_f64_modes_agree():
    c = Case(nsubx=16, p=8, N=16, psf="gauss", sig=500.0, skybrightness=10.0, noiseFloor=6.0)
    a = c.oracle_run(c.oracle("f32"))[0]
    b = c.oracle_run(c.oracle("f64"))[0]
    assert np.abs(a - b).max() < 1e-4


def test_reference_stream_noise_is_reproducible():
    c = Case(nsubx=8, p=8, N=16, sig=2000.0, addPoisson=1, readnoise=2.0, skybrightness=5.0, noiseFloor=4.0)
    a = c.oracle_run(c.oracle())
    b = c.oracle_run(c.oracle())
    np.testing.assert_array_equal(a[1], b[1])
    c.params["nthreads"] = 3
    d = c.oracle_run(c.oracle())
    assert not np.array_equal(a[1], d[1])  # Q6: streams depend on the partition


def test_integration_state_machine():
    c = Case(nsubx=8, p=8, N=16, sig=1e4, nintegrations=3, nlatency=1)
    orc = c.oracle()
    cents = np.full(128, 9.0, np.float32)
    for _ in range(3):
        c.oracle_run(orc, None, cents)
        assert np.all(cents == 9.0)
    c.oracle_run(orc, None, cents)
    assert not np.all(cents == 9.0)
    assert orc.curInteg == 0


# ---- interpolatePhase (cmod/src/centmodule.c:1628-1758) ----

def test_interpolate_phase_known_answers():
    from oracle.shwfs_oracle import interpolate_phase
    rng = np.random.default_rng(4)
    # a constant stays that constant exactly
    c = np.full((50, 50), 3.25, np.float32)
    assert np.array_equal(interpolate_phase(c, 8, 8), np.full((64, 64), 3.25, np.float32))
    # same size: every sample but the pinned last row/column is the input
    # (t = 0 keeps 0.5 * 2 * f[1]); the last one is the t = 1 end of the
    # n-3 .. n cell, equal to the last input sample up to rounding
    a = rng.standard_normal((64, 64)).astype(np.float32)
    b = interpolate_phase(a, 8, 8)
    assert np.array_equal(b[:-1, :-1], a[:-1, :-1])
    assert np.abs(b - a).max() < 1e-5
    # Catmull-Rom reproduces a linear ramp away from the clamped edges
    x = np.arange(50, dtype=np.float64)
    r = np.add.outer(0.3 * x, -0.7 * x).astype(np.float32)
    o = interpolate_phase(r, 8, 8)
    X = np.arange(64) * (49 / 63.0)
    ref = np.add.outer(0.3 * X, -0.7 * X)
    assert np.abs(o[2:-2, 2:-2] - ref[2:-2, 2:-2]).max() < 1e-4
    # and a cubic in the interior of a finer resample (the kernel's order)
    assert interpolate_phase(rng.standard_normal((90, 90)).astype(np.float32), 8, 8).dtype == np.float32


def test_oracle_interpolates_mismatched_phase():
    """A phase of another size gives the centroids of its resampled array,
    and OUTPUTPHASEARR receives the lit subapertures' resampled phase."""
    from oracle.shwfs_oracle import OUTPUTPHASEARR, interpolate_phase
    from dasp_gb300.screens import von_karman_screen
    c = Case(nsubx=8, p=8, N=16)
    inp = von_karman_screen(50, 4.2, 0.15, 30.0, 3, 640.0)
    full = interpolate_phase(inp, 8, 8)
    o1, o2 = c.oracle("f32"), c.oracle("f32")
    out = np.full((64, 64), -7.0, np.float32)
    o1.update(OUTPUTPHASEARR, out)
    c1, _ = c.oracle_run(o1, phs=inp)
    c2, _ = c.oracle_run(o2, phs=full)
    np.testing.assert_array_equal(c1, c2)
    lit = c.lit().reshape(8, 8)
    for sy in range(8):
        for sx in range(8):
            blk = out[sy * 8:(sy + 1) * 8, sx * 8:(sx + 1) * 8]
            if lit[sy, sx]:
                np.testing.assert_array_equal(blk, full[sy * 8:(sy + 1) * 8, sx * 8:(sx + 1) * 8])
            else:
                assert (blk == -7.0).all()
