"""The counter-based noise samplers against their distributions.

Poisson draws are checked by a chi-square goodness-of-fit test against the
exact Poisson pmf on both sides of every sampler boundary (modal inversion
below lambda 64, PTRS transformed rejection above); normal draws by their
moments and a binned chi-square test.  Each test fails with probability
about 1e-6 for a correct sampler."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
stats = pytest.importorskip("scipy.stats")


def _draw(kind, lam, n, seed=11, frame=0):
    from dasp_gb300 import _lib
    lam_t = torch.full((n,), float(lam), device="cuda", dtype=torch.float32)
    out = torch.empty(n, device="cuda", dtype=torch.float32)
    _lib.check(_lib.lib().shwfs_sample_noise(kind, lam_t.data_ptr(), n, seed, frame, out.data_ptr(), None),
               "sample_noise")
    return out.cpu().numpy().astype(np.float64)


def _chi2_poisson(x, lam):
    assert np.all(x == np.floor(x)) and x.min() >= 0
    n = x.size
    # bins: every k with expected count >= 20, tails pooled
    k = np.arange(0, int(lam + 20 * np.sqrt(lam) + 30))
    pk = stats.poisson.pmf(k, lam)
    keep = pk * n >= 20
    lo, hi = k[keep].min(), k[keep].max()
    obs = [np.sum(x < lo + 1) if lo > 0 else np.sum(x == 0)]
    exp_ = [stats.poisson.cdf(lo, lam) * n]
    for kk in range(lo + 1, hi):
        obs.append(np.sum(x == kk))
        exp_.append(pk[kk] * n)
    obs.append(np.sum(x >= hi))
    exp_.append(stats.poisson.sf(hi - 1, lam) * n)
    obs, exp_ = np.array(obs, float), np.array(exp_, float)
    chi2 = ((obs - exp_) ** 2 / exp_).sum()
    return stats.chi2.sf(chi2, len(obs) - 1)


@pytest.mark.parametrize("kind", [0, 2])
@pytest.mark.parametrize("lam", [0.05, 0.7, 1.0, 2.5, 3.99, 4.0, 9.7, 10.0, 17.3, 29.9, 30.5, 63.9, 64.0, 127.5, 150.0,
                                 500.0, 1000.0, 2000.0])
def test_poisson_chi_square(lam, kind):
    """kind 2: the sampler every compute form uses (below 64: tabulated
    Poisson(floor lam) + inversion of the fractional remainder; PTRS above);
    kind 0: the table-free modal inversion below 64 / PTRS."""
    x = _draw(kind, lam, 1 << 21)
    p = _chi2_poisson(x, lam)
    assert p > 1e-6, "chi-square p-value %g at lambda %g" % (p, lam)
    assert abs(x.mean() - lam) < 6 * np.sqrt(lam / x.size)


@pytest.mark.parametrize("kind", [0, 2])
def test_poisson_zero_and_negative_mean(kind):
    from dasp_gb300 import _lib
    lam = torch.tensor([0.0, -1.0, 0.0, float("nan")], device="cuda")
    out = torch.full((4,), 7.0, device="cuda")
    _lib.check(_lib.lib().shwfs_sample_noise(kind, lam.data_ptr(), 4, 1, 0, out.data_ptr(), None), "sample_noise")
    assert out.cpu().tolist() == [0.0, 0.0, 0.0, 0.0]


def test_normal_moments_and_shape():
    x = _draw(1, 0.0, 1 << 21)
    n = x.size
    assert abs(x.mean()) < 6 / np.sqrt(n)
    assert abs(x.var() - 1) < 6 * np.sqrt(2 / n)
    edges = np.linspace(-4, 4, 41)
    obs, _ = np.histogram(x, bins=np.concatenate([[-np.inf], edges, [np.inf]]))
    cdf = stats.norm.cdf(np.concatenate([[-np.inf], edges, [np.inf]]))
    exp_ = np.diff(cdf) * n
    assert stats.chi2.sf(((obs - exp_) ** 2 / exp_).sum(), len(obs) - 1) > 1e-6


def test_streams_depend_on_seed_and_frame():
    a = _draw(0, 9.7, 4096, seed=1, frame=0)
    b = _draw(0, 9.7, 4096, seed=1, frame=0)
    c = _draw(0, 9.7, 4096, seed=1, frame=1)
    d = _draw(0, 9.7, 4096, seed=2, frame=0)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c) and not np.array_equal(a, d)


def test_quad_draws_independent_within_a_quad():
    """The four pixels of a quad share three Philox blocks (two Box-Muller
    pairs, four alias words, four inversion uniforms): the cosine and sine
    normals of one pair, and the Poisson draws of neighbouring pixels, are
    uncorrelated."""
    n = 1 << 21
    g = _draw(1, 0.0, n).reshape(-1, 4)
    for j, k in [(0, 1), (2, 3), (0, 2), (1, 3)]:
        r = np.corrcoef(g[:, j], g[:, k])[0, 1]
        assert abs(r) < 6 / np.sqrt(g.shape[0]), (j, k, r)
    # the pair's squared radius -2 ln u1 is shared: its branches are
    # independent only if g0^2 + g1^2 is Exp(1/2), which it is for exact pairs
    r2 = g[:, 0] ** 2 + g[:, 1] ** 2
    assert stats.kstest(r2 / 2, "expon").pvalue > 1e-6
    p = _draw(2, 9.7, n).reshape(-1, 4)
    for j, k in [(0, 1), (1, 2), (2, 3)]:
        r = np.corrcoef(p[:, j], p[:, k])[0, 1]
        assert abs(r) < 6 / np.sqrt(p.shape[0]), (j, k, r)
