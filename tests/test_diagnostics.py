"""ESS and ARI helpers used by the measurement (CPU)."""
import numpy as np
import pytest

from busseq_gpu_gb300.diagnostics import adjusted_rand_index, ess_geyer


def test_ess_iid_and_ar1():
    rng = np.random.default_rng(0)
    iid = rng.standard_normal((64, 4000))
    e = ess_geyer(iid)
    assert 0.85 * 4000 < np.median(e) < 1.15 * 4000
    rho, n = 0.9, 40000
    z = rng.standard_normal((16, n))
    x = np.empty_like(z)
    x[:, 0] = z[:, 0]
    for t in range(1, n):
        x[:, t] = rho * x[:, t - 1] + np.sqrt(1 - rho * rho) * z[:, t]
    want = n * (1 - rho) / (1 + rho)
    got = ess_geyer(x)
    assert 0.8 * want < np.median(got) < 1.2 * want


def test_ess_constant_row_is_nan():
    d = np.ones((3, 100))
    d[1] = np.arange(100) % 7
    e = ess_geyer(d)
    assert np.isnan(e[0]) and np.isnan(e[2]) and np.isfinite(e[1])


def test_ari_known_values():
    a = np.array([0, 0, 1, 1, 2, 2])
    assert adjusted_rand_index(a, a) == pytest.approx(1.0)
    assert adjusted_rand_index(a, (a + 1) % 3) == pytest.approx(1.0)
    rng = np.random.default_rng(1)
    x, y = rng.integers(0, 5, 20000), rng.integers(0, 5, 20000)
    assert abs(adjusted_rand_index(x, y)) < 0.01
    skm = pytest.importorskip("sklearn.metrics")
    u, v = rng.integers(0, 4, 500), rng.integers(0, 6, 500)
    v[:250] = u[:250]
    assert adjusted_rand_index(u, v) == pytest.approx(skm.adjusted_rand_score(u, v), abs=1e-12)
