"""The Madras-Sokal integrated autocorrelation time estimator on series of
known tau: AR(1) processes (tau = (1 + phi) / (2 (1 - phi))) and white noise."""
import numpy as np
import pytest

from mcx.autocorr import ar1, autocovariance, tau_int


@pytest.mark.parametrize("phi", [0.0, 0.5, 0.9, 0.97])
def test_tau_of_ar1(phi):
    rng = np.random.default_rng(int(phi * 100))
    x = ar1(20000, phi, rng, replicas=8)
    want = (1 + phi) / (2 * (1 - phi))
    got = tau_int(x)
    assert got["reliable"]
    assert abs(got["tau"] - want) < max(4 * got["err"], 0.05 * want), (got, want)


def test_autocovariance_matches_direct_sum():
    rng = np.random.default_rng(1)
    x = rng.normal(size=(3, 200))
    C = autocovariance(x)
    xc = x - x.mean(1, keepdims=True)
    for t in (0, 1, 5, 50):
        direct = np.mean([np.sum(r[:200 - t] * r[t:]) / 200 for r in xc])
        assert abs(C[t] - direct) < 1e-12


def test_short_series_is_flagged():
    rng = np.random.default_rng(2)
    x = ar1(200, 0.99, rng)
    assert not tau_int(x)["reliable"]


def test_constant_series():
    assert tau_int(np.ones((2, 100)))["tau"] == 0.5
