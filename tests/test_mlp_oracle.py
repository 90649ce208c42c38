"""The learned proposal's FP64 reference: gradients by finite differences,
the mixture's normalisation and symmetry, the sampler's law, the MH ratio."""
import numpy as np
import pytest

from oracle import mlp as M


def _batch(rng, B=64):
    nb = rng.normal(size=(B, 6, 3))
    nb /= np.linalg.norm(nb, axis=2, keepdims=True)
    X = M.features(nb, rng.uniform(0.8, 1.2, B))
    n = rng.normal(size=(B, 3))
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    return X, n


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    params = M.init_params(rng, scale=1.5)
    X, n = _batch(rng)
    loss, grads = M.nll_and_grad(params, X, n)
    eps = 1e-6
    for pi, (p, g) in enumerate(zip(params, grads)):
        flat = p.reshape(-1)
        for idx in rng.choice(flat.size, size=min(12, flat.size), replace=False):
            old = flat[idx]
            flat[idx] = old + eps
            lp, _ = M.nll_and_grad(params, X, n)
            flat[idx] = old - eps
            lm, _ = M.nll_and_grad(params, X, n)
            flat[idx] = old
            fd = (lp - lm) / (2 * eps)
            assert g.reshape(-1)[idx] == pytest.approx(fd, rel=1e-5, abs=1e-8), (pi, idx)


def test_density_is_normalised_and_antipodal():
    rng = np.random.default_rng(1)
    for logk in (-3.0, 0.0, 2.0, 5.0):
        Y = np.array([[0.3, -0.2, 0.9, logk]])
        # Monte Carlo over uniform directions: E_uniform[q] * 4 pi = 1
        v = rng.normal(size=(200000, 3))
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        q = np.exp(M.log_density(np.repeat(Y, len(v), 0), v))
        assert np.mean(q) * 4 * np.pi == pytest.approx(1.0, rel=2e-2 if logk < 4 else 8e-2)
        assert np.allclose(M.log_density(np.repeat(Y, 10, 0), v[:10]), M.log_density(np.repeat(Y, 10, 0), -v[:10]))


def test_sampler_follows_the_density():
    rng = np.random.default_rng(2)
    Y = np.repeat(np.array([[0.0, 0.6, 0.8, np.log(4.0)]]), 200000, 0)
    s = M.sample(Y, rng.uniform(size=len(Y)), rng.uniform(size=len(Y)), rng.uniform(size=len(Y)))
    assert np.allclose(np.linalg.norm(s, axis=1), 1, atol=1e-12)
    muhat = np.array([0.0, 0.6, 0.8])
    w = np.abs(s @ muhat)
    # |w| has density proportional to cosh(kappa w) on [0, 1]
    k = 4.0
    hist, edges = np.histogram(w, bins=20, range=(0, 1), density=True)
    mid = 0.5 * (edges[1:] + edges[:-1])
    want = k * np.cosh(k * mid) / np.sinh(k)
    assert np.allclose(hist, want, rtol=0.05, atol=0.02)
    # both hemispheres equally likely
    assert abs(np.mean(s @ muhat > 0) - 0.5) < 0.01


def test_pack_roundtrip():
    rng = np.random.default_rng(3)
    params = M.init_params(rng)
    flat = M.pack_weights(params)
    assert flat.size == M.N_PARAMS
    back = M.unpack_weights(flat)
    for a, b in zip(params, back):
        assert np.allclose(a, b, atol=1e-6)


def test_mh_ratio_detailed_balance_on_a_single_site():
    """With the exact local conditional as the 'energy', the MH chain with the
    mixture proposal samples it: compare <(n.z)^2> against quadrature."""
    rng = np.random.default_rng(4)
    beta = 3.0  # target density ~ exp(beta (n.z)^2)
    Y = np.array([[0.2, 0.1, 1.0, np.log(2.0)]])
    n = np.array([[0.0, 0.0, 1.0]])
    acc = []
    for _ in range(60000):
        s = M.sample(Y, rng.uniform(size=1), rng.uniform(size=1), rng.uniform(size=1))
        dE = -(s[0, 2] ** 2 - n[0, 2] ** 2)
        if np.log(rng.uniform()) < M.mh_log_ratio(Y, n, s, np.array([dE]), 1.0 / beta)[0]:
            n = s
        acc.append(n[0, 2] ** 2)
    x = np.linspace(-1, 1, 20001)
    p = np.exp(beta * x ** 2)
    want = np.sum(x ** 2 * p) / np.sum(p)
    assert np.mean(acc[5000:]) == pytest.approx(want, abs=0.01)
