"""Training of the learned proposal on the GPU against its FP64 reference
(oracle/mlp.py).

- Sample collection: each sample's inputs are exactly the neighbour directors
  and T of the site it names, its target that site's director; augmentations
  preserve what they must (signs only; all pairwise dot products).
- The training kernel's loss and gradient match the FP64 ones (BF16 operands:
  loss within 1e-2 relative, each weight block's gradient within cosine 0.995
  and 5e-2 relative norm).
- Training lowers the loss below the isotropic density's log(4 pi) and the
  trained proposal is accepted far more often than an untrained one."""
import numpy as np
import pytest

import mcx
from oracle import mlp as M
from oracle import oracle as O
from helpers import desc_from_model, neighbours, random_state

pytestmark = pytest.mark.gpu

BLOCKS = ["W1", "b1", "W2", "b2", "W3", "b3"]


def _split_ids(samples):
    ids = samples[:, 22:24].copy().view(np.int32)
    return ids[:, 0], ids[:, 1]


def test_collect_samples_match_states():
    models = [O.Model(nx=16, ny=12, nz=10, potential="ll"),
              O.Model(nx=12, ny=8, nz=6, geometry="slab", potential="ll",
                      surfaces=[O.Surface("fg", 2.0), O.Surface("homeotropic", 3.0)]),
              O.Model(nx=12, ny=12, nz=12, geometry="sphere", potential="ll", surfaces=[O.Surface("fg", 1.0)])]
    Ts = [0.9, 1.1, 1.3]
    lats = [O.Lattice(m) for m in models]
    rng = np.random.default_rng(5)
    with mcx.Engine([desc_from_model(m, T=T, seed=3 + r) for r, (m, T) in enumerate(zip(models, Ts))]) as eng:
        states = []
        for r, (m, lat) in enumerate(zip(models, lats)):
            ni = random_state(m, lat.pt, rng)
            eng.set_state(r, ni)
            lat.ni[:] = eng.get_state(r)
            states.append(lat.ni.copy())
        n = 1500  # not a multiple of 256: a ragged last block
        smp = eng.collect_samples(n, seed=9)
        rep, site = _split_ids(smp)
        assert np.array_equal(rep, (np.arange(n) // 256) % 3)
        for q in range(n):
            r, s = int(rep[q]), int(site[q])
            m, lat = models[r], lats[r]
            assert 0 <= s < m.n and lat.pt[s] != 0
            assert np.array_equal(smp[q, :18], neighbours(lat, m, s).reshape(18).astype(np.float32))
            assert smp[q, 18] == np.float32(Ts[r])
            assert np.array_equal(smp[q, 19:22], states[r][s])
        # distinct sites as many as uniform draws with replacement give: the draw is not stuck
        for r, lat in enumerate(lats):
            k, N = int(np.sum(rep == r)), int(np.sum(lat.pt != 0))
            expect = N * (1 - (1 - 1 / N) ** k)
            assert len(set(site[rep == r].tolist())) > 0.9 * expect
        # flips: each director equals the state's up to sign
        fl = eng.collect_samples(n, seed=9, augment=mcx.AUG_FLIP)
        assert np.array_equal(_split_ids(fl)[1], site)
        for d in range(7):
            cols = slice(3 * d, 3 * d + 3) if d < 6 else slice(19, 22)
            a, b = fl[:, cols], smp[:, cols]
            assert np.all(np.all(a == b, axis=1) | np.all(a == -b, axis=1))
        assert np.mean(np.all(fl[:, 19:22] == -smp[:, 19:22], axis=1)) > 0.3
        with pytest.raises(mcx.McxError):
            eng.collect_samples(16, augment=mcx.AUG_ROTATE)  # surfaces: not a symmetry


def test_collect_rotation_preserves_geometry():
    m = O.Model(nx=16, ny=16, nz=16, potential="ll")
    lat = O.Lattice(m)
    with mcx.Engine([desc_from_model(m, T=1.0, seed=1)]) as eng:
        eng.set_state(0, random_state(m, lat.pt, np.random.default_rng(2)))
        n = 2048
        base = eng.collect_samples(n, seed=4)
        rot = eng.collect_samples(n, seed=4, augment=mcx.AUG_ROTATE)
    assert np.array_equal(_split_ids(rot)[1], _split_ids(base)[1])

    def vecs(x):
        return np.concatenate([x[:, :18].reshape(-1, 6, 3), x[:, None, 19:22]], axis=1).astype(np.float64)

    a, b = vecs(base), vecs(rot)
    ga = np.einsum("nik,njk->nij", a, a)
    gb = np.einsum("nik,njk->nij", b, b)
    assert np.max(np.abs(ga - gb)) < 2e-5
    # the rotations spread the targets over the sphere: mean ~ 0, second moment ~ I/3
    t = b[:, 6]
    assert np.linalg.norm(t.mean(0)) < 0.1
    assert np.max(np.abs(t.T @ t / n - np.eye(3) / 3)) < 0.05


def _synthetic_samples(rng, n):
    """Neighbour directors scattered around a random axis, T in [0.8, 1.3],
    targets near the axis with random signs, some neighbours absent."""
    ax = O.random_directors(n, rng)
    nb = ax[:, None, :] + 0.5 * rng.normal(size=(n, 6, 3))
    nb /= np.linalg.norm(nb, axis=2, keepdims=True)
    nb *= np.sign(rng.normal(size=(n, 6, 1)))
    nb[rng.random((n, 6)) < 0.1] = 0.0
    T = rng.uniform(0.8, 1.3, n)
    tgt = ax + 0.4 * rng.normal(size=(n, 3))
    tgt /= np.linalg.norm(tgt, axis=1, keepdims=True)
    tgt *= np.sign(rng.normal(size=(n, 1)))
    X = M.features(nb, T)
    return np.concatenate([X, tgt], axis=1).astype(np.float32)


@pytest.mark.parametrize("n", [64, 1000, 20000])
def test_gradient_matches_oracle(n):
    rng = np.random.default_rng(n)
    params = M.init_params(rng, scale=1.0)
    params[5] = np.array([0.2, -0.1, 0.3, 1.0])
    smp = _synthetic_samples(rng, n)
    m = O.Model(nx=8, ny=8, nz=8, potential="ll")
    with mcx.Engine([desc_from_model(m)]) as eng:
        w = M.pack_weights(params)
        eng.set_mlp(w)
        loss, g = eng.mlp_grad(smp)
    p32 = M.unpack_weights(w)
    X = smp[:, :19].astype(np.float64)
    lref, gref = M.nll_and_grad(p32, X, smp[:, 19:22].astype(np.float64))
    assert abs(loss - lref) < 1e-2 * abs(lref), (loss, lref)
    gref_flat = M.pack_weights(gref).astype(np.float64)
    off = 0
    sizes = [M.K_IN * M.D_H, M.D_H, M.D_H * M.D_H, M.D_H, M.D_H * M.N_OUT, M.N_OUT]
    for name, sz in zip(BLOCKS, sizes):
        a, b = g[off:off + sz].astype(np.float64), gref_flat[off:off + sz]
        off += sz
        cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert cos > 0.995 and rel < 5e-2, (name, cos, rel)
    # padding carries no gradient
    W1g = g[:M.K_IN * M.D_H].reshape(M.K_IN, M.D_H)
    assert np.all(W1g[M.D_IN:] == 0)


def test_training_learns_the_conditional():
    """LL bulk near the transition: equilibrate with the plain move, train on
    the GPU, then the learned proposal's acceptance must beat an untrained
    network's by far, and the GPU loss must agree with the FP64 loss of the
    downloaded weights on fresh samples."""
    m = O.Model(nx=16, ny=16, nz=16, potential="ll")
    R, T = 4, 1.1
    descs = [desc_from_model(m, T=T, seed=50 + r, stream=r) for r in range(R)]
    with mcx.Engine(descs) as eng:
        for r in range(R):
            eng.init_random(r, 3 + r)
        eng.sweep(300)
        rng = np.random.default_rng(0)
        params = M.init_params(rng, scale=1.0)
        eng.set_mlp(M.pack_weights(params))
        eng.set_proposal("vmf_mlp")
        eng.reset_stats()
        eng.sweep(20, measure=True)
        acc0 = np.mean([eng.stats(r)[mcx.ST_ACC] / (eng.stats(r)[mcx.ST_SWEEPS] * m.n) for r in range(R)])
        eng.set_proposal("plain")
        losses = eng.train_mlp(samples=1 << 16, batch=1024, steps=400, lr=3e-3, seed=11,
                               augment=mcx.AUG_FLIP | mcx.AUG_ROTATE)
        assert np.all(np.isfinite(losses))
        assert losses[-20:].mean() < losses[:5].mean() - 0.1
        assert losses[-20:].mean() < np.log(4 * np.pi) - 0.2
        fresh = eng.collect_samples(8192, seed=99)
        lgpu, _ = eng.mlp_grad(fresh)
        w = eng.get_mlp()
        lref, _ = M.nll_and_grad(M.unpack_weights(w), fresh[:, :19].astype(np.float64),
                                 fresh[:, 19:22].astype(np.float64))
        assert abs(lgpu - lref) < 1e-2 * abs(lref) + 1e-3
        eng.set_proposal("vmf_mlp")
        eng.reset_stats()
        eng.sweep(20, measure=True)
        acc1 = np.mean([eng.stats(r)[mcx.ST_ACC] / (eng.stats(r)[mcx.ST_SWEEPS] * m.n) for r in range(R)])
    assert acc1 > 0.45 and acc1 > acc0 + 0.15, (acc0, acc1)


def test_training_errors():
    m = O.Model(nx=8, ny=8, nz=8, potential="ll")
    with mcx.Engine([desc_from_model(m)]) as eng:
        with pytest.raises(mcx.McxError):
            eng.train_mlp(samples=256, batch=64, steps=1)  # no weights yet
        eng.set_mlp(M.pack_weights(M.init_params(np.random.default_rng(1))))
        with pytest.raises(mcx.McxError):
            eng.train_mlp(samples=0, batch=64, steps=1)
        with pytest.raises(mcx.McxError):
            eng.train_mlp(samples=256, batch=64, steps=1, lr=-1.0)
        with pytest.raises(mcx.McxError):
            eng.collect_samples(16, augment=8)
        eng.train_mlp(samples=256, batch=64, steps=2)


def test_trained_proposal_shortens_autocorrelation():
    """What the trained network gains over the method without it, per sweep:
    LL 16^3 x 32 replicas at T = 1.15, both chains from the same equilibrated
    states with the step size frozen; the learned chain's integrated
    autocorrelation time of S is well below the plain chain's, and the two
    agree on E and S within 3 combined standard errors (exact MH ratio)."""
    from mcx.autocorr import tau_int
    from mcx import gain
    m = O.Model(nx=16, ny=16, nz=16, potential="ll")
    R, T, n = 32, 1.15, 3000
    with mcx.Engine([desc_from_model(m, T=T, seed=70 + r, stream=r) for r in range(R)]) as eng:
        for r in range(R):
            eng.init_random(r, 9 + r)
        eng.sweep(1000)
        eng.set_mlp(gain.init_weights(3))
        eng.train_mlp(samples=1 << 17, batch=4096, steps=800, lr=2e-3, seed=5, augment=mcx.AUG_FLIP | mcx.AUG_ROTATE)
        eng.set_adapt(False)
        saved = [eng.get_state(r) for r in range(R)]
        eng.set_series(n)
        out = {}
        for kind in ("plain", "vmf_mlp"):
            for r in range(R):
                eng.set_state(r, saved[r])
            eng.set_proposal(kind)
            eng.reset_stats()
            eng.sweep(n, measure=True)
            ser = np.array([eng.series(r, n) for r in range(R)])
            out[kind] = (tau_int(ser[:, :, 1])["tau"], ser[:, :, 0].mean(1), ser[:, :, 1].mean(1))
    tp, tl = out["plain"][0], out["vmf_mlp"][0]
    assert tl < 0.7 * tp, (tp, tl)
    for q in (1, 2):
        a, b = out["plain"][q], out["vmf_mlp"][q]
        se = np.hypot(a.std(ddof=1), b.std(ddof=1)) / np.sqrt(R)
        assert abs(a.mean() - b.mean()) <= 3 * se, (q, a.mean(), b.mean(), se)


def test_learned_and_plain_agree_at_every_c4_temperature():
    """The learned-proposal protocol of the 96^3 workload (mcx.gain: plain
    equilibration, training on the plain sampler's states, frozen step, both
    proposals from the same saved states) on 16^3 lattices: at each of
    T = 1.00, 1.10, 1.12, 1.15, over 32 replicas, E and S of the two chains
    agree within 3 combined standard errors, and the trained network shortens
    the integrated autocorrelation time per sweep."""
    from mcx import gain
    res = gain.run(L=16, per_T=32, equil=1500, meas=2000, train_samples=1 << 18,
                   schedule=((600, 2e-3), (300, 5e-4)), batch=4096, seed=3)
    for row in res["rows"]:
        assert row["E_diff_sigma"] <= 3 and row["S_diff_sigma"] <= 3, row
        assert row["tau_ratio"] > 1.0, row
