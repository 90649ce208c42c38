"""The learned proposal on the GPU against its FP64 reference (oracle/mlp.py).

Per red/black pass, for every updated site: the network's outputs match the
FP64 forward pass with the engine's BF16 roundings (within 3e-2, set by BF16
activations and the hardware tanh); the proposal matches the FP64 inverse-CDF
draw from those outputs and the same Philox uniforms; the accept/reject
decision matches the FP64 Metropolis-Hastings ratio evaluated on the GPU's
proposal, except inside the 1e-5 tie band; the state is what the decisions
say.  And the MH correction is exact: with any weights the learned chain
samples the same equilibrium E and S as the plain one."""
import numpy as np
import pytest

import mcx
from oracle import mlp as M
from oracle import oracle as O
from helpers import desc_from_model, neighbours, random_state

pytestmark = pytest.mark.gpu

CASES = {
    "bulk_ll": O.Model(nx=16, ny=8, nz=8, potential="ll"),
    "slab_ghrl_field": O.Model(nx=12, ny=8, nz=6, geometry="slab", potential="ghrl", k11=1.0, k22=0.6, k33=1.4,
                               p0=20, elecA=0.4, elecZ=1.0, elecE=1.5,
                               surfaces=[O.Surface("fg", 2.0), O.Surface("homeotropic", 3.0)]),
    "sphere_ll": O.Model(nx=12, ny=12, nz=12, geometry="sphere", potential="ll", surfaces=[O.Surface("fg", 1.0)]),
}


def _weights(seed, scale=1.5):
    rng = np.random.default_rng(seed)
    params = M.init_params(rng, scale=scale)
    params[5] = np.array([0.0, 0.0, 0.3, 1.0])  # a typical kappa ~ e
    return params


def _vmf_uniforms(site, seed, stream, sweep):
    r = O.philox([site, sweep & 0xFFFFFFFF, sweep >> 32, 2], [seed, stream])
    return O.u24(r)


@pytest.mark.parametrize("name", list(CASES))
def test_learned_pass_parity(name):
    m = CASES[name]
    T, seed, stream = 0.9, 31, 4
    params = _weights(1)
    lat = O.Lattice(m)
    rng = np.random.default_rng(8)
    ni0 = random_state(m, lat.pt, rng)
    with mcx.Engine([desc_from_model(m, T=T, seed=seed, stream=stream)]) as eng:
        eng.set_state(0, ni0)
        eng.set_mlp(M.pack_weights(params))
        eng.set_proposal("vmf_mlp")
        i = np.arange(m.n) % m.nx
        j = (np.arange(m.n) // m.nx) % m.ny
        k = np.arange(m.n) // (m.nx * m.ny)
        ties = 0
        for colour in (0, 1):
            before = eng.get_state(0)
            dE, acc, prop, y = eng.debug_pass_mlp(0, colour)
            after = eng.get_state(0)
            upd = (((i + j + k) & 1) == colour) & (lat.pt != 0)
            assert np.all(acc[~upd] == 255)
            lat.ni[:] = before
            sites = np.nonzero(upd)[0]
            # network outputs
            nbrs = np.zeros((len(sites), 6, 3))
            for q, s in enumerate(sites):
                nbrs[q] = neighbours(lat, m, int(s))
            X = M.features(nbrs, T)
            Yref = M.forward_bf16(params, X)
            assert np.max(np.abs(y[sites] - Yref)) < 3e-2
            for q, s in enumerate(sites):
                u = _vmf_uniforms(int(s), seed, stream, 0)
                Yg = y[s:s + 1].astype(np.float64)
                v = M.sample(Yg, u[0:1], u[1:2], u[2:3])[0]
                assert np.max(np.abs(prop[s] - v)) < 1e-4, (s, prop[s], v)
                e1, a1 = lat.local_energy_abs(int(s), prop[s])
                e0, a0 = lat.local_energy_abs(int(s), before[s])
                assert abs(dE[s] - (e1 - e0)) <= 1e-5 * max(a1 + a0, 1e-3)
                lr = M.mh_log_ratio(Yg, before[s:s + 1].astype(np.float64), prop[s:s + 1].astype(np.float64),
                                    np.array([e1 - e0]), T)[0]
                p = np.exp(min(lr, 50.0))
                if p < 1 and abs(u[3] - p) <= 1e-5 * (1 + p):
                    ties += 1
                    continue
                assert bool(acc[s]) == (u[3] < p), (s, u[3], p)
            want = before.copy()
            want[acc == 1] = prop[acc == 1]
            assert np.array_equal(after, want)


@pytest.mark.parametrize("path", ["tcgen05", "warp"])
@pytest.mark.parametrize("T", [0.8, 1.6])
def test_learned_chain_samples_the_same_equilibrium(T, path):
    """Random (untrained) weights: a poor proposal, but the exact MH ratio
    keeps the Boltzmann distribution -- E and S agree with the plain chain
    within 3 combined standard errors over 32 replicas each, with the learned
    z-march's network on the tensor cores or at warp level."""
    m = O.Model(nx=8, ny=8, nz=8, potential="ll")
    params = _weights(2, scale=1.0)
    R = 32
    res = {}
    for kind in ("plain", "vmf_mlp"):
        descs = [desc_from_model(m, T=T, seed=100 + r, stream=r) for r in range(R)]
        with mcx.Engine(descs) as eng:
            for r in range(R):
                eng.init_random(r, 7 + r)
            if kind == "vmf_mlp":
                eng.set_mlp(M.pack_weights(params))
                eng.mlp_path = path
                eng.set_proposal("vmf_mlp")
            eng.sweep(600)
            eng.reset_stats()
            eng.sweep(600, measure=True)
            st = np.array([eng.stats(r) for r in range(R)])
        n = st[:, mcx.ST_N]
        res[kind] = (st[:, mcx.ST_E1] / n, st[:, mcx.ST_S1] / n)
    for q in range(2):
        a, b = res["plain"][q], res["vmf_mlp"][q]
        se = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
        assert abs(a.mean() - b.mean()) <= 3 * se, (q, a.mean(), b.mean(), se)


IDENTITY_CASES = {**CASES,
                  # a small droplet in a large box: units with no active site around are skipped
                  "droplet_big_box": O.Model(nx=32, ny=32, nz=40, geometry="sphere", potential="ghrl", k11=1.0,
                                             k22=0.6, k33=1.4, p0=20, elecA=0.3, elecZ=1.0, elecE=1.5, radius=6.0,
                                             surfaces=[O.Surface("fg", 1.0)]),
                  # odd lengths: the learned passes built with phantom-slot handling
                  "droplet_odd13": O.Model(nx=13, ny=13, nz=13, geometry="sphere", potential="ghrl", k11=1.0,
                                           k22=0.6, k33=1.4, p0=20, elecA=0.3, elecZ=1.0, elecE=1.5,
                                           surfaces=[O.Surface("fg", 1.0)]),
                  "bulk_ll_odd_free": O.Model(nx=9, ny=8, nz=6, xbound="free", potential="ll")}


@pytest.mark.parametrize("name", list(IDENTITY_CASES))
def test_learned_march_equals_learned_direct_pass(name):
    """The learned z-march with the warp-level network and the learned direct
    pass give bit-identical states, step sizes and acceptance counts after
    measured sweeps."""
    m = IDENTITY_CASES[name]
    params = _weights(4)
    lat = O.Lattice(m)
    out = []
    for kind in ("march", "direct"):
        with mcx.Engine([desc_from_model(m, T=0.9, seed=13, stream=2)]) as eng:
            eng.pass_kind = kind
            eng.set_state(0, random_state(m, lat.pt, np.random.default_rng(6)))
            eng.set_mlp(M.pack_weights(params))
            if kind == "march":
                eng.mlp_path = "warp"
                assert eng.mlp_path == "warp"
            eng.set_proposal("vmf_mlp")
            eng.sweep(11, measure=True)
            out.append((eng.get_state(0), eng.stats(0)))
    (sa, ta), (sb, tb) = out
    assert np.array_equal(sa, sb)
    assert ta[mcx.ST_ANG_VAR] == tb[mcx.ST_ANG_VAR] and ta[mcx.ST_ACC] == tb[mcx.ST_ACC]
    assert ta[mcx.ST_S1] == pytest.approx(tb[mcx.ST_S1], rel=1e-6)


def test_learned_forms_agree_over_long_runs():
    """32 chiral droplets in a field, 50 + 50 measured learned sweeps: the
    learned z-march with the warp-level network runs the learned direct
    pass's chain bit for bit (the same network code, and the MH ratio's
    roundings fixed); the tensor-core network sums in another order, so its
    chain parts from theirs, but it samples the same states: replica-averaged
    S and E agree with the direct pass's within 3 combined standard errors."""
    m = O.Model(nx=64, ny=64, nz=64, geometry="sphere", xbound="free", ybound="free", zbound="free",
                potential="ghrl", k11=1.0, k22=0.6, k33=1.4, p0=20.0, elecA=1.0, elecZ=1.0, elecE=0.5, radius=26.0,
                surfaces=[O.Surface("fg", 1.0)])
    R = 32
    descs = [desc_from_model(m, T=0.8, seed=500 + q, stream=q) for q in range(R)]
    params = _weights(4)
    means, states = [], []
    for kind, path in (("direct", None), ("march", "tcgen05"), ("march", "warp")):
        with mcx.Engine(descs) as eng:
            eng.pass_kind = kind
            for q in range(R):
                eng.init_random(q, 11 + q)
            eng.set_mlp(M.pack_weights(params))
            if path:
                eng.mlp_path = path
            eng.set_proposal("vmf_mlp")
            eng.sweep(50)
            eng.reset_stats()
            eng.sweep(50, measure=True)
            st = [eng.stats(q) for q in range(R)]
            states.append([eng.get_state(q) for q in range(R)])
        means.append((np.array([t[mcx.ST_S1] / t[mcx.ST_N] for t in st]),
                      np.array([t[mcx.ST_E1] / t[mcx.ST_N] for t in st])))
    for q in range(R):  # warp-level learned z-march == learned direct pass
        assert np.array_equal(states[0][q], states[2][q]), q
    for other in means[1:]:
        for a, b in zip(means[0], other):
            se = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
            assert abs(a.mean() - b.mean()) <= 3 * se, (a.mean(), b.mean(), se)


@pytest.mark.parametrize("n", [1, 5, 128, 1000, 40000])
def test_network_on_tensor_cores_matches_the_oracle(n):
    """mcx_mlp_forward: the network on the tcgen05 tensor cores (FP32
    accumulators in tensor memory) and with the learned passes' warp-level
    mma.sync code, on rows of neighbour directors (some absent) and
    temperatures, against the FP64 forward pass with the engine's BF16
    roundings (within 3e-2, as the learned pass's outputs, up to 1000 rows;
    over 40000 rows the tail of BF16 activation roundings reaches further: the
    99.9th percentile within 2e-2 and every output within 5e-2); the two GPU
    paths take the same BF16 operands and differ only in the order of the FP32
    sums, so most outputs agree exactly and every one within those bounds."""
    params = _weights(11)
    rng = np.random.default_rng(n)
    nb = O.random_directors(6 * n, rng).reshape(n, 6, 3)
    nb[rng.random((n, 6)) < 0.15] = 0.0
    X = M.features(nb, rng.uniform(0.5, 1.5, n))
    ref = M.forward_bf16(params, X)
    m = O.Model(nx=8, ny=8, nz=8, potential="ll")
    with mcx.Engine([desc_from_model(m)]) as eng:
        eng.set_mlp(M.pack_weights(params))
        tc = eng.mlp_forward(X, "tcgen05")
        wp = eng.mlp_forward(X, "warp")
        again = eng.mlp_forward(X, "tcgen05")
    bound = 3e-2 if n <= 1000 else 5e-2
    for got in (tc, wp):
        d = np.abs(got - ref)
        assert np.max(d) < bound and np.quantile(d, 0.999) < 2e-2, (np.max(d), np.quantile(d, 0.999))
    assert np.max(np.abs(tc - wp)) < bound
    assert np.mean(tc == wp) > 0.5
    assert np.array_equal(tc, again)  # deterministic run to run
