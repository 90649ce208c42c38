"""Oracle self-checks that need no reference build: Philox known answers,
analytic ground states, eigen-solver and the step-size rule."""
import numpy as np
import pytest

from oracle import oracle as O

# Published Philox4x32-10 known-answer vectors (Random123 distribution,
# kat_vectors: philox4x32 10 rounds).
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox_known_answers(ctr, key, want):
    got = O.philox(ctr, key)
    assert [int(x) for x in got] == list(want)


def test_ll_homogeneous_ground_state():
    # n = z everywhere, periodic LL: each site has 6 bonds of -1.5 A
    m = O.Model(nx=8, ny=6, nz=4, A=1.0)
    lat = O.Lattice(m)
    r = lat.measure()
    assert r["E"] == pytest.approx(-9.0, abs=1e-12)
    assert r["E_valid"] == pytest.approx(-9.0, abs=1e-12)
    assert r["S"] == pytest.approx(1.0, abs=1e-12)
    assert abs(abs(r["director"][2]) - 1) < 1e-12


def test_ll_free_bounds_count_bonds():
    m = O.Model(nx=4, ny=4, nz=4, xbound="free", ybound="free", zbound="free", A=2.0)
    lat = O.Lattice(m)
    # number of directed bonds in a free 4^3 cube: 3 axes * 2 dirs * 3*16
    nb = 3 * 2 * 3 * 16
    assert lat.measure()["E"] == pytest.approx(-1.5 * 2.0 * nb / 64, abs=1e-12)


def test_ghrl_homogeneous_pair_matches_formula():
    m = O.Model(potential="ghrl", k11=1.0, k22=0.8, k33=1.2, p0=0)
    lat = O.Lattice(m)
    lam, mu, nu, rho, sigma = [float(v) for v in O.ghrl_constants(1.0, 0.8, 1.2, 0)]
    n = np.array([0, 0, 1.0])
    # bond along x with ni = nj = z: ai = aj = 0, nij = 1 -> P2 = 1, E1 = -1
    want = -1 * (rho + lam) + mu * (0 - 1 / 9) + nu
    assert lat.pair(n, n, 0) == pytest.approx(want, abs=1e-12)
    # bond along z: ai = aj = 1 -> E1 = 2
    want_z = 2 * (rho + lam) + mu * (1 - 1 / 9) + nu
    assert lat.pair(n, n, 4) == pytest.approx(want_z, abs=1e-12)


def test_eigmax_random_symmetric():
    rng = np.random.default_rng(3)
    for _ in range(50):
        a = rng.normal(size=(3, 3))
        q = a + a.T
        lam, v = O.eigmax(q)
        w, V = np.linalg.eigh(q)
        assert lam == pytest.approx(w[-1], abs=1e-12)
        assert abs(abs(np.dot(v, V[:, -1])) - 1) < 1e-10


def test_adapt_rule():
    # src/evolve.cpp:169-178
    assert O.adapt(0.5, 10, 100) == np.float32(0.5 * 0.99)
    assert O.adapt(0.5, 90, 100) == np.float32(0.5 / 0.99)
    assert O.adapt(0.5, 50, 100) == np.float32(0.5)
    assert O.adapt(np.float32(0.0100001), 0, 100) == np.float32(0.01)
    a = O.adapt(np.float32(0.999), 100, 100)
    assert a == np.float32(np.float32(np.float32(0.999) / 0.99) - 0.5)


def test_sweep_orders_preserve_norm_and_mask():
    rng = np.random.default_rng(1)
    m = O.Model(nx=8, ny=8, nz=8, geometry="sphere", potential="ghrl", k11=1, k22=0.6, k33=1.4, p0=20,
                surfaces=[O.Surface("fg", 2.0)])
    lat = O.Lattice(m)
    ni = O.random_directors(m.n, rng)
    ni[lat.pt == 0] = (0, 0, 1)
    lat.ni[:] = ni
    for order in ("redblack", "eight"):
        acc, a = lat.sweep(1.0, 0.5, 7, 0, 0, order)
        assert 0 < acc <= lat.valid
        assert np.allclose(np.linalg.norm(lat.ni, axis=1), 1, atol=1e-6)
        assert np.all(lat.ni[lat.pt == 0] == np.array([0, 0, 1], np.float32))


def test_parallel_pass_equals_serial():
    rng = np.random.default_rng(2)
    m = O.Model(nx=12, ny=10, nz=8, potential="ghrl", k11=1, k22=0.8, k33=1.2)
    a = O.Lattice(m, ni=O.random_directors(m.n, rng))
    b = O.Lattice(m, ni=a.ni.copy())
    for q in range(2):
        a.run_pass(1.0, 0.4, 11, 3, 5, "redblack", q)
        b.run_pass(1.0, 0.4, 11, 3, 5, "redblack", q, flags=O.F_PARALLEL)
    assert np.array_equal(a.ni, b.ni)
