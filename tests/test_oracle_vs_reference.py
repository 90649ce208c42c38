"""Pins the oracle to the reference's own compiled C++ (oracle/_ref).

Each case runs the reference in a fresh process (it keeps lattice-sized
function statics).  Skipped where the reference tree was not available at
build time."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import refproc

pytestmark = pytest.mark.skipif(not refproc.available(), reason="reference build (oracle/_ref) not present")

ALL_ANCH = ["homeotropic", "fg", "rp", "strong", "homeotropic_ghrl", "fg_ghrl", "rp_ghrl", "strong_ghrl"]
RIJ = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32)


def _ghrl_model(**kw):
    base = dict(nx=8, ny=8, nz=8, potential="ghrl", k11=1.0, k22=0.6, k33=1.4, p0=20.0)
    base.update(kw)
    return O.Model(**base)


@pytest.mark.parametrize("k", [(1.0, 0.8, 1.2, 0.0), (1.0, 0.6, 1.4, 20.0), (1.48, 1.0, 2.28, 0.0), (1, 1, 1, 40.0)])
def test_ghrl_constants_bit_exact(k):
    m = O.Model(nx=4, ny=4, nz=4, potential="ghrl", k11=k[0], k22=k[1], k33=k[2], p0=k[3])
    (g,) = refproc.run(m, [("ghrl",)])
    lam, mu, nu, rho, sigma = O.ghrl_constants(*k)
    assert np.array_equal(g, np.array([lam, mu, nu, rho, sigma], np.float32))


@pytest.mark.parametrize("geo,dims", [("bulk", (6, 4, 5)), ("slab", (6, 4, 5)), ("sphere", (10, 10, 10)),
                                      ("sphere", (9, 8, 11)), ("slab", (4, 4, 1))])
def test_masks_bit_exact(geo, dims):
    nsurf = {"bulk": 0, "slab": 2, "sphere": 1}[geo]
    m = O.Model(nx=dims[0], ny=dims[1], nz=dims[2], geometry=geo,
                surfaces=[O.Surface("homeotropic", 1.0)] * nsurf)
    ((pt, ns),) = refproc.run(m, [("mask",)])
    lat = O.Lattice(m)
    assert np.array_equal(lat.pt, pt)
    assert np.array_equal(lat.ns, ns)


@pytest.mark.parametrize("pot", ["ll", "ghrl", "pear"])
def test_pair_energies(pot):
    rng = np.random.default_rng(5)
    m = _ghrl_model(potential=pot, A=1.3, B1=0.3, C=0.45)
    a = O.random_directors(600, rng)
    b = O.random_directors(600, rng)
    r = np.tile(RIJ, (100, 1))
    (ref,) = refproc.run(m, [("pairs", a, b, r)])
    lat = O.Lattice(m)
    mine = np.array([lat.pair(a[q], b[q], q % 6) for q in range(600)])
    assert np.max(np.abs(mine - ref)) < 4e-6


@pytest.mark.parametrize("pot", ["ll", "ghrl"])
def test_surface_energies_all_anchorings(pot):
    rng = np.random.default_rng(6)
    surfs = [O.Surface(a, 1.7, theta_s=30.0, phi_s=45.0) for a in ALL_ANCH]
    m = _ghrl_model(potential=pot, geometry="bulk", surfaces=surfs)
    n = O.random_directors(200, rng)
    s = O.random_directors(200, rng)
    ops = [("surface", q, n, s) for q in range(len(ALL_ANCH))]
    ref = refproc.run(m, ops)
    lat = O.Lattice(m)
    for q in range(len(ALL_ANCH)):
        mine = np.array([lat.surface(q, n[t], s[t]) for t in range(200)])
        assert np.max(np.abs(mine - ref[q])) < 1e-5, ALL_ANCH[q]


def test_field_energy():
    rng = np.random.default_rng(7)
    m = O.Model(nx=4, ny=4, nz=4, elecA=0.7, elecX=0.2, elecY=0.3, elecZ=1.1, elecE=1.6)
    n = O.random_directors(100, rng)
    (ref,) = refproc.run(m, [("field", n)])
    lat = O.Lattice(m)
    mine = np.array([lat.field(x) for x in n])
    assert np.max(np.abs(mine - ref)) < 2e-6


CASES = [
    dict(geometry="bulk", potential="ll"),
    dict(geometry="bulk", potential="ghrl", elecA=0.5, elecZ=1.0, elecE=1.5),
    dict(geometry="slab", potential="ghrl", xbound="periodic", ybound="periodic",
         surfaces=[O.Surface("homeotropic", 4.0), O.Surface("homeotropic", 4.0)]),
    dict(geometry="slab", potential="ghrl", surfaces=[O.Surface("fg_ghrl", 1.5), O.Surface("homeotropic_ghrl", 2.0)]),
    dict(geometry="sphere", potential="ghrl", surfaces=[O.Surface("fg", 2.0)], elecA=0.3, elecZ=1.0, elecE=2.0),
    dict(geometry="sphere", potential="ll", surfaces=[O.Surface("rp", 1.0, theta_s=60, phi_s=10)]),
    dict(geometry="bulk", potential="pear", B1=0.3, C=0.3),
    dict(geometry="sphere", potential="pear", B1=0.3, C=0.3, surfaces=[O.Surface("homeotropic", 4.0)]),
]


def _lattice_for(case, rng, dims=(8, 8, 8)):
    m = _ghrl_model(nx=dims[0], ny=dims[1], nz=dims[2], **case)
    lat = O.Lattice(m)
    ni = O.random_directors(m.n, rng)
    ni[lat.pt == 0] = (0, 0, 1)
    lat.ni[:] = ni
    return m, lat


@pytest.mark.parametrize("case", range(len(CASES)))
def test_local_energies(case):
    rng = np.random.default_rng(10 + case)
    m, lat = _lattice_for(CASES[case], rng)
    sites = rng.integers(0, m.n, 300)
    newn = O.random_directors(300, rng)
    (ref,) = refproc.run(m, [("local", lat.ni, sites, newn)])
    mine = np.array([lat.local_energy(int(s), newn[q]) for q, s in enumerate(sites)])
    assert np.max(np.abs(mine - ref)) < 2e-5


@pytest.mark.parametrize("case", range(len(CASES)))
def test_sweep_with_fed_uniforms_matches_reference(case):
    """One EvolveN::Monte_Carlo_Step of the reference, fed the oracle's Philox
    uniforms in its visiting order, against the oracle's eight-colour sweep
    without renormalisation: identical accept/reject decisions, directors
    equal to float rounding, identical step-size update."""
    rng = np.random.default_rng(20 + case)
    m, lat = _lattice_for(CASES[case], rng)
    T, a0, seed, stream, sweep = 0.9, np.float32(0.5), 1234, 7, 3
    feed = O.sweep_uniforms(m, lat.pt, seed, stream, sweep, "eight")
    ((ref_ni, ref_a, used),) = refproc.run(m, [("sweep", lat.ni, T, float(a0), feed)])
    assert used == len(feed)
    before = lat.ni.copy()
    ties = 0
    acc = 0
    for q in range(8):
        n_acc, tr = lat.run_pass(T, a0, seed, stream, sweep, "eight", q, flags=O.F_NO_NORMALIZE, trace=True)
        ties += int(tr["tie"].sum())
        acc += n_acc
    assert ties == 0, "tie inside the decision band: pick another seed"
    moved_ref = np.any(ref_ni != before, axis=1)
    moved_orc = np.any(lat.ni != before, axis=1)
    assert np.array_equal(moved_ref, moved_orc)
    assert np.max(np.abs(lat.ni - ref_ni)) < 2e-6
    assert np.float32(O.adapt(a0, acc, lat.valid)) == np.float32(ref_a)


@pytest.mark.parametrize("case", range(len(CASES)))
def test_energy_and_order_parameter(case):
    rng = np.random.default_rng(40 + case)
    m, lat = _lattice_for(CASES[case], rng)
    # a partially ordered field so that S is away from 0
    lat.ni[:] = lat.ni * 0.6 + np.array([0.3, 0.1, 1.0], np.float32)
    lat.ni /= np.linalg.norm(lat.ni, axis=1, keepdims=True)
    lat.ni[lat.pt == 0] = (0, 0, 1)
    E_ref, (S_ref, Q_ref, v_ref) = refproc.run(m, [("energy", lat.ni), ("order", lat.ni)])
    r = lat.measure()
    assert r["E"] == pytest.approx(E_ref, abs=2e-5 * max(1, abs(E_ref)))
    assert r["S"] == pytest.approx(S_ref, abs=2e-5)
    assert np.allclose(r["Q"], Q_ref, atol=2e-5)
