"""Statistical parity with the reference's own CPU path on the c1 anneal and
on reduced GHRL configurations.

tests/golden/c1_ll16_anneal.json holds S(T) and E(T) of the reference's
thermalEvolveN::run (src/evolve_thermal.cpp:30-99) on LL bulk 16^3, random
start, Ti = 1.2 -> Tf = 0.0 in steps of -0.02, MCT = MCS = 100, over 128
independent runs (generated by tests/golden/make_c1_anneal.py from the
reference compiled here).  The GPU runs the same protocol on 32 replicas in
one engine: per temperature 100 sweeps, then 100 sweeps each followed by the
E / S measurement, step size carried across temperatures.

The chains differ (2-colour vs 8-colour order, Philox vs ranlxs0, renormalised
vs unrenormalised proposals), so the comparison is statistical: at every T the
means agree within 3 combined standard errors (plus the systematic of the
reference's director-length drift, measured in its runs and below 1e-5),
except for as many of the 122 comparisons as chance puts beyond 3 sigma at 5%
family-wise (one) and none beyond 4 sigma (helpers.assert_stat_parity), and
chi^2 per temperature over the whole curve stays below 2."""
import json
import os

import numpy as np
import pytest

import mcx
from helpers import assert_stat_parity

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c1_ll16_anneal.json")


def test_c1_anneal_matches_reference_curves():
    g = json.load(open(GOLD))
    temps = g["temps"]
    R, N, MC = 32, 16, 100
    descs = [mcx.replica(nx=N, ny=N, nz=N, potential="ll", A=1.0, T=temps[0], ang_var=0.5, seed=1 + r, stream=r)
             for r in range(R)]
    S = np.zeros((R, len(temps)))
    E = np.zeros((R, len(temps)))
    with mcx.Engine(descs) as eng:
        for r in range(R):
            eng.init_random(r, 500 + r)
        for t, T in enumerate(temps):
            eng.set_temperature(T)
            eng.sweep(MC)
            eng.reset_stats()
            eng.sweep(MC, measure=True)
            for r in range(R):
                st = eng.stats(r)
                S[r, t] = st[mcx.ST_S1] / st[mcx.ST_N]
                E[r, t] = st[mcx.ST_E1] / st[mcx.ST_N]
    assert_stat_parity([(S, g, "S"), (E, g, "E")], temps)
    chi2 = []
    for name, G in (("S", S), ("E", E)):
        m, se = G.mean(0), G.std(0, ddof=1) / np.sqrt(R)
        sig = np.hypot(se, np.array(g[name + "_sem"]))
        chi2.append(float(np.mean(((m - np.array(g[name + "_mean"])) / sig) ** 2)))
    assert max(chi2) < 2.0, chi2


def _ghrl_descs(spec, T0, R):
    surf = [dict(anchoring=a, W=W, theta_s=0.0, phi_s=0.0) for a, W in spec["surfaces"]]
    kw = {k: v for k, v in spec.items() if k not in ("surfaces",)}
    return [mcx.replica(**kw, T=T0, ang_var=0.5, seed=1 + r, stream=r, surfaces=surf) for r in range(R)]


@pytest.mark.parametrize("name", ["ghrl_slab16_anneal", "ghrl_sphere16_field_anneal", "pear_bulk16_anneal"])
def test_ghrl_anneals_match_reference_curves(name):
    """tests/golden/{ghrl,pear}_*_anneal.json: 32 runs of the reference's CPU
    thermal loop on a 16^3 GHRL slab (homeotropic, W = 4), a chiral droplet
    (planar anchoring, field along z) and bulk Pear, made by
    tests/golden/make_ghrl_anneals.py.  The
    GPU runs 32 replicas with the same protocol; at every T the means agree
    within 3 combined standard errors (helpers.assert_stat_parity: one
    chance exceedance of at most 4 sigma allowed among the 22-26
    comparisons)."""
    g = json.load(open(os.path.join(os.path.dirname(GOLD), name + ".json")))
    temps, MC, R = g["temps"], g["mct"], 32
    descs = _ghrl_descs(g["model"], temps[0], R)
    S = np.zeros((R, len(temps)))
    E = np.zeros((R, len(temps)))
    with mcx.Engine(descs) as eng:
        for r in range(R):
            eng.init_random(r, 700 + r)
        for t, T in enumerate(temps):
            eng.set_temperature(T)
            eng.sweep(MC)
            eng.reset_stats()
            eng.sweep(MC, measure=True)
            for r in range(R):
                st = eng.stats(r)
                S[r, t] = st[mcx.ST_S1] / st[mcx.ST_N]
                E[r, t] = st[mcx.ST_E1] / st[mcx.ST_N]
    assert_stat_parity([(S, g, "S"), (E, g, "E")], temps)


def test_droplet_field_sweep_matches_reference_curve():
    """tests/golden/ghrl_sphere16_field_sweep.json: 32 runs of the reference's
    electric-field loop (electricEvolveN::run, src/evolve_electric.cpp:28-90)
    on the chiral GHRL droplet at T = 0.8, field stepped 0 -> 2.0 by 0.2; the
    GPU runs 32 replicas with the same protocol (per field value 100 sweeps,
    then 100 measured ones; step size carried); 3 combined standard errors at
    every field value (helpers.assert_stat_parity)."""
    g = json.load(open(os.path.join(os.path.dirname(GOLD), "ghrl_sphere16_field_sweep.json")))
    fields, MC, R = g["fields"], g["mct"], 32
    descs = _ghrl_descs(g["model"], g["T"], R)
    S = np.zeros((R, len(fields)))
    E = np.zeros((R, len(fields)))
    with mcx.Engine(descs) as eng:
        for r in range(R):
            eng.init_random(r, 900 + r)
        for t, Ef in enumerate(fields):
            eng.set_field(Ef)
            eng.sweep(MC)
            eng.reset_stats()
            eng.sweep(MC, measure=True)
            for r in range(R):
                st = eng.stats(r)
                S[r, t] = st[mcx.ST_S1] / st[mcx.ST_N]
                E[r, t] = st[mcx.ST_E1] / st[mcx.ST_N]
    assert_stat_parity([(S, g, "S"), (E, g, "E")], fields)
