"""The oracle's red/black chain against the reference's own S(T), E(T) on the
c1 anneal (tests/golden/c1_ll16_anneal.json, 32 reference runs): 8 oracle
runs with the GPU's Philox streams, same protocol; at every T the means agree
within 4 combined standard errors plus 1e-3 (S) / 2e-3 (E)."""
import functools
import json
import multiprocessing as mp
import os

import numpy as np

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c1_ll16_anneal.json")


def _run(seed, temps):
    m = O.Model(nx=16, ny=16, nz=16, potential="ll", A=1.0)
    ni0 = O.random_directors(m.n, np.random.default_rng(2000 + seed)).astype(np.float32)
    return O.anneal(m, temps, 100, 100, seed, seed, ni0)


def test_oracle_anneal_matches_reference_curves():
    g = json.load(open(GOLD))
    temps = g["temps"]
    R = 8
    with mp.get_context("spawn").Pool(R) as pool:
        rows = np.array(pool.map(functools.partial(_run, temps=temps), range(1, R + 1)))
    for col, name, tol in ((1, "S", 1e-3), (2, "E", 2e-3)):
        G = rows[:, :, col]
        m, se = G.mean(0), G.std(0, ddof=1) / np.sqrt(R)
        rm, rse = np.array(g[name + "_mean"]), np.array(g[name + "_sem"])
        sig = np.hypot(se, rse)
        bad = np.nonzero(np.abs(m - rm) > 4 * sig + tol)[0]
        assert len(bad) == 0, [(temps[i], m[i], rm[i], sig[i]) for i in bad]
