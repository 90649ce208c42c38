"""The oracle's red/black chain against the reference's own S(T), E(T) on the
c1 anneal (tests/golden/c1_ll16_anneal.json, 128 reference runs): 32 oracle
runs with the GPU's Philox streams, same protocol; at every T the means agree
within 3 combined standard errors, up to the exceedances chance allows among
all the comparisons (helpers.assert_stat_parity)."""
import functools
import json
import multiprocessing as mp
import os

import numpy as np

from oracle import oracle as O
from helpers import assert_stat_parity

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c1_ll16_anneal.json")


def _run(seed, temps):
    m = O.Model(nx=16, ny=16, nz=16, potential="ll", A=1.0)
    ni0 = O.random_directors(m.n, np.random.default_rng(2000 + seed)).astype(np.float32)
    return O.anneal(m, temps, 100, 100, seed, seed, ni0)


def test_oracle_anneal_matches_reference_curves():
    g = json.load(open(GOLD))
    temps = g["temps"]
    R = 32
    with mp.get_context("spawn").Pool(min(R, os.cpu_count() or 1)) as pool:
        rows = np.array(pool.map(functools.partial(_run, temps=temps), range(1, R + 1)))
    assert_stat_parity([(rows[:, :, 1], g, "S"), (rows[:, :, 2], g, "E")], temps)
