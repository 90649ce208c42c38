"""The oracle's red/black chain against the reference's own S(T), E(T) on the
reduced GHRL and Pear configurations (tests/golden/{ghrl,pear}_*_anneal.json,
32 reference runs each, made by tests/golden/make_ghrl_anneals.py): a slab
with homeotropic anchoring, a chiral droplet with planar anchoring in a
field, bulk Pear across its transition, and the droplet's field sweep at
fixed T (electricEvolveN::run).
32 oracle runs per case with the GPU's Philox streams, same protocol; at every
T the means agree within 3 combined standard errors, up to the exceedances
chance allows among all the comparisons (helpers.assert_stat_parity)."""
import functools
import json
import multiprocessing as mp
import os

import numpy as np
import pytest

from oracle import oracle as O
from helpers import assert_stat_parity

HERE = os.path.dirname(os.path.abspath(__file__))
R = 32


def _model(spec):
    kw = dict(spec)
    kw["surfaces"] = [O.Surface(a, W) for a, W in kw.pop("surfaces")]
    return O.Model(**kw)


def _run(seed, spec, steps, mc, T):
    m = _model(spec)
    pt = O.Lattice(m).pt
    ni0 = O.random_directors(m.n, np.random.default_rng(3000 + seed)).astype(np.float32)
    ni0[pt == 0] = (0.0, 0.0, 1.0)
    if T is not None:  # a field sweep at fixed T
        return O.field_sweep(m, T, steps, mc, mc, seed, seed, ni0)
    return O.anneal(m, steps, mc, mc, seed, seed, ni0)


@pytest.mark.parametrize("name", ["ghrl_slab16_anneal", "ghrl_sphere16_field_anneal", "pear_bulk16_anneal",
                                  "ghrl_sphere16_field_sweep"])
def test_oracle_ghrl_anneal_matches_reference_curves(name):
    g = json.load(open(os.path.join(HERE, "golden", name + ".json")))
    temps = g.get("temps", g.get("fields"))
    with mp.get_context("spawn").Pool(min(R, os.cpu_count() or 1)) as pool:
        rows = np.array(pool.map(functools.partial(_run, spec=g["model"], steps=temps, mc=g["mct"], T=g.get("T")),
                                 range(1, R + 1)))
    assert_stat_parity([(rows[:, :, 1], g, "S"), (rows[:, :, 2], g, "E")], temps)
