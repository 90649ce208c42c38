"""The batched configurations beside the headline anneal, reduced in size,
against the oracle's red/black sweeps (same Philox streams): every replica of
an uneven GHRL slab batch (the c3 shape) and of a droplet batch with chiral
GHRL, planar anchoring and a field (the c5 shape) ends four measured sweeps
in the oracle's state (2e-5) with the oracle's step size."""
import numpy as np
import pytest

import mcx
from oracle import oracle as O
from helpers import desc_from_model, random_state

pytestmark = pytest.mark.gpu


def _batch_vs_oracle(models, Ts, sweeps=4):
    descs = [desc_from_model(m, T=T, seed=30 + r, stream=r, ang_var=0.5) for r, (m, T) in enumerate(zip(models, Ts))]
    lats = [O.Lattice(m) for m in models]
    with mcx.Engine(descs) as eng:
        starts = []
        for r, (m, lat) in enumerate(zip(models, lats)):
            ni = random_state(m, lat.pt, np.random.default_rng(r))
            eng.set_state(r, ni)
            starts.append(eng.get_state(r))
        eng.sweep(sweeps, measure=True)
        for r, (m, lat, T) in enumerate(zip(models, lats, Ts)):
            lat.ni[:] = starts[r]
            a = np.float32(0.5)
            for sw in range(sweeps):
                _, a = lat.sweep(T, a, 30 + r, r, sw, "redblack")
            got = eng.get_state(r)
            assert np.max(np.abs(got - lat.ni)) < 2e-5, r
            assert np.float32(eng.stats(r)[mcx.ST_ANG_VAR]) == np.float32(a), r


def test_ghrl_slab_batch_of_uneven_sizes():
    rng = np.random.default_rng(3)
    sides = [16, 24, 16, 32, 24, 16]
    hom = [O.Surface("homeotropic", 4.0), O.Surface("homeotropic", 4.0)]
    models = [O.Model(nx=L, ny=L, nz=L, geometry="slab", potential="ghrl", k11=1.0, k22=0.8, k33=1.2, surfaces=hom)
              for L in sides]
    _batch_vs_oracle(models, list(rng.uniform(0.8, 1.2, len(sides))))


def test_droplet_field_chiral_batch():
    m = O.Model(nx=24, ny=24, nz=24, geometry="sphere", potential="ghrl", k11=1.0, k22=0.6, k33=1.4, p0=20,
                elecA=1.0, elecZ=1.0, elecE=1.0, radius=9.0, surfaces=[O.Surface("fg", 1.0)])
    _batch_vs_oracle([m, m, m], [0.8, 0.8, 0.8])
