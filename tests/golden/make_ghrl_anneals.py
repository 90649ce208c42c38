"""Generates the GHRL and Pear golden curves: S(T) and E(T) of the reference's own CPU
thermal run (thermalEvolveN::run, src/evolve_thermal.cpp:30-99, through the
reference compiled here as oracle/_ref) on reduced versions of the GHRL
configurations, over independent runs:

  ghrl_slab16_anneal.json          slab 16^3 (free z, periodic x/y), GHRL
                                   k = (1, 0.8, 1.2), p0 = 0, homeotropic
                                   anchoring W = 4 on both faces;
                                   T = 1.2 -> 0.6, dT = -0.05
  ghrl_sphere16_field_anneal.json  droplet in 16^3 (the reference's sphere:
                                   all bounds free), GHRL k = (1, 0.6, 1.4),
                                   p0 = 20, planar (fg) anchoring W = 1,
                                   field along z (elecA = 1, E = 1);
                                   T = 1.0 -> 0.5, dT = -0.05
  pear_bulk16_anneal.json          bulk 16^3 periodic, Pear A = 1, B1 = 0.04,
                                   C = 0.3; T = 1.2 -> 0.6, dT = -0.05
  ghrl_sphere16_field_sweep.json   the droplet above at T = 0.8 with the field
                                   stepped E = 0 -> 2.0 by 0.2
                                   (electricEvolveN::run)

MCT = MCS = 100 per temperature, the step size carried across temperatures,
generators seeded seed * 104729 + thread (one thread per run).  Initial
directors: uniform on the sphere from numpy at active sites, +z at inactive
ones (the engine's convention; the initial condition is not on the compared
path, but inactive directors enter the all-site field energy).

Run from the repository root, where the reference tree is present
(`make -C oracle ref` first):
    python tests/golden/make_ghrl_anneals.py [case ...]
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from oracle import refproc  # noqa: E402

RUNS = 32
MCT = MCS = 100
HERE = os.path.dirname(os.path.abspath(__file__))

CASES = {
    "ghrl_slab16_anneal": dict(
        model=dict(nx=16, ny=16, nz=16, geometry="slab", potential="ghrl", k11=1.0, k22=0.8, k33=1.2, p0=0.0,
                   surfaces=[("homeotropic", 4.0), ("homeotropic", 4.0)]),
        ti=1.2, tf=0.6, dt=-0.05),
    "ghrl_sphere16_field_anneal": dict(
        model=dict(nx=16, ny=16, nz=16, geometry="sphere", xbound="free", ybound="free", zbound="free",
                   potential="ghrl", k11=1.0, k22=0.6, k33=1.4, p0=20.0, elecA=1.0, elecZ=1.0, elecE=1.0,
                   surfaces=[("fg", 1.0)]),
        ti=1.0, tf=0.5, dt=-0.05),
    "pear_bulk16_anneal": dict(
        model=dict(nx=16, ny=16, nz=16, potential="pear", A=1.0, B1=0.04, C=0.3, surfaces=[]),
        ti=1.2, tf=0.6, dt=-0.05),
    # the droplet configuration's protocol: a field sweep at fixed T
    # (electricEvolveN::run, src/evolve_electric.cpp:28-90)
    "ghrl_sphere16_field_sweep": dict(
        model=dict(nx=16, ny=16, nz=16, geometry="sphere", xbound="free", ybound="free", zbound="free",
                   potential="ghrl", k11=1.0, k22=0.6, k33=1.4, p0=20.0, elecA=1.0, elecZ=1.0, elecE=0.0,
                   surfaces=[("fg", 1.0)]),
        T=0.8, ei=0.0, ef=2.0, de=0.2),
}


def temperatures(ti, tf, dt):
    """The reference's float loops (src/evolve_thermal.cpp:58,
    src/evolve_electric.cpp:59)."""
    f = np.float32
    out = []
    T = f(ti)
    sign = int(-dt / abs(dt))
    while int(1e6 * sign * (float(T) - tf)) >= 0:
        out.append(float(T))
        T = f(T + f(dt))
    return out


def build_model(spec):
    kw = dict(spec)
    kw["surfaces"] = [O.Surface(a, W) for a, W in kw.pop("surfaces")]
    return O.Model(**kw)


def one_run(args):
    name, seed = args
    c = CASES[name]
    m = build_model(c["model"])
    pt = O.Lattice(m).pt
    rng = np.random.default_rng(2000 + seed)
    ni = O.random_directors(m.n, rng).astype(np.float32)
    ni[pt == 0] = (0.0, 0.0, 1.0)
    if "T" in c:
        fields = temperatures(c["ei"], c["ef"], c["de"])
        return refproc._worker(refproc.model_dict(m), [("field_sweep", ni, c["T"], fields, MCT, MCS, seed, 1)])[0]
    temps = temperatures(c["ti"], c["tf"], c["dt"])
    return refproc._worker(refproc.model_dict(m), [("anneal", ni, temps, MCT, MCS, seed, 1)])[0]


def main():
    if not refproc.available():
        raise SystemExit("oracle/_ref/libref_mcx.so is missing: build it with `make -C oracle ref`")
    ctx = mp.get_context("spawn")
    only = sys.argv[1:]
    for name, c in CASES.items():
        if only and name not in only:
            continue
        temps = temperatures(c["ei"], c["ef"], c["de"]) if "T" in c else temperatures(c["ti"], c["tf"], c["dt"])
        with ctx.Pool(min(RUNS, os.cpu_count() or 1), maxtasksperchild=1) as pool:
            runs = pool.map(one_run, [(name, s) for s in range(1, RUNS + 1)])
        arr = np.array(runs)  # [run, step, (T or field, S, E)]
        S, E, D = arr[:, :, 1], arr[:, :, 2], arr[:, :, 3]
        out = {
            "config": name, "model": c["model"], "mct": MCT, "mcs": MCS, "runs": RUNS,
            **({"T": c["T"], "fields": temps} if "T" in c else {"temps": temps}),
            "S_mean": S.mean(0).tolist(), "S_sem": (S.std(0, ddof=1) / np.sqrt(RUNS)).tolist(),
            "E_mean": E.mean(0).tolist(), "E_sem": (E.std(0, ddof=1) / np.sqrt(RUNS)).tolist(),
            # the reference's director-length drift (mean |n|^2 - 1 over active sites)
            "len2_drift_mean": D.mean(0).tolist(), "len2_drift_absmax": np.abs(D).max(0).tolist(),
        }
        path = os.path.join(HERE, name + ".json")
        with open(path, "w") as f:
            json.dump(out, f, indent=1)
        print(f"wrote {path}: {len(temps)} temperatures x {RUNS} runs")


if __name__ == "__main__":
    main()
