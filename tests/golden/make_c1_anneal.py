"""Generates tests/golden/c1_ll16_anneal.json: S(T) and E(T) of the
reference's own CPU thermal run on the c1 configuration (LL bulk 16^3,
periodic, A = 1, random initial directors, Ti = 1.2 -> Tf = 0.0, dT = -0.02,
MCT = MCS = 100), over independent runs.

Each run calls the reference's EvolveN::Monte_Carlo_Step, energy_calculator
and order parameter (oracle/_ref, compiled from the reference tree by
`make -C oracle ref`) with the thermal loop of src/evolve_thermal.cpp:30-99:
step size 0.5 carried across temperatures, generators seeded
seed * 104729 + thread (one thread per run, so a run is deterministic), and the
float temperature stepping of the reference.  Initial directors are uniform on
the sphere from numpy (the reference draws them with gsl_ran_dir_3d; the
initial condition is not on the compared path).

Run from the repository root, where the reference tree is present:
    python tests/golden/make_c1_anneal.py
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

RUNS = 128
N = 16
MCT = MCS = 100
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c1_ll16_anneal.json")


def temperatures(ti=1.2, tf=0.0, dt=-0.02):
    """The reference's float loop (src/evolve_thermal.cpp:58)."""
    f = np.float32
    out = []
    T = f(ti)
    sign = int(-dt / abs(dt))
    while int(1e6 * sign * (float(T) - tf)) >= 0:
        out.append(float(T))
        T = f(T + f(dt))
    return out


def one_run(seed):
    m = O.Model(nx=N, ny=N, nz=N, potential="ll", A=1.0)
    rng = np.random.default_rng(1000 + seed)
    ni = O.random_directors(m.n, rng).astype(np.float32)
    # a fresh process per run (maxtasksperchild=1): the reference keeps
    # lattice state in function-local statics
    return refproc._worker(refproc.model_dict(m), [("anneal", ni, temperatures(), MCT, MCS, seed, 1)])[0]


def main():
    if not refproc.available():
        raise SystemExit("oracle/_ref/libref_mcx.so is missing: build it with `make -C oracle ref`")
    temps = temperatures()
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(RUNS, os.cpu_count() or 1), maxtasksperchild=1) as pool:
        runs = pool.map(one_run, range(1, RUNS + 1))
    arr = np.array(runs)  # [run, T, (T, S, E)]
    S, E, D = arr[:, :, 1], arr[:, :, 2], arr[:, :, 3]
    out = {
        "config": "LL bulk 16^3 periodic, A=1, random ic, Ti=1.2 Tf=0.0 dT=-0.02, MCT=MCS=100 "
                  "(thermalEvolveN::run on the reference's CPU path)",
        "runs": RUNS, "temps": temps,
        "S_mean": S.mean(0).tolist(), "S_sem": (S.std(0, ddof=1) / np.sqrt(RUNS)).tolist(),
        "E_mean": E.mean(0).tolist(), "E_sem": (E.std(0, ddof=1) / np.sqrt(RUNS)).tolist(),
        # the reference's director-length drift (mean |n|^2 - 1 over active sites)
        "len2_drift_mean": D.mean(0).tolist(), "len2_drift_absmax": np.abs(D).max(0).tolist(),
    }
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {OUT}: {len(temps)} temperatures x {RUNS} runs")


if __name__ == "__main__":
    main()
