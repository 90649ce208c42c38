"""Generates the run-loop golden files: po.dat rows written by the reference's
own CPU program (./mc_sim, its `make CPU` build compiled here as
oracle/_ref/ref_mc_sim against the test-only GSL shim) in each of its four
modes, over independent runs that differ only in `seed`:

  run_thermal_sphere25.json   the reference's test4.txt droplet (25^3 sphere,
                              all bounds free, GHRL k = (1.48, 1, 2.28),
                              p0 = 0, homeotropic W = 4), T = 1.3 -> 0.8 by
                              -0.1 (thermalEvolveN::run,
                              src/evolve_thermal.cpp:30-99), MCT = MCS = 100
                              instead of 3000 / 400
  run_electric_sphere13.json  a chiral droplet in 13^3 (GHRL k = (1, 0.6, 1.4),
                              p0 = 10, planar (fg) W = 1) at T = 0.8 with the
                              field along z stepped E = 0 -> 1 by 0.25
                              (electricEvolveN::run,
                              src/evolve_electric.cpp:28-90)
  run_step_slab11.json        an 11 x 12 x 9 slab (free x and z, periodic y),
                              LL, homeotropic W = 2 on both faces, homogeneous
                              start along z, 4 blocks at T = 0.9
                              (stepEvolveN::run, src/evolve_step.cpp:28-89)
  run_quench_bulk12.json      bulk 12^3 LL, homogeneous start, 3 blocks of
                              MCT sweeps at Ti = 0.5 then MCT*dT = 30 sweeps
                              at Tf = 0.9 before the measured ones
                              (quenchEvolveN::run, src/evolve_quench.cpp:28-94,
                              with its MCT*dT count at :62)

Each file holds the parameter file, the first run's po.dat text (the layout
the engine's files must reproduce) and, per po.dat row, the mean and standard
error over the runs of S, varS, E and varE.  One OpenMP thread per run (the
sweep's generator count follows the thread count).

Run from the repository root after building the reference programs
(`make -C oracle ref REF=<McLiCS source tree>`):
    python tests/golden/make_run_loops.py [case ...]
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
HERE = os.path.dirname(os.path.abspath(__file__))
REF_MC_SIM = os.path.join(ROOT, "oracle", "_ref", "ref_mc_sim")
RUNS = 32

CASES = {
    "run_thermal_sphere25": """\
Nx 25
Ny 25
Nz 25
MCS 100
MCT 100
Ti 1.3
Tf 0.8
dT -0.1
potential ghrl
k11 1.48
k22 1
k33 2.28
p0 0
evol thermal
ic random
geometry sphere
anchoring_type 0 homeotropic
W 0 4
""",
    "run_electric_sphere13": """\
Nx 13
Ny 13
Nz 13
MCS 100
MCT 100
Ti 0.8
potential ghrl
k11 1
k22 0.6
k33 1.4
p0 10
evol electric
Ei 0
Ef 1
dE 0.25
Electric_field_z 1
Aniso_E 1
ic random
geometry sphere
anchoring_type 0 fg
W 0 1
""",
    "run_step_slab11": """\
Nx 11
Ny 12
Nz 9
MCS 60
MCT 60
Ti 0.9
potential ll
A 1
evol step
fn 4
first_file_number 0
ic homogeneous
theta_0 0
phi_0 0
geometry slab
xbound free
ybound periodic
anchoring_type 0 homeotropic
W 0 2
anchoring_type 1 homeotropic
W 1 2
""",
    "run_quench_bulk12": """\
Nx 12
Ny 12
Nz 12
MCS 60
MCT 60
Ti 0.5
Tf 0.9
dT 0.5
potential ll
A 1
evol quench
fn 3
first_file_number 1
ic homogeneous
theta_0 0
phi_0 0
geometry bulk
""",
}


def read_po(path):
    with open(path) as f:
        text = f.read()
    lines = text.splitlines()
    rows = [ln.split() for ln in lines[1:] if ln.strip()]
    return text, lines[0], [r[0] for r in rows], np.array([[float(x) for x in r[1:5]] for r in rows])


def one_run(args):
    name, seed = args
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "params.txt")
        with open(p, "w") as f:
            f.write(CASES[name] + f"seed {seed}\n")
        env = dict(os.environ, OMP_NUM_THREADS="1")
        subprocess.run([REF_MC_SIM, p], cwd=d, env=env, check=True, stdout=subprocess.DEVNULL)
        snaps = sorted(f for f in os.listdir(d) if f.startswith("director_field_"))
        return read_po(os.path.join(d, "po.dat")) + (snaps,)


def main():
    if not os.path.exists(REF_MC_SIM):
        raise SystemExit("oracle/_ref/ref_mc_sim is missing: build it with `make -C oracle ref REF=<tree>`")
    only = sys.argv[1:]
    ctx = mp.get_context("spawn")
    for name in CASES:
        if only and name not in only:
            continue
        with ctx.Pool(min(RUNS, os.cpu_count() or 1)) as pool:
            runs = pool.map(one_run, [(name, s) for s in range(1, RUNS + 1)])
        text0, header, labels, _, snaps = runs[0]
        for r in runs[1:]:
            assert r[1] == header and r[2] == labels and r[4] == snaps
        vals = np.array([r[3] for r in runs])  # [run, row, (S, varS, E, varE)]
        mean = vals.mean(0)
        sem = vals.std(0, ddof=1) / np.sqrt(RUNS)
        out = {
            "config": name, "params": CASES[name], "runs": RUNS, "seeds": list(range(1, RUNS + 1)),
            "po_dat_run1": text0, "header": header, "labels": labels, "snapshots": snaps,
            "columns": ["S", "varS", "E", "varE"],
            "mean": mean.tolist(), "sem": sem.tolist(),
        }
        path = os.path.join(HERE, name + ".json")
        with open(path, "w") as f:
            json.dump(out, f, indent=1)
        print(f"wrote {path}: {len(labels)} rows x {RUNS} runs")


if __name__ == "__main__":
    main()
