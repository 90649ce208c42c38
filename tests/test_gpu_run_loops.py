"""The parameter-file drop-in in all four run modes against po.dat files the
reference's own CPU program wrote (tests/golden/run_*.json, made by
tests/golden/make_run_loops.py from the reference compiled here).

mcx_run_file runs each golden's parameter file with 32 replicas (seeds 1..32,
as the golden's 32 runs): its po.dat must have the reference's layout byte for
byte -- the header line, the row labels (the reference's float temperature /
field loops and block numbers, with the quench loop's MCT*dT sweep count), the
column count and %g formatting -- and the same snapshot file names; and at
every row the mean over replicas of S and of E must agree with the
reference's within 3 combined standard errors.  The two chains differ in
colour order (2 colours, not 8), random numbers and the proposal's
renormalisation, so only the statistics are compared."""
import json
import os
import re

import numpy as np
import pytest

import mcx
from helpers import assert_stat_parity

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ["run_thermal_sphere25", "run_electric_sphere13", "run_step_slab11", "run_quench_bulk12"]
NUM = re.compile(r"^-?(\d+(\.\d*)?|\.\d+)(e[-+]\d+)?$|^-?(nan|inf)$")


def _golden(name):
    with open(os.path.join(HERE, "golden", name + ".json")) as f:
        return json.load(f)


def _read(path):
    with open(path) as f:
        lines = f.read().splitlines()
    return lines[0], [ln.split() for ln in lines[1:] if ln.strip()]


@pytest.mark.parametrize("name", CASES)
def test_run_file_matches_reference_program(name, tmp_path):
    g = _golden(name)
    runs = g["runs"]
    p = tmp_path / "params.txt"
    p.write_text(g["params"] + f"seed 1\nreplicas {runs}\n")
    out = tmp_path / "out"
    out.mkdir()
    mcx.run_file(str(p), str(out))
    # layout: header, labels, columns, number format, snapshot names
    vals = []
    for r in range(runs):
        header, rows = _read(out / ("po.dat" if r == 0 else f"po_r{r}.dat"))
        assert header == g["header"]
        assert [row[0] for row in rows] == g["labels"]
        for row in rows:
            assert len(row) == 5
            assert all(NUM.match(x) for x in row), row
        vals.append([[float(x) for x in row[1:5]] for row in rows])
    got = sorted(f for f in os.listdir(out) if f.startswith("director_field_"))
    assert got == g["snapshots"]
    assert (out / "ic.csv").exists()
    # statistics: S and E per row within 3 combined standard errors (at most
    # 10 comparisons per file: no chance exceedance is allowed)
    vals = np.array(vals)  # [replica, row, (S, varS, E, varE)]
    rm, rs = np.array(g["mean"]), np.array(g["sem"])
    gold = {"S_mean": rm[:, 0], "S_sem": rs[:, 0], "E_mean": rm[:, 2], "E_sem": rs[:, 2]}
    assert_stat_parity([(vals[:, :, 0], gold, "S"), (vals[:, :, 2], gold, "E")], g["labels"])
