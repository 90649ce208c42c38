"""Generates tests/golden/replica_avg.json: po.dat files of synthetic
replicas and the table the reference's own average_replicas.py makes of them.

Cases (seeded): five-column LL-style files with a shared temperature grid;
six-column Pear-style files; files of unequal length (only the common prefix
is combined); a temperature that differs by more than 1e-3 in one file (that
row is skipped); a single replica.  The values are written with %g, as the
reference's po.dat writer does, and the script reads them back.

Run from the repository root, where the reference tree is present:
    python tests/golden/make_replica_avg.py
"""
from __future__ import annotations

import contextlib
import io
import json
import os
import sys
import tempfile

import numpy as np

# the McLiCS source tree whose average_replicas.py this script runs
REF = os.environ.get("MCLICS_REFERENCE_TREE", "/root/reference")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "replica_avg.json")


def po_text(rows, pear):
    head = "T S varS E varE P" if pear else "T S varS E varE"
    return head + "\n" + "".join(" ".join("%g" % v for v in r) + "\n" for r in rows)


def synth(rng, n_rep, n_t, pear, lengths=None, bad=None):
    T = np.round(np.arange(1.2, 1.2 - 0.02 * n_t, -0.02)[:n_t], 6)
    files = []
    for r in range(n_rep):
        m = n_t if lengths is None else lengths[r]
        rows = []
        for i in range(m):
            S = float(np.clip(0.9 - 0.5 * T[i] + rng.normal(0, 0.05), 0, 1))
            E = float(-9 * S + rng.normal(0, 0.1))
            row = [float(T[i]), S, float(abs(rng.normal(1e-4, 5e-5))), E, float(abs(rng.normal(2e-3, 1e-3)))]
            if bad is not None and (r, i) == bad:
                row[0] += 0.01
            if pear:
                row.append(float(abs(rng.normal(0.2, 0.1))))
            rows.append(row)
        files.append(po_text(rows, pear))
    return files


def main():
    sys.path.insert(0, REF)
    import average_replicas as ar  # the reference's own script

    rng = np.random.default_rng(20240607)
    cases = {
        "ll_8x12": synth(rng, 8, 12, False),
        "pear_4x6": synth(rng, 4, 6, True),
        "ragged_3": synth(rng, 3, 7, False, lengths=[7, 5, 6]),
        "t_mismatch": synth(rng, 4, 5, False, bad=(2, 3)),
        "single": synth(rng, 1, 4, False),
    }
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for name, files in cases.items():
            paths = []
            for q, text in enumerate(files):
                p = os.path.join(d, f"{name}_{q}.dat")
                with open(p, "w") as f:
                    f.write(text)
                paths.append(p)
            with contextlib.redirect_stdout(io.StringIO()):
                header, combined = ar.combine(paths)
            out[name] = {"files": files, "header": header, "combined": [[float(v) for v in r] for r in combined]}
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print(OUT)


if __name__ == "__main__":
    main()
