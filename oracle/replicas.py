"""Replica combination of po.dat rows (TEST INFRASTRUCTURE ONLY).

Restates average_replicas.py:57-103 (the reference's combiner of po.dat files
from runs that differ only in their seed) in NumPy:

  * every file must have the same number of columns (5, or 6 for Pear runs:
    T S varS E varE [P]); only the first min(rows) rows are combined;
  * a row whose temperatures differ by more than 1e-3 across files is skipped;
  * T = mean of the files' T; S = mean S_r; varS = mean varS_r + var(S_r)
    (ddof 0, the law of total variance); the same for E; P = mean P_r.

po_rows() turns the running sums of mcx_get_stats into the po.dat row of one
replica, as src/evolve_thermal.cpp:78-86 forms it from its measured sweeps.
"""
from __future__ import annotations

import numpy as np


class CombineError(ValueError):
    pass


def combine(per_file):
    """per_file: one list of rows per replica (each row a list of floats).
    Returns the combined rows (the script's `combined`)."""
    ncols = len(per_file[0][0])
    if not all(len(r) == ncols for rows in per_file for r in rows):
        raise CombineError("replicas with different column counts")
    n_points = min(len(rows) for rows in per_file)
    out = []
    for i in range(n_points):
        T_vals = [rows[i][0] for rows in per_file]
        if max(T_vals) - min(T_vals) > 1e-3:
            continue
        col = lambda c: np.array([rows[i][c] for rows in per_file])  # noqa: E731
        S_r, varS_r, E_r, varE_r = col(1), col(2), col(3), col(4)
        row = [np.mean(T_vals), S_r.mean(), varS_r.mean() + S_r.var(ddof=0), E_r.mean(),
               varE_r.mean() + E_r.var(ddof=0)]
        if ncols >= 6:
            row.append(col(5).mean())
        out.append(row)
    return out


def po_row(T, stats, P=None):
    """The po.dat row of one replica from its running sums (the MCX_ST_*
    layout: N, sum S, sum S^2, sum E, sum E^2)."""
    n = stats[0]
    S1, S2, E, E2 = stats[1] / n, stats[2] / n, stats[3] / n, stats[4] / n
    row = [T, S1, S2 - S1 * S1, E, E2 - E * E]
    if P is not None:
        row.append(P)
    return row


def read_po(path):
    """The rows of a po.dat file, skipping its header line."""
    rows = []
    with open(path) as f:
        for line in f:
            line = line.strip()
            if not line or not line[0].replace(".", "").replace("-", "").isdigit():
                continue
            rows.append([float(x) for x in line.split()])
    return rows
