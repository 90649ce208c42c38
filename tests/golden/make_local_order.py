"""Writes local_order.npz: director states, the local order parameter that
the reference's own lattice_order_parameter (src/parameter_order.cpp:62-113),
compiled in oracle/_ref, returns for them at every active site (NaN
elsewhere), and, for the bulk, the droplet and the slab, the snapshot file its print_n
(src/io.cpp:50-80) writes for them.  Four cases: periodic LL bulk, a
droplet with free bounds and a GHRL slab, each with seeded random directors
tilted towards (0.1, 0.2, 0.9) (S about 0.86-0.99, an ordered snapshot), and
the bulk with untilted random directors (low S, nearly degenerate Q).

    make -C oracle ref REF=<McLiCS source tree>
    python tests/golden/make_local_order.py
"""
from __future__ import annotations

import dataclasses
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402
from oracle import refproc  # noqa: E402

MODELS = {
    "bulk": O.Model(nx=10, ny=8, nz=6, potential="ll"),
    "sphere": O.Model(nx=10, ny=10, nz=10, geometry="sphere", xbound="free", ybound="free", zbound="free",
                      potential="ll", surfaces=[O.Surface("fg", 1.0)]),
    "slab": O.Model(nx=12, ny=8, nz=6, geometry="slab", potential="ghrl",
                    surfaces=[O.Surface("homeotropic", 2.0), O.Surface("fg", 1.0)]),
    "bulk_random": O.Model(nx=10, ny=8, nz=6, potential="ll"),
}

CSV_CASES = ("bulk", "sphere", "slab")  # snapshot text kept for these (periodic; inactive sites; surfaces)


def state(m: O.Model, pt: np.ndarray, seed: int, tilt: bool) -> np.ndarray:
    ni = O.random_directors(m.n, np.random.default_rng(seed))
    if tilt:
        ni = 0.3 * ni + np.array([0.1, 0.2, 0.9], np.float32)
    ni /= np.linalg.norm(ni, axis=1, keepdims=True)
    ni[pt == 0] = (0, 0, 1)
    return ni.astype(np.float32)


def main():
    if not refproc.available():
        raise SystemExit("build the reference first: make -C oracle ref REF=<McLiCS source tree>")
    arrays = {}
    spec = {}
    for q, (name, m) in enumerate(MODELS.items()):
        ((pt, _),) = refproc.run(m, [("mask",)])
        ni = state(m, pt, 40 + q, tilt=name != "bulk_random")
        with tempfile.TemporaryDirectory() as d:
            S, csv = refproc.run(m, [("local_order", ni), ("print_n", ni, os.path.join(d, "snap.csv"))])
        if name in CSV_CASES:
            arrays[f"{name}_csv"] = np.frombuffer(csv.encode(), np.uint8)
        arrays[f"{name}_ni"] = ni
        arrays[f"{name}_pt"] = pt.astype(np.uint8)
        arrays[f"{name}_S"] = S
        d = dataclasses.asdict(m)
        spec[name] = d
    arrays["models"] = np.array(json.dumps(spec))
    np.savez_compressed(os.path.join(HERE, "local_order.npz"), **arrays)
    print("wrote local_order.npz:", {k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    main()
