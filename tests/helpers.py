"""Shared test helpers: descriptors from oracle models, the GPU fixture."""
import json
import os

import numpy as np

import mcx
from oracle import oracle as O


def desc_from_model(m: O.Model, T=1.0, seed=1, stream=0, ang_var=0.5):
    return mcx.replica(nx=m.nx, ny=m.ny, nz=m.nz, geometry=m.geometry, xbound=m.xbound, ybound=m.ybound,
                       zbound=m.zbound, potential=m.potential, A=m.A, k11=m.k11, k22=m.k22, k33=m.k33, p0=m.p0,
                       elecA=m.elecA, elecX=m.elecX, elecY=m.elecY, elecZ=m.elecZ, elecE=m.elecE, T=T,
                       ang_var=ang_var, seed=seed, stream=stream,
                       surfaces=[dict(anchoring=s.anchoring, W=s.W, theta_s=s.theta_s, phi_s=s.phi_s)
                                 for s in m.surfaces], radius=m.radius, B1=m.B1, C=m.C)


def random_state(m: O.Model, pt: np.ndarray, rng) -> np.ndarray:
    ni = O.random_directors(m.n, rng)
    ni[pt == 0] = (0, 0, 1)
    return ni


def neighbours(lat, m, s):
    """The six neighbour directors of site s in slot order, zero when the bond
    is absent or the neighbour inactive."""
    i, j, k = s % m.nx, (s // m.nx) % m.ny, s // (m.nx * m.ny)
    xb, yb, zb = m.effective_bounds()
    N = [m.nx, m.ny, m.nz]
    B = [xb, yb, zb]
    out = np.zeros((6, 3))
    for d in range(6):
        c = [i, j, k]
        ax = d >> 1
        c[ax] += -1 if d & 1 else 1
        if c[ax] < 0 or c[ax] >= N[ax]:
            if B[ax] != "periodic":
                continue
            c[ax] %= N[ax]
        t = c[0] + m.nx * (c[1] + m.ny * c[2])
        if lat.pt[t] == 0:
            continue
        out[d] = lat.ni[t]
    return out


def stat_parity_failures(G: np.ndarray, g: dict, key: str):
    """Rows where the mean over runs of G (runs x rows) and the golden's mean
    g[key + "_mean"] differ by more than 3 combined standard errors plus the
    systematic of the reference's unrenormalised directors, as
    (row, mean, golden mean, combined standard error, deviation in those
    errors beyond the systematic).

    The reference's CPU sweep does not renormalise its proposals
    (src/evolve.cpp:139-151), so its director lengths drift by float rounding;
    the golden files record the drift measured in the reference's own runs
    (len2_drift_absmax, the largest |mean |n|^2 - 1| over runs, per row; about
    1e-7).  With |n|^2 = 1 + eps the order parameter moves by at most
    1.5 eps and each bond or site energy term of degree <= 4 in the directors by
    at most 2 eps of its size, so the allowance is 2 eps for S and
    4 eps (|E| + 1) for E: below 1e-5 in every golden."""
    R = G.shape[0]
    m, se = G.mean(0), G.std(0, ddof=1) / np.sqrt(R)
    rm, rse = np.asarray(g[key + "_mean"]), np.asarray(g[key + "_sem"])
    sig = np.hypot(se, rse)
    eps = np.asarray(g.get("len2_drift_absmax", np.zeros_like(rm)))
    sysm = 2 * eps if key == "S" else 4 * eps * (np.abs(rm) + 1)
    z = np.maximum(np.abs(m - rm) - sysm, 0.0) / sig
    return [(int(i), float(m[i]), float(rm[i]), float(sig[i]), float(z[i])) for i in np.nonzero(z > 3)[0]]


P_BEYOND_3SIGMA = 0.0026997961  # two-sided normal tail beyond 3 standard errors


def chance_exceedances(n: int, alpha: float = 0.05) -> int:
    """How many of n independent comparisons may lie beyond 3 standard errors
    by chance: the smallest k with P(Binomial(n, p3) > k) < alpha, p3 the
    two-sided normal tail beyond 3 sigma.  0 for up to 18 comparisons (every
    row within 3 sigma), 1 for 19..131 (e.g. both S and E of the 61
    temperatures of the LL anneal)."""
    from math import comb
    k, tail = 0, 1.0
    while True:
        tail -= comb(n, k) * P_BEYOND_3SIGMA ** k * (1 - P_BEYOND_3SIGMA) ** (n - k)
        if tail < alpha:
            return k
        k += 1


def assert_stat_parity(checks, labels):
    """checks: (G, golden, key) triples compared row by row against the same
    labels.  Every row must lie within 3 combined standard errors
    (stat_parity_failures), except for as many rows as chance alone puts
    beyond 3 sigma among all the comparisons made (chance_exceedances, 5%
    family-wise), and none beyond 4 sigma."""
    bad, n = [], 0
    for G, g, key in checks:
        n += G.shape[1]
        bad += [(key, labels[i], *rest) for i, *rest in stat_parity_failures(G, g, key)]
    allowed = chance_exceedances(n)
    assert len(bad) <= allowed and all(b[-1] <= 4.0 for b in bad), (n, allowed, bad)
    return bad


def load_local_order():
    """tests/golden/local_order.npz (make_local_order.py): per lattice its
    model, point types, directors, the reference's local S and the text of
    the reference's snapshot file of that state (None where not kept)."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "local_order.npz")
    z = np.load(path)
    out = {}
    for name, d in json.loads(str(z["models"])).items():
        d = dict(d)
        d["surfaces"] = [O.Surface(**s) for s in d["surfaces"]]
        csv = z[f"{name}_csv"].tobytes().decode() if f"{name}_csv" in z.files else None
        out[name] = (O.Model(**d), z[f"{name}_pt"], z[f"{name}_ni"], z[f"{name}_S"], csv)
    return out
