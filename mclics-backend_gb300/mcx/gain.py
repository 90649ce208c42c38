"""What the learned proposal gains over plain Metropolis: effectively
independent samples per second of E and S (no counterpart in the reference).

Protocol (Lebwohl-Lasher bulk, periodic, one engine holding every replica):
  1. every replica starts along z and is equilibrated with the plain move and
     the reference's adaptive step;
  2. training samples are drawn from those plain-sampler equilibrium states
     (all temperatures at once, head-tail flips and global rotations as
     augmentation) and the network is trained on the GPU;
  3. the step size is frozen, the states are saved, and each proposal runs
     `meas` measured sweeps from the same saved states; the per-sweep E and S
     series give tau_int (Madras-Sokal, over the replicas at each T) and the
     per-replica means give E(T), S(T) with standard errors;
  4. independent samples/s at T = (replicas at T) * sweeps/s / (2 tau), with
     tau the larger of tau_E and tau_S, and sweeps/s the wall-clock rate of the
     measured run of the whole engine.
The two chains have the same stationary law (exact MH ratio); their E and S
means must agree within 3 combined standard errors at every T.
"""
from __future__ import annotations

import time
from typing import Dict, Sequence

import numpy as np

from . import AUG_FLIP, AUG_ROTATE, ST_ACC, ST_SWEEPS, Engine, replica
from .autocorr import tau_int

MLP_FLOP_PER_UPDATE = 2 * (19 * 64 + 64 * 64 + 64 * 4)  # 11,136


def init_weights(seed: int) -> np.ndarray:
    """He-style random weights in the flat layout (rows 19..31 of W1 and
    columns 4..7 of W3 zero), log-kappa bias 1."""
    rng = np.random.default_rng(seed)
    W1 = np.zeros((32, 64))
    W1[:19] = rng.normal(0, 1 / np.sqrt(19), (19, 64))
    W2 = rng.normal(0, 1 / np.sqrt(64), (64, 64))
    W3 = np.zeros((64, 8))
    W3[:, :4] = rng.normal(0, 1 / np.sqrt(64), (64, 4))
    b3 = np.zeros(8)
    b3[3] = 1.0
    return np.concatenate([W1.ravel(), np.zeros(64), W2.ravel(), np.zeros(64), W3.ravel(), b3]).astype(np.float32)


def run(L: int = 96, temps: Sequence[float] = (1.00, 1.10, 1.12, 1.15), per_T: int = 32, equil: int = 3000,
        meas: int = 8000, train_samples: int = 1_000_000, schedule=((1500, 2e-3), (1000, 5e-4), (500, 1e-4)),
        batch: int = 8192, seed: int = 1, log=None) -> Dict:
    def say(*a):
        if log:
            log(" ".join(str(x) for x in a))

    nT = len(temps)
    R = nT * per_T
    descs = [replica(nx=L, ny=L, nz=L, potential="ll", T=temps[q // per_T], seed=seed + q, stream=q)
             for q in range(R)]
    out: Dict = {"lattice": [L, L, L], "temps": list(temps), "replicas_per_T": per_T, "equil_sweeps": equil,
                 "meas_sweeps": meas, "train_samples": train_samples}
    with Engine(descs) as eng:
        for q in range(R):
            eng.init_homogeneous(q, 0.0, 0.0)
        t0 = time.perf_counter()
        eng.sweep(equil)
        eng.sync()
        say(f"equilibrated {equil} sweeps in {time.perf_counter() - t0:.1f}s")
        # the plain sampler runs with the pass shape the autotuner picks for this batch
        out["plain_pass"] = list(eng.autotune()[:2]) + [eng.pass_kind]
        # training on plain-sampler equilibrium configurations
        eng.set_mlp(init_weights(seed))
        t0 = time.perf_counter()
        losses = []
        first = True
        for steps, lr in schedule:
            losses.append(eng.train_mlp(samples=train_samples if first else 0, batch=batch, steps=steps, lr=lr,
                                        seed=seed, augment=AUG_FLIP | AUG_ROTATE))
            first = False
        losses = np.concatenate(losses)
        out["train_seconds"] = time.perf_counter() - t0
        out["train_steps"] = int(len(losses))
        out["train_batch"] = batch
        out["loss_first"] = float(losses[:10].mean())
        out["loss_last"] = float(losses[-50:].mean())
        out["loss_uniform"] = float(np.log(4 * np.pi))
        say(f"trained {len(losses)} steps in {out['train_seconds']:.1f}s, loss {out['loss_first']:.4f} -> "
            f"{out['loss_last']:.4f}")
        eng.set_adapt(False)
        saved = [eng.get_state(q) for q in range(R)]
        eng.set_series(meas)
        runs = {}
        for kind in ("plain", "vmf_mlp"):
            for q in range(R):
                eng.set_state(q, saved[q])
            eng.set_proposal(kind)
            eng.reset_stats()
            eng.sync()
            t0 = time.perf_counter()
            eng.sweep(meas, measure=True)
            eng.sync()
            dt = time.perf_counter() - t0
            st = np.array([eng.stats(q) for q in range(R)])
            ser = np.array([eng.series(q, meas) for q in range(R)])  # [R, meas, 2]
            acc = st[:, ST_ACC] / (st[:, ST_SWEEPS] * L ** 3)
            runs[kind] = dict(seconds=dt, sweeps_per_s=meas / dt, series=ser, acc=acc)
            say(f"{kind}: {meas} measured sweeps in {dt:.1f}s ({meas / dt:.1f} sweeps/s), "
                f"acceptance {acc.mean():.3f}")
        rows = []
        for t, T in enumerate(temps):
            sl = slice(t * per_T, (t + 1) * per_T)
            row = {"T": T}
            for kind, rr in runs.items():
                ser = rr["series"][sl]
                tE, tS = tau_int(ser[:, :, 0]), tau_int(ser[:, :, 1])
                tau = max(tE["tau"], tS["tau"])
                mE, mS = ser[:, :, 0].mean(1), ser[:, :, 1].mean(1)
                row[kind] = {
                    "tau_E": tE["tau"], "tau_E_err": tE["err"], "tau_S": tS["tau"], "tau_S_err": tS["err"],
                    "reliable": tE["reliable"] and tS["reliable"],
                    "E": float(mE.mean()), "E_sem": float(mE.std(ddof=1) / np.sqrt(per_T)),
                    "S": float(mS.mean()), "S_sem": float(mS.std(ddof=1) / np.sqrt(per_T)),
                    "acceptance": float(rr["acc"][sl].mean()),
                    "indep_samples_per_s": per_T * rr["sweeps_per_s"] / (2 * tau),
                }
            p, lrn = row["plain"], row["vmf_mlp"]
            for o in ("E", "S"):
                se = np.hypot(p[o + "_sem"], lrn[o + "_sem"])
                row[o + "_diff_sigma"] = float(abs(p[o] - lrn[o]) / se) if se > 0 else 0.0
            row["gain"] = lrn["indep_samples_per_s"] / p["indep_samples_per_s"]
            row["tau_ratio"] = max(p["tau_E"], p["tau_S"]) / max(lrn["tau_E"], lrn["tau_S"])
            rows.append(row)
            say(f"T={T}: tau plain E {p['tau_E']:.1f} S {p['tau_S']:.1f} | learned E {lrn['tau_E']:.1f} "
                f"S {lrn['tau_S']:.1f} | gain {row['gain']:.2f} | dE {row['E_diff_sigma']:.2f} sigma, "
                f"dS {row['S_diff_sigma']:.2f} sigma")
        out["rows"] = rows
        out["sweeps_per_s"] = {k: v["sweeps_per_s"] for k, v in runs.items()}
        sites = R * L ** 3
        out["site_updates_per_s"] = {k: v["sweeps_per_s"] * sites for k, v in runs.items()}
        out["mlp_tflops"] = runs["vmf_mlp"]["sweeps_per_s"] * sites * MLP_FLOP_PER_UPDATE / 1e12
        out["parity_3sigma"] = all(r["E_diff_sigma"] < 3 and r["S_diff_sigma"] < 3 for r in rows)
    return out


if __name__ == "__main__":
    import argparse
    import json

    ap = argparse.ArgumentParser(description="learned vs plain proposal: independent samples/s")
    ap.add_argument("--side", type=int, default=96)
    ap.add_argument("--per-T", type=int, default=32)
    ap.add_argument("--equil", type=int, default=6000)
    ap.add_argument("--meas", type=int, default=12000)
    ap.add_argument("--samples", type=int, default=1_000_000)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    res = run(L=a.side, per_T=a.per_T, equil=a.equil, meas=a.meas, train_samples=a.samples, seed=a.seed,
              log=lambda m: print(m, flush=True))
    txt = json.dumps(res)
    if a.out:
        with open(a.out, "w") as f:
            f.write(txt + "\n")
    print(txt)
