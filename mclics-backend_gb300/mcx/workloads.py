"""The batched workloads beside the headline anneal, timed on the GPU (one
JSON line each):

  c3  GHRL slab batch: R independent replicas in one engine, cubic sides drawn
      uniformly from {16, 24, 32, 48, 64} (fixed seed), slab geometry (free z,
      periodic x/y), homeotropic anchoring W = 4 on both z faces,
      k11 = 1.0, k22 = 0.8, k33 = 1.2, p0 = 0, T uniform in [0.8, 1.2], random
      start; MCT unmeasured + MCS measured sweeps.
  c5  droplet + field: R replicas of a radius-40 droplet centred in a 96^3
      box (free outer bounds, planar (fg) anchoring W = 1 on the droplet
      surface), GHRL k11 = 1.0, k22 = 0.6, k33 = 1.4, p0 = 20, field along z
      (elecA = 1) stepped E = 0 -> 2.0 by 0.1 at T = 0.8, random start; per
      field value MCT + MCS sweeps, with the plain or the learned proposal
      (trained first on samples of the plain chain's states, head-tail flips
      as augmentation).

Throughput is site-updates/s over all sites of the batch (inactive droplet
sites included, as the kernels visit them); the roofline figure uses the
masked pass's algorithmic 19 B per site per pass (18 B of directors + 1 B of
point types).  The full configurations run MCT = MCS = 1000; the defaults
here time fewer sweeps per step so that a run takes seconds, which does not
change the per-sweep cost.

    PYTHONPATH=mclics-backend_gb300 python -m mcx.workloads c3 [--replicas 256] [--sweeps 50] [--pass-shape march:64:16]
    PYTHONPATH=mclics-backend_gb300 python -m mcx.workloads c5 [--replicas 64] [--sweeps 20] [--proposal vmf_mlp]
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import AUG_FLIP, ST_ACC, ST_N, ST_S1, ST_SWEEPS, Engine, replica

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
BYTES_PER_SITE_PASS_MASKED = 19


def _peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return json.load(open(p))["hbm_gbs"], "measured"
    return 6800.0, "fallback"


def c3_descs(n: int, seed: int = 3):
    rng = np.random.default_rng(seed)
    sides = rng.choice([16, 24, 32, 48, 64], size=n)
    temps = rng.uniform(0.8, 1.2, size=n)
    hom = dict(anchoring="homeotropic", W=4.0, theta_s=0.0, phi_s=0.0)
    return [replica(nx=int(L), ny=int(L), nz=int(L), geometry="slab", potential="ghrl", k11=1.0, k22=0.8, k33=1.2,
                    p0=0.0, T=float(T), seed=100 + q, stream=q, surfaces=[hom, hom])
            for q, (L, T) in enumerate(zip(sides, temps))]


def c5_descs(n: int, side: int = 96, radius: float = 40.0):
    fg = dict(anchoring="fg", W=1.0, theta_s=0.0, phi_s=0.0)
    return [replica(nx=side, ny=side, nz=side, geometry="sphere", potential="ghrl", k11=1.0, k22=0.6, k33=1.4,
                    p0=20.0, elecA=1.0, elecX=0.0, elecY=0.0, elecZ=1.0, elecE=0.0, T=0.8, seed=500 + q, stream=q,
                    surfaces=[fg], radius=radius) for q in range(n)]


def _time_blocks(eng, steps, mct, mcs, per_step=None):
    eng.sync()
    t0 = time.perf_counter()
    for s in range(steps):
        if per_step:
            per_step(s)
        eng.sweep(mct)
        eng.reset_stats()
        eng.sweep(mcs, measure=True)
    eng.sync()
    return time.perf_counter() - t0


def _shape(eng, pass_shape):
    """The autotuner's pass shape, or KIND:BLOCK:PLANES as given (profiling
    runs, where a profiler's serialisation would distort the autotuner)."""
    if not pass_shape:
        return eng.autotune()
    kind, blk, planes = pass_shape.split(":")
    eng.pass_kind = kind
    eng.set_march_shape(int(blk), int(planes))
    return int(blk), int(planes), None


def run_c3(replicas=256, sweeps=50, steps=3, seed=3, pass_shape=None):
    descs = c3_descs(replicas, seed)
    sites = sum(d.nx * d.ny * d.nz for d in descs)
    with Engine(descs) as eng:
        for q in range(replicas):
            eng.init_random(q, 7 + q)
        tuned = _shape(eng, pass_shape)
        _time_blocks(eng, 1, sweeps, sweeps)  # warm-up: graphs built
        dt = _time_blocks(eng, steps, sweeps, sweeps)
        sw_ms = None
        import ctypes as C
        from . import lib
        ms = C.c_float()
        if lib().mcx_sweep_timing(eng._h, 160, C.byref(ms)) == 0:
            sw_ms = ms.value / 160
        S = np.mean([eng.stats(q)[ST_S1] / max(eng.stats(q)[ST_N], 1) for q in range(replicas)])
    ups = 2 * sweeps * steps * sites / dt
    peak, src = _peak()
    ach = BYTES_PER_SITE_PASS_MASKED * sites / (sw_ms / 2 * 1e-3) / 1e9 if sw_ms else None
    return {"workload": "c3: GHRL slab batch", "replicas": replicas, "sites": int(sites),
            "sides": sorted(set(int(d.nx) for d in descs)), "site_updates_per_s": ups,
            "sweep_ms": sw_ms,
            "pass_kernel": f"z-march {tuned[0]} x {tuned[1]} ({'given' if pass_shape else 'autotuned'})",
            "roofline": {"achieved_gbs": ach, "peak_gbs": peak, "frac": ach / peak if ach else None,
                         "peak_source": src, "bytes_per_site_pass": BYTES_PER_SITE_PASS_MASKED},
            "mean_S": float(S)}


def run_c5(replicas=64, sweeps=20, proposal="plain", side=96, radius=40.0, train_samples=1_000_000, pass_shape=None):
    from . import gain
    descs = c5_descs(replicas, side, radius)
    sites = replicas * side ** 3
    fields = [round(0.1 * i, 1) for i in range(21)]
    out = {"workload": "c5: droplet r=40 in 96^3, GHRL p0=20, field sweep E=0..2.0 at T=0.8",
           "replicas": replicas, "sites": int(sites), "proposal": proposal, "field_values": len(fields)}
    with Engine(descs) as eng:
        for q in range(replicas):
            eng.init_random(q, 11 + q)
        tuned = _shape(eng, pass_shape)
        out["pass_kernel"] = f"{eng.pass_kind} {tuned[0]} x {tuned[1]}" + ("" if pass_shape else " (autotuned)")
        eng.sweep(200)
        if proposal != "plain":
            eng.set_mlp(gain.init_weights(5))
            loss = eng.train_mlp(samples=train_samples, batch=8192, steps=1500, lr=2e-3, seed=5, augment=AUG_FLIP)
            eng.train_mlp(samples=0, batch=8192, steps=500, lr=3e-4, seed=6, augment=AUG_FLIP)
            out["train_loss"] = [float(loss[:10].mean()), float(loss[-50:].mean())]
            eng.set_proposal(proposal)
        eng.reset_stats()
        dt = _time_blocks(eng, len(fields), sweeps, sweeps, per_step=lambda s: eng.set_field(fields[s]))
        st = [eng.stats(q) for q in range(replicas)]
        valid = eng.measure(0)["valid"]  # active sites of a droplet (every replica has the same mask)
        out["active_sites_per_replica"] = int(valid)
        out["acceptance"] = float(np.mean([x[ST_ACC] / (x[ST_SWEEPS] * valid) for x in st]))
        out["mean_S_last_field"] = float(np.mean([x[ST_S1] / max(x[ST_N], 1) for x in st]))
        if proposal == "plain":
            # the pass against the HBM roofline as for c3: 19 B per site of the
            # box per pass (dead units load nothing, so this counts more than
            # the pass moves), over the unmeasured sweep time
            import ctypes as C
            from . import lib
            ms = C.c_float()
            if lib().mcx_sweep_timing(eng._h, 80, C.byref(ms)) == 0:
                sw_ms = ms.value / 80
                peak, src = _peak()
                ach = BYTES_PER_SITE_PASS_MASKED * sites / (sw_ms / 2 * 1e-3) / 1e9
                out["sweep_ms"] = sw_ms
                out["roofline"] = {"achieved_gbs": ach, "peak_gbs": peak, "frac": ach / peak, "peak_source": src,
                                   "bytes_per_site_pass": BYTES_PER_SITE_PASS_MASKED,
                                   "sites": "every site of the box"}
    out["site_updates_per_s"] = 2 * sweeps * len(fields) * sites / dt
    out["active_site_updates_per_s"] = 2 * sweeps * len(fields) * replicas * out["active_sites_per_replica"] / dt
    out["seconds"] = dt
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("which", choices=["c3", "c5"])
    ap.add_argument("--replicas", type=int, default=None)
    ap.add_argument("--sweeps", type=int, default=None)
    ap.add_argument("--proposal", default="plain", choices=["plain", "vmf_mlp"])
    ap.add_argument("--steps", type=int, default=3, help="c3: timed blocks")
    ap.add_argument("--pass-shape", default=None, help="KIND:BLOCK:PLANES instead of the autotuner's choice")
    a = ap.parse_args()
    if a.which == "c3":
        res = run_c3(replicas=a.replicas or 256, sweeps=a.sweeps or 50, steps=a.steps, pass_shape=a.pass_shape)
    else:
        res = run_c5(replicas=a.replicas or 64, sweeps=a.sweeps or 20, proposal=a.proposal, pass_shape=a.pass_shape)
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
