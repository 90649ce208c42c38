#!/usr/bin/env python3
"""Benchmark of the GB300 Metropolis engine on the McLiCS 128^3 anneal.

Workload (the configuration the headline metric is quoted on): Lebwohl-Lasher
bulk 128x128x128, periodic, A = 1, homogeneous initial directors along z,
thermal anneal Ti = 1.20 -> Tf = 0.90 in steps of dT = -0.01 (31 temperatures,
float stepping as the reference's run loop), MCT = 2000 unmeasured + MCS = 2000
measured sweeps per temperature, fp32 directors, FP64 E / Q / S reductions
after every measured sweep.

One step = one temperature block (4000 red/black sweeps of 2,097,152 sites,
2000 of them followed by the E/Q/S measurement).  Metric: site-updates/s.

  value      device time (CUDA events on the engine's stream) of K steps with
             the lattice already resident; L2 is flushed (256 MiB write)
             between steps, outside the timed windows.
  e2e        the same K steps through the C ABI with host buffers: each step
             uploads the AoS director field from pinned host memory
             (mcx_set_state), runs the block, and reads back the running sums
             and the AoS field (mcx_get_stats, mcx_get_state); wall clock.
  roofline   the red/black pass kernel: 18 algorithmic bytes per site per
             launch (read both colours 12 B, write the updated half 6 B) over
             its mean launch time, from CUDA events around each pass launch
             (mcx_pass_timing) right after the timed region.
  cpu_baseline  the reference CPU path on the host cores on a bounded sample
             of the same lattice (the reference's own EvolveN::Monte_Carlo_Step
             when oracle/_ref is loadable, else the oracle's C port of it).

--impl reference times only that CPU path, per step a bounded sample.
Multi-GPU runs (torchrun) are replicas: each rank anneals its own lattice.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "mclics-backend_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

NX = NY = NZ = 128
SITES = NX * NY * NZ
TI, TF, DT = 1.20, 0.90, -0.01
MCT = MCS = 2000
BYTES_PER_SITE_PASS = 18
# pass forms of the plain proposal: roofline kernel name, description
FORMS = {"march": ("k_march<LL> (red/black pass)", "z-march"),
         "march_async": ("k_amarch<LL> (red/black pass, cp.async prefetch)", "z-march with cp.async prefetch"),
         "march_tma": ("k_tmarch<LL> (red/black pass, bulk-copy staged)", "z-march with bulk-copy staging"),
         "march_persistent": ("k_pmarch<LL> (red/black passes, one cooperative launch)", "persistent z-march"),
         "direct": ("k_pass<LL> (red/black pass)", "direct pass"),
         "staged": ("k_tpass<LL> (red/black pass)", "staged pass")}
WORKLOAD = ("LL bulk 128^3 periodic, A=1, homogeneous ic along z, anneal Ti=1.20 -> Tf=0.90 dT=-0.01, "
            "MCT=2000 MCS=2000 per temperature")


def temperatures():
    """The reference's float loop (src/evolve_thermal.cpp:58)."""
    f = np.float32
    out = []
    T = f(TI)
    sign = int(-DT / abs(DT))
    while f(1e6 * sign) * (T - f(TF)) >= 0:
        out.append(float(T))
        T = f(T + f(DT))
    return out


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    lrank = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, lrank


class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(seconds: float = 12.0):
    """Site-updates/s of the reference CPU sweep on the host cores, on a
    bounded sample of the same 128^3 lattice (homogeneous along z, T = 1.20)."""
    cores = os.cpu_count() or 1
    try:
        from oracle import refproc
        if refproc.available():
            return _cpu_reference(seconds, cores)
    except Exception:
        pass
    return _cpu_port(seconds, cores)


def _cpu_reference_worker(seconds, cores, q):
    import ctypes as C

    from oracle import oracle as O
    from oracle import refproc
    L = C.CDLL(refproc.REF_LIB_PATH)
    m = O.Model(nx=NX, ny=NY, nz=NZ)
    devnull = os.open(os.devnull, os.O_WRONLY)
    old = os.dup(1)
    os.dup2(devnull, 1)
    refproc._setup(L, refproc.model_dict(m))
    os.dup2(old, 1)
    ni = np.zeros((SITES, 3), np.float32)
    ni[:, 2] = 1
    L.ref_set_state(ni.ctypes.data_as(C.c_void_p))
    L.ref_sweeps_inplace(1, C.c_float(TI), C.c_float(0.5), cores)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds or n < 2:
        L.ref_sweeps_inplace(1, C.c_float(TI), C.c_float(0.5), cores)
        n += 1
    dt = time.perf_counter() - t0
    q.put((n, dt))


def _cpu_reference(seconds, cores):
    import multiprocessing as mp
    # the worker's OpenMP runtime reads this when the library loads (a
    # launcher such as torchrun sets it to 1 for every rank)
    os.environ["OMP_NUM_THREADS"] = str(cores)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_cpu_reference_worker, args=(seconds, cores, q))
    p.start()
    n, dt = q.get(timeout=seconds * 20 + 120)
    p.join()
    return {"value": n * SITES / dt, "unit": "site-updates/s", "cores": cores, "kind": "reference",
            "sample": f"{n} sweeps of the 128^3 LL lattice at T=1.20 (reference EvolveN::Monte_Carlo_Step, "
                      f"8-colour OpenMP, test-only GSL shim RNG), {dt:.1f} s"}


def _cpu_port(seconds, cores):
    from oracle import oracle as O
    m = O.Model(nx=NX, ny=NY, nz=NZ)
    os.environ["OMP_NUM_THREADS"] = str(cores)  # before the oracle library's OpenMP runtime loads
    lat = O.Lattice(m)
    a = np.float32(0.5)
    lat.sweep(TI, a, 1, 0, 0, "eight", O.F_PARALLEL | O.F_NO_NORMALIZE)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds or n < 2:
        _, a = lat.sweep(TI, a, 1, 0, n + 1, "eight", O.F_PARALLEL | O.F_NO_NORMALIZE)
        n += 1
    dt = time.perf_counter() - t0
    return {"value": n * SITES / dt, "unit": "site-updates/s", "cores": cores, "kind": "port",
            "sample": f"{n} sweeps of the 128^3 LL lattice at T=1.20 (oracle C port of "
                      f"EvolveN::Monte_Carlo_Step, 8-colour, OpenMP), {dt:.1f} s"}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    sample = 2  # sweeps of the 128^3 lattice per step
    use_ref = False
    try:
        from oracle import refproc
        use_ref = refproc.available()
    except Exception:
        use_ref = False
    times = []
    kind = "reference" if use_ref else "port"
    if use_ref:
        for s in range(args.warmup + args.steps):
            r = _cpu_reference(0.0, cores)  # one bounded sample per step (>= 2 sweeps)
            if s >= args.warmup:
                times.append(SITES / r["value"] * 2)
        sample = 2
    else:
        os.environ["OMP_NUM_THREADS"] = str(cores)  # before the oracle library's OpenMP runtime loads
        from oracle import oracle as O
        lat = O.Lattice(O.Model(nx=NX, ny=NY, nz=NZ))
        a = np.float32(0.5)
        sweep = 0
        for s in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            for _ in range(sample):
                _, a = lat.sweep(TI, a, 1, 0, sweep, "eight", O.F_PARALLEL | O.F_NO_NORMALIZE)
                sweep += 1
            if s >= args.warmup:
                times.append(time.perf_counter() - t0)
    per_step = float(np.mean(times))
    value = sample * SITES / per_step
    line = {
        "impl": "reference", "metric": "site-updates/s", "value": value, "unit": "site-updates/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if use_ref else "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "step": f"bounded sample: {sample} sweeps of the {NX}^3 lattice at T=1.20"},
        "cpu_baseline": {"value": value, "unit": "site-updates/s", "cores": cores, "kind": kind,
                         "sample": f"{sample} sweeps per step, all {cores} host threads"},
        "e2e": {"value": value, "unit": "site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=31)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--side", type=int, default=128,
                    help="lattice side (default 128, the headline workload; other sides are for profiling)")
    ap.add_argument("--sweeps", type=int, default=2000,
                    help="MCT = MCS per temperature (default 2000, the headline workload)")
    ap.add_argument("--replicas", type=int, default=1,
                    help="independent lattices in one engine (default 1, the headline workload; more for profiling "
                         "the batched pass)")
    ap.add_argument("--pass-shape", default=None,
                    help="KIND:BLOCK:PLANES (e.g. march:256:0) instead of the autotuner's choice; for profiling "
                         "runs, where a profiler's serialisation would distort the autotuner's timings")
    ap.add_argument("--proposal", default="plain", choices=["plain", "vmf_mlp"],
                    help="plain (the reference's move; default) or the learned proposal with untrained weights "
                         "(for profiling its pass)")
    args = ap.parse_args()
    global NX, NY, NZ, SITES, MCT, MCS, WORKLOAD
    R = max(1, args.replicas)
    if args.side != 128 or args.sweeps != 2000 or R != 1 or args.proposal != "plain":
        NX = NY = NZ = args.side
        SITES = NX * NY * NZ
        MCT = MCS = args.sweeps
        WORKLOAD = (f"LL bulk {NX}^3 periodic x {R} replicas, A=1, homogeneous ic along z, anneal Ti=1.20 -> "
                    f"Tf=0.90 dT=-0.01, MCT={MCT} MCS={MCS} per temperature, {args.proposal} proposal (profiling "
                    f"variant of the headline workload)")
    ws, rank, lrank = dist_info()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    import torch
    torch.cuda.set_device(lrank)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import mcx
    from mcx.shard import max_over_ranks

    temps = temperatures()
    descs = [mcx.replica(nx=NX, ny=NY, nz=NZ, potential="ll", A=1.0, T=temps[0], ang_var=0.5, seed=1 + rank * R + q,
                         stream=rank * R + q) for q in range(R)]
    eng = mcx.Engine(descs)
    stream = torch.cuda.ExternalStream(mcx.lib().mcx_stream(eng._h))
    # the engine's autotuner picks the z-march pass shape (on a scratch copy of
    # the state, before anything is timed)
    for q in range(R):
        eng.init_homogeneous(q, 0.0, 0.0)
    if args.pass_shape:
        kind, blk, planes = args.pass_shape.split(":")
        eng.pass_kind = kind
        eng.set_march_shape(int(blk), int(planes))
        tuned = (int(blk), int(planes), None)
    else:
        tuned = eng.autotune()
    form, how = eng.pass_kind, "given" if args.pass_shape else "autotuned"
    if args.proposal != "plain":
        from mcx import gain
        eng.set_mlp(gain.init_weights(1))
        eng.set_proposal(args.proposal)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def reset():
        for q in range(R):
            eng.init_homogeneous(q, 0.0, 0.0)
        eng.set_step(0.5)

    def block(T):
        eng.set_temperature(T)
        eng.sweep(MCT, measure=False)
        eng.reset_stats()
        eng.sweep(MCS, measure=True)

    # warm-up: W temperature blocks (graphs built, clocks up)
    reset()
    for s in range(args.warmup):
        block(temps[s % len(temps)])
    eng.sync()

    # timed region: K temperature blocks of the anneal from the initial state
    reset()
    nsteps = args.steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
    rows = []
    clocks = ClockSampler(lrank)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    eng.sync()
    launches0 = eng.kernel_launches
    clocks.start()
    for s in range(nsteps):
        with torch.cuda.stream(stream):
            flush.add_(1)
            ev[s][0].record(stream)
        block(temps[s % len(temps)])
        ev[s][1].record(stream)
        st = eng.stats(0)
        n = st[mcx.ST_N]
        rows.append((temps[s % len(temps)], st[mcx.ST_S1] / n, st[mcx.ST_E1] / n))
    eng.sync()
    torch.cuda.synchronize()
    clk = clocks.stop()
    if dist:
        dist.barrier()
    launches = eng.kernel_launches - launches0
    total_ms = sum(a.elapsed_time(b) for a, b in ev)
    total_ms = max_over_ranks(total_ms)  # the slowest rank's time (identity on one GPU)
    per_step_ms = total_ms / nsteps
    updates_per_step = (MCT + MCS) * SITES * R
    value = ws * updates_per_step * nsteps / (total_ms / 1e3)

    # live pass-kernel timing for the roofline
    import ctypes as C
    # (a) the pass kernel's average duration in the production sequence: 400
    # unmeasured sweeps replayed from the engine's graphs between two events
    # on its stream (launch gaps included, so this is conservative); (b) for
    # reference, the mean of per-launch event brackets around directly
    # launched passes (these include the host submission gap of each launch)
    sw_ms = C.c_float()
    n_prof = 400
    st = mcx.lib().mcx_sweep_timing(eng._h, n_prof, C.byref(sw_ms))
    if st:
        raise RuntimeError(mcx.lib().mcx_last_error(eng._h).decode())
    per_launch_ms = sw_ms.value / (2 * n_prof)
    pass_ms, all_ms = C.c_float(), C.c_float()
    st = mcx.lib().mcx_pass_timing(eng._h, 100, C.byref(pass_ms), C.byref(all_ms))
    if st:
        raise RuntimeError(mcx.lib().mcx_last_error(eng._h).decode())
    per_launch_isolated_ms = pass_ms.value / 200
    bytes_per_launch = BYTES_PER_SITE_PASS * SITES * R
    achieved = bytes_per_launch / (per_launch_ms * 1e-3) / 1e9
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        pk = json.load(open(peaks_path))
        peak, bf16_peak = pk["hbm_gbs"], pk.get("bf16_tflops_sustained", pk.get("bf16_tflops"))
        peak_src = "measured"
    else:
        peak, bf16_peak, peak_src = 6800.0, 1700.0, "fallback"
    from mcx.gain import MLP_FLOP_PER_UPDATE
    flops_per_launch = MLP_FLOP_PER_UPDATE * SITES * R / 2  # one colour: half the sites
    mlp_tflops = flops_per_launch / (per_launch_ms * 1e-3) / 1e12
    traffic = None
    tpath = os.path.join(ROOT, "profiles", f"sweep_pass_ll{NX}.md" if R == 1 else f"sweep_pass_ll{NX}x{R}.md")
    if os.path.exists(tpath):
        for ln in open(tpath):
            if ln.startswith("dram_bytes_per_launch:"):
                traffic = float(ln.split(":", 1)[1].split()[0])

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        host_in = torch.zeros((SITES, 3), dtype=torch.float32).pin_memory()
        host_in[:, 2] = 1.0
        host_out = torch.empty((SITES, 3), dtype=torch.float32).pin_memory()
        import ctypes as C2
        L = mcx.lib()
        pin = C2.c_void_p(host_in.data_ptr())
        pout = C2.c_void_p(host_out.data_ptr())
        stats = np.zeros(16)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        eng.set_step(0.5)
        t0 = time.perf_counter()
        for s in range(nsteps):
            for q in range(R):
                if L.mcx_set_state(eng._h, q, pin):
                    raise RuntimeError(L.mcx_last_error(eng._h).decode())
            block(temps[s % len(temps)])
            if L.mcx_get_stats(eng._h, 0, stats.ctypes.data_as(C2.c_void_p)):
                raise RuntimeError(L.mcx_last_error(eng._h).decode())
            for q in range(R):
                if L.mcx_get_state(eng._h, q, pout):
                    raise RuntimeError(L.mcx_last_error(eng._h).decode())
        e2e_s = time.perf_counter() - t0
        e2e_s = max_over_ranks(e2e_s)
        e2e = {"value": ws * updates_per_step * nsteps / e2e_s, "unit": "site-updates/s",
               "h2d_bytes_per_step": 12 * SITES * R, "d2h_bytes_per_step": 12 * SITES * R + 16 * 8}

    if rank != 0:
        eng.close()
        if dist:
            dist.destroy_process_group()
        return
    cpu = None if args.no_cpu_baseline or ws > 1 else cpu_baseline()
    line = {
        "metric": "site-updates/s", "value": value, "unit": "site-updates/s", "n_gpus": ws, "steps": nsteps,
        "warmup": args.warmup, "ms_per_step": per_step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD,
                   "step": f"one temperature block: {MCT} sweeps + {MCS} sweeps each followed by FP64 E/Q/S",
                   "l2": "flushed (256 MiB write) between steps outside the timed windows; the 25 MB lattice "
                         "stays L2-resident within a step",
                   "parallelism": (f"replicas x{ws} ranks" if ws > 1 else "one GPU") + f", {R} lattice(s) per engine",
                   "pass_kernel": ((f"{FORMS[form][1]}, {tuned[0]} threads x {tuned[1]} planes per CTA ({how})"
                                    if tuned[1] > 0
                                    else f"{FORMS[form][1]}, {tuned[0]} threads x balanced chunks filling "
                                         f"{max(1, -tuned[1])} wave(s) of resident CTAs ({how})")
                                   if args.proposal == "plain" else "learned-proposal z-march (k_lmarch, BF16 MLP)"),
                   "S_E_last_step": [rows[-1][0], rows[-1][1], rows[-1][2]] if rows else None},
        "roofline": ({"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                      "traffic": traffic, "peak_source": peak_src, "kernel": FORMS[form][0],
                      "bytes_per_launch": bytes_per_launch}
                     if args.proposal == "plain" else
                     # the learned pass is bound by its BF16 MLP: 11.1 kFLOP per site-update against
                     # the sustained dense BF16 rate (the pass runs for seconds back to back)
                     {"bound": "tensor", "achieved": mlp_tflops, "peak": bf16_peak, "unit": "TFLOP/s",
                      "frac": mlp_tflops / bf16_peak, "traffic": None, "peak_source": peak_src,
                      "kernel": "k_lmarch<LL> (learned proposal, mma.sync BF16 MLP)",
                      "flops_per_launch": flops_per_launch, "hbm_achieved_gbs": achieved}) | {
                     "launch_ms": per_launch_ms,
                     "launch_ms_isolated": per_launch_isolated_ms,
                     "launch_ms_method": ("400 unmeasured sweeps in cooperative launches between two CUDA events "
                                          "on the engine stream / 800 passes" if form == "march_persistent" else
                                          "400 graph-replayed unmeasured sweeps between two CUDA events on the "
                                          "engine stream / 800 pass launches (launch gaps included)"),
                     "pass_share_of_sweep": pass_ms.value / all_ms.value if all_ms.value else None},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clk,
        "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)
    eng.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
