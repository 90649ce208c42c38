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
             when oracle/_ref is loadable, else its C port, oracle/mcx_port.c,
             which reproduces the reference's sweeps bit for bit and runs
             within 10% of its speed); the host CPU model is recorded.
  c3, c5, indep_samples  the other configurations, each a bounded run after
             the headline (--no-workloads skips them): the 256-replica GHRL
             slab batch and the droplet field sweep (site-updates/s and the
             masked pass's roofline), and the learned proposal against the
             plain one on 128 x 96^3 at T = 1.00, 1.10, 1.12, 1.15
             (effectively independent samples/s by tau_int of E and S).

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
         "march_quad": ("k_qmarch<LL> (red/black pass, four sites per thread)", "z-march with four sites per thread"),
         "direct": ("k_pass<LL> (red/black pass)", "direct pass"),
         "staged": ("k_tpass<LL> (red/black pass)", "staged pass")}
WORKLOAD = ("LL bulk 128^3 periodic, A=1, homogeneous ic along z, anneal Ti=1.20 -> Tf=0.90 dT=-0.01, "
            "MCT=2000 MCS=2000 per temperature")
# dram__bytes_read.sum + dram__bytes_write.sum per launch of the pass kernel
# on the 128^3 lattice, from one ncu capture (cold-cache replay: every launch
# starts with the lattice outside L2; in the timed run it stays L2-resident)
NCU_DRAM_BYTES_128 = {
    "march": (25.19e6, "ncu capture of k_march<LL> on 128^3 (dram__bytes_read.sum + dram__bytes_write.sum, "
                       "cold-cache replay)"),
}


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


def host_cpu() -> str:
    """The host's CPU model (lscpu's "Model name", else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith(("model name", "cpu model")):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


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
            "cpu_model": host_cpu(),
            "sample": f"{n} sweeps of the {NX}^3 LL lattice at T=1.20 (reference EvolveN::Monte_Carlo_Step, "
                      f"8-colour OpenMP, test-only GSL shim RNG), {dt:.1f} s"}


def _port(cores):
    """The reference's sweep ported operation for operation (oracle/mcx_port.c),
    on a homogeneous 128^3 LL lattice, with one generator per host thread."""
    from oracle import oracle as O
    os.environ["OMP_NUM_THREADS"] = str(cores)  # before the oracle library's OpenMP runtime loads
    lat = O.Lattice(O.Model(nx=NX, ny=NY, nz=NZ))
    return O.Port(lat, seed=1, threads=cores)


def _cpu_port(seconds, cores):
    port = _port(cores)
    a = port.sweep(TI, 0.5)[1]
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds or n < 2:
        a = port.sweep(TI, a)[1]
        n += 1
    dt = time.perf_counter() - t0
    return {"value": n * SITES / dt, "unit": "site-updates/s", "cores": cores, "kind": "port",
            "cpu_model": host_cpu(),
            "sample": f"{n} sweeps of the {NX}^3 LL lattice at T=1.20 (C port of EvolveN::Monte_Carlo_Step: "
                      f"the reference's float/double arithmetic, 8-colour OpenMP loop and per-thread generators; "
                      f"bit-identical to the reference's own build on one thread, within 10% of its speed), "
                      f"{dt:.1f} s"}


def other_workloads():
    """Bounded runs of the configurations beside the headline anneal, each
    with what it reduces from the full configuration named."""
    from mcx import gain, workloads
    out = {}
    c3 = workloads.run_c3(replicas=256, sweeps=50, steps=3)
    out["c3"] = {"workload": "256 GHRL slab replicas, sides 16-64, homeotropic W=4, T in [0.8, 1.2], random ic",
                 "reduced": "3 blocks of 50 + 50 sweeps (the configuration runs 1000 + 1000)",
                 "site_updates_per_s": c3["site_updates_per_s"], "sweep_ms": c3["sweep_ms"],
                 "pass_kernel": c3["pass_kernel"], "roofline": c3["roofline"]}
    c5 = {}
    for prop in ("vmf_mlp", "plain"):
        r = workloads.run_c5(replicas=64, sweeps=20, proposal=prop)
        c5[prop] = {k: r[k] for k in ("site_updates_per_s", "active_site_updates_per_s", "acceptance",
                                      "pass_kernel", "seconds", "sweep_ms", "roofline") if k in r}
        if "train_loss" in r:
            c5[prop]["train_loss_first_last"] = r["train_loss"]
    out["c5"] = {"workload": "64 droplets r=40 in 96^3, GHRL p0=20, planar W=1, field E=0..2.0 by 0.1 at T=0.8",
                 "reduced": "20 + 20 sweeps per field value (the configuration runs 1000 + 1000)", **c5}
    g = gain.run(L=96, per_T=32, equil=3000, meas=4000, train_samples=1_000_000)
    rows = []
    for r in g["rows"]:
        p, lrn = r["plain"], r["vmf_mlp"]
        rows.append({"T": r["T"], "tau_plain": [p["tau_E"], p["tau_S"]], "tau_learned": [lrn["tau_E"], lrn["tau_S"]],
                     "acceptance": [p["acceptance"], lrn["acceptance"]],
                     "indep_samples_per_s": [p["indep_samples_per_s"], lrn["indep_samples_per_s"]],
                     "gain": r["gain"], "E_diff_sigma": r["E_diff_sigma"], "S_diff_sigma": r["S_diff_sigma"],
                     "tau_reliable": p["reliable"] and lrn["reliable"]})
    out["indep_samples"] = {
        "workload": "LL bulk 96^3 periodic, 32 replicas at each of T = 1.00, 1.10, 1.12, 1.15; learned vMF "
                    "proposal (19-64-64-4 BF16 MLP trained on 10^6 plain-sampler samples) vs plain Metropolis",
        "reduced": "3000 equilibration and 4000 measured sweeps per proposal (the full protocol: 6000 and 12000)",
        "metric": "replicas x sweeps/s / (2 max(tau_E, tau_S)), tau_int by Madras-Sokal windowing",
        "sweeps_per_s": g["sweeps_per_s"], "site_updates_per_s": g["site_updates_per_s"],
        "mlp_tflops": g["mlp_tflops"], "rows": rows,
        "gain_min": min(r["gain"] for r in rows), "parity_3sigma": g["parity_3sigma"]}
    return out


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
        port = _port(cores)
        a = 0.5
        for s in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            for _ in range(sample):
                a = port.sweep(TI, a)[1]
            if s >= args.warmup:
                times.append(time.perf_counter() - t0)
    per_step = float(np.mean(times))
    value = sample * SITES / per_step
    line = {
        "impl": "reference", "metric": "site-updates/s", "value": value, "unit": "site-updates/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "step": f"bounded sample: {sample} sweeps of the {NX}^3 lattice at T=1.20 "
                                                 f"(the same per-site-update metric as the headline's anneal block)"},
        "cpu_baseline": {"value": value, "unit": "site-updates/s", "cores": cores, "kind": kind,
                         "cpu_model": host_cpu(),
                         "sample": f"{sample} sweeps per step, all {cores} host threads"
                                   + ("" if use_ref else "; C port of the reference's sweep (bit-identical to its "
                                                         "own build on one thread, within 10% of its speed)")},
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
    ap.add_argument("--no-workloads", action="store_true",
                    help="skip the bounded runs of the other configurations (c3, c5, learned vs plain)")
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
    # DRAM bytes per launch cannot be counted inside the timed run; for the
    # headline lattice they come from one ncu capture of this kernel (and are
    # labelled so), for other shapes they are not reported
    traffic, traffic_src = None, "not measured for this lattice"
    if NX == 128 and R == 1 and args.proposal == "plain" and form in NCU_DRAM_BYTES_128:
        traffic, traffic_src = NCU_DRAM_BYTES_128[form]

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
    headline = NX == 128 and R == 1 and MCT == 2000 and args.proposal == "plain"
    extra = {}
    if headline and ws == 1 and not args.no_workloads:
        eng.close()
        extra = other_workloads()
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
                      "traffic": traffic, "traffic_source": traffic_src, "peak_source": peak_src,
                      "kernel": FORMS[form][0],
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
        **extra,
    }
    print(json.dumps(line), flush=True)
    eng.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
