"""The CPU baseline's port of the reference sweep (oracle/mcx_port.c) against
the reference's own build (oracle/_ref, compiled here from the reference's
sources; skipped where it is absent, as on the GPU host).

On one thread, fed by the same generator (the test-only GSL shim's splitmix64
seeded seed * 104729 + thread), the port reproduces the reference's sweeps bit
for bit -- directors and step size -- for every pair potential, a field, and
masked geometries with anchoring; and timed back to back on the same cores it
runs within 10% of the reference's speed, so a speed-up measured against the
port is the speed-up against the reference."""
import ctypes as C
import multiprocessing as mp
import os
import time

import numpy as np
import pytest

from oracle import oracle as O
from oracle import refproc

pytestmark = pytest.mark.skipif(not refproc.available(), reason="the reference's own build (oracle/_ref) is absent")

MODELS = {
    "ll_bulk": O.Model(nx=12, ny=10, nz=8, potential="ll", A=1.0),
    "ghrl_chiral_field": O.Model(nx=10, ny=8, nz=6, potential="ghrl", k11=1.0, k22=0.6, k33=1.4, p0=20, elecA=0.5,
                                 elecZ=1.0, elecE=1.5),
    "pear_bulk": O.Model(nx=8, ny=8, nz=8, potential="pear", A=1.0, B1=0.3, C=0.3),
    "ghrl_slab": O.Model(nx=10, ny=8, nz=7, geometry="slab", potential="ghrl", k11=1.0, k22=0.8, k33=1.2,
                         surfaces=[O.Surface("homeotropic", 4.0), O.Surface("fg_ghrl", 1.5)]),
    "ll_sphere_odd": O.Model(nx=11, ny=11, nz=11, geometry="sphere", potential="ll",
                             surfaces=[O.Surface("rp", 1.0, 60, 10)]),
}


def _ref_sweeps(md, ni, T, n, seed):
    os.environ["OMP_NUM_THREADS"] = "1"
    import ctypes as C2
    from oracle import refproc as rp
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    L = C2.CDLL(rp.REF_LIB_PATH)
    rp._setup(L, md)
    L.ref_seed.argtypes = [C2.c_ulong]
    L.ref_seed(seed)
    ni = ni.copy()
    a = C2.c_float(0.5)
    for _ in range(n):
        L.ref_sweep(ni.ctypes.data_as(C2.c_void_p), C2.c_float(T), C2.byref(a), None, 0, 1)
    return ni, a.value


@pytest.mark.parametrize("name", list(MODELS))
def test_port_reproduces_the_reference_bit_for_bit(name):
    m = MODELS[name]
    lat = O.Lattice(m)
    ni0 = O.random_directors(m.n, np.random.default_rng(4)).astype(np.float32)
    ni0[lat.pt == 0] = (0, 0, 1)
    with mp.get_context("spawn").Pool(1) as pool:
        want, a_want = pool.apply(_ref_sweeps, (refproc.model_dict(m), ni0, 0.9, 5, 7))
    lat.ni[:] = ni0
    port = O.Port(lat, seed=7, threads=1)
    a = 0.5
    for _ in range(5):
        _, a = port.sweep(0.9, a)
    assert np.array_equal(lat.ni, want)
    assert np.float32(a) == np.float32(a_want)


def _time_ref(side, threads, seconds, q):
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import ctypes as C2
    from oracle import refproc as rp
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    m = O.Model(nx=side, ny=side, nz=side)
    L = C2.CDLL(rp.REF_LIB_PATH)
    rp._setup(L, rp.model_dict(m))
    ni = np.zeros((m.n, 3), np.float32)
    ni[:, 2] = 1
    L.ref_set_state(ni.ctypes.data_as(C2.c_void_p))
    L.ref_sweeps_inplace.restype = C2.c_float
    L.ref_sweeps_inplace(1, C2.c_float(1.2), C2.c_float(0.5), threads)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        L.ref_sweeps_inplace(1, C2.c_float(1.2), C2.c_float(0.5), threads)
        n += 1
    q.put(n * m.n / (time.perf_counter() - t0))


def _time_port(side, threads, seconds, q):
    os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle import oracle as O2
    lat = O2.Lattice(O2.Model(nx=side, ny=side, nz=side))
    port = O2.Port(lat, seed=1, threads=threads)
    a = port.sweep(1.2, 0.5)[1]
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        a = port.sweep(1.2, a)[1]
        n += 1
    q.put(n * lat.model.n / (time.perf_counter() - t0))


def test_port_runs_at_the_reference_speed():
    """Best of five alternating rounds each, one thread, a 64^3 LL lattice
    (the best round filters out time the host spent on other work)."""
    ctx = mp.get_context("spawn")
    rates = {"ref": [], "port": []}
    for _ in range(5):
        for key, fn in (("ref", _time_ref), ("port", _time_port)):
            q = ctx.Queue()
            p = ctx.Process(target=fn, args=(64, 1, 1.5, q))
            p.start()
            rates[key].append(q.get(timeout=120))
            p.join()
    ratio = np.max(rates["port"]) / np.max(rates["ref"])
    assert 0.9 <= ratio <= 1.1, (ratio, rates)
