"""Runs the reference's own compiled C++ (oracle/_ref/libref_mcx.so) in a fresh
process (TEST INFRASTRUCTURE ONLY).

The reference keeps lattice-sized state in function-local statics
(src/evolve.cpp:28,66-68; src/parameter_order.cpp:31-33), so each model gets
its own spawned process.  ``available()`` is False where the reference tree
was not present at build time (the GPU host), and callers skip.
"""
from __future__ import annotations

import ctypes as C
import multiprocessing as mp
import os
from typing import Any, List, Sequence

import numpy as np

from oracle.oracle import REF_LIB_PATH, Model


def available() -> bool:
    return os.path.exists(REF_LIB_PATH)


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _setup(L, m: dict):
    V = C.c_void_p
    L.ref_setup.restype = C.c_int
    L.ref_pair.restype = C.c_float
    L.ref_surface.restype = C.c_float
    L.ref_field.restype = C.c_float
    L.ref_local_energy.restype = C.c_float
    L.ref_local_energy.argtypes = [V, C.c_long, V]
    L.ref_sweep.restype = C.c_long
    L.ref_sweep.argtypes = [V, C.c_float, C.POINTER(C.c_float), V, C.c_long, C.c_int]
    L.ref_energy.restype = C.c_float
    L.ref_order.restype = C.c_float
    L.ref_sweeps_inplace.restype = C.c_float
    L.ref_sweeps_inplace.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int]
    surfs = m["surfaces"]
    ns = len(surfs)
    anch = (C.c_char_p * max(ns, 1))(*[s["anchoring"].encode() for s in surfs])
    W = np.array([s["W"] for s in surfs] + [0], np.float32)
    th = np.array([s["theta_s"] for s in surfs] + [0], np.float32)
    ph = np.array([s["phi_s"] for s in surfs] + [0], np.float32)
    f = C.c_float
    rc = L.ref_setup(m["nx"], m["ny"], m["nz"], m["geometry"].encode(), m["xbound"].encode(), m["ybound"].encode(),
                     m["zbound"].encode(), m["potential"].encode(), f(m["A"]), f(m["k11"]), f(m["k22"]), f(m["k33"]),
                     f(m["p0"]), f(m["elecA"]), f(m["elecX"]), f(m["elecY"]), f(m["elecZ"]), f(m["elecE"]), ns, anch,
                     _p(W), _p(th), _p(ph), m.get("bound_file", b"").encode() if m.get("bound_file") else None)
    if rc != 0:
        raise RuntimeError("ref_setup failed")
    if m["potential"] == "pear":
        L.ref_set_pear.argtypes = [C.c_float, C.c_float]
        L.ref_set_pear(f(m["B1"]), f(m["C"]))


def _active(L, n: int) -> np.ndarray:
    pt = np.zeros(n, np.int32)
    ns = np.zeros((n, 3), np.float32)
    L.ref_get_mask(_p(pt), _p(ns))
    return pt != 0


def _length_drift(ni: np.ndarray, act: np.ndarray) -> float:
    """Mean of |n|^2 - 1 over the active sites: the reference's CPU sweep
    does not renormalise its proposals (src/evolve.cpp:139-151), so director
    lengths drift by float rounding, and E and S with them."""
    v = ni.reshape(-1, 3)[act].astype(np.float64)
    return float(np.mean(np.sum(v * v, axis=1) - 1.0))


def _worker(m: dict, ops: List[tuple]) -> List[Any]:
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)  # the reference prints its setup banner to stdout
    L = C.CDLL(REF_LIB_PATH)
    _setup(L, m)
    n = m["nx"] * m["ny"] * m["nz"]
    out = []
    for op in ops:
        kind = op[0]
        if kind == "mask":
            pt = np.zeros(n, np.int32)
            ns = np.zeros((n, 3), np.float32)
            L.ref_get_mask(_p(pt), _p(ns))
            out.append((pt, ns))
        elif kind == "ghrl":
            g = np.zeros(5, np.float32)
            L.ref_get_ghrl(_p(g))
            out.append(g)
        elif kind == "pairs":
            a, b, r = [np.ascontiguousarray(x, np.float32) for x in op[1:4]]
            out.append(np.array([L.ref_pair(_p(a[q]), _p(b[q]), _p(r[q])) for q in range(len(a))], np.float32))
        elif kind == "surface":
            sid = op[1]
            a, s = [np.ascontiguousarray(x, np.float32) for x in op[2:4]]
            out.append(np.array([L.ref_surface(sid, _p(a[q]), _p(s[q])) for q in range(len(a))], np.float32))
        elif kind == "field":
            a = np.ascontiguousarray(op[1], np.float32)
            out.append(np.array([L.ref_field(_p(a[q])) for q in range(len(a))], np.float32))
        elif kind == "local":
            fld = np.ascontiguousarray(op[1], np.float32)
            sites = op[2]
            nn = np.ascontiguousarray(op[3], np.float32)
            out.append(np.array([L.ref_local_energy(_p(fld), int(sites[q]), _p(nn[q])) for q in range(len(sites))],
                                np.float32))
        elif kind == "sweep":
            ni = np.ascontiguousarray(op[1], np.float32).copy()
            T, a = op[2], C.c_float(op[3])
            feed = op[4]
            if feed is not None:
                feed = np.ascontiguousarray(feed, np.float64)
                used = L.ref_sweep(_p(ni), T, C.byref(a), _p(feed), len(feed), 1)
            else:
                used = L.ref_sweep(_p(ni), T, C.byref(a), None, 0, op[5] if len(op) > 5 else 0)
            out.append((ni, a.value, used))
        elif kind == "local_order":
            ni = np.ascontiguousarray(op[1], np.float32)
            S = np.zeros(n, np.float32)
            L.ref_local_order.argtypes = [C.c_void_p, C.c_void_p]
            L.ref_local_order(_p(ni), _p(S))
            out.append(S)
        elif kind == "print_n":
            ni = np.ascontiguousarray(op[1], np.float32)
            L.ref_print_n.argtypes = [C.c_void_p, C.c_char_p]
            if L.ref_print_n(_p(ni), op[2].encode()) != 0:
                raise RuntimeError("print_n failed")
            with open(op[2]) as f:
                out.append(f.read())
        elif kind == "energy":
            ni = np.ascontiguousarray(op[1], np.float32)
            out.append(float(L.ref_energy(_p(ni))))
        elif kind == "anneal":
            # thermalEvolveN::run (src/evolve_thermal.cpp:30-99): per temperature
            # MCT sweeps, then MCS sweeps each followed by energy_calculator and
            # the order parameter; the step size carries across temperatures.
            ni = np.ascontiguousarray(op[1], np.float32).copy()
            temps, mct, mcs, seed, nth = op[2], op[3], op[4], op[5], op[6]
            L.ref_seed.argtypes = [C.c_ulong]
            L.ref_seed(seed)
            a = C.c_float(0.5)
            rows = []
            Q = np.zeros(9, np.float32)
            v = np.zeros(3, np.float32)
            act = _active(L, n)
            for T in temps:
                for _ in range(mct):
                    L.ref_sweep(_p(ni), C.c_float(T), C.byref(a), None, 0, nth)
                S1 = E1 = 0.0
                for _ in range(mcs):
                    L.ref_sweep(_p(ni), C.c_float(T), C.byref(a), None, 0, nth)
                    E1 += float(L.ref_energy(_p(ni)))
                    S1 += float(L.ref_order(_p(ni), _p(Q), _p(v)))
                rows.append((T, S1 / mcs, E1 / mcs, _length_drift(ni, act)))
            out.append(np.array(rows))
        elif kind == "field_sweep":
            # electricEvolveN::run (src/evolve_electric.cpp:28-90): at T = Ti, per
            # field value MCT sweeps, then MCS sweeps each followed by
            # energy_calculator and the order parameter; the step size carries.
            ni = np.ascontiguousarray(op[1], np.float32).copy()
            T, fields, mct, mcs, seed, nth = op[2], op[3], op[4], op[5], op[6], op[7]
            L.ref_seed.argtypes = [C.c_ulong]
            L.ref_seed(seed)
            L.ref_set_field.argtypes = [C.c_float]
            a = C.c_float(0.5)
            rows = []
            Q = np.zeros(9, np.float32)
            v = np.zeros(3, np.float32)
            act = _active(L, n)
            for Ef in fields:
                L.ref_set_field(C.c_float(Ef))
                for _ in range(mct):
                    L.ref_sweep(_p(ni), C.c_float(T), C.byref(a), None, 0, nth)
                S1 = E1 = 0.0
                for _ in range(mcs):
                    L.ref_sweep(_p(ni), C.c_float(T), C.byref(a), None, 0, nth)
                    E1 += float(L.ref_energy(_p(ni)))
                    S1 += float(L.ref_order(_p(ni), _p(Q), _p(v)))
                rows.append((Ef, S1 / mcs, E1 / mcs, _length_drift(ni, act)))
            out.append(np.array(rows))
        elif kind == "order":
            ni = np.ascontiguousarray(op[1], np.float32)
            Q = np.zeros(9, np.float32)
            v = np.zeros(3, np.float32)
            S = L.ref_order(_p(ni), _p(Q), _p(v))
            out.append((float(S), Q.reshape(3, 3), v))
        else:
            raise ValueError(kind)
    return out


def model_dict(model: Model) -> dict:
    d = dict(model.__dict__)
    d["surfaces"] = [dict(s.__dict__) for s in model.surfaces]
    return d


def pool_run(md: dict, ops: Sequence[tuple], timeout: float = 300.0) -> List[Any]:
    ctx = mp.get_context("spawn")
    with ctx.Pool(1) as pool:
        return pool.apply_async(_worker, (md, list(ops))).get(timeout)


def run(model: Model, ops: Sequence[tuple], timeout: float = 300.0) -> List[Any]:
    """Set up `model` in a fresh process with the reference's own code and run
    the ops (see _worker) there."""
    return pool_run(model_dict(model), ops, timeout)
