"""Python bindings for the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a plain-C FP64 restatement of the McLiCS Metropolis hot path
(oracle/mcx_oracle.c).  Only the tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module: it is the checker, never
the thing measured or shipped.

Layout is the reference's natural AoS: site s = i + Nx*(j + Ny*k), director
``ni[s, 0:3]`` (include/define.h:10-12).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmcx_oracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libref_mcx.so")

POT = {"ll": 0, "lebwohl-lahser": 0, "ghrl": 1, "grun-hess": 1, "pear": 2}
GEO = {"bulk": 0, "slab": 1, "sphere": 2, "custom": 3}
BOUND = {"free": 0, "periodic": 1}
ANCH = {
    "homeotropic": 0,
    "fg": 1,
    "rp": 2,
    "strong": 3,
    "homeotropic_ghrl": 4,
    "fg_ghrl": 5,
    "rp_ghrl": 6,
    "strong_ghrl": 7,
}
ORDER = {"redblack": 0, "eight": 1}
F_NO_NORMALIZE = 1
F_PARALLEL = 2
MAX_SURF = 16


class _Params(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("xb", C.c_int), ("yb", C.c_int), ("zb", C.c_int),
        ("potential", C.c_int),
        ("A", C.c_double),
        ("lam", C.c_double), ("mu", C.c_double), ("nu", C.c_double), ("rho", C.c_double), ("sigma", C.c_double),
        ("elecA", C.c_double), ("elecE", C.c_double), ("ex", C.c_double), ("ey", C.c_double), ("ez", C.c_double),
        ("nsurf", C.c_int),
        ("anch", C.c_int * MAX_SURF),
        ("W", C.c_double * MAX_SURF),
        ("dir", (C.c_double * 3) * MAX_SURF),
        ("B1", C.c_double), ("C", C.c_double),
    ]


class _Trace(C.Structure):
    _fields_ = [("dE", C.c_void_p), ("scale", C.c_void_p), ("acc", C.c_void_p), ("tie", C.c_void_p),
                ("visited", C.c_void_p)]


def ghrl_constants(k11: float, k22: float, k33: float, p0: float):
    """setGHRL (src/io.cpp:277-302) with the reference's float/double rounding.

    Returns (lambda, mu, nu, rho, sigma) as float32 values."""
    f = np.float32
    k11, k22, k33, p0 = f(k11), f(k22), f(k33), f(p0)
    den = f(f(k11 - f(f(3) * k22)) - k33)
    scale = f(abs(9.0 / float(den)))
    if p0 != 0:
        sigma = f(float(f(-scale * k22)) * (2 * np.pi / float(p0)))
    else:
        sigma = f(0)
    s9 = f(scale / f(9))
    lam = f(s9 * f(f(f(f(2) * k11) - f(f(3) * k22)) + k33))
    mu = f(scale * f(k22 - k11))
    rho = f(s9 * f(k11 - k33))
    nu = f(s9 * f(f(k11 - f(f(3) * k22)) - k33))
    return lam, mu, nu, rho, sigma


def angles_to_dir(theta_deg: float, phi_deg: float):
    """Anchoring easy axis from (theta_s, phi_s) in degrees
    (src/anchoring_rp.cpp:43-45)."""
    t = np.float32(np.pi / 180)
    th = float(np.float32(t * np.float32(theta_deg)))
    ph = float(np.float32(t * np.float32(phi_deg)))
    return (float(np.float32(np.cos(ph) * np.sin(th))), float(np.float32(np.sin(ph) * np.sin(th))),
            float(np.float32(np.cos(th))))


@dataclass
class Surface:
    anchoring: str = "homeotropic"
    W: float = 1.0
    theta_s: float = 0.0
    phi_s: float = 0.0


@dataclass
class Model:
    """One lattice's physics, named after the reference's parameter keys."""
    nx: int = 16
    ny: int = 16
    nz: int = 16
    geometry: str = "bulk"
    xbound: str = "periodic"
    ybound: str = "periodic"
    zbound: str = "periodic"
    potential: str = "ll"
    A: float = 1.0
    k11: float = 1.0
    k22: float = 1.0
    k33: float = 1.0
    p0: float = 0.0
    elecA: float = 0.0
    elecX: float = 0.0
    elecY: float = 0.0
    elecZ: float = 0.0
    elecE: float = 1.0
    surfaces: List[Surface] = field(default_factory=list)
    radius: float = 0.0
    B1: float = 0.04  # Pear potential (include/parameters.h:34-36 defaults)
    C: float = 0.3

    @property
    def n(self) -> int:
        return self.nx * self.ny * self.nz

    def effective_bounds(self):
        """Slab forces z free (src/geometry_slab.cpp:23); sphere forces all
        three free (src/geometry_sphere.cpp:19-21)."""
        xb, yb, zb = self.xbound, self.ybound, self.zbound
        if self.geometry == "slab":
            zb = "free"
        if self.geometry == "sphere":
            xb = yb = zb = "free"
        return xb, yb, zb

    def cparams(self) -> _Params:
        p = _Params()
        p.nx, p.ny, p.nz = self.nx, self.ny, self.nz
        xb, yb, zb = self.effective_bounds()
        p.xb, p.yb, p.zb = BOUND[xb], BOUND[yb], BOUND[zb]
        p.potential = POT[self.potential]
        p.A = float(np.float32(self.A))
        if p.potential == 1:
            lam, mu, nu, rho, sigma = ghrl_constants(self.k11, self.k22, self.k33, self.p0)
        else:
            lam, mu, nu, rho, sigma = 0.0, 0.0, 1.0, 0.0, 0.0
        p.lam, p.mu, p.nu, p.rho, p.sigma = float(lam), float(mu), float(nu), float(rho), float(sigma)
        f = lambda v: float(np.float32(v))
        p.elecA, p.elecE, p.ex, p.ey, p.ez = f(self.elecA), f(self.elecE), f(self.elecX), f(self.elecY), f(self.elecZ)
        p.B1, p.C = f(self.B1), f(self.C)
        p.nsurf = len(self.surfaces)
        for i, s in enumerate(self.surfaces):
            p.anch[i] = ANCH[s.anchoring.lower()]
            p.W[i] = f(s.W)
            d = angles_to_dir(s.theta_s, s.phi_s)
            for c in range(3):
                p.dir[i][c] = d[c]
        return p


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P, D, F, I, V = C.POINTER(_Params), C.c_double, C.c_float, C.c_int, C.c_void_p
        L.orc_philox.argtypes = [V, V, V]
        L.orc_site_uniforms.argtypes = [I, I, C.c_long, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, V]
        L.orc_pair.argtypes = [P, V, V, I, V]
        L.orc_pair.restype = D
        L.orc_surface.argtypes = [P, I, V, V, V]
        L.orc_surface.restype = D
        L.orc_field.argtypes = [P, V]
        L.orc_field.restype = D
        L.orc_local_energy.argtypes = [P, V, V, V, C.c_long, V, V]
        L.orc_local_energy.restype = D
        L.orc_pass.argtypes = [P, V, V, V, F, F, C.c_uint32, C.c_uint32, C.c_uint64, I, I, I, D, V,
                               C.POINTER(_Trace)]
        L.orc_pass.restype = C.c_long
        L.orc_propose.argtypes = [V, D, D, F, I, V]
        L.orc_adapt.argtypes = [F, C.c_long, C.c_long]
        L.orc_adapt.restype = F
        L.orc_sweep.argtypes = [P, V, V, V, F, C.POINTER(F), C.c_uint32, C.c_uint32, C.c_uint64, I, I]
        L.orc_sweep.restype = C.c_long
        L.orc_eigmax.argtypes = [V, V]
        L.orc_eigmax.restype = D
        L.orc_measure.argtypes = [P, V, V, V, V]
        L.orc_geometry.argtypes = [I, I, I, I, F, V, V]
        L.orc_count_valid.argtypes = [P, V]
        L.orc_count_valid.restype = C.c_long
        L.orc_port_rngs.argtypes = [C.c_ulong, I]
        L.orc_port_rngs.restype = V
        L.orc_port_sweep.argtypes = [P, V, V, V, F, C.POINTER(F), C.c_long, V, I, V]
        L.orc_port_sweep.restype = C.c_long
        _lib = L
    return _lib


def build():
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def philox(ctr: Sequence[int], key: Sequence[int]) -> np.ndarray:
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox(_ptr(c), _ptr(k), _ptr(out))
    return out


class Port:
    """The reference's CPU sweep ported operation for operation (mcx_port.c:
    EvolveN::Monte_Carlo_Step with its float / double arithmetic, 8-colour
    OpenMP loop and per-thread generators), on a Lattice's field: the CPU
    baseline where the reference's own build is absent."""

    def __init__(self, lat: "Lattice", seed: int = 1, threads: int = 1):
        import atexit
        self.lat = lat
        self.threads = max(1, int(threads))
        self._rngs = lib().orc_port_rngs(seed, self.threads)
        self._scratch = np.zeros_like(lat.ni)
        self.valid = lib().orc_count_valid(C.byref(lat.p), _ptr(lat.pt))
        libc = C.CDLL(None)
        libc.free.argtypes = [C.c_void_p]
        atexit.register(libc.free, self._rngs)

    def sweep(self, T: float, ang_var: float):
        a = C.c_float(ang_var)
        L = self.lat
        acc = lib().orc_port_sweep(C.byref(L.p), _ptr(L.ni), _ptr(L.pt), _ptr(L.ns), T, C.byref(a), self.valid,
                                   self._rngs, self.threads, _ptr(self._scratch))
        return acc, a.value


class Lattice:
    """A director field plus its mask for one Model, on the CPU."""

    def __init__(self, model: Model, ni: Optional[np.ndarray] = None, pt: Optional[np.ndarray] = None,
                 ns: Optional[np.ndarray] = None):
        self.model = model
        self.p = model.cparams()
        n = model.n
        if pt is None:
            pt = np.zeros(n, dtype=np.int32)
            ns = np.zeros((n, 3), dtype=np.float32)
            lib().orc_geometry(model.nx, model.ny, model.nz, GEO[model.geometry], float(model.radius), _ptr(pt),
                               _ptr(ns))
        self.pt = np.ascontiguousarray(pt, dtype=np.int32)
        self.ns = np.ascontiguousarray(ns if ns is not None else np.zeros((n, 3)), dtype=np.float32).reshape(n, 3)
        if ni is None:
            ni = np.zeros((n, 3), dtype=np.float32)
            ni[:, 2] = 1
        self.ni = np.ascontiguousarray(ni, dtype=np.float32).reshape(n, 3)

    @property
    def valid(self) -> int:
        return int((self.pt != 0).sum())

    def pair(self, a, b, d: int) -> float:
        a = np.asarray(a, np.float64)
        b = np.asarray(b, np.float64)
        return lib().orc_pair(C.byref(self.p), _ptr(a), _ptr(b), d, None)

    def surface(self, sid: int, n, s) -> float:
        n = np.asarray(n, np.float64)
        s = np.asarray(s, np.float64)
        return lib().orc_surface(C.byref(self.p), sid, _ptr(n), _ptr(s), None)

    def field(self, n) -> float:
        n = np.asarray(n, np.float64)
        return lib().orc_field(C.byref(self.p), _ptr(n))

    def local_energy(self, s: int, n=None) -> float:
        return self.local_energy_abs(s, n)[0]

    def local_energy_abs(self, s: int, n=None):
        """(E_local, sum of |terms|) of site s with director n (FP64)."""
        if n is None:
            n = self.ni[s]
        n = np.asarray(n, np.float64)
        a = C.c_double()
        e = lib().orc_local_energy(C.byref(self.p), _ptr(self.ni), _ptr(self.pt), _ptr(self.ns), s, _ptr(n),
                                   C.byref(a))
        return e, a.value

    def run_pass(self, T: float, ang_var: float, seed: int, stream: int, sweep: int, order: str, pass_: int,
                 flags: int = 0, tie_eps: float = 1e-5, feed: Optional[np.ndarray] = None, trace: bool = False):
        n = self.model.n
        tr = None
        bufs = None
        if trace:
            bufs = dict(dE=np.zeros(n), scale=np.zeros(n), acc=np.zeros(n, np.uint8), tie=np.zeros(n, np.uint8),
                        visited=np.zeros(n, np.uint8))
            tr = _Trace(*[b.ctypes.data for b in bufs.values()])
        f = None
        if feed is not None:
            feed = np.ascontiguousarray(feed, dtype=np.float64)
            f = _ptr(feed)
        acc = lib().orc_pass(C.byref(self.p), _ptr(self.ni), _ptr(self.pt), _ptr(self.ns), T, ang_var, seed, stream,
                             sweep, ORDER[order], pass_, flags, tie_eps, f, C.byref(tr) if tr is not None else None)
        return acc, bufs

    def sweep(self, T: float, ang_var: float, seed: int, stream: int, sweep: int, order: str = "redblack",
              flags: int = 0):
        a = C.c_float(ang_var)
        acc = lib().orc_sweep(C.byref(self.p), _ptr(self.ni), _ptr(self.pt), _ptr(self.ns), T, C.byref(a), seed,
                              stream, sweep, ORDER[order], flags)
        return acc, a.value

    def measure(self) -> dict:
        out = np.zeros(16)
        lib().orc_measure(C.byref(self.p), _ptr(self.ni), _ptr(self.pt), _ptr(self.ns), _ptr(out))
        return dict(E=out[0], E_valid=out[1], Q=out[2:11].reshape(3, 3), S=out[11], director=out[12:15],
                    valid=int(out[15]))


def propose(n, u0: float, u1: float, ang_var: float, flags: int = 0) -> np.ndarray:
    """The rotated proposal of src/evolve.cpp:136-152 in FP64 (renormalised
    unless F_NO_NORMALIZE)."""
    n = np.ascontiguousarray(n, np.float32)
    out = np.zeros(3)
    lib().orc_propose(_ptr(n), u0, u1, ang_var, flags, _ptr(out))
    return out


def site_uniforms(model_or_nx, ny_or_site, *args, tag: int = 0) -> np.ndarray:
    """The (u0, u1, u2) a site update draws: site_uniforms(model, site, seed,
    stream, sweep) or site_uniforms(nx, ny, site, seed, stream, sweep)."""
    if isinstance(model_or_nx, Model):
        nx, ny, site = model_or_nx.nx, model_or_nx.ny, ny_or_site
        seed, stream, sweep = args
    else:
        nx, ny = model_or_nx, ny_or_site
        site, seed, stream, sweep = args
    u = np.zeros(3)
    lib().orc_site_uniforms(nx, ny, int(site), seed, stream, sweep, tag, _ptr(u))
    return u


def adapt(ang_var: float, acc: int, valid: int) -> float:
    return lib().orc_adapt(ang_var, acc, valid)


def eigmax(Q) -> tuple:
    q = np.ascontiguousarray(Q, dtype=np.float64).reshape(9)
    v = np.zeros(3)
    lam = lib().orc_eigmax(_ptr(q), _ptr(v))
    return lam, v


def local_order(ni: np.ndarray, pt: np.ndarray, m: Model) -> np.ndarray:
    """The local order parameter of the reference's snapshots
    (lattice_order_parameter, src/parameter_order.cpp:62-113) at every site:
    Q = sum (3 n n^T - I) / (2 points) over the site and its six neighbours
    that exist (bounds) and are active, largest eigenvalue; FP64.  NaN at
    inactive sites (the reference evaluates only active ones)."""
    nx, ny, nz = m.nx, m.ny, m.nz
    N = [nx, ny, nz]
    B = list(m.effective_bounds())
    out = np.full(m.n, np.nan)
    for s in np.nonzero(pt)[0]:
        i, j, k = s % nx, (s // nx) % ny, s // (nx * ny)
        Q = np.zeros((3, 3))
        pts = 0
        for d in ((0, 0, 0), (-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)):
            c = [i + d[0], j + d[1], k + d[2]]
            ok = True
            for ax in range(3):
                if c[ax] < 0 or c[ax] >= N[ax]:
                    if B[ax] == "periodic":
                        c[ax] %= N[ax]
                    else:
                        ok = False
            if not ok:
                continue
            t = c[0] + nx * (c[1] + ny * c[2])
            if pt[t] == 0:
                continue
            n = ni[t].astype(np.float64)
            Q += 3 * np.outer(n, n) - np.eye(3)
            pts += 1
        out[s] = np.linalg.eigvalsh(Q / (2 * pts))[-1]
    return out


def random_directors(n: int, rng: np.random.Generator) -> np.ndarray:
    """Uniform on the sphere (z uniform in [-1,1], azimuth uniform)."""
    z = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    r = np.sqrt(1 - z * z)
    return np.stack([r * np.cos(ph), r * np.sin(ph), z], axis=1).astype(np.float32)


def u24(x: np.ndarray) -> np.ndarray:
    return (np.asarray(x, np.uint32) >> 8).astype(np.float64) / 16777216.0


def sweep_uniforms(model: Model, pt: np.ndarray, seed: int, stream: int, sweep: int, order: str = "eight",
                   tag: int = 0) -> np.ndarray:
    """The (u0, u1, u2) triples the oracle draws for one sweep, in the order
    the sites are visited (pass by pass, natural index order within a pass,
    inactive sites skipped) -- the order in which the reference's
    single-threaded Monte_Carlo_Step consumes uniforms (src/evolve.cpp:89-167)."""
    nx, ny, nz = model.nx, model.ny, model.nz
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    s = i + nx * (j + ny * k)
    out = []
    npass = 8 if order == "eight" else 2
    for q in range(npass):
        if order == "eight":
            m = ((i & 1) == (q & 1)) & ((j & 1) == ((q >> 1) & 1)) & ((k & 1) == (q >> 2))
        else:
            m = ((i + j + k) & 1) == q
        m &= pt[s] != 0
        for site in s[m]:
            out.append(site_uniforms(nx, ny, int(site), seed, stream, sweep, tag=tag))
    return np.array(out, dtype=np.float64).reshape(-1)


def field_sweep(model: Model, T: float, fields: Sequence[float], mct: int, mcs: int, seed: int, stream: int,
                ni0: np.ndarray, order: str = "redblack") -> np.ndarray:
    """electricEvolveN::run (src/evolve_electric.cpp:28-90) on the oracle: at
    temperature T, per field value mct sweeps, then mcs sweeps each followed
    by E and S; the step size (starting at 0.5) carries across field values.
    Returns rows (E_field, mean S, mean E)."""
    lat = Lattice(model)
    lat.ni[:] = ni0
    a = np.float32(0.5)
    sw = 0
    rows = []
    for Ef in fields:
        lat.p.elecE = float(np.float32(Ef))
        for _ in range(mct):
            _, a = lat.sweep(T, a, seed, stream, sw, order)
            sw += 1
        S1 = E1 = 0.0
        for _ in range(mcs):
            _, a = lat.sweep(T, a, seed, stream, sw, order)
            sw += 1
            r = lat.measure()
            S1 += r["S"]
            E1 += r["E"]
        rows.append((Ef, S1 / mcs, E1 / mcs))
    return np.array(rows)


def anneal(model: Model, temps: Sequence[float], mct: int, mcs: int, seed: int, stream: int, ni0: np.ndarray,
           order: str = "redblack") -> np.ndarray:
    """thermalEvolveN::run (src/evolve_thermal.cpp:30-99) on the oracle: per
    temperature mct sweeps, then mcs sweeps each followed by E and S; the
    step size (starting at 0.5) carries across temperatures.  Returns rows
    (T, mean S, mean E)."""
    lat = Lattice(model)
    lat.ni[:] = ni0
    a = np.float32(0.5)
    sw = 0
    rows = []
    for T in temps:
        for _ in range(mct):
            _, a = lat.sweep(T, a, seed, stream, sw, order)
            sw += 1
        S1 = E1 = 0.0
        for _ in range(mcs):
            _, a = lat.sweep(T, a, seed, stream, sw, order)
            sw += 1
            r = lat.measure()
            S1 += r["S"]
            E1 += r["E"]
        rows.append((T, S1 / mcs, E1 / mcs))
    return np.array(rows)
