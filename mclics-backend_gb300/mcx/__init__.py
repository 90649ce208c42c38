"""Python host interface to the GB300 Metropolis engine for the McLiCS
nematic lattice model: ctypes over the C ABI in include/mcx.h
(_build/libmcx.so).

The engine runs only on the GPU: importing works anywhere, but creating an
Engine needs the compiled library and a CUDA device, and fails loudly
otherwise -- there is no CPU fallback.

Names follow the reference's parameter keys (include/parameters.h:11-83);
directors cross the boundary in the reference's AoS layout
ni[(i + Nx*(j + Ny*k)), 0:3] (include/define.h:10-12).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, Iterable, List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.environ.get("MCX_LIB") or os.path.join(PKG, "_build", "libmcx.so")
CLI_PATH = os.path.join(PKG, "_build", "mc_sim_gb300")

MAX_SURFACES = 16
POTENTIALS = {"ll": 0, "lebwohl-lahser": 0, "ghrl": 1, "grun-hess": 1, "pear": 2}
GEOMETRIES = {"bulk": 0, "slab": 1, "sphere": 2, "custom": 3}
BOUNDS = {"free": 0, "periodic": 1}
ANCHORINGS = {"homeotropic": 0, "fg": 1, "rp": 2, "strong": 3, "homeotropic_ghrl": 4, "fg_ghrl": 5, "rp_ghrl": 6,
              "strong_ghrl": 7}
PROPOSALS = {"plain": 0, "vmf_mlp": 1}
PASSES = {"march": 0, "direct": 1, "staged": 2, "march_tma": 3, "march_async": 4, "march_persistent": 5,
          "march_quad": 6}
MLP_PARAMS = 6792
SAMPLE_FLOATS = 24
AUG_FLIP, AUG_ROTATE = 1, 2
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "unsupported", 5: "I/O error",
          6: "parse error"}

# mcx_measure / mcx_get_stats layouts
M_E, M_E_VALID, M_Q, M_S, M_DIRECTOR, M_VALID = 0, 1, 2, 11, 12, 15
ST_N, ST_S1, ST_S2, ST_E1, ST_E2, ST_EV1, ST_EV2, ST_ACC, ST_SWEEPS, ST_LAST_E, ST_LAST_S, ST_ANG_VAR, ST_SWEEP_INDEX = \
    range(13)
# mcx_combine_stats layout
CB_T, CB_S, CB_VAR_S, CB_E, CB_VAR_E, CB_P, CB_N, CB_T_SPREAD = range(8)
COMBINED_LEN = 8


class McxError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"mcx: {STATUS.get(status, status)}: {msg}")
        self.status = status


class ReplicaDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("geometry", C.c_int),
        ("xbound", C.c_int), ("ybound", C.c_int), ("zbound", C.c_int),
        ("potential", C.c_int),
        ("A", C.c_float),
        ("k11", C.c_float), ("k22", C.c_float), ("k33", C.c_float), ("p0", C.c_float),
        ("elecA", C.c_float), ("elecX", C.c_float), ("elecY", C.c_float), ("elecZ", C.c_float), ("elecE", C.c_float),
        ("T", C.c_float),
        ("ang_var", C.c_float),
        ("seed", C.c_uint), ("stream", C.c_uint),
        ("n_surfaces", C.c_int),
        ("anchoring", C.c_int * MAX_SURFACES),
        ("W", C.c_float * MAX_SURFACES),
        ("theta_s", C.c_float * MAX_SURFACES),
        ("phi_s", C.c_float * MAX_SURFACES),
        ("radius", C.c_float),
        ("B1", C.c_float), ("C", C.c_float),
    ]


class TrainConfig(C.Structure):
    """mcx_train_config of include/mcx.h."""
    _fields_ = [("samples", C.c_int), ("batch", C.c_int), ("steps", C.c_int), ("lr", C.c_float),
                ("seed", C.c_uint), ("augment", C.c_int)]


def replica(nx=16, ny=16, nz=16, geometry="bulk", xbound="periodic", ybound="periodic", zbound="periodic",
            potential="ll", A=1.0, k11=1.0, k22=1.0, k33=1.0, p0=0.0, elecA=0.0, elecX=0.0, elecY=0.0, elecZ=0.0,
            elecE=1.0, T=1.0, ang_var=0.5, seed=1, stream=0, surfaces: Sequence[dict] = (), radius=0.0,
            B1=0.04, C=0.3) -> ReplicaDesc:
    """A replica descriptor from the reference's parameter names.  `surfaces`
    is a list of dicts with keys anchoring, W, theta_s, phi_s (surface id =
    list index = pt - 2)."""
    d = ReplicaDesc()
    d.nx, d.ny, d.nz = nx, ny, nz
    d.geometry = GEOMETRIES[geometry.lower()]
    d.xbound, d.ybound, d.zbound = BOUNDS[xbound.lower()], BOUNDS[ybound.lower()], BOUNDS[zbound.lower()]
    d.potential = POTENTIALS[potential.lower()]
    d.A, d.k11, d.k22, d.k33, d.p0 = A, k11, k22, k33, p0
    d.elecA, d.elecX, d.elecY, d.elecZ, d.elecE = elecA, elecX, elecY, elecZ, elecE
    d.T, d.ang_var, d.seed, d.stream = T, ang_var, seed, stream
    d.n_surfaces = len(surfaces)
    for i, s in enumerate(surfaces):
        d.anchoring[i] = ANCHORINGS[s.get("anchoring", "homeotropic").lower()]
        d.W[i] = s.get("W", 1.0)
        d.theta_s[i] = s.get("theta_s", 0.0)
        d.phi_s[i] = s.get("phi_s", 0.0)
    d.radius = radius
    d.B1, d.C = B1, C
    return d


_lib = None


def lib() -> C.CDLL:
    """The engine library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise McxError(5, f"{LIB_PATH} is missing: build it with mclics-backend_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        V, I, F, D = C.c_void_p, C.c_int, C.c_float, C.c_double
        L.mcx_version.restype = I
        L.mcx_last_error.restype = C.c_char_p
        L.mcx_last_error.argtypes = [V]
        L.mcx_create.argtypes = [I, C.POINTER(ReplicaDesc), C.POINTER(V)]
        L.mcx_destroy.argtypes = [V]
        L.mcx_num_replicas.argtypes = [V]
        L.mcx_get_desc.argtypes = [V, I, C.POINTER(ReplicaDesc), V]
        for name in ("mcx_set_state", "mcx_get_state"):
            getattr(L, name).argtypes = [V, I, V]
        L.mcx_init_random.argtypes = [V, I, C.c_uint]
        L.mcx_init_homogeneous.argtypes = [V, I, F, F]
        L.mcx_set_mask.argtypes = [V, I, V, V]
        L.mcx_get_mask.argtypes = [V, I, V, V]
        L.mcx_set_temperature.argtypes = [V, I, F]
        L.mcx_set_field.argtypes = [V, I, F]
        L.mcx_set_step.argtypes = [V, I, F]
        L.mcx_set_adapt.argtypes = [V, I, I]
        L.mcx_sweep.argtypes = [V, I, I]
        L.mcx_sync.argtypes = [V]
        L.mcx_measure.argtypes = [V, I, V]
        L.mcx_get_stats.argtypes = [V, I, V]
        L.mcx_reset_stats.argtypes = [V, I]
        L.mcx_set_series.argtypes = [V, I]
        L.mcx_get_series.argtypes = [V, I, I, V]
        L.mcx_debug_pass.argtypes = [V, I, I, V, V, V]
        L.mcx_kernel_launches.argtypes = [V]
        L.mcx_kernel_launches.restype = C.c_longlong
        L.mcx_run_file.argtypes = [C.c_char_p, C.c_char_p]
        L.mcx_set_staged.argtypes = [V, I]
        L.mcx_set_pass.argtypes = [V, I]
        L.mcx_get_pass.argtypes = [V]
        L.mcx_set_march_shape.argtypes = [V, I, I]
        L.mcx_autotune.argtypes = [V, C.POINTER(I), C.POINTER(I), C.POINTER(F)]
        L.mcx_get_staged.argtypes = [V]
        L.mcx_stream.argtypes = [V]
        L.mcx_stream.restype = V
        L.mcx_pass_timing.argtypes = [V, I, C.POINTER(F), C.POINTER(F)]
        L.mcx_sweep_timing.argtypes = [V, I, C.POINTER(F)]
        L.mcx_debug_barrier_timeout.argtypes = [V]
        L.mcx_local_order.argtypes = [V, I, V]
        L.mcx_print_n.argtypes = [V, I, C.c_char_p]
        L.mcx_polarization.argtypes = [V, I, C.POINTER(C.c_double)]
        L.mcx_save.argtypes = [V, C.c_char_p]
        L.mcx_load.argtypes = [V, C.c_char_p]
        L.mcx_exchange.argtypes = [V, I, V, C.c_uint, C.c_ulonglong, V]
        L.mcx_combine_stats.argtypes = [V, I, V, V]
        L.mcx_set_mlp.argtypes = [V, V, I]
        L.mcx_get_mlp.argtypes = [V, V]
        L.mcx_set_proposal.argtypes = [V, I]
        L.mcx_debug_pass_mlp.argtypes = [V, I, I, V, V, V, V]
        L.mcx_mlp_params.restype = I
        L.mcx_collect_samples.argtypes = [V, I, C.c_uint, I, V]
        L.mcx_train_mlp.argtypes = [V, C.POINTER(TrainConfig), V]
        L.mcx_mlp_grad.argtypes = [V, V, I, V, V]
        L.mcx_mlp_forward.argtypes = [V, V, I, V, I]
        L.mcx_set_mlp_path.argtypes = [V, I]
        L.mcx_get_mlp_path.argtypes = [V]
        L.mcx_get_mlp_path.restype = I
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Engine:
    """A batch of replicas resident on the GPU (mcx_create ... mcx_destroy)."""

    def __init__(self, descs: Iterable[ReplicaDesc]):
        descs = list(descs)
        arr = (ReplicaDesc * len(descs))(*descs)
        h = C.c_void_p()
        self._L = lib()
        st = self._L.mcx_create(len(descs), arr, C.byref(h))
        if st:
            raise McxError(st, self._L.mcx_last_error(None).decode())
        self._h = h
        self.descs = descs
        self.n = len(descs)

    def _ck(self, st: int):
        if st:
            raise McxError(st, self._L.mcx_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.mcx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def sites(self, r: int) -> int:
        if not 0 <= r < self.n:
            raise McxError(1, f"replica {r} out of range [0, {self.n})")
        d = self.descs[r]
        return d.nx * d.ny * d.nz

    def desc(self, r: int):
        d = ReplicaDesc()
        g = np.zeros(5, np.float32)
        self._ck(self._L.mcx_get_desc(self._h, r, C.byref(d), _p(g)))
        return d, g

    def set_state(self, r: int, ni: np.ndarray):
        ni = np.ascontiguousarray(ni, dtype=np.float32).reshape(-1, 3)
        if ni.shape[0] != self.sites(r):
            raise ValueError("director array has the wrong number of sites")
        self._ck(self._L.mcx_set_state(self._h, r, _p(ni)))

    def get_state(self, r: int) -> np.ndarray:
        out = np.empty((self.sites(r), 3), np.float32)
        self._ck(self._L.mcx_get_state(self._h, r, _p(out)))
        return out

    def init_random(self, r: int, seed: int):
        self._ck(self._L.mcx_init_random(self._h, r, seed))

    def init_homogeneous(self, r: int, theta_0: float = 0.0, phi_0: float = 0.0):
        self._ck(self._L.mcx_init_homogeneous(self._h, r, theta_0, phi_0))

    def set_mask(self, r: int, pt: np.ndarray, ns: Optional[np.ndarray] = None):
        pt = np.ascontiguousarray(pt, dtype=np.int32).reshape(-1)
        nsp = None
        if ns is not None:
            ns = np.ascontiguousarray(ns, dtype=np.float32).reshape(-1, 3)
            nsp = _p(ns)
        self._ck(self._L.mcx_set_mask(self._h, r, _p(pt), nsp))

    def get_mask(self, r: int):
        pt = np.empty(self.sites(r), np.int32)
        ns = np.empty((self.sites(r), 3), np.float32)
        self._ck(self._L.mcx_get_mask(self._h, r, _p(pt), _p(ns)))
        return pt, ns

    def set_temperature(self, T: float, r: int = -1):
        self._ck(self._L.mcx_set_temperature(self._h, r, T))

    def set_field(self, E: float, r: int = -1):
        self._ck(self._L.mcx_set_field(self._h, r, E))

    def set_step(self, ang_var: float, r: int = -1):
        self._ck(self._L.mcx_set_step(self._h, r, ang_var))

    def set_adapt(self, on: bool, r: int = -1):
        self._ck(self._L.mcx_set_adapt(self._h, r, 1 if on else 0))

    def sweep(self, n: int, measure: bool = False):
        self._ck(self._L.mcx_sweep(self._h, n, 1 if measure else 0))

    def sync(self):
        self._ck(self._L.mcx_sync(self._h))

    def measure(self, r: int) -> Dict:
        out = np.zeros(16)
        self._ck(self._L.mcx_measure(self._h, r, _p(out)))
        return dict(E=out[M_E], E_valid=out[M_E_VALID], Q=out[M_Q:M_Q + 9].reshape(3, 3), S=out[M_S],
                    director=out[M_DIRECTOR:M_DIRECTOR + 3], valid=int(out[M_VALID]))

    def stats(self, r: int) -> np.ndarray:
        out = np.zeros(16)
        self._ck(self._L.mcx_get_stats(self._h, r, _p(out)))
        return out

    def reset_stats(self, r: int = -1):
        self._ck(self._L.mcx_reset_stats(self._h, r))

    def set_series(self, capacity: int):
        self._ck(self._L.mcx_set_series(self._h, capacity))

    def series(self, r: int, count: int) -> np.ndarray:
        out = np.zeros((count, 2))
        self._ck(self._L.mcx_get_series(self._h, r, count, _p(out)))
        return out

    def debug_pass(self, r: int, colour: int):
        n = self.sites(r)
        dE = np.zeros(n, np.float32)
        acc = np.zeros(n, np.uint8)
        prop = np.zeros((n, 3), np.float32)
        self._ck(self._L.mcx_debug_pass(self._h, r, colour, _p(dE), _p(acc), _p(prop)))
        return dE, acc, prop

    def set_mlp(self, weights: np.ndarray):
        w = np.ascontiguousarray(weights, np.float32).reshape(-1)
        self._ck(self._L.mcx_set_mlp(self._h, _p(w), int(w.size)))

    def get_mlp(self) -> np.ndarray:
        w = np.zeros(MLP_PARAMS, np.float32)
        self._ck(self._L.mcx_get_mlp(self._h, _p(w)))
        return w

    def set_proposal(self, kind: str):
        self._ck(self._L.mcx_set_proposal(self._h, PROPOSALS[kind]))

    def debug_pass_mlp(self, r: int, colour: int):
        n = self.sites(r)
        dE = np.zeros(n, np.float32)
        acc = np.zeros(n, np.uint8)
        prop = np.zeros((n, 3), np.float32)
        y = np.zeros((n, 4), np.float32)
        self._ck(self._L.mcx_debug_pass_mlp(self._h, r, colour, _p(dE), _p(acc), _p(prop), _p(y)))
        return dE, acc, prop, y

    def collect_samples(self, n: int, seed: int = 0, augment: int = 0) -> np.ndarray:
        """n training samples from the current states: [n, 24] float32 (19
        inputs, the director, then replica and natural site index as int32
        bit patterns in columns 22, 23)."""
        out = np.zeros((n, SAMPLE_FLOATS), np.float32)
        self._ck(self._L.mcx_collect_samples(self._h, int(n), int(seed) & 0xFFFFFFFF, int(augment), _p(out)))
        return out

    def train_mlp(self, samples: int, batch: int, steps: int, lr: float = 1e-3, seed: int = 0,
                  augment: int = 0) -> np.ndarray:
        """Collects `samples` samples and runs `steps` Adam steps on the GPU;
        returns each step's minibatch loss."""
        cfg = TrainConfig(int(samples), int(batch), int(steps), float(lr), int(seed) & 0xFFFFFFFF, int(augment))
        loss = np.zeros(max(1, steps), np.float32)
        self._ck(self._L.mcx_train_mlp(self._h, C.byref(cfg), _p(loss)))
        return loss[:steps]

    def mlp_grad(self, samples: np.ndarray):
        """(loss, gradient) of the mean negative log-likelihood at the current
        weights over host samples [n, >= 22] (columns 0..21 read)."""
        s = np.zeros((samples.shape[0], SAMPLE_FLOATS), np.float32)
        s[:, :22] = samples[:, :22]
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = np.zeros(1, np.float32)
        self._ck(self._L.mcx_mlp_grad(self._h, _p(s), int(s.shape[0]), _p(g), _p(loss)))
        return float(loss[0]), g

    def mlp_forward(self, inputs: np.ndarray, path: str = "tcgen05") -> np.ndarray:
        """The network on rows of its 19 inputs -> [n, 4] outputs, on the
        tcgen05 tensor cores ("tcgen05") or with the learned passes' warp-level
        mma.sync code ("warp")."""
        x = np.ascontiguousarray(inputs, np.float32).reshape(-1, 19)
        y = np.zeros((x.shape[0], 4), np.float32)
        self._ck(self._L.mcx_mlp_forward(self._h, _p(x), int(x.shape[0]), _p(y), {"warp": 0, "tcgen05": 1}[path]))
        return y

    @property
    def mlp_path(self) -> str:
        """The learned z-march's network code: "tcgen05" or "warp"."""
        return "tcgen05" if self._L.mcx_get_mlp_path(self._h) == 1 else "warp"

    @mlp_path.setter
    def mlp_path(self, path: str):
        self._ck(self._L.mcx_set_mlp_path(self._h, {"warp": 0, "tcgen05": 1}[path]))

    def polarization(self, r: int) -> float:
        P = C.c_double()
        self._ck(self._L.mcx_polarization(self._h, r, C.byref(P)))
        return P.value

    def local_order(self, r: int) -> np.ndarray:
        """Per-site local order parameter (NaN at inactive sites)."""
        out = np.zeros(self.sites(r), np.float32)
        self._ck(self._L.mcx_local_order(self._h, r, _p(out)))
        return out

    def print_n(self, r: int, path: str):
        """The replica's current state as the reference's snapshot file
        (print_n): x,y,z,nx,ny,nz,S,pt."""
        self._ck(self._L.mcx_print_n(self._h, r, path.encode()))

    def save(self, path: str):
        self._ck(self._L.mcx_save(self._h, path.encode()))

    def load(self, path: str):
        self._ck(self._L.mcx_load(self._h, path.encode()))

    def exchange(self, pairs, seed: int = 0, round: int = 0) -> np.ndarray:
        """Replica-exchange attempts for the given (a, b) pairs; returns the
        acceptance decisions."""
        pr = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
        acc = np.zeros(len(pr), np.int32)
        self._ck(self._L.mcx_exchange(self._h, len(pr), _p(pr), int(seed) & 0xFFFFFFFF, int(round), _p(acc)))
        return acc

    def combine_stats(self, replicas=None) -> dict:
        """One po.dat row combining independent replicas (all when None) by the
        law of total variance, on the GPU: T, S, varS, E, varE and, for Pear,
        P (NaN otherwise)."""
        out = np.zeros(COMBINED_LEN, np.float64)
        if replicas is None:
            self._ck(self._L.mcx_combine_stats(self._h, 0, None, _p(out)))
        else:
            idx = np.ascontiguousarray(replicas, np.int32).ravel()
            self._ck(self._L.mcx_combine_stats(self._h, len(idx), _p(idx), _p(out)))
        return {"T": out[CB_T], "S": out[CB_S], "varS": out[CB_VAR_S], "E": out[CB_E], "varE": out[CB_VAR_E],
                "P": out[CB_P], "n": int(out[CB_N]), "T_spread": out[CB_T_SPREAD]}

    @property
    def pass_kind(self) -> str:
        return {v: k for k, v in PASSES.items()}[int(self._L.mcx_get_pass(self._h))]

    @pass_kind.setter
    def pass_kind(self, kind: str):
        self._ck(self._L.mcx_set_pass(self._h, PASSES[kind]))

    def set_march_shape(self, block: int, planes: int):
        self._ck(self._L.mcx_set_march_shape(self._h, int(block), int(planes)))

    def autotune(self):
        """Chooses the z-march pass's block size and chunk depth by timing;
        returns (block, planes, microseconds per pass)."""
        b, k, us = C.c_int(), C.c_int(), C.c_float()
        self._ck(self._L.mcx_autotune(self._h, C.byref(b), C.byref(k), C.byref(us)))
        return b.value, k.value, us.value

    @property
    def staged(self) -> bool:
        return bool(self._L.mcx_get_staged(self._h))

    @staged.setter
    def staged(self, on: bool):
        self._ck(self._L.mcx_set_staged(self._h, 1 if on else 0))

    @property
    def kernel_launches(self) -> int:
        return int(self._L.mcx_kernel_launches(self._h))


def run_file(param_file: str, out_dir: Optional[str] = None) -> None:
    """./mc_sim <param_file> on the GPU (src/main.cpp:63-83 of the reference)."""
    L = lib()
    st = L.mcx_run_file(param_file.encode(), out_dir.encode() if out_dir else None)
    if st:
        raise McxError(st, L.mcx_last_error(None).decode())


def exported_symbols() -> List[str]:
    """Every entry point declared in include/mcx.h."""
    hdr = os.path.join(os.path.dirname(PKG), "include", "mcx.h")
    import re
    names = re.findall(r"\b(mcx_[a-z_]+)\s*\(", open(hdr).read())
    return sorted(set(names))
