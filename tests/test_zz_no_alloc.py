"""mcx_measure_noalloc: the allocation-free measurement, for callers that
cannot allocate device memory themselves (a host framework that owns every
device allocation, a latency-critical loop where cudaMalloc would stall).

Called through the C ABI on director fields held in caller-owned device
memory, on two calls in a row -- the second call reuses the shared scratch
the first one left behind -- it must agree with the FP64 oracle's measurement
of the same field and with the engine's mcx_measure (E within 2e-6 relative,
Q and S within 2e-6), for every pair potential and for odd lattice sides."""
import ctypes as C

import numpy as np
import pytest

import mcx
from oracle import oracle as O
from helpers import desc_from_model, random_state

pytestmark = pytest.mark.gpu

CASES = [
    O.Model(nx=16, ny=16, nz=16, potential="ll"),
    O.Model(nx=12, ny=10, nz=8, geometry="slab", potential="ghrl", k11=1.0, k22=0.8, k33=1.2, p0=12, elecA=0.4,
            elecZ=1.0, elecE=1.3, surfaces=[O.Surface("homeotropic", 4.0), O.Surface("fg_ghrl", 1.5)]),
    O.Model(nx=14, ny=14, nz=14, geometry="sphere", potential="ghrl", k11=1.0, k22=0.6, k33=1.4, p0=20,
            surfaces=[O.Surface("fg", 2.0)]),
    O.Model(nx=12, ny=8, nz=6, potential="pear", A=1.0, B1=0.3, C=0.3, elecA=0.4, elecZ=1.0, elecE=1.0),
    O.Model(nx=13, ny=11, nz=9, geometry="sphere", potential="pear", B1=0.2, C=0.4,
            surfaces=[O.Surface("homeotropic", 3.0)]),
]


def _noalloc(L, d, ni, pt, ns, out, stream):
    return L.mcx_measure_noalloc(C.byref(d), C.c_void_p(ni.data_ptr()), C.c_void_p(pt.data_ptr()),
                                 C.c_void_p(ns.data_ptr()), C.c_void_p(out.data_ptr()), C.c_void_p(stream))


@pytest.mark.parametrize("case", range(len(CASES)))
def test_measure_noalloc_matches_engine(case):
    torch = pytest.importorskip("torch")
    L = mcx.lib()
    L.mcx_measure_noalloc.argtypes = [C.POINTER(mcx.ReplicaDesc), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p]
    m = CASES[case]
    d = desc_from_model(m, T=1.0, seed=3)
    lat = O.Lattice(m)
    rng = np.random.default_rng(40 + case)
    with mcx.Engine([d]) as eng:
        ni = random_state(m, lat.pt, rng)
        ni = ni * 0.6 + np.array([0.1, -0.2, 0.9], np.float32)
        ni /= np.linalg.norm(ni, axis=1, keepdims=True)
        ni[lat.pt == 0] = (0, 0, 1)
        eng.set_state(0, ni)
        ref = eng.measure(0)
    lat.ni[:] = ni
    orc = lat.measure()
    dev = torch.device("cuda:0")
    t_ni = torch.from_numpy(np.ascontiguousarray(ni, np.float32)).to(dev)
    t_pt = torch.from_numpy(np.ascontiguousarray(lat.pt, np.int32)).to(dev)
    t_ns = torch.from_numpy(np.ascontiguousarray(lat.ns, np.float32)).to(dev)
    t_out = torch.zeros(mcx.M_VALID + 1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        t_out.fill_(-7.0)
        assert _noalloc(L, d, t_ni, t_pt, t_ns, t_out, stream) == 0, L.mcx_last_error(None).decode()
        torch.cuda.synchronize()
        out = t_out.cpu().numpy()
        # the FP64 oracle
        assert out[mcx.M_VALID] == orc["valid"]
        assert out[mcx.M_E] == pytest.approx(orc["E"], rel=2e-6, abs=1e-6), call
        assert out[mcx.M_E_VALID] == pytest.approx(orc["E_valid"], rel=2e-6, abs=1e-6), call
        assert np.allclose(out[mcx.M_Q:mcx.M_Q + 9].reshape(3, 3), orc["Q"], atol=2e-6), call
        assert out[mcx.M_S] == pytest.approx(orc["S"], abs=2e-6), call
        # and the engine's own measurement
        assert out[mcx.M_VALID] == ref["valid"]
        assert out[mcx.M_E] == pytest.approx(ref["E"], rel=2e-6, abs=1e-6), call
        assert out[mcx.M_E_VALID] == pytest.approx(ref["E_valid"], rel=2e-6, abs=1e-6), call
        assert np.allclose(out[mcx.M_Q:mcx.M_Q + 9].reshape(3, 3), ref["Q"], atol=2e-6), call
        assert out[mcx.M_S] == pytest.approx(ref["S"], abs=2e-6), call
        assert abs(abs(np.dot(out[mcx.M_DIRECTOR:mcx.M_DIRECTOR + 3], ref["director"])) - 1) < 1e-5


def test_measure_noalloc_rejects_oversized_lattice():
    torch = pytest.importorskip("torch")
    L = mcx.lib()
    L.mcx_measure_noalloc.argtypes = [C.POINTER(mcx.ReplicaDesc), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p]
    d = mcx.replica(nx=1024, ny=1024, nz=1024)
    buf = torch.zeros(16, dtype=torch.float64, device="cuda:0")
    rc = L.mcx_measure_noalloc(C.byref(d), C.c_void_p(buf.data_ptr()), None, None, C.c_void_p(buf.data_ptr()), None)
    assert rc == 1
    assert "exceed the maximum" in L.mcx_last_error(None).decode()


def test_measure_noalloc_rejects_bad_descriptors():
    torch = pytest.importorskip("torch")
    L = mcx.lib()
    L.mcx_measure_noalloc.argtypes = [C.POINTER(mcx.ReplicaDesc), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p]
    buf = torch.zeros(16 * 3, dtype=torch.float64, device="cuda:0")
    d = mcx.replica(nx=2, ny=2, nz=2, geometry="slab", surfaces=[dict(anchoring="fg", W=1.0)] * 2)
    d.anchoring[1] = 9
    rc = L.mcx_measure_noalloc(C.byref(d), C.c_void_p(buf.data_ptr()), None, None, C.c_void_p(buf.data_ptr()), None)
    assert rc == 1 and "unknown anchoring 9 on surface 1" in L.mcx_last_error(None).decode()
    d = mcx.replica(nx=2, ny=2, nz=2)
    d.potential = 5
    rc = L.mcx_measure_noalloc(C.byref(d), C.c_void_p(buf.data_ptr()), None, None, C.c_void_p(buf.data_ptr()), None)
    assert rc == 1 and "unknown potential" in L.mcx_last_error(None).decode()
