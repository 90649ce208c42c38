"""The batched workloads that bench.py times (mcx/workloads.py) are the
configurations they name: the GHRL slab batch (256 replicas, cubic sides
drawn from {16, 24, 32, 48, 64}, slab geometry with homeotropic W = 4 on the
z faces, k = (1, 0.8, 1.2), p0 = 0, T uniform in [0.8, 1.2]) and the droplet
field sweep (64 droplets of radius 40 in 96^3, GHRL k = (1, 0.6, 1.4),
p0 = 20, planar anchoring W = 1, the field along z, T = 0.8).  Host-side
checks only: descriptors, and the droplet's mask from the engine's own
builder against the oracle's."""
import ctypes as C

import numpy as np

import mcx
from mcx import workloads
from oracle import oracle as O


def test_slab_batch_descriptors():
    ds = workloads.c3_descs(256)
    assert len(ds) == 256
    sides = {d.nx for d in ds}
    assert sides == {16, 24, 32, 48, 64}
    for q, d in enumerate(ds):
        assert d.nx == d.ny == d.nz
        assert d.geometry == mcx.GEOMETRIES["slab"] and d.potential == mcx.POTENTIALS["ghrl"]
        assert (d.k11, d.k22, d.k33, d.p0) == (1.0, np.float32(0.8), np.float32(1.2), 0.0)
        assert 0.8 <= d.T <= 1.2
        assert d.n_surfaces == 2
        for s in range(2):
            assert d.anchoring[s] == mcx.ANCHORINGS["homeotropic"] and d.W[s] == 4.0
        assert (d.seed, d.stream) == (100 + q, q)  # independent streams


def test_droplet_batch_descriptors_and_mask():
    ds = workloads.c5_descs(64)
    assert len(ds) == 64
    d = ds[0]
    assert (d.nx, d.ny, d.nz) == (96, 96, 96) and d.radius == 40.0
    assert d.geometry == mcx.GEOMETRIES["sphere"] and d.potential == mcx.POTENTIALS["ghrl"]
    assert (d.k11, d.k22, d.k33, d.p0) == (1.0, np.float32(0.6), np.float32(1.4), 20.0)
    assert (d.elecX, d.elecY, d.elecZ, d.T) == (0.0, 0.0, 1.0, np.float32(0.8))
    assert d.n_surfaces == 1 and d.anchoring[0] == mcx.ANCHORINGS["fg"] and d.W[0] == 1.0
    assert len({(x.seed, x.stream) for x in ds}) == 64
    pt = np.zeros(96 ** 3, np.int32)
    ns = np.zeros((96 ** 3, 3), np.float32)
    assert mcx.lib().mcx_build_mask(C.byref(d), pt.ctypes.data_as(C.c_void_p), ns.ctypes.data_as(C.c_void_p)) == 0
    m = O.Model(nx=96, ny=96, nz=96, geometry="sphere", potential="ghrl", radius=40.0, surfaces=[O.Surface("fg", 1.0)])
    assert np.array_equal(pt, O.Lattice(m).pt)
    # the droplet's active sites (bulk and surface shell), as the engine reports them on the GPU
    assert int(np.count_nonzero(pt)) == 288113
