"""The C-ABI library (no GPU needed): it loads, exports every entry point
include/mcx.h declares, lays out mcx_replica_desc as the header does, and its
host-only helpers agree with the oracle and the reference."""
import ctypes as C
import os
import subprocess
import textwrap

import numpy as np
import pytest

import mcx
from oracle import oracle as O
from oracle import refproc
from helpers import desc_from_model

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    L = mcx.lib()
    names = mcx.exported_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_replica_desc_layout_matches_header(tmp_path):
    src = tmp_path / "sz.c"
    src.write_text(textwrap.dedent("""
        #include <stdio.h>
        #include <stddef.h>
        #include "mcx.h"
        int main(void) {
          printf("%zu %zu %zu %zu\\n", sizeof(mcx_replica_desc), offsetof(mcx_replica_desc, anchoring),
                 offsetof(mcx_replica_desc, phi_s), offsetof(mcx_replica_desc, radius));
          return 0;
        }"""))
    exe = tmp_path / "sz"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    D = mcx.ReplicaDesc
    assert got == [C.sizeof(D), D.anchoring.offset, D.phi_s.offset, D.radius.offset]


@pytest.mark.parametrize("k", [(1.0, 0.8, 1.2, 0.0), (1.0, 0.6, 1.4, 20.0), (1.48, 1.0, 2.28, 0.0), (1, 1, 1, 40.0)])
def test_ghrl_constants_match_oracle(k):
    out = np.zeros(5, np.float32)
    mcx.lib().mcx_ghrl_constants(*[C.c_float(x) for x in k], out.ctypes.data_as(C.c_void_p))
    assert np.array_equal(out, np.array(O.ghrl_constants(*k), np.float32))


@pytest.mark.parametrize("geo,dims,radius", [("bulk", (6, 4, 5), 0), ("slab", (6, 4, 5), 0), ("sphere", (10, 10, 10), 0),
                                             ("sphere", (12, 8, 11), 0), ("sphere", (24, 24, 24), 7.5),
                                             ("slab", (4, 4, 1), 0)])
def test_build_mask_matches_oracle(geo, dims, radius):
    nsurf = {"bulk": 0, "slab": 2, "sphere": 1}[geo]
    m = O.Model(nx=dims[0], ny=dims[1], nz=dims[2], geometry=geo, radius=radius,
                surfaces=[O.Surface("fg", 1.0)] * nsurf)
    d = desc_from_model(m)
    pt = np.zeros(m.n, np.int32)
    ns = np.zeros((m.n, 3), np.float32)
    st = mcx.lib().mcx_build_mask(C.byref(d), pt.ctypes.data_as(C.c_void_p), ns.ctypes.data_as(C.c_void_p))
    assert st == 0
    lat = O.Lattice(m)
    assert np.array_equal(pt, lat.pt)
    assert np.array_equal(ns, lat.ns)


def _check(path):
    d = mcx.ReplicaDesc()
    st = mcx.lib().mcx_check_file(str(path).encode(), C.byref(d))
    return st, d, mcx.lib().mcx_last_error(None).decode()


def _samples():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "reference_samples.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("name", sorted(_samples()))
def test_every_reference_sample_file_is_accepted(name, tmp_path):
    """The reference's eight sample parameter files (key/value lines kept by
    tests/golden/make_sample_params.py) parse and validate, including the
    odd-sided droplets of test4.txt (25^3) and input_parameters.txt (61^3)."""
    text = _samples()[name]
    p = tmp_path / name
    p.write_text(text)
    st, d, err = _check(p)
    assert st == 0, err
    kv = {ln.split()[0].lower(): ln.split()[1] for ln in text.splitlines()}
    assert (d.nx, d.ny, d.nz) == (int(kv["nx"]), int(kv["ny"]), int(kv["nz"]))


def test_odd_periodic_axis_is_refused_with_a_reason(tmp_path):
    p = tmp_path / "p.txt"
    p.write_text("Nx 15\nNy 16\nNz 16\nxbound periodic\n")
    st, d, err = _check(p)
    assert st == 4 and "odd" in err and "periodic" in err
    p.write_text("Nx 15\nNy 16\nNz 16\nxbound free\n")
    st, d, err = _check(p)
    assert st == 0, err


def test_parser_reads_reference_sample_style(tmp_path):
    p = tmp_path / "p.txt"
    p.write_text(textwrap.dedent("""\
        # comment line
        Nx 20
        ny  20   # trailing comment
        NZ 30
        Nk 1
        potential  ghrl
        k11 1.48
        k22 1
        k33 2.28
        p0  0
        evol thermalGPU
        Ti 1.3
        Tf 0.8
        dT -0.1
        MCT 3000
        MCS 400
        ic random
        geometry slab
        xbound periodic
        ybound periodic
        anchoring_type 0 homeotropic
        W       0 4
        anchoring_type 1 homeotropic_ghrl
        W       1 2.5
        Electric_field_z 1
        Aniso_E 0.3
        """))
    st, d, err = _check(p)
    assert st == 0, err
    assert (d.nx, d.ny, d.nz) == (20, 20, 30)
    assert d.potential == 1 and d.geometry == 1 and d.n_surfaces == 2
    assert d.anchoring[0] == 0 and d.anchoring[1] == 4
    assert d.W[1] == pytest.approx(2.5)
    assert d.k11 == pytest.approx(1.48) and d.elecA == pytest.approx(0.3) and d.elecZ == 1


@pytest.mark.parametrize("body,code,msg", [
    ("Nx 16\nbogus 3\n", 6, "unknown parameter"),
    ("Nx sixteen\n", 6, "invalid value"),
    ("nk 2\n", 6, "neighbour_kind"),
    ("geometry slab\nanchoring_type 0 homeotropic\nW 0 1\n", 6, "define 2 boundaries"),
    ("geometry sphere\nanchoring_type 0 nonsense\nW 0 1\n", 6, "not defined"),
    ("geometry sphere\nanchoring_type 0 rp\nW 0 1\n", 6, "phi_s"),
    ("potential gay_berne\n", 6, "ll | ghrl | pear"),
    ("Nx 15\nxbound periodic\n", 4, "even lengths on periodic axes"),
    ("evol sideways\n", 6, "evol mode"),
    ("dT 0\n", 6, "dT"),
])
def test_parser_errors(tmp_path, body, code, msg):
    p = tmp_path / "p.txt"
    p.write_text(body)
    st, _, err = _check(p)
    assert st == code
    assert msg in err


def test_missing_file_is_io_error(tmp_path):
    st, _, err = _check(tmp_path / "nope.txt")
    assert st == 5 and "cannot open" in err


def test_custom_geometry_reader(tmp_path):
    f = tmp_path / "geo.csv"
    f.write_text("x,y,z,nx,ny,nz,pt\n0,0,0,0,0,1,2\n1,0,0,0,1,0,3\n1,1,1,0,0,0,0\n")
    n = 4 * 2 * 2
    pt = np.zeros(n, np.int32)
    ns = np.zeros((n, 3), np.float32)
    k = C.c_int()
    st = mcx.lib().mcx_read_geometry(str(f).encode(), 4, 2, 2, pt.ctypes.data_as(C.c_void_p),
                                     ns.ctypes.data_as(C.c_void_p), C.byref(k))
    assert st == 0 and k.value == 2
    assert pt[0] == 2 and pt[1] == 3 and pt[1 + 4 * (1 + 2)] == 0 and pt[2] == 1
    assert tuple(ns[1]) == (0, 1, 0)
    f.write_text("x,y,z,nx,ny,nz,pt\n9,0,0,0,0,1,2\n")
    st = mcx.lib().mcx_read_geometry(str(f).encode(), 4, 2, 2, pt.ctypes.data_as(C.c_void_p),
                                     ns.ctypes.data_as(C.c_void_p), C.byref(k))
    assert st == 6 and "out of simulation box" in mcx.lib().mcx_last_error(None).decode()


@pytest.mark.skipif(not refproc.available(), reason="reference build (oracle/_ref) not present")
def test_custom_geometry_matches_reference(tmp_path):
    f = tmp_path / "geo.csv"
    rng = np.random.default_rng(4)
    lines = ["x,y,z,nx,ny,nz,pt"]
    for _ in range(40):
        i, j, k = rng.integers(0, 6), rng.integers(0, 4), rng.integers(0, 4)
        v = O.random_directors(1, rng)[0]
        lines.append(f"{i},{j},{k},{v[0]:.6f},{v[1]:.6f},{v[2]:.6f},{rng.integers(0, 4)}")
    f.write_text("\n".join(lines) + "\n")
    n = 6 * 4 * 4
    pt = np.zeros(n, np.int32)
    ns = np.zeros((n, 3), np.float32)
    k = C.c_int()
    assert mcx.lib().mcx_read_geometry(str(f).encode(), 6, 4, 4, pt.ctypes.data_as(C.c_void_p),
                                       ns.ctypes.data_as(C.c_void_p), C.byref(k)) == 0
    m = O.Model(nx=6, ny=4, nz=4, geometry="custom", surfaces=[O.Surface("fg", 1.0)] * max(k.value, 1))
    md = refproc.model_dict(m)
    md["bound_file"] = str(f)
    ((rpt, rns),) = refproc.pool_run(md, [("mask",)])
    assert np.array_equal(pt, rpt)
    assert np.allclose(ns, rns, atol=1e-6)
