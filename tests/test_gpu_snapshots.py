"""Snapshots, checkpoints, replica exchange and the parameter-file driver.

- mcx_local_order against the reference's own lattice_order_parameter
  (src/parameter_order.cpp:62-113) on committed golden states, and against
  the oracle's FP64 restatement: Q over the site and its existing active
  neighbours, largest eigenvalue; NaN at inactive sites.
- mcx_save / mcx_load: a loaded engine continues the saved trajectory bit for
  bit (same states, step sizes and running sums after more sweeps).
- mcx_exchange: the decisions are min(1, exp((1/Ta - 1/Tb)(Ha - Hb))) against
  the documented Philox uniform; accepted pairs swap T.
- mcx_run_file: ./mc_sim on a small parameter file writes po.dat and the
  director_field_*.csv snapshots in the reference's formats.
- mcx_combine_stats: the GPU combination of replicas equals the oracle's
  restatement of average_replicas.py applied to each replica's po.dat row;
  with `replicas R` the driver's po_avg.dat equals the oracle's combination of
  the po.dat files it wrote (to their %g rounding)."""
import os

import numpy as np
import pytest

import mcx
from oracle import oracle as O
from oracle import replicas as OR
from helpers import desc_from_model, load_local_order, random_state

pytestmark = pytest.mark.gpu

LOCAL_ORDER = load_local_order()


@pytest.mark.parametrize("name", list(LOCAL_ORDER))
def test_local_order_against_reference(name):
    m, pt, ni, S, _ = LOCAL_ORDER[name]
    with mcx.Engine([desc_from_model(m)]) as eng:
        eng.set_state(0, ni)
        got = eng.local_order(0)
    assert np.array_equal(np.isnan(got), np.isnan(S))
    ok = ~np.isnan(S)
    assert np.max(np.abs(got[ok] - S[ok])) < 1e-6


@pytest.mark.parametrize("name", [k for k, v in LOCAL_ORDER.items() if v[4] is not None])
def test_print_n_against_reference(name, tmp_path):
    """mcx_print_n writes the reference's print_n file for the same state:
    the same header, and per line the same coordinates, directors (the same
    floats through %g), point type and nan text; S as the reference prints
    it to within its FP32 evaluation (the two solve Q in different code, so
    the sixth significant digit can differ)."""
    m, pt, ni, S, csv = LOCAL_ORDER[name]
    path = tmp_path / "snap.csv"
    with mcx.Engine([desc_from_model(m)]) as eng:
        eng.set_state(0, ni)
        eng.print_n(0, str(path))
    got, want = path.read_text().splitlines(), csv.splitlines()
    assert got[0] == want[0] == "x,y,z,nx,ny,nz,S,pt"
    assert len(got) == len(want) == m.n + 1
    for a, b in zip(got[1:], want[1:]):
        fa, fb = a.split(","), b.split(",")
        assert fa[:6] == fb[:6] and fa[7] == fb[7], (a, b)
        if fb[6] == "nan":
            assert fa[6] == "nan", (a, b)
        else:
            assert abs(float(fa[6]) - float(fb[6])) <= 2e-6, (a, b)


def test_print_n_reports_an_unwritable_path(tmp_path):
    m, pt, ni, S, _ = LOCAL_ORDER["bulk"]
    with mcx.Engine([desc_from_model(m)]) as eng:
        with pytest.raises(mcx.McxError) as err:
            eng.print_n(0, str(tmp_path / "missing_dir" / "snap.csv"))
        assert err.value.status == 5  # MCX_ERR_IO
        assert "cannot write" in str(err.value)


@pytest.mark.parametrize("m", [O.Model(nx=12, ny=10, nz=8, potential="ll"),
                               O.Model(nx=16, ny=16, nz=16, geometry="sphere", potential="ll",
                                       surfaces=[O.Surface("fg", 1.0)]),
                               O.Model(nx=12, ny=8, nz=6, geometry="slab", potential="ghrl",
                                       surfaces=[O.Surface("homeotropic", 2.0), O.Surface("fg", 1.0)])],
                         ids=["bulk", "sphere", "slab"])
def test_local_order_parameter(m):
    lat = O.Lattice(m)
    with mcx.Engine([desc_from_model(m)]) as eng:
        ni = random_state(m, lat.pt, np.random.default_rng(4))
        ni = 0.3 * ni + np.array([0.1, 0.2, 0.9], np.float32)
        ni /= np.linalg.norm(ni, axis=1, keepdims=True)
        eng.set_state(0, ni)
        got = eng.local_order(0)
        ni = eng.get_state(0)
    want = O.local_order(ni, lat.pt, m)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    ok = ~np.isnan(want)
    assert np.max(np.abs(got[ok] - want[ok])) < 2e-6


def test_checkpoint_continues_the_trajectory(tmp_path):
    m = O.Model(nx=12, ny=8, nz=6, geometry="slab", potential="ghrl", k11=1.0, k22=0.6, k33=1.4, p0=20, elecA=0.5,
                elecZ=1.0, elecE=1.0, surfaces=[O.Surface("homeotropic", 2.0), O.Surface("fg", 1.0)])
    descs = [desc_from_model(m, T=0.9 + 0.1 * r, seed=11 + r, stream=r) for r in range(3)]
    path = str(tmp_path / "ck.bin")
    with mcx.Engine(descs) as a:
        for r in range(3):
            a.init_random(r, 5 + r)
        a.sweep(7, measure=True)
        a.save(path)
        a.sweep(9, measure=True)
        want = [(a.get_state(r), a.stats(r)) for r in range(3)]
    with mcx.Engine(descs) as b:
        b.load(path)
        b.sweep(9, measure=True)
        got = [(b.get_state(r), b.stats(r)) for r in range(3)]
    for (sa, ta), (sb, tb) in zip(want, got):
        assert np.array_equal(sa, sb)
        assert ta[mcx.ST_ANG_VAR] == tb[mcx.ST_ANG_VAR]
        assert ta[mcx.ST_SWEEP_INDEX] == tb[mcx.ST_SWEEP_INDEX] == 16
        assert ta[mcx.ST_N] == tb[mcx.ST_N] == 16
        assert ta[mcx.ST_S1] == pytest.approx(tb[mcx.ST_S1], rel=1e-12)
        assert ta[mcx.ST_E1] == pytest.approx(tb[mcx.ST_E1], rel=1e-12)
    with mcx.Engine(descs[:2]) as c:
        with pytest.raises(mcx.McxError):
            c.load(path)


def test_failed_checkpoint_load_leaves_the_engine_unchanged(tmp_path):
    """A truncated checkpoint, one made with another seed and one made for
    other physics are refused, and the engine keeps its own directors, mask,
    counters and running sums (the file is read and checked before anything
    is applied)."""
    m = O.Model(nx=10, ny=8, nz=6, geometry="slab", potential="ghrl", k11=1.0, k22=0.8, k33=1.2,
                surfaces=[O.Surface("homeotropic", 2.0), O.Surface("fg", 1.0)])
    descs = [desc_from_model(m, T=0.9, seed=4 + r, stream=r) for r in range(3)]
    path = str(tmp_path / "ck.bin")
    with mcx.Engine(descs) as a:
        for r in range(3):
            a.init_random(r, 50 + r)
        a.sweep(5, measure=True)
        a.save(path)
    data = open(path, "rb").read()
    bad = {"truncated": data[:len(data) - 1000]}
    other_seed = [desc_from_model(m, T=0.9, seed=4 + r + (r == 2), stream=r) for r in range(3)]
    m2 = O.Model(**{**m.__dict__, "k22": 0.7})
    other_phys = [desc_from_model(m2, T=0.9, seed=4 + r, stream=r) for r in range(3)]
    for name, text in bad.items():
        p = tmp_path / (name + ".bin")
        p.write_bytes(text)
        bad[name] = str(p)
    for engine_descs, ck in ((descs, bad["truncated"]), (other_seed, path), (other_phys, path)):
        with mcx.Engine(engine_descs) as b:
            for r in range(3):
                b.init_random(r, 90 + r)
            b.sweep(3, measure=True)
            before = [(b.get_state(r), b.get_mask(r), b.stats(r)) for r in range(3)]
            with pytest.raises(mcx.McxError):
                b.load(ck)
            for r in range(3):
                ni, (pt, ns), st = before[r]
                assert np.array_equal(b.get_state(r), ni)
                gp, gn = b.get_mask(r)
                assert np.array_equal(gp, pt) and np.array_equal(gn, ns)
                assert np.array_equal(b.stats(r), st)
            b.sweep(1)  # still usable


def test_replica_exchange_decisions():
    m = O.Model(nx=8, ny=8, nz=8, potential="ll")
    Ts = [0.6, 0.9, 1.2, 1.5]
    descs = [desc_from_model(m, T=T, seed=3 + r, stream=r) for r, T in enumerate(Ts)]
    with mcx.Engine(descs) as eng:
        for r in range(4):
            eng.init_random(r, 20 + r)
        eng.sweep(30)
        seed, rnd = 77, 5
        pairs = [(0, 1), (2, 3)]
        H = [eng.measure(r)["E"] * m.n for r in range(4)]
        acc = eng.exchange(pairs, seed=seed, round=rnd)
        for i, (a, b) in enumerate(pairs):
            u = float(O.u24(O.philox([i, rnd, 0, 4], [seed, 0]))[0])
            lr = (1 / Ts[a] - 1 / Ts[b]) * (H[a] - H[b])
            assert bool(acc[i]) == (lr >= 0 or u < np.exp(lr))
            if acc[i]:
                assert eng.desc(a)[0].T == np.float32(Ts[b]) and eng.desc(b)[0].T == np.float32(Ts[a])
            else:
                assert eng.desc(a)[0].T == np.float32(Ts[a])
        # equal temperatures always swap
        eng.set_temperature(1.0)
        assert np.all(eng.exchange([(0, 1), (2, 3)], seed=1, round=9) == 1)
        with pytest.raises(mcx.McxError):
            eng.exchange([(0, 0)])
    other = [desc_from_model(m, T=1.0), desc_from_model(O.Model(nx=8, ny=8, nz=8, potential="ll", A=2.0), T=1.0)]
    with mcx.Engine(other) as eng:
        with pytest.raises(mcx.McxError):
            eng.exchange([(0, 1)])


PARAMS = """Nx  8
Ny  8
Nz  8
potential  ll
evol  thermalGPU
Ti    1.2
Tf    1.0
dT    -0.1
MCT  20
MCS  20
ic  random
geometry  bulk
xbound    periodic
ybound    periodic
zbound    periodic
"""


def test_run_file_writes_reference_outputs(tmp_path):
    pf = tmp_path / "params.txt"
    pf.write_text(PARAMS)
    mcx.run_file(str(pf), str(tmp_path) + "/")
    rows = [ln.split() for ln in (tmp_path / "po.dat").read_text().splitlines()]
    assert rows[0] == ["T", "S", "varS", "E", "varE"]
    data = np.array(rows[1:], float)
    assert data.shape == (3, 5)
    assert np.allclose(data[:, 0], [1.2, 1.1, 1.0], atol=1e-5)
    assert np.all((data[:, 1] > 0) & (data[:, 1] <= 1)) and np.all(data[:, 3] < 0)
    snaps = sorted(f for f in os.listdir(tmp_path) if f.startswith("director_field_"))
    assert len(snaps) >= 3
    lines = (tmp_path / snaps[0]).read_text().splitlines()
    assert lines[0] == "x,y,z,nx,ny,nz,S,pt"
    assert len(lines) == 1 + 8 ** 3
    S = np.array([float(l.split(",")[6]) for l in lines[1:]])
    assert np.all((S >= -0.5) & (S <= 1.0))


def test_polarization():
    m = O.Model(nx=12, ny=10, nz=8, potential="pear", B1=0.3, C=0.3)
    with mcx.Engine([desc_from_model(m)]) as eng:
        ni = random_state(m, np.ones(m.n, np.int32), np.random.default_rng(9))
        ni = 0.5 * ni + np.array([0.0, 0.3, 0.8], np.float32)
        ni /= np.linalg.norm(ni, axis=1, keepdims=True)
        eng.set_state(0, ni)
        got = eng.polarization(0)
        ni = eng.get_state(0).astype(np.float64)
    assert got == pytest.approx(np.linalg.norm(ni.sum(0)) / m.n, rel=1e-9)


def test_run_file_pear_adds_polarization(tmp_path):
    pf = tmp_path / "params.txt"
    pf.write_text(PARAMS.replace("potential  ll", "potential  pear\nA 1.0\nB1 0.3\nC 0.3"))
    mcx.run_file(str(pf), str(tmp_path) + "/")
    rows = [ln.split() for ln in (tmp_path / "po.dat").read_text().splitlines()]
    assert rows[0] == ["T", "S", "varS", "E", "varE", "P"]
    data = np.array(rows[1:], float)
    assert data.shape == (3, 6) and np.all((data[:, 5] >= 0) & (data[:, 5] <= 1))


def _replica_rows(eng, idx, pear=False):
    return [OR.po_row(float(eng.desc(r)[0].T), eng.stats(r), eng.polarization(r) if pear else None) for r in idx]


def test_combine_stats_matches_oracle_combiner():
    m = O.Model(nx=8, ny=8, nz=8, potential="ll")
    descs = [desc_from_model(m, T=1.0, seed=40 + r, stream=r) for r in range(6)]
    with mcx.Engine(descs) as eng:
        for r in range(6):
            eng.init_random(r, 90 + r)
        eng.sweep(20)
        eng.reset_stats()
        eng.sweep(30, measure=True)
        for idx in (list(range(6)), [0, 2, 5], [3]):
            got = eng.combine_stats(None if len(idx) == 6 else idx)
            want = OR.combine([[row] for row in _replica_rows(eng, idx)])[0]
            assert got["n"] == len(idx) and np.isnan(got["P"])
            np.testing.assert_allclose([got[k] for k in ("T", "S", "varS", "E", "varE")], want, rtol=1e-12)
        # a replica without measured sweeps, and temperatures more than 1e-3 apart
        eng.reset_stats(4)
        with pytest.raises(mcx.McxError, match="without measured sweeps"):
            eng.combine_stats()
        eng.combine_stats([0, 1])
        eng.set_temperature(1.01, 1)
        with pytest.raises(mcx.McxError, match="temperatures differ"):
            eng.combine_stats([0, 1])
        with pytest.raises(mcx.McxError):
            eng.combine_stats([0, 6])


def test_combine_stats_pear_polarization():
    m = O.Model(nx=8, ny=6, nz=10, potential="pear", B1=0.3, C=0.3)
    descs = [desc_from_model(m, T=0.8, seed=7 + r, stream=r) for r in range(3)]
    with mcx.Engine(descs) as eng:
        for r in range(3):
            eng.init_random(r, 5 + r)
        eng.sweep(10)
        eng.reset_stats()
        eng.sweep(12, measure=True)
        got = eng.combine_stats()
        want = OR.combine([[row] for row in _replica_rows(eng, range(3), pear=True)])[0]
    np.testing.assert_allclose([got[k] for k in ("T", "S", "varS", "E", "varE", "P")], want, rtol=1e-12)


def test_run_file_replicas_writes_combined_table(tmp_path):
    pf = tmp_path / "params.txt"
    pf.write_text(PARAMS + "replicas  3\n")
    mcx.run_file(str(pf), str(tmp_path) + "/")
    files = ["po.dat", "po_r1.dat", "po_r2.dat"]
    want = np.array(OR.combine([OR.read_po(str(tmp_path / f)) for f in files]))
    lines = (tmp_path / "po_avg.dat").read_text().splitlines()
    assert lines[0].split() == ["T", "S", "varS", "E", "varE"]
    got = np.array([[float(x) for x in ln.split()] for ln in lines[1:]])
    assert got.shape == want.shape == (3, 5)
    np.testing.assert_allclose(got, want, rtol=1e-3, atol=1e-7)
