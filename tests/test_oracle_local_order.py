"""The oracle's local order parameter against the reference's own
lattice_order_parameter (src/parameter_order.cpp:62-113): the committed
golden (tests/golden/local_order.npz, made by make_local_order.py from the
reference compiled in oracle/_ref) and, where that build is present, a fresh
run of the reference on the same states."""
import numpy as np
import pytest

from helpers import load_local_order
from oracle import oracle as O
from oracle import refproc

CASES = load_local_order()


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_local_order_matches_reference_golden(name):
    m, pt, ni, S, _ = CASES[name]
    assert np.array_equal(O.Lattice(m).pt != 0, pt != 0)  # the oracle's mask is the reference's
    want = O.local_order(ni, pt, m)
    assert np.array_equal(np.isnan(S), np.isnan(want))
    ok = ~np.isnan(S)
    # the reference sums and solves in FP32: within a few ulps of S
    assert np.max(np.abs(S[ok] - want[ok])) < 5e-7


@pytest.mark.skipif(not refproc.available(), reason="reference build (oracle/_ref) not present")
def test_local_order_golden_is_the_reference_output(tmp_path):
    for name, (m, pt, ni, S, csv) in CASES.items():
        got, text = refproc.run(m, [("local_order", ni), ("print_n", ni, str(tmp_path / f"{name}.csv"))])
        assert np.array_equal(got, S, equal_nan=True), name
        assert csv is None or text == csv, name
