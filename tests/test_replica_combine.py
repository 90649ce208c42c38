"""The replica combiner of the oracle (oracle/replicas.py) against the table
the reference's own average_replicas.py made of the same po.dat files
(tests/golden/replica_avg.json): equal columns, the common prefix of ragged
files, the skipped row whose temperatures differ, Pear's P column and a single
replica."""
import json
import os

import numpy as np
import pytest

from oracle import replicas as OR

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "replica_avg.json")


def _cases():
    return json.load(open(GOLD))


@pytest.mark.parametrize("name", sorted(_cases()))
def test_oracle_combine_matches_reference_script(name, tmp_path):
    case = _cases()[name]
    per_file = []
    for q, text in enumerate(case["files"]):
        p = tmp_path / f"po_{q}.dat"
        p.write_text(text)
        per_file.append(OR.read_po(str(p)))
    got = OR.combine(per_file)
    want = case["combined"]
    assert len(got) == len(want)
    np.testing.assert_allclose(np.array(got), np.array(want), rtol=1e-14, atol=0)


def test_oracle_combine_rejects_mixed_columns():
    with pytest.raises(OR.CombineError):
        OR.combine([[[1.0, 0.5, 0.1, -1.0, 0.2]], [[1.0, 0.5, 0.1, -1.0, 0.2, 0.3]]])


def test_po_row_from_running_sums():
    st = [4, 2.0, 1.1, -8.0, 16.4]
    row = OR.po_row(1.1, st, P=0.25)
    assert row == pytest.approx([1.1, 0.5, 1.1 / 4 - 0.25, -2.0, 16.4 / 4 - 4.0, 0.25])
