"""The oracle restatement against golden vectors produced by the reference itself."""
import pytest
import sys, os
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from graphaligner_gb300.extend import ExtendParams
from golden_sets import MAX_CELLS, compare, golden_case, load_digests


@pytest.mark.parametrize("name,bandwidth", [("vg50k", 10), ("vg50k", 5), ("vg50k_hi", 10), ("dbg100k", 5), ("dbg100k", 10),
                                               ("iupac20k", 10), ("iupac20k", 5)])
def test_oracle_matches_reference(oracle_lib, name, bandwidth):
    g, batch = golden_case(name)
    expected = load_digests(name, bandwidth)
    res = oracle_lib.extend(g, ExtendParams(bandwidth=bandwidth, max_cells_per_slice=MAX_CELLS.get(name, 2**64 - 1)), batch, threads=4)
    bad = compare(res, expected)
    assert not bad, f"{len(bad)} of {len(expected)} extensions differ from the reference, first {bad[:5]}"
    if not name.startswith("iupac"):
        assert all(e[0] == 0 for e in expected)
