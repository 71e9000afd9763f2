"""The oracle restatement against golden vectors produced by the reference itself."""
import pytest
import sys, os
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from graphaligner_gb300.extend import ExtendParams
from golden_sets import MAX_CELLS, compare, golden_case, load_digests

CASES = [("vg50k", 10, None), ("vg50k", 5, None), ("vg50k_hi", 10, None), ("dbg100k", 5, None), ("dbg100k", 10, None),
         ("iupac20k", 10, None), ("iupac20k", 5, None), ("dbg1m", 5, None), ("dbg1m", 10, None)]
# bandwidths 1-40 and X-drop cutoffs 1500 / 3000 on extensions that they change
CASES += [("vg50k_px", bw, None) for bw in (10, 1, 3, 17, 40)] + [("vg50k_px", 10, x) for x in (1500, 3000)]


@pytest.mark.parametrize("name,bandwidth,xdrop", CASES)
def test_oracle_matches_reference(oracle_lib, name, bandwidth, xdrop):
    g, batch = golden_case(name)
    expected = load_digests(name, bandwidth, xdrop)
    p = ExtendParams(bandwidth=bandwidth, max_cells_per_slice=MAX_CELLS.get(name, 2**64 - 1))
    if xdrop is not None:
        p.xdrop = xdrop
    res = oracle_lib.extend(g, p, batch, threads=4)
    bad = compare(res, expected)
    assert not bad, f"{len(bad)} of {len(expected)} extensions differ from the reference, first {bad[:5]}"
    if not name.startswith("iupac"):
        assert all(e[0] == 0 for e in expected)
