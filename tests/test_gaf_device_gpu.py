"""Alignment selection and GAF lines on the GPU, through their C ABI: ga_aligner_select_alignments
against SelectAlignments' rules, and ga_aligner_format_gaf on hand-made traces.  (Every GAF
golden of the read-level GPU tests also goes through both.)"""
import ctypes
import gzip
import os
import sys
import tempfile

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from golden_sets import GOLDEN  # noqa: E402

pytestmark = pytest.mark.gpu


def quickstart_aligner():
    from graphaligner_gb300 import graph as gg
    from graphaligner_gb300.align import Aligner, preset
    from graphaligner_gb300.extend import DeviceGraph, Extender
    with tempfile.NamedTemporaryFile(suffix=".gag") as f:
        f.write(gzip.open(os.path.join(GOLDEN, "test_graph.gag.gz")).read())
        f.flush()
        g = gg.load_gag(f.name)
    return g, Aligner(Extender(DeviceGraph(g)), g, preset("vg"))


def incompatible(l, r):
    """AlignmentSelection::alignmentIncompatible in float32, as the reference computes it."""
    min_overlap = np.float32(min(l[1] - l[0], r[1] - r[0])) * np.float32(0.05)
    (ls, le), (rs, re_) = sorted([(l[0], l[1]), (r[0], r[1])])
    overlap = le - rs if le > rs else 0
    return np.float32(overlap) > min_overlap


def select_ref(alns, min_score, fraction):
    """AlignmentSelection::SelectAlignments without the E-value filter, as kept flags."""
    idx = list(range(len(alns)))
    if min_score > -2**31:
        idx = [i for i in idx if alns[i][2] >= min_score]
    if fraction != 0:
        idx = [i for i in idx if not any(j != i and incompatible(alns[i], alns[j]) and alns[i][2] < alns[j][2] * fraction for j in idx)]
    keep = [False] * len(alns)
    for i in idx:
        keep[i] = True
    return keep


def test_gpu_select_alignments_matches_rules(cuda_lib):
    """Random reads of 1-12 alignments with overlapping spans and close X-scores, at several
    score cuts and multimap fractions."""
    _, a = quickstart_aligner()
    rng = np.random.default_rng(5)
    reads = []
    for _ in range(400):
        k = int(rng.integers(1, 13))
        alns = []
        for _ in range(k):
            s = int(rng.integers(0, 20000))
            e = s + int(rng.integers(1, 8000))
            alns.append((s, e, float(np.round(rng.uniform(-50, 300), 2))))
        reads.append(alns)
    for min_score, fraction in ((0, 0.9), (-2**31, 0.9), (100, 0.5), (0, 0.0), (-2**31, 0.0)):
        got = a.select_alignments(reads, min_score, fraction)
        want = [select_ref(r, min_score, fraction) for r in reads]
        assert got == want, (min_score, fraction)


def gaf_call(a, lines, items, names, lens, merge=0):
    from graphaligner_gb300._lib import check
    L = cuda_lib_handle()
    ln = np.array(lines, dtype=[("first_item", "<u8"), ("item_count", "<u4"), ("read", "<u4"), ("xscore100", "<i4"), ("mapq", "<i4")])
    it = np.array(items, dtype=[("node", "<i4"), ("node_offset", "<u4"), ("seq_pos", "<u4"), ("node_switch", "u1"), ("seq_char", "u1"),
                                ("graph_char", "u1"), ("pad", "u1")])
    cnames = (ctypes.c_char_p * len(names))(*[n.encode() for n in names])
    clens = (ctypes.c_uint32 * len(lens))(*lens)
    text = ctypes.c_char_p()
    nbytes = ctypes.c_uint64()
    ends = ctypes.POINTER(ctypes.c_uint64)()
    failed = ctypes.POINTER(ctypes.c_uint8)()
    check(L.ga_aligner_format_gaf(a.handle, len(lines), ln.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint64(len(items)),
                                  it.ctypes.data_as(ctypes.c_void_p), len(names), cnames, clens, ctypes.c_uint8(merge), ctypes.byref(text),
                                  ctypes.byref(nbytes), ctypes.byref(ends), ctypes.byref(failed)))
    body = ctypes.string_at(text, nbytes.value).decode()
    return body, [ends[k] for k in range(len(lines))], [failed[k] for k in range(len(lines))]


def cuda_lib_handle():
    from graphaligner_gb300._lib import lib
    return lib()


def test_gpu_format_gaf_lines(cuda_lib):
    """Hand-made traces on the quickstart graph: a run of matches, a mismatch, an insertion and a
    deletion, a node switch, AS:f left out for an X-score of -1, and a character outside the
    IUPAC set (the reference would assert: the line is marked failed)."""
    g, a = quickstart_aligner()
    lookup = {int(x): i for i, x in enumerate(g.lookup_ids)}
    size = {b: int(g.original_size[i]) for b, i in lookup.items()}
    # GFA nodes 1 and 2, forward strand (bigraph ids 2 and 4); unnamed nodes print their GFA id
    node1, node2 = 2, 4
    assert node1 in lookup and node2 in lookup and g.names[lookup[node1]] in ("", "1") and g.names[lookup[node2]] in ("", "2")
    # the formatter only compares the read and graph characters of an item; A throughout
    items = []
    # line 0: 4 matches on node 1
    for k in range(4):
        items.append((node1, k, k, 0, ord("A"), ord("A"), 0))
    # line 1: match, mismatch, insertion (same node offset), deletion (same read position), switch to node 2
    base = len(items)
    items += [(node1, 0, 0, 0, ord("A"), ord("A"), 0), (node1, 1, 1, 0, ord("C"), ord("A"), 0), (node1, 1, 2, 0, ord("A"), ord("A"), 0),
              (node1, 2, 2, 0, ord("A"), ord("A"), 0), (node1, size[node1] - 1, 3, 1, ord("A"), ord("A"), 0), (node2, 0, 4, 0, ord("A"), ord("A"), 0)]
    # line 2: a bad character
    bad = len(items)
    items += [(node1, 0, 0, 0, ord("!"), ord("A"), 0)]
    lines = [(0, 4, 0, 350, 60), (base, 6, 1, -100, 7), (bad, 1, 0, 100, 60)]
    body, ends, failed = gaf_call(a, lines, items, ["r0", "r1"], [4, 5])
    assert failed == [0, 0, 1]
    out = body.split("\n")
    assert out[0] == f"r0\t4\t0\t4\t+\t>1\t{size[node1]}\t0\t4\t4\t4\t60\tNM:i:0\tAS:f:3.5\tdv:f:0\tid:f:1\tcg:Z:4="
    f = out[1].split("\t")
    assert f[:5] == ["r1", "5", "0", "5", "+"] and f[5] == ">1>2"
    assert f[9] == "3" and f[10] == "6" and f[11] == "7" and f[12] == "NM:i:3" and not any(x.startswith("AS:f:") for x in f)
    assert f[-1] == "cg:Z:1=1X1I1D2="
    assert out[2] == "" and ends[-1] == len(body)
