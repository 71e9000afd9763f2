"""The workload generators' graph side: the de Bruijn compactor and the GFA builder,
against brute force and against the reference-built graph of the same GFA."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from golden_sets import load_graph  # noqa: E402

from graphaligner_gb300 import datagen as dg  # noqa: E402
from graphaligner_gb300 import graph as gg  # noqa: E402


def _rc(s: str) -> str:
    return dg.revcomp(np.frombuffer(s.encode(), dtype=np.uint8)).tobytes().decode()


def _canon(x: str) -> str:
    return min(x, _rc(x))


def test_compact_dbg_brute_force():
    k = 33
    genome = dg.make_repeat_genome(20_000, 8, 800, 0.01, 0.03, 10, tandem_len=(100, 400), seed=3)
    gfa = dg.compact_dbg(genome, k)
    seqs, links = {}, []
    for line in gfa.splitlines():
        f = line.split("\t")
        if f[0] == "S":
            seqs[int(f[1])] = f[2]
        else:
            links.append((int(f[1]), f[2], int(f[3]), f[4], f[5]))
    gs = genome.tobytes().decode()
    owner = {}
    for u, s in seqs.items():
        for i in range(len(s) - k + 1):
            c = _canon(s[i:i + k])
            assert c not in owner, "a k-mer in two unitigs"
            owner[c] = u
    assert set(owner) == {_canon(gs[i:i + k]) for i in range(len(gs) - k + 1)}
    oriented = lambda u, o: seqs[u] if o == "+" else _rc(seqs[u])  # noqa: E731
    edges = set()
    for a, ao, b, bo, ov in links:
        assert ov == f"{k - 1}M"
        x, y = oriented(a, ao), oriented(b, bo)
        assert x[-(k - 1):] == y[:k - 1]
        edges.add((x[-k:], y[:k]))
        edges.add((_rc(y[:k]), _rc(x[-k:])))
    inside = set()
    for s in seqs.values():
        for i in range(len(s) - k):
            inside.add((s[i:i + k], s[i + 1:i + 1 + k]))
            inside.add((_rc(s[i + 1:i + 1 + k]), _rc(s[i:i + k])))
    for i in range(len(gs) - k):
        e = (gs[i:i + k], gs[i + 1:i + 1 + k])
        assert e in inside or e in edges


def test_dbg_positions_and_read_truth():
    genome = dg.small_dbg_genome(0)
    d = dg.compact_dbg(genome, 63, with_positions=True)
    seqs = {}
    for line in d.gfa.splitlines():
        f = line.split("\t")
        if f[0] == "S":
            seqs[int(f[1])] = f[2]
    strand = lambda bn: seqs[bn // 2] if bn % 2 == 0 else _rc(seqs[bn // 2])  # noqa: E731
    for p in range(0, len(genome), 97):
        assert strand(int(d.pos_bignode[p]))[int(d.pos_offset[p])] == chr(genome[p])
    for r in dg.dbg_reads(genome, 4, 3000, 0.12, 9, dbg=d):
        for j in np.nonzero(r.exact)[0][::11]:
            assert strand(int(r.bignode[j]))[int(r.bigoffset[j])] == chr(r.seq[j])


def _structure(g):
    key = [(int(g.node_ids[i]), int(g.node_offset[i]), int(g.node_length[i])) for i in range(g.num_nodes)]
    edges = set()
    for v in range(g.num_nodes):
        for e in range(int(g.out_offsets[v]), int(g.out_offsets[v + 1])):
            w = int(g.out_neighbors[e])
            edges.add((key[v], key[w], bool(g.component[v] == g.component[w]), bool(g.component[v] <= g.component[w])))
    return set(key), edges, len(set(g.component.tolist()))


def test_build_from_gfa_overlaps_matches_reference_graph():
    """Pieces, edges, strongly connected components and the topological direction of
    every edge equal those of the reference's build of the same k-1-overlap GFA."""
    d = dg.compact_dbg(dg.small_dbg_genome(0), 63)
    mine = _structure(gg.build_from_gfa(d))
    ref = _structure(load_graph("dbg100k"))
    assert mine == ref


def test_build_from_gfa_variation_graph_matches_reference_graph():
    mine = _structure(gg.build_from_gfa(dg.small_vg(0).to_gfa()))
    ref = _structure(load_graph("vg50k"))
    assert mine == ref


def test_build_from_gfa_iupac_matches_reference_graph():
    """Ambiguous (IUPAC) nodes: renumbered to the end, stored as 4-mask sequences; pieces,
    edges and components equal the reference's build of the same GFA."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(os.path.dirname(__file__), "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    g_src, _ = mg.iupac_edge_set(5)
    mine = gg.build_from_gfa(g_src.to_gfa())
    ref = load_graph("iupac20k")
    assert _structure(mine) == _structure(ref)
    assert mine.num_nodes - mine.first_ambiguous == ref.num_nodes - ref.first_ambiguous > 0
    # the same sequence masks for every ambiguous piece
    def amb(g):
        out = {}
        for k in range(g.num_nodes - g.first_ambiguous):
            i = g.first_ambiguous + k
            out[(int(g.node_ids[i]), int(g.node_offset[i]))] = tuple(int(x) for x in g.seq_ambiguous[4 * k:4 * k + 4])
        return out
    assert amb(mine) == amb(ref)


GRAPH_FIELDS = ["num_nodes", "first_ambiguous", "node_length", "node_ids", "node_offset", "reverse", "linearizable",
                "component", "chain_number", "chain_approx_pos", "seq2bit", "seq_ambiguous", "in_offsets", "in_neighbors",
                "out_offsets", "out_neighbors", "lookup_ids", "original_size", "lookup_offsets", "lookup_nodes", "names",
                "bp_size"]


def _differing_fields(a, b):
    bad = []
    for f in GRAPH_FIELDS:
        x, y = getattr(a, f), getattr(b, f)
        if isinstance(x, np.ndarray):
            if x.dtype != y.dtype or x.shape != y.shape or not np.array_equal(x, y):
                bad.append(f)
        elif x != y:
            bad.append(f)
    return bad


# numeric and named segments, links on both strands, overlaps, lower case, U, IUPAC codes,
# a segment longer than one piece, a self-loop and a bubble
HAND_GFA_NUMERIC = "\n".join([
    "H\tVN:Z:1.0",
    "S\t1\tACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTAC",
    "S\t2\tacgtnACGUu",
    "S\t3\tGGGCCCTTTAAA",
    "S\t4\tTTTT",
    "S\t5\tRYKMSWBDHVNacgt",
    "L\t1\t+\t2\t+\t0M",
    "L\t1\t+\t3\t+\t0M",
    "L\t2\t+\t4\t+\t0M",
    "L\t3\t+\t4\t+\t0M",
    "L\t4\t+\t4\t+\t0M",
    "L\t4\t-\t5\t+\t*",
    "L\t3\t+\t1\t-\t2M",
]) + "\n"
HAND_GFA_NAMED = HAND_GFA_NUMERIC.replace("\t1\t", "\tseg_one\t").replace("\t4\t", "\tfour\t")


def test_native_builder_equals_the_restatement():
    """graph.build_from_gfa (native, csrc/gfa_build.cpp) gives exactly the arrays of the
    Python restatement (tests/gfa_restatement.py): numbering, edges in order, components,
    chains and chain positions, sequences and names."""
    import gfa_restatement as gr
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(os.path.dirname(__file__), "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    cases = {
        "vg": dg.small_vg(0).to_gfa(),
        "vg_1m": dg.make_variation_graph(1_000_000, 100, 0.7, 20, 5).to_gfa(),
        "dbg": dg.compact_dbg(dg.small_dbg_genome(0), 63),
        "iupac": mg.iupac_edge_set(5)[0].to_gfa(),
        "hand_numeric": HAND_GFA_NUMERIC,
        "hand_named": HAND_GFA_NAMED,
        "crlf": HAND_GFA_NUMERIC.replace("\n", "\r\n"),
    }
    for name, text in cases.items():
        a, b = gg.build_from_gfa(text), gr.build_from_gfa(text)
        assert a.num_nodes > 0
        assert not _differing_fields(a, b), (name, _differing_fields(a, b))


def test_native_builder_refuses_what_it_cannot_build():
    import pytest
    from graphaligner_gb300._lib import GAError
    for bad in ["S\t1\tACGT\nL\t1\t+\t9\t+\t0M\n",          # link to an unknown segment
                "S\t1\tACGT\nS\t2\tACGT\nL\t1\t+\t2\t+\t4M\n",  # overlap not smaller than both
                "S\t1\t\n",                                    # empty segment
                "S\t1\tAC-GT\n",                               # not an IUPAC code
                "S\t1\tACGT\nS\t2\tACGT\nL\t1\t+\t2\t+\tx\n"]:  # overlap not a number
        with pytest.raises(GAError):
            gg.build_from_gfa(bad)


def _random_gfa(rng, numeric: bool) -> str:
    """Random segments (ACGT with some lower case, U and IUPAC codes), random links in
    both orientations with 0-bp or small overlaps, self-links and repeated links."""
    n = int(rng.integers(5, 40))
    names = [str(int(x)) for x in rng.choice(10_000, n, replace=False) + 1] if numeric else [f"s{k}x" for k in range(n)]
    alphabet = np.frombuffer(b"ACGTACGTACGTACGTacgtUNRYKMSWBDHV", dtype=np.uint8)
    weights = np.array([8.0] * 16 + [1.0] * 4 + [0.2] * 12)
    weights /= weights.sum()
    lens = rng.integers(1, 300, n)
    lines = []
    for name, length in zip(names, lens):
        seq = rng.choice(alphabet, int(length), p=weights).tobytes().decode()
        lines.append(f"S\t{name}\t{seq}")
    for _ in range(int(rng.integers(0, 3 * n))):
        a, b = int(rng.integers(0, n)), int(rng.integers(0, n))
        limit = int(min(lens[a], lens[b]))
        ov = 0 if rng.random() < 0.6 or limit <= 1 else int(rng.integers(1, limit))
        ov_text = "*" if ov == 0 and rng.random() < 0.2 else f"{ov}M"
        lines.append(f"L\t{names[a]}\t{'+-'[int(rng.integers(0, 2))]}\t{names[b]}\t{'+-'[int(rng.integers(0, 2))]}\t{ov_text}")
    return "\n".join(lines) + "\n"


def test_native_builder_equals_the_restatement_on_random_gfas():
    import gfa_restatement as gr
    rng = np.random.default_rng(2024)
    for k in range(60):
        text = _random_gfa(rng, numeric=k % 2 == 0)
        a, b = gg.build_from_gfa(text), gr.build_from_gfa(text)
        assert not _differing_fields(a, b), (k, _differing_fields(a, b), text)


def test_gag_round_trip(tmp_path):
    """save_gag then load_gag gives back every array of a built graph (the layout the
    reference-graph dumper writes and the harness reads)."""
    g = gg.build_from_gfa(HAND_GFA_NAMED)
    path = os.path.join(tmp_path, "g.gag")
    gg.save_gag(g, path)
    assert not _differing_fields(gg.load_gag(path), g)
    ref = load_graph("iupac20k")
    gg.save_gag(ref, path)
    assert not _differing_fields(gg.load_gag(path), ref)
