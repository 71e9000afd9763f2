"""The multiseed DP (--multiseed-DP 1) on the GPU: ga_multiseed_batch against the oracle's
multiseed DP trace for trace, and ga_align_reads with multiseed_dp against the reference's
GAF byte for byte."""
import gzip
import os
import subprocess
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from golden_sets import GOLDEN, graph_file, load_graph  # noqa: E402
from test_read_pipeline_host import MULTISEED_CASES, harness  # noqa: E402,F401  (the host read-level harness)

pytestmark = pytest.mark.gpu


def read_fasta(name):
    text = gzip.open(os.path.join(GOLDEN, f"{name}.fa.gz"), "rt").read().split("\n")
    names = [line[1:].split()[0] for line in text if line.startswith(">")]
    seqs = [line.encode() for line in text if line and not line.startswith(">")]
    return names, seqs


def multiseed_seeds(exe, graph, reads, dbg, tmp_path):
    """prepareSeedsForMultiseeding's (slice, split node) pairs per read, from the harness."""
    fa = os.path.join(tmp_path, "reads.fa")
    open(fa, "wb").write(gzip.open(os.path.join(GOLDEN, f"{reads}.fa.gz")).read())
    out = subprocess.run([exe, graph_file(graph, str(tmp_path)), fa, "msseedsdbg" if dbg else "msseeds"], check=True,
                         capture_output=True, text=True).stdout.splitlines()
    seeds = []
    for line in out:
        f = line.split()
        v = list(map(int, f[2:]))
        seeds.append([(v[2 * k], v[2 * k + 1]) for k in range(int(f[1]))])
    return seeds


TRACE_CASES = [("vg50k", "vg50k_chimera_reads", False, 10), ("vg50k", "vg50k_reads", False, 5), ("dbg100k", "dbg100k_reads", True, 5)]


@pytest.mark.parametrize("graph,reads,dbg,bandwidth", TRACE_CASES)
def test_gpu_multiseed_traces_match_oracle(cuda_lib, oracle_lib, harness, tmp_path, graph, reads, dbg, bandwidth):  # noqa: F811
    """Every read's status, number of traces, and each trace's score and packed items (in the
    reference's order) equal the oracle's multiseed DP: seeds started in their slices, seed-start
    columns merged into the node columns, local maxima over slices and neighbours, traces that
    end at a seed start."""
    from graphaligner_gb300.extend import DeviceGraph, Extender, ExtendParams, MultiseedBatch
    g = load_graph(graph)
    _, seqs = read_fasta(reads)
    seeds = multiseed_seeds(harness[0], graph, reads, dbg, tmp_path)
    assert len(seeds) == len(seqs)
    batch = MultiseedBatch.pack(seqs, seeds, max_traces=256, items_per_bp=64)
    p = ExtendParams(bandwidth=bandwidth, max_cells_per_slice=10000 if dbg else 2**64 - 1)
    gpu = Extender(DeviceGraph(g)).multiseed(p, batch)
    cpu = oracle_lib.multiseed(g, p, batch, threads=8)
    assert (cpu.status == 0).all()
    assert np.array_equal(gpu.status, cpu.status), np.nonzero(gpu.status != cpu.status)[0][:10]
    assert np.array_equal(gpu.num_traces, cpu.num_traces)
    bad = []
    for i in range(batch.num):
        for (gs, gi), (cs, ci) in zip(gpu.traces(i), cpu.traces(i)):
            if gs != cs or not np.array_equal(gi, ci):
                bad.append(i)
                break
    assert not bad, f"reads {bad[:10]} differ"
    assert int(cpu.num_traces.sum()) > batch.num
    # with exact room: removeDuplicateTraces' survivors of the same traces, in room sized to them
    ex = Extender(DeviceGraph(g)).multiseed_exact(p, batch)
    assert np.array_equal(ex.status, cpu.status)
    assert int(ex.trace_len.sum()) == len(ex.trace_items)
    for i in range(batch.num):
        assert_deduplicated(ex.traces(i), cpu.traces(i), p.xscore_error_cost)
    assert int(ex.num_traces.sum()) <= int(cpu.num_traces.sum())


def _start_cell(items):
    return int(items[-1]) & ~(1 << 38)


def _sort_score(score, items, cost):
    first, last = (int(items[0]) >> 39) - 1, (int(items[-1]) >> 39) - 1
    return ((first - last + 1) * 100 - score * cost + 2**31) % 2**32 - 2**31


def assert_deduplicated(got, traces, cost):
    """got is removeDuplicateTraces applied to traces: one trace per start cell, each one of the
    given traces, and where a start cell's traces differ in their sort key the survivor has the
    greatest (ties go by std::sort's arrangement, which the GAF goldens pin)."""
    cells = {}
    for score, items in traces:
        cells.setdefault(_start_cell(items), []).append((_sort_score(score, items, cost), score, items))
    seen = set()
    for score, items in got:
        cell = _start_cell(items)
        assert cell not in seen
        seen.add(cell)
        group = cells[cell]
        assert any(score == s and np.array_equal(items, it) for _, s, it in group)
        best = max(k for k, _, _ in group)
        if sum(1 for k, _, _ in group if k == best) == 1:
            assert _sort_score(score, items, cost) == best
    assert seen == set(cells)


def test_gpu_multiseed_reports_capacity(cuda_lib, oracle_lib, harness, tmp_path):  # noqa: F811
    """With room for eight traces per read, the chimeric reads that have more report GA_CAPACITY,
    as the oracle does, and the others keep their traces."""
    from graphaligner_gb300.extend import DeviceGraph, Extender, ExtendParams, MultiseedBatch
    g = load_graph("vg50k")
    _, seqs = read_fasta("vg50k_chimera_reads")
    seeds = multiseed_seeds(harness[0], "vg50k", "vg50k_chimera_reads", False, tmp_path)
    batch = MultiseedBatch.pack(seqs, seeds, max_traces=8, items_per_bp=64)
    p = ExtendParams(bandwidth=10)
    gpu = Extender(DeviceGraph(g)).multiseed(p, batch)
    cpu = oracle_lib.multiseed(g, p, batch, threads=8)
    assert np.array_equal(gpu.status, cpu.status)
    assert 0 < int((cpu.status == 3).sum()) < batch.num
    # the room the overflowing reads need, counted on the device as the oracle counts it
    assert np.array_equal(gpu.items_needed, cpu.items_needed) and np.array_equal(gpu.traces_needed, cpu.traces_needed)
    for i in np.nonzero(cpu.status == 0)[0]:
        assert [(s, list(t)) for s, t in gpu.traces(int(i))] == [(s, list(t)) for s, t in cpu.traces(int(i))]


def test_gpu_multiseed_exact_room_over_several_passes(cuda_lib, harness, tmp_path):  # noqa: F811
    """With a DP-table arena far too small for the batch, reads that find it exhausted run
    again in later passes, each pass giving its finished reads their room after the earlier
    passes' traces; statuses, trace counts and every trace equal a run with room to spare, in
    both the exact-room and the caller's-room forms."""
    from graphaligner_gb300.extend import DeviceGraph, Extender, ExtendParams, MultiseedBatch
    g = load_graph("vg50k")
    _, seqs = read_fasta("vg50k_chimera_reads")
    seeds = multiseed_seeds(harness[0], "vg50k", "vg50k_chimera_reads", False, tmp_path)
    batch = MultiseedBatch.pack(seqs, seeds, max_traces=256, items_per_bp=64)
    p = ExtendParams(bandwidth=10)
    dg = DeviceGraph(g)
    roomy = Extender(dg)
    want = roomy.multiseed_exact(p, batch)
    need = roomy.last_arena_bytes()
    want_cap = roomy.multiseed(p, batch)
    # two thirds of what the batch takes: the reads that are short of it when it runs out go
    # again with a fresh arena
    tight = Extender(dg, arena_bytes=max(need * 2 // 3, 1 << 20))
    got = tight.multiseed_exact(p, batch)
    passes = sum(tight.last_layout_counts())
    got_cap = tight.multiseed(p, batch)
    assert passes > batch.num, "the small arena should have sent reads to a second pass"
    assert (want.status == 0).all()
    assert np.array_equal(got.status, want.status) and np.array_equal(got.num_traces, want.num_traces)
    for i in range(batch.num):
        assert [(s, list(t)) for s, t in got.traces(i)] == [(s, list(t)) for s, t in want.traces(i)]
    assert np.array_equal(got_cap.status, want_cap.status) and np.array_equal(got_cap.num_traces, want_cap.num_traces)
    for i in range(batch.num):
        assert [(s, list(t)) for s, t in got_cap.traces(i)] == [(s, list(t)) for s, t in want_cap.traces(i)]


def test_gpu_multiseed_rejects_bad_seeds(cuda_lib):
    """Seeds outside the graph, beyond their read or out of slice order are GA_ERR_ARGUMENT."""
    from graphaligner_gb300._lib import GAError
    from graphaligner_gb300.extend import DeviceGraph, Extender, ExtendParams, MultiseedBatch
    g = load_graph("vg50k")
    x = Extender(DeviceGraph(g))
    seq = [b"ACGT" * 100]
    for seeds in ([(0, g.num_nodes)], [(7, 0)], [(2, 0), (1, 0)]):
        with pytest.raises(GAError, match="seed"):
            x.multiseed(ExtendParams(bandwidth=10), MultiseedBatch.pack(seq, [seeds]))


@pytest.mark.parametrize("graph,reads,mode,bandwidth,gaf", MULTISEED_CASES)
def test_gpu_multiseed_gaf_matches_reference(cuda_lib, graph, reads, mode, bandwidth, gaf):
    """ga_align_reads with multiseed_dp: GAF bytes equal to the reference's --multiseed-DP 1."""
    from graphaligner_gb300.align import Aligner, preset
    from graphaligner_gb300.extend import DeviceGraph, Extender
    g = load_graph(graph)
    names, seqs = read_fasta(reads)
    dbg = mode.endswith("dbg")
    a = Aligner(Extender(DeviceGraph(g)), g, preset("dbg" if dbg else "vg", bandwidth=bandwidth, multiseed=True))
    out = a.align(names, seqs)
    assert a.stats()["failed_reads"] == 0
    assert out == gzip.open(os.path.join(GOLDEN, f"{gaf}.gaf.gz"), "rt").read()
