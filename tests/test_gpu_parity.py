"""GPU kernels against the reference's golden vectors and against the oracle."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from golden_sets import MAX_CELLS, compare, golden_case, load_digests  # noqa: E402

from graphaligner_gb300 import datagen as dg  # noqa: E402
from graphaligner_gb300 import graph as gg  # noqa: E402
from graphaligner_gb300.extend import DeviceGraph, Extender, ExtendParams, pack_batch  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden_vg():
    g, batch = golden_case("vg50k")
    dgraph = DeviceGraph(g)
    ext = Extender(dgraph)
    yield g, batch, ext
    ext.close()
    dgraph.close()


@pytest.mark.parametrize("bandwidth", [10, 5])
def test_gpu_matches_reference_golden(cuda_lib, golden_vg, bandwidth):
    g, batch, ext = golden_vg
    res = ext.run(ExtendParams(bandwidth=bandwidth), batch)
    bad = compare(res, load_digests("vg50k", bandwidth))
    assert not bad, f"{len(bad)} extensions differ from the reference, first {bad[:5]}"


def test_gpu_matches_reference_golden_high_error(cuda_lib):
    g, batch = golden_case("vg50k_hi")
    with_graph = DeviceGraph(g)
    ext = Extender(with_graph)
    res = ext.run(ExtendParams(bandwidth=10), batch)
    bad = compare(res, load_digests("vg50k_hi", 10))
    assert not bad, f"{len(bad)} extensions differ, first {bad[:5]}"


@pytest.mark.parametrize("bandwidth", [5, 10])
def test_gpu_matches_reference_golden_dbg(cuda_lib, bandwidth):
    """Cyclic components (k=63 de Bruijn graph with repeats and tandem arrays) at tangle effort 10000."""
    g, batch = golden_case("dbg100k")
    ext = Extender(DeviceGraph(g))
    res = ext.run(ExtendParams(bandwidth=bandwidth, max_cells_per_slice=MAX_CELLS["dbg100k"]), batch)
    bad = compare(res, load_digests("dbg100k", bandwidth))
    assert not bad, f"{len(bad)} extensions differ, first {bad[:5]}"


@pytest.fixture(scope="module")
def golden_px():
    g, batch = golden_case("vg50k_px")
    ext = Extender(DeviceGraph(g))
    yield batch, ext
    ext.close()


@pytest.mark.parametrize("bandwidth,xdrop", [(10, None), (1, None), (3, None), (17, None), (40, None), (10, 1500), (10, 3000)])
def test_gpu_matches_reference_golden_parameters(cuda_lib, golden_px, bandwidth, xdrop):
    """Bandwidths 1-40 (band admission, GraphAlignerBitvectorBanded.h:449-471) and X-drop cutoffs
    1500 and 3000 (the X-drop stop, :651-669) on extensions whose results they change: reads at
    12-25 % error, half of them with a random block the low cutoffs stop at."""
    batch, ext = golden_px
    p = ExtendParams(bandwidth=bandwidth)
    if xdrop is not None:
        p.xdrop = xdrop
    res = ext.run(p, batch)
    bad = compare(res, load_digests("vg50k_px", bandwidth, xdrop))
    assert not bad, f"{len(bad)} extensions differ from the reference, first {bad[:5]}"


@pytest.mark.parametrize("bandwidth", [5, 10])
def test_gpu_matches_reference_golden_dbg1m(cuda_lib, bandwidth):
    """The de Bruijn stress shape at 1 Mbp (20 copies of a 5 kbp repeat at 1-3 %, 40 tandem
    arrays; k=63): extensions of 20 kbp reads at 12 % error at tangle effort 10000, against the
    reference.  Extensions whose bands outgrow the shared-memory tables are re-run with larger
    ones, so the digests also pin that path."""
    g, batch = golden_case("dbg1m")
    ext = Extender(DeviceGraph(g))
    res = ext.run(ExtendParams(bandwidth=bandwidth, max_cells_per_slice=MAX_CELLS["dbg1m"]), batch)
    bad = compare(res, load_digests("dbg1m", bandwidth))
    assert not bad, f"{len(bad)} extensions differ, first {bad[:5]}"
    print("layout counts", ext.last_layout_counts())


def test_gpu_matches_oracle_dbg_generated(cuda_lib, oracle_lib):
    """A second de Bruijn graph built here (own numbering), GPU against the oracle on the same arrays,
    with tangle efforts that do and do not cut the band."""
    genome = dg.make_repeat_genome(60_000, 12, 1_500, 0.01, 0.03, 15, tandem_len=(200, 800), seed=21)
    d = dg.compact_dbg(genome, 63, with_positions=True)
    g = gg.build_from_gfa(d.gfa)
    reads = dg.sample_genome_reads(genome, 60, 22, dg.uniform_length(300, 10_000), dg.uniform_error(0.05, 0.15), dbg=d)
    ext = dg.seed_extensions(reads, d.node_len, 15, 23, per_read=2)
    batch = pack_batch(g, ext.seqs, ext.bignode, ext.offset)
    x = Extender(DeviceGraph(g))
    for bw, cells, xdrop in ((5, 10000, None), (10, 10000, None), (5, 500, None), (1, 10000, None), (3, 10000, None),
                             (17, 10000, None), (40, 2000, None), (5, 10000, 1500), (5, 10000, 3000)):
        p = ExtendParams(bandwidth=bw, max_cells_per_slice=cells)
        if xdrop is not None:
            p.xdrop = xdrop
        gpu = x.run(p, batch)
        ref = oracle_lib.extend(g, p, batch, threads=8)
        _assert_same(gpu, ref, batch.num)


def _assert_same(a, b, n):
    assert np.array_equal(a.status[:n], b.status[:n])
    assert np.array_equal(a.score[:n], b.score[:n])
    assert np.array_equal(a.trace_len[:n], b.trace_len[:n])
    for i in range(n):
        assert np.array_equal(a.items(i), b.items(i)), f"trace {i} differs"


def test_gpu_matches_oracle_generated(cuda_lib, oracle_lib):
    vg = dg.small_vg(11)
    g = gg.build_from_gfa(vg.to_gfa())
    nl = np.zeros(len(vg.node_seqs) + 1, dtype=np.int64)
    nl[1:] = [len(s) for s in vg.node_seqs]
    reads = dg.sample_reads(vg, 80, 12, dg.uniform_length(200, 12_000), dg.uniform_error(0.03, 0.2))
    ext = dg.seed_extensions(reads, nl, 15, 13, per_read=2)
    batch = pack_batch(g, ext.seqs, ext.bignode, ext.offset)
    dgraph = DeviceGraph(g)
    x = Extender(dgraph)
    unlimited = 2**64 - 1
    for bw, cells, xdrop in ((10, unlimited, None), (5, unlimited, None), (10, 300, None), (1, unlimited, None),
                             (3, unlimited, None), (17, unlimited, None), (40, unlimited, None), (10, unlimited, 1500),
                             (10, unlimited, 3000)):
        p = ExtendParams(bandwidth=bw, max_cells_per_slice=cells)
        if xdrop is not None:
            p.xdrop = xdrop
        gpu = x.run(p, batch)
        ref = oracle_lib.extend(g, p, batch, threads=8)
        _assert_same(gpu, ref, batch.num)


def test_launch_shapes_do_not_change_results(cuda_lib):
    """How the kernels are launched never changes a result: every launch shape (warps per block,
    resident blocks, first table layout, arena chunk, including chunks smaller than one slice
    record) gives the reference's digests."""
    from graphaligner_gb300._lib import GAError
    g, batch = golden_case("vg50k")
    x = Extender(DeviceGraph(g))
    expected = load_digests("vg50k", 10)
    for shape in [(4, 0, 0, 64), (1, 1, 0, 128), (2, 0, 1, 64), (3, 2, 2, 8), (4, 0, 0, 1)]:
        x.set_launch_shape(*shape)
        res = x.run(ExtendParams(bandwidth=10), batch)
        bad = compare(res, expected)
        assert not bad, f"shape {shape}: {len(bad)} extensions differ"
    with pytest.raises(GAError):
        x.set_launch_shape(0, 0, 0, 128)
    with pytest.raises(GAError):
        x.set_launch_shape(5, 0, 0, 128)
    with pytest.raises(GAError):
        x.set_launch_shape(4, 0, 3, 128)
    with pytest.raises(GAError):
        x.set_launch_shape(4, 0, 0, 0)
    cands = [(4, 0, 0, 64), (1, 0, 0, 16), (2, 2, 1, 128)]
    tuned = x.autotune(ExtendParams(bandwidth=10), batch, candidates=cands, sample_every=2, repeats=1)
    assert len(tuned["candidates_ms"]) == len(cands) and all(ms > 0 for ms, _ in tuned["candidates_ms"])
    best_ms = min(ms for ms, _ in tuned["candidates_ms"])
    chosen = tuple(tuned["chosen"].values())
    assert chosen in [tuple(c) for ms, c in tuned["candidates_ms"] if ms == best_ms]
    assert not compare(x.run(ExtendParams(bandwidth=10), batch), expected)
    with pytest.raises(GAError):
        x.autotune(ExtendParams(bandwidth=10), batch, candidates=[(8, 0, 0, 128)])


def test_table_layouts_agree_on_dbg(cuda_lib):
    """The de Bruijn set outgrows the shared-memory tables: whichever layout a run starts with,
    the extensions that overflow are re-run with larger tables and every digest is the reference's."""
    g, batch = golden_case("dbg100k")
    x = Extender(DeviceGraph(g))
    expected = load_digests("dbg100k", 10)
    p = ExtendParams(bandwidth=10, max_cells_per_slice=MAX_CELLS["dbg100k"])
    for layout in (0, 1, 2):
        x.set_launch_shape(4, 0, layout, 64)
        res = x.run(p, batch)
        bad = compare(res, expected)
        assert not bad, f"first layout {layout}: {len(bad)} extensions differ"
        counts = x.last_layout_counts()
        assert counts[layout] == batch.num and all(c == 0 for c in counts[:layout])


@pytest.mark.parametrize("bandwidth", [10, 5])
def test_gpu_matches_reference_golden_iupac_edges(cuda_lib, bandwidth):
    """IUPAC codes in graph nodes (ambiguous-node storage) and in reads, lower case (on which
    the reference's traceback asserts), and edge requests: lengths 1-2, 63-65, 127-129,
    starts on a node's first and last base.  Statuses, including the asserts, must match."""
    g, batch = golden_case("iupac20k")
    assert g.first_ambiguous < g.num_nodes
    ext = Extender(DeviceGraph(g))
    res = ext.run(ExtendParams(bandwidth=bandwidth), batch)
    expected = load_digests("iupac20k", bandwidth)
    bad = compare(res, expected)
    assert not bad, f"{len(bad)} extensions differ, first {bad[:5]}"
    assert sum(1 for e in expected if e[0] == 2) > 0 and sum(1 for e in expected if e[0] == 0) > 0
