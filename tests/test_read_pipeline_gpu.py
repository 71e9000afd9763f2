"""The read-level path on the GPU (k-mer lookups and extensions as kernels)
against the reference's GAF."""
import gzip
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from golden_sets import GOLDEN, graph_file, load_gaf, load_graph, load_reads  # noqa: E402
from test_read_pipeline_host import INDEX_CASES, harness  # noqa: E402,F401  (the host read-level harness)
import subprocess  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bandwidth", [10, 5])
def test_gpu_gaf_matches_reference(cuda_lib, bandwidth):
    from graphaligner_gb300.align import Aligner, preset
    from graphaligner_gb300.extend import DeviceGraph, Extender
    g = load_graph("vg50k")
    names, seqs = load_reads("vg50k")
    x = Extender(DeviceGraph(g))
    a = Aligner(x, g, preset("vg", bandwidth=bandwidth))
    gaf = a.align(names, seqs)
    st = a.stats()
    assert st["failed_reads"] == 0
    assert gaf == load_gaf("vg50k", bandwidth)


def test_gpu_gaf_matches_reference_dbg(cuda_lib):
    """-x dbg (bandwidth 5, tangle effort 10000) on a k=63 de Bruijn graph with cyclic components."""
    from graphaligner_gb300.align import Aligner, preset
    from graphaligner_gb300.extend import DeviceGraph, Extender
    g = load_graph("dbg100k")
    names, seqs = load_reads("dbg100k")
    a = Aligner(Extender(DeviceGraph(g)), g, preset("dbg"))
    gaf = a.align(names, seqs)
    assert a.stats()["failed_reads"] == 0
    assert gaf == load_gaf("dbg100k", 5)


def test_gpu_gaf_matches_reference_dbg1m(cuda_lib):
    """-x dbg on the 1 Mbp de Bruijn stress graph (20 copies of a 5 kbp repeat, 40 tandem
    arrays): 20 reads of 20 kbp at 12 % error, GAF bytes against the reference's."""
    from graphaligner_gb300.align import Aligner, preset
    from graphaligner_gb300.extend import DeviceGraph, Extender
    g = load_graph("dbg1m")
    names, seqs = load_reads("dbg1m")
    a = Aligner(Extender(DeviceGraph(g)), g, preset("dbg"))
    gaf = a.align(names, seqs)
    assert a.stats()["failed_reads"] == 0
    assert gaf == load_gaf("dbg1m", 5)


def test_gpu_seeds_match_reference_on_edge_reads(cuda_lib):
    """getSeeds through the k-mer lookup kernel (one warp per read) on reads with homopolymer
    runs longer than k (iterateKmers' window rule for repeated k-mers), N runs and IUPAC codes
    (restarts), lower case, and lengths below, at and just above k, plus the golden reads: every
    read's seeds, in order, equal the reference's."""
    import hashlib
    from graphaligner_gb300.align import Aligner, preset
    from graphaligner_gb300.extend import DeviceGraph, Extender
    g = load_graph("vg50k")
    a = Aligner(Extender(DeviceGraph(g)), g, preset("vg"))
    for fasta, digest in (("vg50k_seed_edges.fa.gz", "vg50k_seed_edges_seeds.digest"), ("vg50k_reads.fa.gz", "vg50k_seeds.digest")):
        text = gzip.open(os.path.join(GOLDEN, fasta), "rt").read().split("\n")
        names = [line[1:].split()[0] for line in text if line.startswith(">")]
        seqs = [line.encode() for line in text if line and not line.startswith(">")]
        lines = []
        for name, seeds in zip(names, a.seeds(seqs)):
            lines.append(f"R {name} {len(seeds)}" + "".join(f" {s[0]},{s[1]},{s[2]},{s[3]},{s[4]},{s[5]},{s[6]},{s[7]}" for s in seeds))
        ref = open(os.path.join(GOLDEN, digest)).read().split()
        # the reference's output: a maxCount line, then per read its getSeeds line and its OrderSeeds line
        want = ref[1::2][:len(lines)]
        got = [hashlib.sha1(line.encode()).hexdigest() for line in lines]
        assert got == want, f"{fasta}: reads {[i for i, (x, y) in enumerate(zip(got, want)) if x != y][:5]} differ"


@pytest.mark.parametrize("name,k,w,discard", INDEX_CASES)
def test_gpu_index_matches_host_build(cuda_lib, harness, tmp_path, name, k, w, discard):  # noqa: F811
    """The minimizer index built on the GPU (per-node minimizer walk, radix sort by k-mer,
    reversed groups, maxCount, device lookup table) equals the host build array for array,
    and every key of the table the lookup kernel probes is found: the seeds of the golden
    reads through it equal the reference's on vg50k."""
    import numpy as np
    from graphaligner_gb300.align import Aligner, preset
    from graphaligner_gb300.extend import DeviceGraph, Extender
    exe = harness[0]
    gag = graph_file(name, str(tmp_path))
    prefix = os.path.join(tmp_path, "host")
    out = subprocess.run([exe, gag, harness[2], "indexdump", str(k), str(w), str(discard), prefix], check=True, capture_output=True,
                         text=True).stdout.split()
    f = dict(zip(out[0::2], (int(v) for v in out[1::2])))
    g = load_graph(name)
    p = preset("vg")
    p.minimizer_length, p.minimizer_window, p.minimizer_discard_fraction = k, w, discard
    a = Aligner(Extender(DeviceGraph(g)), g, p)
    info, keys, start, pos = a.index(arrays=True)
    assert info["max_count"] == f["maxCount"] and info["num_keys"] == f["keys"] and info["num_positions"] == f["positions"]
    assert info["table_capacity"] >= 2 * info["num_keys"]
    assert np.array_equal(keys, np.fromfile(prefix + ".keys", dtype=np.uint64))
    assert np.array_equal(start, np.fromfile(prefix + ".start", dtype=np.uint64))
    assert np.array_equal(pos, np.fromfile(prefix + ".pos", dtype=np.uint64))


def test_gpu_index_rejects_out_of_range_windows(cuda_lib):
    """Minimizer windows of more than 64 positions are refused with GA_ERR_ARGUMENT and a message."""
    from graphaligner_gb300._lib import GAError
    from graphaligner_gb300.align import Aligner, preset
    from graphaligner_gb300.extend import DeviceGraph, Extender
    g = load_graph("vg50k")
    p = preset("vg")
    p.minimizer_length, p.minimizer_window = 15, 79
    with pytest.raises(GAError, match="window"):
        Aligner(Extender(DeviceGraph(g)), g, p)


def test_gpu_quickstart(cuda_lib, tmp_path):
    from graphaligner_gb300 import graph as gg
    from graphaligner_gb300.align import Aligner, preset
    from graphaligner_gb300.extend import DeviceGraph, Extender
    path = os.path.join(tmp_path, "t.gag")
    open(path, "wb").write(gzip.open(os.path.join(GOLDEN, "test_graph.gag.gz")).read())
    g = gg.load_gag(path)
    lines = open(os.path.join(GOLDEN, "test_read.fa")).read().split()
    x = Extender(DeviceGraph(g))
    a = Aligner(x, g, preset("vg"))
    assert a.align([lines[0][1:]], [lines[1].encode()]) == open(os.path.join(GOLDEN, "test_graph.gaf")).read()


def test_gpu_two_lanes_gaf_matches_reference(cuda_lib):
    """400 reads take the two-extender path (two groups whose rounds alternate between the GPU
    and the host): the golden reads and renamed copies of them, each read's GAF the reference's."""
    from graphaligner_gb300.align import Aligner, preset
    from graphaligner_gb300.extend import DeviceGraph, Extender
    g = load_graph("vg50k")
    names, seqs = load_reads("vg50k")
    want = {}
    for line in load_gaf("vg50k", 10).splitlines(keepends=True):
        want.setdefault(line.split("\t", 1)[0], []).append(line)
    copies = [n + "_copy" for n in names]
    a = Aligner(Extender(DeviceGraph(g)), g, preset("vg"))
    gaf = a.align(names + copies, seqs + seqs)
    expected = "".join("".join(want.get(n, [])) for n in names)
    expected += "".join("".join(l.replace(n + "\t", n + "_copy\t", 1) for l in want.get(n, [])) for n in names)
    assert gaf == expected
    assert a.stats()["failed_reads"] == 0


def test_gpu_sequences_over_the_trace_limit_are_rejected(cuda_lib, tmp_path):
    """A sequence longer than GA_MAX_SEQ_LEN (its read positions would not fit the trace item)
    is refused with GA_ERR_ARGUMENT before anything is copied or launched, by the extension,
    read-level and serving entry points; the handles stay usable."""
    from graphaligner_gb300 import graph as gg
    from graphaligner_gb300._lib import GAError
    from graphaligner_gb300.align import Aligner, preset
    from graphaligner_gb300.extend import DeviceGraph, Extender, ExtendParams
    from graphaligner_gb300.serve import Server
    max_len = 33554431
    path = os.path.join(tmp_path, "t.gag")
    open(path, "wb").write(gzip.open(os.path.join(GOLDEN, "test_graph.gag.gz")).read())
    g = gg.load_gag(path)
    lines = open(os.path.join(GOLDEN, "test_read.fa")).read().split()
    x = Extender(DeviceGraph(g))
    a = Aligner(x, g, preset("vg"))
    long_read = b"A" * (max_len + 1)
    with pytest.raises(GAError):
        x.extend(ExtendParams(bandwidth=10), [long_read], [int(g.node_ids[0])], [0])
    with pytest.raises(GAError):
        a.align(["too_long"], [long_read])
    with Server(a) as srv:
        with pytest.raises(GAError):
            srv.submit("too_long", long_read)
    assert a.align([lines[0][1:]], [lines[1].encode()]) == open(os.path.join(GOLDEN, "test_graph.gaf")).read()
    res = x.extend(ExtendParams(bandwidth=10), [lines[1].encode()[:40]], [int(g.node_ids[0])], [0])
    assert res.status[0] in (0, 1)
