"""The package's read-level host logic (minimizer index, seed selection and
ordering, the seed loop, trace fix-up and merge, selection, GAF) driven by the
oracle's extensions, against the reference's own seeds and GAF."""
import hashlib
import os
import subprocess
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from golden_sets import GOLDEN, graph_file, load_gaf  # noqa: E402

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
BUILD = os.path.join(ROOT, "tests", "_build")
HARNESS = os.path.join(BUILD, "pipeline")
SOURCES = [os.path.join(ROOT, "tests", "harness", "pipeline.cpp"),
           os.path.join(ROOT, "graphaligner_gb300", "csrc", "readalign.cpp"),
           os.path.join(ROOT, "graphaligner_gb300", "csrc", "seeding.cpp"),
           os.path.join(ROOT, "oracle", "ga_oracle.cpp")]


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    os.makedirs(BUILD, exist_ok=True)
    deps = SOURCES + [os.path.join(ROOT, "graphaligner_gb300", "csrc", "readalign.h"), os.path.join(ROOT, "graphaligner_gb300", "csrc", "index_walk.cuh"), os.path.join(ROOT, "graphaligner_gb300", "csrc", "gaf_format.cuh"), os.path.join(ROOT, "graphaligner_gb300", "csrc", "seed_table.h"), os.path.join(ROOT, "graphaligner_gb300", "csrc", "trace_dedupe.h"), os.path.join(ROOT, "include", "graphaligner_gb300.h")]
    if not os.path.exists(HARNESS) or os.path.getmtime(HARNESS) < max(os.path.getmtime(d) for d in deps):
        subprocess.run(["g++", "-std=c++17", "-O2", "-o", HARNESS, *SOURCES, "-lpthread"], check=True)
    d = tmp_path_factory.mktemp("pipeline")
    import gzip
    reads = os.path.join(d, "reads.fa")
    open(reads, "wb").write(gzip.open(os.path.join(GOLDEN, "vg50k_reads.fa.gz")).read())
    return HARNESS, graph_file("vg50k", str(d)), reads, d


def test_seeds_match_reference(harness):
    exe, gag, reads, _ = harness
    out = subprocess.run([exe, gag, reads, "seeds", "15", "20", "10", "0.001"], check=True, capture_output=True, text=True).stdout
    mine = [hashlib.sha1(line.encode()).hexdigest() for line in out.splitlines()]
    ref = open(os.path.join(GOLDEN, "vg50k_seeds.digest")).read().split()
    assert mine == ref


def test_seeds_match_reference_on_edge_reads(harness, tmp_path):
    """getSeeds and OrderSeeds on reads with homopolymer runs longer than k (iterateKmers' window
    rule for repeated k-mers), N runs and IUPAC codes (restarts), lower case, and lengths below,
    at and just above k: every output line equals the reference's."""
    import gzip
    exe, gag, _, _ = harness
    reads = os.path.join(tmp_path, "edges.fa")
    open(reads, "wb").write(gzip.open(os.path.join(GOLDEN, "vg50k_seed_edges.fa.gz")).read())
    out = subprocess.run([exe, gag, reads, "seeds", "15", "20", "10", "0.001"], check=True, capture_output=True, text=True).stdout
    mine = [hashlib.sha1(line.encode()).hexdigest() for line in out.splitlines()]
    assert mine == open(os.path.join(GOLDEN, "vg50k_seed_edges_seeds.digest")).read().split()


@pytest.mark.parametrize("name,k,w,discard", [("vg50k", 15, 20, 0.001), ("dbg100k", 19, 30, 0.0002)])
def test_seed_table_finds_every_key(harness, tmp_path, name, k, w, discard):
    """The k-mer table the lookup kernel probes, built on all cores: every k-mer of the index
    is found with its group, and k-mers outside the index are not."""
    exe, _, reads, _ = harness
    out = subprocess.run([exe, graph_file(name, str(tmp_path)), reads, "table", str(k), str(w), str(discard)],
                         check=True, capture_output=True, text=True).stdout.split()
    f = dict(zip(out[0::2], (int(v) for v in out[1::2])))
    assert f["keys"] > 10000 and f["used"] == f["keys"] and f["capacity"] >= 2 * f["keys"]
    assert f["bad"] == 0 and f["absent_found"] == 0


INDEX_CASES = [("vg50k", 15, 20, 0.001), ("dbg100k", 19, 30, 0.0002), ("iupac20k", 15, 20, 0.001), ("dbg1m", 19, 30, 0.0002),
               ("vg50k", 11, 11, 0.001), ("vg50k", 5, 8, 0.001), ("vg50k", 31, 94, 0.01), ("iupac20k", 11, 40, 0.001)]


@pytest.mark.parametrize("name,k,w,discard", INDEX_CASES)
def test_index_walk_matches_host_build(harness, tmp_path, name, k, w, discard):
    """The GPU index build's per-node minimizer walk (index_walk.cuh, compiled for the host),
    its occurrences grouped by k-mer with insertion order reversed, gives the host build's
    keys, start positions and positions: IUPAC pieces, nodes exactly one window long (the
    initial window reads the end of the node), windows of 1 and of 64 minimizer positions,
    k = 5 (groups of hundreds of occurrences)."""
    exe, _, reads, _ = harness
    out = subprocess.run([exe, graph_file(name, str(tmp_path)), reads, "walk", str(k), str(w), str(discard)],
                         check=True, capture_output=True, text=True).stdout.split()
    f = dict(zip(out[0::2], (int(v) for v in out[1::2])))
    assert f["bad"] == 0 and f["occurrences"] > 1000 and f["equal"] == 1, f


@pytest.mark.parametrize("bandwidth", [10, 5])
def test_gaf_matches_reference(harness, oracle_lib, bandwidth):
    exe, gag, reads, _ = harness
    out = subprocess.run([exe, gag, reads, "gaf", str(bandwidth)], check=True, capture_output=True, text=True).stdout
    assert out == load_gaf("vg50k", bandwidth)


def test_gaf_same_when_reads_join_between_rounds(harness, oracle_lib):
    """Reads admitted 7 per round (the serving loop's continuous batching): every
    read's GAF is the reference's, byte for byte."""
    exe, gag, reads, _ = harness
    out = subprocess.run([exe, gag, reads, "gafmix", "10"], check=True, capture_output=True, text=True).stdout
    assert out == load_gaf("vg50k", 10)


def test_gaf_same_with_two_alternating_groups(harness, oracle_lib):
    """The two-lane driver (reads in two groups, one group's round on the worker while the
    other is finished) gives the reference's GAF."""
    exe, gag, reads, _ = harness
    out = subprocess.run([exe, gag, reads, "gaf2", "10"], check=True, capture_output=True, text=True).stdout
    assert out == load_gaf("vg50k", 10)


def test_reads_without_seeds(harness, oracle_lib, tmp_path):
    """Reads that give no seed (shorter than k, all N, empty between others) write no GAF line
    and leave every other read's lines unchanged."""
    import gzip
    exe, gag, reads, _ = harness
    text = gzip.open(os.path.join(GOLDEN, "vg50k_reads.fa.gz"), "rt").read().splitlines()
    extra = [">tiny", "ACGTACGTAC", ">alln", "N" * 3000, ">one", "A"]
    mixed = text[:40] + extra + text[40:]
    path = os.path.join(tmp_path, "mixed.fa")
    open(path, "w").write("\n".join(mixed) + "\n")
    out = subprocess.run([exe, gag, path, "gaf", "10"], check=True, capture_output=True, text=True)
    assert out.stdout == load_gaf("vg50k", 10)
    assert " failed 0 " in out.stderr


@pytest.mark.parametrize("name", ["dbg100k", "dbg1m"])
def test_gaf_matches_reference_dbg(harness, oracle_lib, tmp_path, name):
    """-x dbg on k=63 de Bruijn graphs with cyclic components (100 kbp and 1 Mbp genomes)."""
    exe = harness[0]
    import gzip
    reads = os.path.join(tmp_path, "reads.fa")
    open(reads, "wb").write(gzip.open(os.path.join(GOLDEN, f"{name}_reads.fa.gz")).read())
    out = subprocess.run([exe, graph_file(name, str(tmp_path)), reads, "gafdbg", "5"], check=True, capture_output=True, text=True).stdout
    assert out == load_gaf(name, 5)


MULTISEED_CASES = [("vg50k", "vg50k_reads", "gafms", 10, "vg50k_ms_b10"), ("vg50k", "vg50k_reads", "gafms", 5, "vg50k_ms_b5"),
                   ("vg50k", "vg50k_chimera_reads", "gafms", 10, "vg50k_chimera_ms_b10"),
                   ("dbg100k", "dbg100k_reads", "gafmsdbg", 5, "dbg100k_ms_b5")]


@pytest.mark.parametrize("graph,reads,mode,bandwidth,gaf", MULTISEED_CASES)
def test_multiseed_gaf_matches_reference(harness, oracle_lib, tmp_path, graph, reads, mode, bandwidth, gaf):
    """--multiseed-DP 1: prepareSeedsForMultiseeding, the oracle's multiseed DP (seeds started
    in their slices, local-maximum traces), duplicate removal, clipping, backward extensions,
    mapping qualities, selection and GAF, byte for byte against the reference's GAF; the
    chimeric reads give two or three alignments each."""
    import gzip
    exe = harness[0]
    fa = os.path.join(tmp_path, "reads.fa")
    open(fa, "wb").write(gzip.open(os.path.join(GOLDEN, f"{reads}.fa.gz")).read())
    out = subprocess.run([exe, graph_file(graph, str(tmp_path)), fa, mode, str(bandwidth)], check=True, capture_output=True, text=True)
    assert out.stdout == gzip.open(os.path.join(GOLDEN, f"{gaf}.gaf.gz"), "rt").read()
    assert " failed 0 " in out.stderr


GAF_HOOK_CASES = [("vg50k", "vg50k_reads", "gaf", 10, "vg50k_b10"), ("vg50k", "vg50k_reads", "gaf2", 5, "vg50k_b5"),
                  ("dbg100k", "dbg100k_reads", "gafdbg", 5, "dbg100k_b5"), ("vg50k", "vg50k_chimera_reads", "gafms", 10, "vg50k_chimera_ms_b10"),
                  ("dbg100k", "dbg100k_reads", "gafmsdbg", 5, "dbg100k_ms_b5")]


@pytest.mark.parametrize("graph,reads,mode,bandwidth,gaf", GAF_HOOK_CASES)
def test_gaf_formatter_hook_matches_reference(harness, oracle_lib, tmp_path, graph, reads, mode, bandwidth, gaf):
    """The selection and GAF line code the device runs (gaf_format.cuh: select_read, gaf_line),
    compiled for the host and plugged into the read flow's formatter hooks: GAF bytes equal to
    the reference's."""
    import gzip
    exe = harness[0]
    fa = os.path.join(tmp_path, "reads.fa")
    open(fa, "wb").write(gzip.open(os.path.join(GOLDEN, f"{reads}.fa.gz")).read())
    env = dict(os.environ, GAF_LINE_FORMATTER="1")
    out = subprocess.run([exe, graph_file(graph, str(tmp_path)), fa, mode, str(bandwidth)], check=True, capture_output=True, text=True, env=env)
    assert out.stdout == gzip.open(os.path.join(GOLDEN, f"{gaf}.gaf.gz"), "rt").read()


def test_multiseed_reports_room_needed(harness, oracle_lib, tmp_path):
    """A read whose multiseed traces outgrow max_traces reports GA_CAPACITY with the items and
    traces it needs, which equal what a run with room enough returns."""
    import gzip
    import numpy as np
    from graphaligner_gb300.extend import ExtendParams, MultiseedBatch
    from golden_sets import load_graph
    exe = harness[0]
    fa = os.path.join(tmp_path, "reads.fa")
    open(fa, "wb").write(gzip.open(os.path.join(GOLDEN, "vg50k_chimera_reads.fa.gz")).read())
    out = subprocess.run([exe, graph_file("vg50k", str(tmp_path)), fa, "msseeds"], check=True, capture_output=True, text=True).stdout.splitlines()
    seeds = []
    for line in out[:20]:
        f = line.split()
        v = list(map(int, f[2:]))
        seeds.append([(v[2 * k], v[2 * k + 1]) for k in range(int(f[1]))])
    seqs = [line.encode() for line in open(fa).read().split("\n") if line and not line.startswith(">")][:20]
    g = load_graph("vg50k")
    p = ExtendParams(bandwidth=10)
    tight = oracle_lib.multiseed(g, p, MultiseedBatch.pack(seqs, seeds, max_traces=2, items_per_bp=64), threads=4)
    roomy = oracle_lib.multiseed(g, p, MultiseedBatch.pack(seqs, seeds, max_traces=4096, items_per_bp=64), threads=4)
    assert (roomy.status == 0).all() and (tight.status == 3).any()
    for i in range(len(seqs)):
        if tight.status[i] == 3:
            assert tight.traces_needed[i] == roomy.num_traces[i]
            assert tight.items_needed[i] == sum(len(t) for _, t in roomy.traces(i))
        else:
            assert tight.items_needed[i] == 0 and tight.traces_needed[i] == 0


def test_gaf_number_formatting_matches_ostream():
    """gaf_format.cuh's double formatting (six significant digits from the exact binary value,
    ties to even, fixed or scientific as %g) and integer formatting equal std::ostream's on X-scores,
    identity ratios and doubles over the whole exponent range."""
    exe = os.path.join(BUILD, "gaf_fmt")
    src = os.path.join(ROOT, "tests", "harness", "gaf_fmt.cpp")
    hdr = os.path.join(ROOT, "graphaligner_gb300", "csrc", "gaf_format.cuh")
    os.makedirs(BUILD, exist_ok=True)
    if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(src), os.path.getmtime(hdr)):
        subprocess.run(["g++", "-std=c++17", "-O2", "-o", exe, src], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout[-2000:]
    assert "mismatches 0" in out.stdout


def test_quickstart_gaf(harness, tmp_path):
    exe, _, _, _ = harness
    import gzip
    gag = os.path.join(tmp_path, "t.gag")
    open(gag, "wb").write(gzip.open(os.path.join(GOLDEN, "test_graph.gag.gz")).read())
    out = subprocess.run([exe, gag, os.path.join(GOLDEN, "test_read.fa"), "gaf", "10"], check=True, capture_output=True, text=True).stdout
    assert out == open(os.path.join(GOLDEN, "test_graph.gaf")).read()
    fields = out.split("\t")
    assert fields[5] == ">1>2>4" and fields[2:4] == ["0", "71"] and fields[6] == "87"
