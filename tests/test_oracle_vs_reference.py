"""The oracle restatement against the reference's own source (oracle/_ref/ga_ref, which
__graft_entry__.build() compiles where that source is present) on inputs generated at
test time: other graph seeds, bandwidths, X-drop cutoffs and tangle efforts than the
committed golden vectors hold.  Skipped where the reference build is absent."""
import importlib.util
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from golden_sets import compare  # noqa: E402

from graphaligner_gb300 import datagen as dg  # noqa: E402
from graphaligner_gb300 import graph as gg  # noqa: E402
from graphaligner_gb300.extend import ExtendParams, pack_batch  # noqa: E402

ROOT = os.path.abspath(os.path.join(HERE, ".."))
REF = os.path.join(ROOT, "oracle", "_ref", "ga_ref")
UNLIMITED = 2**64 - 1

pytestmark = pytest.mark.skipif(not os.path.exists(REF), reason="the reference's own build (oracle/_ref) is not here")


def _make_golden():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


def _vg_case(seed):
    g = dg.make_variation_graph(30_000, 150, 0.6, 30, seed)
    reads = dg.sample_reads(g, 40, seed + 1, dg.uniform_length(300, 8_000), dg.uniform_error(0.03, 0.2))
    nl = np.zeros(len(g.node_seqs) + 1, dtype=np.int64)
    nl[1:] = [len(s) for s in g.node_seqs]
    return g.to_gfa(), dg.seed_extensions(reads, nl, 15, seed + 2, per_read=1)


def _iupac_case(seed):
    g, ext = _make_golden().iupac_edge_set(seed)
    return g.to_gfa(), ext


def _dbg_case(seed):
    genome = dg.make_repeat_genome(40_000, 6, 1_500, 0.01, 0.04, 10, tandem_len=(200, 800), seed=seed)
    d = dg.compact_dbg(genome, 63, with_positions=True)
    reads = dg.sample_genome_reads(genome, 30, seed + 1, dg.uniform_length(300, 6_000), lambda rng: 0.1, dbg=d)
    return d.gfa, dg.seed_extensions(reads, d.node_len, 15, seed + 2)


# (kind, seed, bandwidth, xdrop, tangle effort)
CASES = [
    ("vg", 21, 3, 14705, UNLIMITED),
    ("vg", 22, 17, 14705, UNLIMITED),
    ("vg", 23, 8, 1500, UNLIMITED),
    ("dbg", 24, 5, 14705, 2000),
    ("dbg", 25, 9, 4000, 20000),
    ("vg", 26, 1, 14705, UNLIMITED),
    ("vg", 27, 40, 14705, UNLIMITED),
    ("dbg", 28, 3, 14705, 500),
    ("iupac", 29, 7, 3000, UNLIMITED),
    ("iupac", 30, 12, 14705, UNLIMITED),
]


@pytest.mark.parametrize("kind,seed,bandwidth,xdrop,max_cells", CASES)
def test_oracle_matches_reference_on_generated_inputs(oracle_lib, kind, seed, bandwidth, xdrop, max_cells):
    mg = _make_golden()
    gfa_text, ext = {"vg": _vg_case, "dbg": _dbg_case, "iupac": _iupac_case}[kind](seed)
    with tempfile.TemporaryDirectory() as td:
        gfa = os.path.join(td, "g.gfa")
        open(gfa, "w").write(gfa_text)
        gag = os.path.join(td, "g.gag")
        subprocess.run([REF, "graphdump", gfa, gag], check=True)
        tsv = os.path.join(td, "ext.tsv")
        open(tsv, "w").write(ext.to_tsv())
        out = os.path.join(td, "out.txt")
        subprocess.run([REF, "extend", gfa, tsv, out, str(bandwidth), str(xdrop), str(max_cells), "0.66"], check=True)
        expected = [tuple(x if k == 3 else int(x) for k, x in enumerate(line.split("\t")))
                    for line in mg.digest_ref_output(out).splitlines()]
        g = gg.load_gag(gag)
    batch = pack_batch(g, list(ext.seqs), ext.bignode, ext.offset)
    res = oracle_lib.extend(g, ExtendParams(bandwidth=bandwidth, xdrop=xdrop, max_cells_per_slice=max_cells), batch, threads=4)
    assert len(expected) == batch.num > 20
    bad = compare(res, expected)
    assert not bad, f"{len(bad)} of {batch.num} extensions differ from the reference, first {bad[:5]}"


from test_read_pipeline_host import harness  # noqa: E402,F401  (the host read-level harness fixture)


# (kind, seed, bandwidth): reads from freshly generated graphs, -x vg at the bandwidth or -x dbg
READ_CASES = [("vg", 31, 10), ("vg", 32, 5), ("vg", 33, 15), ("vg", 35, 3), ("vg", 36, 25), ("dbg", 34, 5), ("dbg", 37, 5)]


@pytest.mark.parametrize("kind,seed,bandwidth", READ_CASES)
def test_read_level_matches_reference_on_generated_inputs(harness, oracle_lib, tmp_path, kind, seed, bandwidth):  # noqa: F811
    """Seeds (getSeeds + OrderSeeds) and GAF of the package's host read-level code, driven by
    the oracle's extensions, against the reference's own on graphs and reads made here."""
    exe = harness[0]
    if kind == "vg":
        g = dg.make_variation_graph(40_000, 150, 0.7, 20, seed)
        gfa_text = g.to_gfa()
        reads = dg.sample_reads(g, 30, seed + 1, dg.uniform_length(300, 9_000), dg.uniform_error(0.04, 0.16))
        k, w, density, discard, mode = "15", "20", "10", "0.001", "gaf"
    else:
        genome = dg.make_repeat_genome(40_000, 6, 1_500, 0.01, 0.04, 10, tandem_len=(200, 800), seed=seed)
        gfa_text = dg.compact_dbg(genome, 63)
        reads = dg.dbg_reads(genome, 12, 8_000, 0.1, seed + 1)
        k, w, density, discard, mode = "19", "30", "5", "0.0002", "gafdbg"
    gfa = os.path.join(tmp_path, "g.gfa")
    open(gfa, "w").write(gfa_text)
    gag = os.path.join(tmp_path, "g.gag")
    subprocess.run([REF, "graphdump", gfa, gag], check=True)
    fa = os.path.join(tmp_path, "reads.fa")
    open(fa, "w").write(dg.write_fasta(reads))
    ref_seeds = os.path.join(tmp_path, "seeds.txt")
    subprocess.run([REF, "seeds", gfa, fa, ref_seeds, k, w, density, discard], check=True)
    mine = subprocess.run([exe, gag, fa, "seeds", k, w, density, discard], check=True, capture_output=True, text=True).stdout
    assert mine == open(ref_seeds).read()
    ref_gaf = os.path.join(tmp_path, "ref.gaf")
    subprocess.run([REF, "align", gfa, fa, ref_gaf] + (["vg", str(bandwidth)] if kind == "vg" else ["dbg"]), check=True)
    mine = subprocess.run([exe, gag, fa, mode, str(bandwidth)], check=True, capture_output=True, text=True).stdout
    expected = open(ref_gaf).read()
    assert expected.count("\n") >= len(reads) // 2
    assert mine == expected


def test_integration_adapter_compiles_against_reference_headers():
    """The reference-side binding INTEGRATION.md shows (oracle/integration_adapter.cpp, the body of
    GraphAlignerBitvectorBanded::getReverseTraceFromSeed over ga_extend_batch) compiles against the
    reference's own headers and include/graphaligner_gb300.h."""
    import oracle
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "adapter", f"GA_REFERENCE={oracle.REFERENCE_ROOT}"], check=True)
