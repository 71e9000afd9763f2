"""Regenerates the golden vectors in this directory from the REFERENCE itself.

Runs oracle/_ref/ga_ref — GraphAligner's own hot-path source compiled by
oracle/Makefile from /root/reference/src with dependency shims — on seeded
synthetic inputs and stores what it produced:

  *_graph.gag.gz   the reference-built AlignmentGraph (GAG1 layout)
  *_ext.tsv.gz     extension requests "bigraphNodeId offset sequence"
  *_ext_bN.digest  per request: status score n_items sha1(packed items)
                   from getReverseTraceFromSeed at bandwidth N
  test_graph.gaf   GAF of the reference's own quickstart (test/graph.gfa, test/read.fa),
                   with the read as test_read.fa and the graph as test_graph.gag.gz
  vg50k_reads.fa.gz, vg50k_b{10,5}.gaf.gz   reads and the reference's GAF (-x vg, -b 10 / 5)
  vg50k_seeds.digest  sha1 of every line of MinimizerSeeder::getSeeds + OrderSeeds output
  dbg100k_*        the same for a k=63 de Bruijn graph with repeats and tandem arrays
                   (cyclic components), extensions at tangle effort 10000, GAF at -x dbg

The packed item layout is the one include/graphaligner_gb300.h documents, so
the oracle restatement and the GPU kernels are compared byte for byte.

Usage: python tests/golden/make_golden.py   (needs /root/reference; run in the build container)
"""
from __future__ import annotations

import gzip
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from graphaligner_gb300 import datagen as dg  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "ga_ref")
XDROP = 14705
UNLIMITED = 2**64 - 1


def pack(node, off, seq, sw):
    sp1 = 0 if seq < 0 else seq + 1
    return (node & 0xffffffff) | ((off & 63) << 32) | ((sw & 1) << 38) | (sp1 << 39)


def digest_ref_output(path):
    lines = []
    for line in open(path):
        if not line.startswith("E "):
            continue
        f = line.split()
        status, score, n = int(f[2]), int(f[3]), int(f[4])
        items = np.array([pack(*(int(x) for x in t.split(","))) for t in f[5:5 + n]], dtype=np.uint64)
        lines.append(f"{status}\t{score}\t{n}\t{hashlib.sha1(items.tobytes()).hexdigest()}")
    return "\n".join(lines) + "\n"


def run_ext(gfa, tsv, bandwidth, max_cells=UNLIMITED):
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "out.txt")
        subprocess.run([REF, "extend", gfa, tsv, out, str(bandwidth), str(XDROP), str(max_cells), "0.66"], check=True)
        return digest_ref_output(out)


def digest_lines(text: str) -> str:
    """sha1 of every line (seed lists are long; their digests pin them)."""
    return "".join(hashlib.sha1(line.encode()).hexdigest() + "\n" for line in text.splitlines())


def gz_write(path, data: bytes):
    with open(path, "wb") as raw, gzip.GzipFile(fileobj=raw, mode="wb", mtime=0) as g:
        g.write(data)


def make_set(name, graph, ext, bandwidths, max_cells=UNLIMITED, write_graph=True):
    with tempfile.TemporaryDirectory() as td:
        gfa = os.path.join(td, "g.gfa")
        open(gfa, "w").write(graph if isinstance(graph, str) else graph.to_gfa())
        gag = os.path.join(td, "g.gag")
        subprocess.run([REF, "graphdump", gfa, gag], check=True)
        if write_graph:
            gz_write(os.path.join(HERE, f"{name}_graph.gag.gz"), open(gag, "rb").read())
        tsv = os.path.join(td, "ext.tsv")
        open(tsv, "w").write(ext.to_tsv())
        gz_write(os.path.join(HERE, f"{name}_ext.tsv.gz"), ext.to_tsv().encode())
        for bw in bandwidths:
            open(os.path.join(HERE, f"{name}_ext_b{bw}.digest"), "w").write(run_ext(gfa, tsv, bw, max_cells))


def node_lengths(g):
    nl = np.zeros(len(g.node_seqs) + 1, dtype=np.int64)
    nl[1:] = [len(s) for s in g.node_seqs]
    return nl


def main():
    if not os.path.exists(REF):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-j8"], check=True)
    # variation graph: 50 kbp backbone, bubble every ~200 bp; reads 5-15 kbp at 10% error
    g = dg.small_vg(0)
    reads = dg.small_vg_reads(g, 200, 1)
    ext = dg.seed_extensions(reads[:150], node_lengths(g), 15, 3, per_read=1)
    make_set("vg50k", g, ext, [10, 5])
    # same graph, reads 0.5-20 kbp at 5-25% error
    reads2 = dg.sample_reads(g, 60, 7, dg.uniform_length(500, 20_000), dg.uniform_error(0.05, 0.25))
    ext2 = dg.seed_extensions(reads2, node_lengths(g), 15, 4, per_read=1)
    make_set("vg50k_hi", g, ext2, [10], write_graph=False)   # graph: vg50k_graph.gag.gz
    # read-level GAF (seeding + seed loop + selection + GAF) on the same graph, -x vg at bandwidth 10 and 5
    with tempfile.TemporaryDirectory() as td:
        gfa = os.path.join(td, "g.gfa")
        open(gfa, "w").write(g.to_gfa())
        fa = os.path.join(td, "reads.fa")
        open(fa, "w").write(dg.write_fasta(reads))
        gz_write(os.path.join(HERE, "vg50k_reads.fa.gz"), dg.write_fasta(reads).encode())
        for bw in (10, 5):
            out = os.path.join(td, f"b{bw}.gaf")
            subprocess.run([REF, "align", gfa, fa, out, "vg", str(bw)], check=True)
            gz_write(os.path.join(HERE, f"vg50k_b{bw}.gaf.gz"), open(out, "rb").read())
        out = os.path.join(td, "seeds.txt")
        subprocess.run([REF, "seeds", gfa, fa, out, "15", "20", "10", "0.001"], check=True)
        open(os.path.join(HERE, "vg50k_seeds.digest"), "w").write(digest_lines(open(out).read()))
    # de Bruijn graph (k=63, cyclic): 100 kbp genome + 10 copies of a 2 kbp repeat at 1-3 %
    # divergence + 20 tandem arrays; -x dbg (bandwidth 5, tangle effort 10000)
    genome = dg.small_dbg_genome(0)
    d = dg.compact_dbg(genome, 63, with_positions=True)
    ext_reads = dg.sample_genome_reads(genome, 60, 5, dg.uniform_length(500, 20_000), lambda rng: 0.12, dbg=d)
    make_set("dbg100k", d.gfa, dg.seed_extensions(ext_reads, d.node_len, 15, 4), [5, 10], max_cells=10000)
    reads = dg.dbg_reads(genome, 30, 20_000, 0.12, 1)
    with tempfile.TemporaryDirectory() as td:
        gfa = os.path.join(td, "g.gfa")
        open(gfa, "w").write(d.gfa)
        fa = os.path.join(td, "reads.fa")
        open(fa, "w").write(dg.write_fasta(reads))
        gz_write(os.path.join(HERE, "dbg100k_reads.fa.gz"), dg.write_fasta(reads).encode())
        out = os.path.join(td, "b5.gaf")
        subprocess.run([REF, "align", gfa, fa, out, "dbg"], check=True)
        gz_write(os.path.join(HERE, "dbg100k_b5.gaf.gz"), open(out, "rb").read())
    # the reference's quickstart
    ref_test = "/root/reference/test"
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "aln.gaf")
        subprocess.run([REF, "align", os.path.join(ref_test, "graph.gfa"), os.path.join(ref_test, "read.fa"), out, "vg"], check=True)
        open(os.path.join(HERE, "test_graph.gaf"), "w").write(open(out).read())
        open(os.path.join(HERE, "test_read.fa"), "w").write(open(os.path.join(ref_test, "read.fa")).read())
        subprocess.run([REF, "graphdump", os.path.join(ref_test, "graph.gfa"), os.path.join(td, "t.gag")], check=True)
        gz_write(os.path.join(HERE, "test_graph.gag.gz"), open(os.path.join(td, "t.gag"), "rb").read())


if __name__ == "__main__":
    main()
