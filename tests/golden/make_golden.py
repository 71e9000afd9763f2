"""Regenerates the golden vectors in this directory from the REFERENCE itself.

Runs oracle/_ref/ga_ref — GraphAligner's own hot-path source compiled by
oracle/Makefile from the reference checkout's src/ (GA_REFERENCE, default
/root/reference) with dependency shims — on seeded
synthetic inputs and stores what it produced:

  *_graph.gag.gz   the reference-built AlignmentGraph (GAG1 layout)
  *_ext.tsv.gz     extension requests "bigraphNodeId offset sequence"
  *_ext_bN.digest  per request: status score n_items sha1(packed items)
                   from getReverseTraceFromSeed at bandwidth N
  test_graph.gaf   GAF of the reference's own quickstart (test/graph.gfa, test/read.fa),
                   with the read as test_read.fa and the graph as test_graph.gag.gz
  vg50k_reads.fa.gz, vg50k_b{10,5}.gaf.gz   reads and the reference's GAF (-x vg, -b 10 / 5)
  vg50k_seeds.digest  sha1 of every line of MinimizerSeeder::getSeeds + OrderSeeds output
  iupac20k_*       IUPAC codes in 6 % of the graph's nodes and 1 % of the read bases, lower
                   case, and edge requests (lengths 1-2, 63-65, 127-129; node first/last base)
  dbg100k_*        the same for a k=63 de Bruijn graph with repeats and tandem arrays
                   (cyclic components), extensions at tangle effort 10000, GAF at -x dbg
  vg50k_px_*       on the vg50k graph, extensions of reads at 12-25 % error, every other one
                   with a random block of 30-150 bp inside (low X-drop cutoffs stop there,
                   the default one passes it), at bandwidths 10, 1, 3, 17 and 40 and at
                   X-drop cutoffs 1500 and 3000 (bandwidth 10)
  vg50k_seed_edges.fa.gz, vg50k_seed_edges_seeds.digest
                   MinimizerSeeder::getSeeds + OrderSeeds (sha1 per output line) on reads
                   with homopolymer runs longer than k, N runs, IUPAC codes, lower case and
                   lengths below, at and just above k (-x vg minimizers)
  dbg1m_*          a k=63 de Bruijn graph of a 1 Mbp genome (20 copies of a 5 kbp repeat,
                   40 tandem arrays): extensions of 20 kbp reads at 12 % error at tangle
                   effort 10000 (bandwidths 5 and 10), and the GAF of 20 such reads at -x dbg
  *_ms_b*.gaf.gz   GAF of the --multiseed-DP branch (PrepareMultiseeds, AlignMultiseed,
                   AddMappingQualities): vg50k reads at bandwidths 10 and 5, dbg100k reads at
                   -x dbg, and vg50k_chimera_reads.fa.gz (two or three pieces of reads from
                   different places, some reverse-complemented, joined by random blocks)

The packed item layout is the one include/graphaligner_gb300.h documents, so
the oracle restatement and the GPU kernels are compared byte for byte.

Usage: [GA_REFERENCE=<GraphAligner checkout>] python tests/golden/make_golden.py [set ...]
       (sets: base params dbg1m seeds multiseed; default: all)
"""
from __future__ import annotations

import gzip
import hashlib
import os
import subprocess
import sys
import tempfile
import types

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


def run_ext(gfa, tsv, bandwidth, max_cells=UNLIMITED, xdrop=XDROP):
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "out.txt")
        subprocess.run([REF, "extend", gfa, tsv, out, str(bandwidth), str(xdrop), str(max_cells), "0.66"], check=True)
        return digest_ref_output(out)


def digest_lines(text: str) -> str:
    """sha1 of every line (seed lists are long; their digests pin them)."""
    return "".join(hashlib.sha1(line.encode()).hexdigest() + "\n" for line in text.splitlines())


def gz_write(path, data: bytes):
    with open(path, "wb") as raw, gzip.GzipFile(fileobj=raw, mode="wb", mtime=0) as g:
        g.write(data)


def make_set(name, graph, ext, bandwidths, max_cells=UNLIMITED, write_graph=True, xdrops=(), write_requests=True):
    """Digests of the reference's extensions of ext on graph: {name}_ext_b{bw}.digest per bandwidth
    and {name}_ext_b{bw}_x{xdrop}.digest per (first bandwidth, X-drop cutoff) in xdrops."""
    with tempfile.TemporaryDirectory() as td:
        gfa = os.path.join(td, "g.gfa")
        open(gfa, "w").write(graph if isinstance(graph, str) else graph.to_gfa())
        gag = os.path.join(td, "g.gag")
        subprocess.run([REF, "graphdump", gfa, gag], check=True)
        if write_graph:
            gz_write(os.path.join(HERE, f"{name}_graph.gag.gz"), open(gag, "rb").read())
        tsv = os.path.join(td, "ext.tsv")
        open(tsv, "w").write(ext.to_tsv())
        if write_requests:
            gz_write(os.path.join(HERE, f"{name}_ext.tsv.gz"), ext.to_tsv().encode())
        for bw in bandwidths:
            open(os.path.join(HERE, f"{name}_ext_b{bw}.digest"), "w").write(run_ext(gfa, tsv, bw, max_cells))
        for x in xdrops:
            open(os.path.join(HERE, f"{name}_ext_b{bandwidths[0]}_x{x}.digest"), "w").write(run_ext(gfa, tsv, bandwidths[0], max_cells, x))


def node_lengths(g):
    nl = np.zeros(len(g.node_seqs) + 1, dtype=np.int64)
    nl[1:] = [len(s) for s in g.node_seqs]
    return nl


IUPAC = np.frombuffer(b"NRYKMSWBDHV", dtype=np.uint8)


def iupac_edge_set(seed: int = 5):
    """A 20 kbp variation graph with IUPAC codes in ~6 % of its nodes (a few nodes all N),
    reads with N / IUPAC codes and lower case, and extension requests at the edges: lengths
    1, 2, 63-65, 127-129 and starts on a node's first and last base."""
    rng = np.random.default_rng(seed)
    g = dg.make_variation_graph(20_000, 100, 0.7, 20, seed)
    clean = [s.copy() for s in g.node_seqs]
    for i in range(len(g.node_seqs)):
        s = g.node_seqs[i] = g.node_seqs[i].copy()
        if rng.random() < 0.06:
            if len(s) <= 3 and rng.random() < 0.5:
                s[:] = ord("N")
            else:
                pos = rng.choice(len(s), size=min(len(s), int(rng.integers(1, 4))), replace=False)
                s[pos] = IUPAC[rng.integers(0, len(IUPAC), len(pos))]
    # reads from the ACGT graph, then N / IUPAC codes and lower case
    g_clean = dg.VariationGraph(clean, g.edges, g.sites, g.backbone_nodes)
    reads = dg.sample_reads(g_clean, 40, seed + 1, dg.uniform_length(200, 6_000), dg.uniform_error(0.03, 0.12))
    out_reads = []
    for r in reads:
        b = np.frombuffer(r.seq, dtype=np.uint8).copy()
        amb = rng.random(len(b)) < 0.01
        b[amb] = IUPAC[rng.integers(0, len(IUPAC), int(amb.sum()))]
        low = rng.random(len(b)) < 0.1
        b[low] = b[low] + 32          # every base is an upper-case letter here
        out_reads.append(dg.Read(r.name, b.tobytes(), r.bignode, r.bigoffset, r.exact))
    ext = dg.seed_extensions(out_reads, node_lengths(g), 15, seed + 2, per_read=2)
    seqs, nodes, offs = list(ext.seqs), list(ext.bignode), list(ext.offset)
    nl = node_lengths(g)
    for k in range(120):
        nid = int(rng.integers(1, len(g.node_seqs) + 1))
        strand = int(rng.integers(0, 2))
        L = int(nl[nid])
        off = 0 if k % 2 == 0 else L - 1
        length = [1, 2, 63, 64, 65, 127, 128, 129][k % 8]
        s_ = dg._BASES[rng.integers(0, 4, length)]
        if k % 3 == 0:
            s_[rng.integers(0, length)] = ord("N")
        seqs.append(s_.tobytes())
        nodes.append(nid * 2 + strand)
        offs.append(off)
    return g, dg.ExtensionSet(seqs, np.array(nodes, dtype=np.int64), np.array(offs, dtype=np.int64))


def vg50k_requests():
    """The vg50k graph (50 kbp backbone, bubble every ~200 bp), its 200 reads (5-15 kbp at
    10 % error) and the extension requests of the first 150."""
    g = dg.small_vg(0)
    reads = dg.small_vg_reads(g, 200, 1)
    return g, reads, dg.seed_extensions(reads[:150], node_lengths(g), 15, 3, per_read=1)


def params_sets():
    """Extensions on the vg50k graph that the parameters change: reads at 12-25 % error, every
    other one with a random block of 30-150 bp inserted at 20-60 % of its length (an X-drop
    cutoff of 1500 or 3000 stops the extension there; the default one, 14705, passes the block
    and its best end lies beyond it), at bandwidths 10, 1, 3, 17 and 40
    (band admission, GraphAlignerBitvectorBanded.h:449-471) and at X-drop cutoffs 1500 and 3000
    with bandwidth 10 (the X-drop stop, :651-669)."""
    g, _, _ = vg50k_requests()
    reads = dg.sample_reads(g, 80, 11, dg.uniform_length(2_000, 12_000), dg.uniform_error(0.12, 0.25))
    ext = dg.seed_extensions(reads, node_lengths(g), 15, 12, per_read=2)
    rng = np.random.default_rng(13)
    seqs = list(ext.seqs)
    for i in range(0, len(seqs), 2):
        s = np.frombuffer(bytes(seqs[i]), dtype=np.uint8)
        cut = int(len(s) * rng.uniform(0.2, 0.6))
        block = dg._BASES[rng.integers(0, 4, int(rng.integers(30, 151)))]
        seqs[i] = np.concatenate([s[:cut], block, s[cut:]]).tobytes()
    make_set("vg50k_px", g, dg.ExtensionSet(seqs, ext.bignode, ext.offset), [10, 1, 3, 17, 40], write_graph=False,
             xdrops=[1500, 3000])


def seed_edge_reads(seed: int = 17):
    """Reads on which iterateKmers' rules all fire: 30 vg50k reads (cut to 3 kbp) with
    homopolymer runs of 16-80 bp (repeated k-mers: the window rule), N runs and single IUPAC
    codes (restarts), lower-case stretches, plus reads of 1, 14, 15, 16 and 40 bp, an all-N
    read and a 200 bp homopolymer."""
    rng = np.random.default_rng(seed)
    g = dg.small_vg(0)
    base = dg.small_vg_reads(g, 30, seed)
    out = []
    for r in base:
        b = np.frombuffer(r.seq[:3000], dtype=np.uint8).copy()
        for _ in range(3):
            pos = int(rng.integers(0, len(b) - 100))
            run = int(rng.integers(16, 81))
            b[pos:pos + run] = dg._BASES[rng.integers(0, 4)]
        pos = int(rng.integers(0, len(b) - 20))
        b[pos:pos + int(rng.integers(1, 12))] = ord("N")
        iu = rng.random(len(b)) < 0.002
        b[iu] = IUPAC[rng.integers(0, len(IUPAC), int(iu.sum()))]
        pos = int(rng.integers(0, len(b) - 200))
        seg = b[pos:pos + 200]
        seg[seg < 97] += 32          # lower case (IUPAC and N too)
        out.append(dg.Read(r.name + "_edges", b.tobytes(), r.bignode, r.bigoffset, r.exact))
    for i, n in enumerate((1, 14, 15, 16, 40)):
        out.append(dg.Read(f"short{i}", dg._BASES[rng.integers(0, 4, n)].tobytes(), 0, 0, False))
    out.append(dg.Read("alln", b"N" * 300, 0, 0, False))
    out.append(dg.Read("homopolymer", b"C" * 200, 0, 0, False))
    return g, out


def seed_sets():
    g, reads = seed_edge_reads()
    with tempfile.TemporaryDirectory() as td:
        gfa = os.path.join(td, "g.gfa")
        open(gfa, "w").write(g.to_gfa())
        fa = os.path.join(td, "reads.fa")
        open(fa, "w").write(dg.write_fasta(reads))
        gz_write(os.path.join(HERE, "vg50k_seed_edges.fa.gz"), dg.write_fasta(reads).encode())
        out = os.path.join(td, "seeds.txt")
        subprocess.run([REF, "seeds", gfa, fa, out, "15", "20", "10", "0.001"], check=True)
        open(os.path.join(HERE, "vg50k_seed_edges_seeds.digest"), "w").write(digest_lines(open(out).read()))


def dbg1m_sets():
    """A k=63 de Bruijn graph of a 1 Mbp genome: extensions of 20 kbp reads at 12 % error at
    tangle effort 10000 (bandwidths 5 and 10), and the GAF of 20 such reads at -x dbg."""
    genome = dg.mid_dbg_genome(0)
    d = dg.compact_dbg(genome, 63, with_positions=True)
    ext_reads = dg.sample_genome_reads(genome, 60, 5, lambda rng: 20_000, lambda rng: 0.12, dbg=d)
    make_set("dbg1m", d.gfa, dg.seed_extensions(ext_reads, d.node_len, 15, 4), [5, 10], max_cells=10000)
    reads = dg.dbg_reads(genome, 20, 20_000, 0.12, 1)
    with tempfile.TemporaryDirectory() as td:
        gfa = os.path.join(td, "g.gfa")
        open(gfa, "w").write(d.gfa)
        fa = os.path.join(td, "reads.fa")
        open(fa, "w").write(dg.write_fasta(reads))
        gz_write(os.path.join(HERE, "dbg1m_reads.fa.gz"), dg.write_fasta(reads).encode())
        out = os.path.join(td, "b5.gaf")
        subprocess.run([REF, "align", gfa, fa, out, "dbg"], check=True)
        gz_write(os.path.join(HERE, "dbg1m_b5.gaf.gz"), open(out, "rb").read())


def chimeric_reads(g, n: int = 60, seed: int = 21):
    """Reads made of two or three pieces of vg50k reads (2-8 kbp at 5-20 % error), the later
    pieces from elsewhere in the graph and every other one reverse-complemented, with a random
    block of 0-400 bp between pieces: the multiseed DP finds a local maximum per piece."""
    parts = dg.sample_reads(g, 3 * n, seed, dg.uniform_length(2_000, 8_000), dg.uniform_error(0.05, 0.20))
    rng = np.random.default_rng(seed + 1)
    reads = []
    for i in range(n):
        pieces = [np.frombuffer(bytes(parts[3 * i].seq), dtype=np.uint8)]
        for k in range(1, 2 + int(rng.integers(0, 2))):
            block = dg._BASES[rng.integers(0, 4, int(rng.integers(0, 401)))]
            piece = np.frombuffer(bytes(parts[3 * i + k].seq), dtype=np.uint8)
            if k % 2 == 1:
                piece = dg.revcomp(piece)
            pieces += [block, piece]
        reads.append(types.SimpleNamespace(name=f"chimera{i}", seq=np.concatenate(pieces).tobytes()))
    return reads


def multiseed_sets():
    """GAF of the reference's --multiseed-DP branch (ga_ref align ... multiseed): the vg50k reads
    at bandwidths 10 and 5, chimeric vg50k reads at bandwidth 10, and the dbg100k reads at -x dbg."""
    g, reads, _ = vg50k_requests()
    chim = chimeric_reads(g)
    with tempfile.TemporaryDirectory() as td:
        gfa = os.path.join(td, "g.gfa")
        open(gfa, "w").write(g.to_gfa())
        fa = os.path.join(td, "reads.fa")
        open(fa, "w").write(dg.write_fasta(reads))
        for bw in (10, 5):
            out = os.path.join(td, f"ms{bw}.gaf")
            subprocess.run([REF, "align", gfa, fa, out, "vg", str(bw), "-", "multiseed"], check=True)
            gz_write(os.path.join(HERE, f"vg50k_ms_b{bw}.gaf.gz"), open(out, "rb").read())
        fa = os.path.join(td, "chim.fa")
        open(fa, "w").write(dg.write_fasta(chim))
        gz_write(os.path.join(HERE, "vg50k_chimera_reads.fa.gz"), dg.write_fasta(chim).encode())
        out = os.path.join(td, "chim.gaf")
        subprocess.run([REF, "align", gfa, fa, out, "vg", "10", "-", "multiseed"], check=True)
        gz_write(os.path.join(HERE, "vg50k_chimera_ms_b10.gaf.gz"), open(out, "rb").read())
    genome = dg.small_dbg_genome(0)
    d = dg.compact_dbg(genome, 63, with_positions=True)
    reads = dg.dbg_reads(genome, 30, 20_000, 0.12, 1)
    with tempfile.TemporaryDirectory() as td:
        gfa = os.path.join(td, "g.gfa")
        open(gfa, "w").write(d.gfa)
        fa = os.path.join(td, "reads.fa")
        open(fa, "w").write(dg.write_fasta(reads))
        out = os.path.join(td, "ms.gaf")
        subprocess.run([REF, "align", gfa, fa, out, "dbg", "-", "-", "multiseed"], check=True)
        gz_write(os.path.join(HERE, "dbg100k_ms_b5.gaf.gz"), open(out, "rb").read())


def main():
    if not os.path.exists(REF):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-j8"], check=True)
    groups = sys.argv[1:] or ["base", "params", "dbg1m", "seeds", "multiseed"]
    if "multiseed" in groups:
        multiseed_sets()
    if "seeds" in groups:
        seed_sets()
    if "params" in groups:
        params_sets()
    if "dbg1m" in groups:
        dbg1m_sets()
    if "base" not in groups:
        return
    g, reads, ext = vg50k_requests()
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
    # IUPAC codes in graph and reads, lower case, edge lengths and start offsets
    g_iu, ext_iu = iupac_edge_set(5)
    make_set("iupac20k", g_iu, ext_iu, [10, 5])
    # the reference's quickstart
    ref_test = os.path.join(os.environ.get("GA_REFERENCE", "/root/reference"), "test")
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "aln.gaf")
        subprocess.run([REF, "align", os.path.join(ref_test, "graph.gfa"), os.path.join(ref_test, "read.fa"), out, "vg"], check=True)
        open(os.path.join(HERE, "test_graph.gaf"), "w").write(open(out).read())
        open(os.path.join(HERE, "test_read.fa"), "w").write(open(os.path.join(ref_test, "read.fa")).read())
        subprocess.run([REF, "graphdump", os.path.join(ref_test, "graph.gfa"), os.path.join(td, "t.gag")], check=True)
        gz_write(os.path.join(HERE, "test_graph.gag.gz"), open(os.path.join(td, "t.gag"), "rb").read())


if __name__ == "__main__":
    main()
