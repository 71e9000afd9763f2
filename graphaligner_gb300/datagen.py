"""Seeded synthetic workloads for the seed-extension path.

No public dataset is named for this path, so graphs, reads and seeds are
generated here with the shapes the workloads call for:

* variation graph: a uniform-random ACGT backbone with one variant site every
  ``spacing`` bp on average; a site is a SNP (two 1-bp alleles) with
  probability ``snp_frac`` and otherwise an insertion or deletion of
  1..``indel_max`` bp (a bubble with an empty branch).  Nodes are split at
  variant sites and written as GFA with ``0M`` links.
* reads: a random allele per site gives a haplotype path; a read is a window of
  that path on a random strand with per-base errors (60% substitution, 20%
  insertion, 20% deletion of the error budget).
* seeds: exact k-mers of the read that map to consecutive, unedited path bases;
  the seed position is the k-mer's last base, as MinimizerSeeder reports it
  (MinimizerSeeder.cpp:82,545-555).

Everything is a pure function of the seed, so the same inputs are rebuilt on
any machine.
"""
from __future__ import annotations

import dataclasses
import numpy as np

_BASES = np.frombuffer(b"ACGT", dtype=np.uint8)
_COMP = np.zeros(256, dtype=np.uint8)
for _a, _b in zip(b"ACGTacgtN", b"TGCAtgcaN"):
    _COMP[_a] = _b


def revcomp(seq: bytes | np.ndarray) -> np.ndarray:
    arr = np.frombuffer(seq, dtype=np.uint8) if isinstance(seq, (bytes, bytearray)) else seq
    return _COMP[arr[::-1]]


@dataclasses.dataclass
class VariationGraph:
    """A bidirected GFA graph in forward orientation (ids start at 1)."""
    node_seqs: list            # list of np.uint8 arrays, index = id - 1
    edges: list                # list of (from_id, to_id), both '+' strand
    sites: list                # per site: (kind, [allele node id lists])
    backbone_nodes: list       # ordered backbone segment ids between sites

    def to_gfa(self) -> str:
        lines = []
        for i, s in enumerate(self.node_seqs):
            lines.append(f"S\t{i + 1}\t{s.tobytes().decode()}")
        for a, b in self.edges:
            lines.append(f"L\t{a}\t+\t{b}\t+\t0M")
        return "\n".join(lines) + "\n"

    @property
    def total_bp(self) -> int:
        return int(sum(len(s) for s in self.node_seqs))


def make_variation_graph(genome_len: int, spacing: int, snp_frac: float = 0.7,
                         indel_max: int = 20, seed: int = 0) -> VariationGraph:
    """Backbone of ``genome_len`` bp with a variant roughly every ``spacing`` bp."""
    rng = np.random.default_rng(seed)
    backbone = _BASES[rng.integers(0, 4, genome_len)]
    node_seqs: list = []
    edges: list = []
    sites: list = []
    backbone_nodes: list = []

    def new_node(seq):
        node_seqs.append(np.ascontiguousarray(seq, dtype=np.uint8))
        return len(node_seqs)

    # previous "ends": node ids whose right end connects to the next segment
    prev_ends: list = []
    seg_start = 0
    pos = int(rng.integers(spacing // 2, spacing + 1))
    while True:
        if pos >= genome_len - indel_max - 2:
            break
        r = rng.random()
        if r < snp_frac:
            kind, length = "snp", 1
        elif r < snp_frac + (1 - snp_frac) / 2:
            kind, length = "ins", int(rng.integers(1, indel_max + 1))
        else:
            kind, length = "del", int(rng.integers(1, indel_max + 1))
        if pos <= seg_start:
            pos = seg_start + 1
        seg = new_node(backbone[seg_start:pos])
        backbone_nodes.append(seg)
        for p in prev_ends:
            edges.append((p, seg))
        if kind == "snp":
            ref = backbone[pos:pos + 1]
            alt = _BASES[(int(np.searchsorted(_BASES, ref[0])) + int(rng.integers(1, 4))) % 4:][:1]
            a = new_node(ref)
            b = new_node(alt)
            edges.append((seg, a))
            edges.append((seg, b))
            sites.append(("snp", [[a], [b]]))
            prev_ends = [a, b]
            seg_start = pos + 1
        elif kind == "del":
            d = new_node(backbone[pos:pos + length])
            edges.append((seg, d))
            sites.append(("del", [[d], []]))
            prev_ends = [d, seg]
            seg_start = pos + length
        else:
            ins = new_node(_BASES[rng.integers(0, 4, length)])
            edges.append((seg, ins))
            sites.append(("ins", [[], [ins]]))
            prev_ends = [ins, seg]
            seg_start = pos
        step = int(rng.integers(max(1, spacing // 2), spacing + spacing // 2 + 1))
        pos = seg_start + max(step, 2)
    last = new_node(backbone[seg_start:])
    backbone_nodes.append(last)
    for p in prev_ends:
        edges.append((p, last))
    return VariationGraph(node_seqs, edges, sites, backbone_nodes)


@dataclasses.dataclass
class Haplotype:
    seq: np.ndarray        # path sequence (uint8 ASCII)
    node: np.ndarray       # GFA node id of each path base
    offset: np.ndarray     # offset of each path base inside its node


def sample_haplotype(g: VariationGraph, seed: int) -> Haplotype:
    """One allele per site, chosen uniformly."""
    rng = np.random.default_rng(seed)
    choice = rng.integers(0, 2, len(g.sites))
    order = []
    for i, seg in enumerate(g.backbone_nodes):
        order.append(seg)
        if i < len(g.sites):
            order.extend(g.sites[i][1][choice[i]])
    seqs = [g.node_seqs[n - 1] for n in order]
    lens = np.array([len(s) for s in seqs], dtype=np.int64)
    seq = np.concatenate(seqs)
    node = np.repeat(np.array(order, dtype=np.int64), lens)
    starts = np.repeat(np.cumsum(lens) - lens, lens)
    offset = np.arange(len(seq), dtype=np.int64) - starts
    return Haplotype(seq, node, offset)


@dataclasses.dataclass
class Read:
    name: str
    seq: bytes
    # per read base: bigraph node id (GFA id*2 + strand) and offset on that strand,
    # or -1 for inserted / substituted bases
    bignode: np.ndarray
    bigoffset: np.ndarray
    exact: np.ndarray      # True where the base is an unedited copy of the path


def _apply_errors(rng, truth: np.ndarray, rate: float):
    """Returns (read bases, source index into truth or -1, exact flag)."""
    n = len(truth)
    u = rng.random(n)
    kind = np.full(n, 0, dtype=np.int8)            # 0 keep, 1 sub, 2 ins, 3 del
    err = u < rate
    t = rng.random(n)
    kind[err & (t < 0.6)] = 1
    kind[err & (t >= 0.6) & (t < 0.8)] = 2
    kind[err & (t >= 0.8)] = 3
    out_bases = []
    out_src = []
    out_exact = []
    subs = (np.searchsorted(_BASES, truth) + rng.integers(1, 4, n)) % 4
    ins_bases = _BASES[rng.integers(0, 4, n)]
    keep = kind != 3
    # build per source position a list of emitted bases: optional inserted base then the base
    emit_ins = kind == 2
    total = int(keep.sum() + emit_ins.sum())
    bases = np.empty(total, dtype=np.uint8)
    src = np.empty(total, dtype=np.int64)
    exact = np.empty(total, dtype=bool)
    counts = keep.astype(np.int64) + emit_ins.astype(np.int64)
    pos = np.cumsum(counts) - counts
    ins_pos = pos[emit_ins]
    bases[ins_pos] = ins_bases[emit_ins]
    src[ins_pos] = -1
    exact[ins_pos] = False
    base_pos = pos[keep] + emit_ins[keep].astype(np.int64)
    kb = truth[keep].copy()
    is_sub = (kind[keep] == 1)
    kb[is_sub] = _BASES[subs[keep][is_sub]]
    bases[base_pos] = kb
    src[base_pos] = np.nonzero(keep)[0]
    exact[base_pos] = ~is_sub
    return bases, src, exact


def sample_reads(g: VariationGraph, n_reads: int, seed: int, length_fn, error_fn,
                 prefix: str = "read") -> list:
    """Reads along one haplotype per read, on a random strand."""
    rng = np.random.default_rng(seed)
    node_len = np.array([len(s) for s in g.node_seqs], dtype=np.int64)
    reads = []
    hap_cache = {}
    for r in range(n_reads):
        hap_seed = int(rng.integers(0, 4))
        if hap_seed not in hap_cache:
            hap_cache[hap_seed] = sample_haplotype(g, seed * 1000003 + hap_seed)
        hap = hap_cache[hap_seed]
        length = int(min(length_fn(rng), len(hap.seq) - 1))
        start = int(rng.integers(0, len(hap.seq) - length + 1))
        truth = hap.seq[start:start + length]
        node = hap.node[start:start + length]
        off = hap.offset[start:start + length]
        reverse = bool(rng.integers(0, 2))
        if reverse:
            truth = revcomp(truth)
            node = node[::-1]
            off = node_len[node - 1] - 1 - off[::-1]
            bignode = node * 2 + 1
        else:
            bignode = node * 2
        bases, src, exact = _apply_errors(rng, truth, float(error_fn(rng)))
        bn = np.where(src >= 0, bignode[np.maximum(src, 0)], -1)
        bo = np.where(src >= 0, off[np.maximum(src, 0)], -1)
        bn[~exact] = -1
        bo[~exact] = -1
        reads.append(Read(f"{prefix}{r}", bases.tobytes(), bn, bo, exact))
    return reads


def exact_seed_positions(read: Read, k: int) -> np.ndarray:
    """Read positions q such that read[q-k+1..q] copies path bases with no edit
    inside a node (prefix-sum test over the exact flags and offset continuity)."""
    n = len(read.exact)
    if n < k:
        return np.zeros(0, dtype=np.int64)
    bad = ~read.exact
    step = np.zeros(n, dtype=bool)
    same = read.bignode[1:] == read.bignode[:-1]
    step[1:] = same & (read.bigoffset[1:] != read.bigoffset[:-1] + 1)
    cb = np.concatenate([[0], np.cumsum(bad)])
    cs = np.concatenate([[0], np.cumsum(step)])
    q = np.arange(k - 1, n)
    ok = (cb[q + 1] - cb[q + 1 - k] == 0) & (cs[q + 1] - cs[q + 2 - k] == 0)
    return q[ok]


def lognormal_length(mean: float, sigma: float, lo: int, hi: int):
    mu = np.log(mean) - sigma * sigma / 2

    def fn(rng):
        return int(np.clip(rng.lognormal(mu, sigma), lo, hi))
    return fn


def uniform_length(lo: int, hi: int):
    def fn(rng):
        return int(rng.integers(lo, hi + 1))
    return fn


def uniform_error(lo: float, hi: float):
    def fn(rng):
        return float(rng.uniform(lo, hi))
    return fn


@dataclasses.dataclass
class ExtensionSet:
    """Seed extensions in the form GraphAlignerBitvectorBanded::getReverseTraceFromSeed
    takes them (GraphAlignerBitvectorBanded.h:59): a sequence, a bigraph node id and
    an offset on that node."""
    seqs: list             # list of bytes
    bignode: np.ndarray    # int64
    offset: np.ndarray     # int64

    def __len__(self):
        return len(self.seqs)

    def to_tsv(self) -> str:
        return "".join(f"{int(n)}\t{int(o)}\t{s.decode()}\n" for n, o, s in zip(self.bignode, self.offset, self.seqs))


def seed_extensions(reads: list, node_len_by_id: np.ndarray, k: int, seed: int,
                    per_read: int = 1) -> ExtensionSet:
    """Two extensions per chosen seed, exactly as GraphAligner::getTwoDirectionalTrace
    forms them (GraphAligner.h:475-506): the forward part read[q+1:] from the seed's
    node and offset, and the reverse complement of read[:q] from the reverse-strand
    position of the seed base."""
    rng = np.random.default_rng(seed)
    seqs, nodes, offs = [], [], []
    for read in reads:
        q_all = exact_seed_positions(read, k)
        if len(q_all) == 0:
            continue
        for q in rng.choice(q_all, size=min(per_read, len(q_all)), replace=False):
            q = int(q)
            fw_node = int(read.bignode[q])
            fw_off = int(read.bigoffset[q])
            size = int(node_len_by_id[fw_node // 2])
            if q > 0:
                bw_node = fw_node ^ 1
                bw_off = size - fw_off - 1
                seqs.append(revcomp(read.seq[:q]).tobytes())
                nodes.append(bw_node)
                offs.append(bw_off)
            if q < len(read.seq) - 1:
                seqs.append(read.seq[q + 1:])
                nodes.append(fw_node)
                offs.append(fw_off)
    return ExtensionSet(seqs, np.array(nodes, dtype=np.int64), np.array(offs, dtype=np.int64))


def write_fasta(reads: list) -> str:
    return "".join(f">{r.name}\n{r.seq.decode()}\n" for r in reads)


# Named workloads ------------------------------------------------------------

def small_vg(seed: int = 0):
    """50 kbp backbone, a bubble every ~200 bp, 70% SNP / 30% indels of 1-20 bp."""
    return make_variation_graph(50_000, 200, 0.7, 20, seed)


def small_vg_reads(g: VariationGraph, n: int = 200, seed: int = 1):
    """Reads of 5-15 kbp at 10% error."""
    return sample_reads(g, n, seed, uniform_length(5_000, 15_000), lambda rng: 0.10)


def batch_vg(seed: int = 0):
    """5 Mbp backbone, a variant every ~100 bp."""
    return make_variation_graph(5_000_000, 100, 0.7, 20, seed)


def batch_vg_reads(g: VariationGraph, n: int, seed: int = 1):
    """Log-normal lengths with mean 10 kbp clipped to 1-50 kbp, error U[5%, 15%]."""
    return sample_reads(g, n, seed, lognormal_length(10_000, 0.6, 1_000, 50_000), uniform_error(0.05, 0.15))


def _extension_chunk(args):
    graph_seed, genome_len, spacing, chunk_index, n, read_seed, k = args
    g = make_variation_graph(genome_len, spacing, 0.7, 20, graph_seed)
    nl = np.zeros(len(g.node_seqs) + 1, dtype=np.int64)
    nl[1:] = [len(x) for x in g.node_seqs]
    reads = sample_reads(g, n, read_seed * 1_000_003 + chunk_index,
                         lognormal_length(10_000, 0.6, 1_000, 50_000), uniform_error(0.05, 0.15),
                         prefix=f"c{chunk_index}_")
    return seed_extensions(reads, nl, k, read_seed * 7919 + chunk_index)


def batch_extension_workload(n_reads: int, graph_seed: int = 0, read_seed: int = 1, k: int = 15,
                             genome_len: int = 5_000_000, spacing: int = 100, chunk: int = 1000,
                             workers: int | None = None) -> ExtensionSet:
    """Seed extensions of the batched-extension workload: one exact k-mer seed per read,
    both directions, reads log-normal (mean 10 kbp, 1-50 kbp) at U[5%,15%] error.
    Reads are made in fixed chunks with per-chunk seeds, so the result does not depend
    on the number of worker processes."""
    import multiprocessing as mp
    import os
    chunks = [(graph_seed, genome_len, spacing, c, min(chunk, n_reads - c * chunk), read_seed, k)
              for c in range((n_reads + chunk - 1) // chunk)]
    workers = workers or min(len(chunks), os.cpu_count() or 1)
    if workers > 1 and len(chunks) > 1:
        with mp.get_context("spawn").Pool(workers) as pool:
            parts = pool.map(_extension_chunk, chunks)
    else:
        parts = [_extension_chunk(c) for c in chunks]
    seqs = [x for p in parts for x in p.seqs]
    return ExtensionSet(seqs, np.concatenate([p.bignode for p in parts]), np.concatenate([p.offset for p in parts]))


# De Bruijn graph workload ----------------------------------------------------

def _is_rc_rotation(unit: np.ndarray) -> bool:
    """True when the reverse complement of a tandem unit is one of its rotations,
    i.e. the tandem array reads the same on both strands."""
    rc = revcomp(unit).tobytes()
    doubled = (unit.tobytes() * 2)
    return rc in doubled


def _mutate(rng, seq: np.ndarray, divergence: float) -> np.ndarray:
    """A diverged copy: substitutions (80 %) and 1-bp indels (20 %) at the given rate."""
    n = len(seq)
    u = rng.random(n)
    t = rng.random(n)
    out = seq.copy()
    sub = (u < divergence) & (t < 0.8)
    out[sub] = _BASES[(np.searchsorted(_BASES, seq[sub]) + rng.integers(1, 4, int(sub.sum()))) % 4]
    dele = (u < divergence) & (t >= 0.8) & (t < 0.9)
    ins = (u < divergence) & (t >= 0.9)
    keep = ~dele
    counts = keep.astype(np.int64) + ins.astype(np.int64)
    res = np.empty(int(counts.sum()), dtype=np.uint8)
    pos = np.cumsum(counts) - counts
    res[pos[ins]] = _BASES[rng.integers(0, 4, int(ins.sum()))]
    res[pos[keep] + ins[keep].astype(np.int64)] = out[keep]
    return res


def make_repeat_genome(genome_len: int, n_copies: int, repeat_len: int, div_lo: float, div_hi: float,
                       n_tandem: int, tandem_period: tuple = (2, 50), tandem_len: tuple = (500, 3000),
                       seed: int = 0) -> np.ndarray:
    """A uniform-random genome of ``genome_len`` bp with ``n_copies`` inserted copies of
    one ``repeat_len`` bp repeat family (each copy diverged by U[div_lo, div_hi], random
    strand) and ``n_tandem`` tandem arrays of a random unit of period U[tandem_period].
    Units that read the same on both strands are redrawn."""
    rng = np.random.default_rng(seed)
    parts = [_BASES[rng.integers(0, 4, genome_len)]]
    family = _BASES[rng.integers(0, 4, repeat_len)]
    inserts = []
    for _ in range(n_copies):
        c = _mutate(rng, family, float(rng.uniform(div_lo, div_hi)))
        if rng.integers(0, 2):
            c = revcomp(c)
        inserts.append(c)
    for _ in range(n_tandem):
        p = int(rng.integers(tandem_period[0], tandem_period[1] + 1))
        while True:
            unit = _BASES[rng.integers(0, 4, p)]
            if not _is_rc_rotation(unit):
                break
        length = int(rng.integers(tandem_len[0], tandem_len[1] + 1))
        inserts.append(np.resize(unit, length))
    order = rng.permutation(len(inserts))
    cuts = np.sort(rng.integers(1, genome_len, len(inserts)))
    out = []
    prev = 0
    base = parts[0]
    for cut, idx in zip(cuts, order):
        out.append(base[prev:cut])
        out.append(inserts[idx])
        prev = cut
    out.append(base[prev:])
    return np.concatenate(out)


def _windows(codes: np.ndarray, m: int) -> np.ndarray:
    """w[i] = 2-bit packing of codes[i:i+m], first base most significant."""
    n = len(codes) - m + 1
    w = np.zeros(n, dtype=np.uint64)
    for j in range(m):
        w = (w << np.uint64(2)) | codes[j:j + n]
    return w


@dataclasses.dataclass
class DbgGraph:
    """A compacted de Bruijn graph with the place of every genome base in it."""
    gfa: str
    node_len: np.ndarray     # int64 [U + 1], length of unitig id (index 0 unused)
    pos_bignode: np.ndarray  # int64 [genome length], bigraph node holding the base in genome orientation
    pos_offset: np.ndarray   # int64 [genome length], offset of the base on that node


def compact_dbg(genome: np.ndarray, k: int = 63, with_positions: bool = False):
    """The compacted de Bruijn graph of one linear genome as GFA (k-1 bp overlaps).

    Edge-centric: the edges are the genome's (k+1)-mers on both strands.  A unitig is a
    maximal path whose inner edges go from an oriented k-mer with one successor to one
    with one predecessor (and not to its own reverse complement).  Every genome walk
    between two non-compactable edges is then exactly one unitig, so unitigs are cut
    from the genome directly: a unitig is named by the smaller canonical id of its two
    end k-mers, numbered by first occurrence, and written in the orientation whose
    first k-mer has the smaller id (a single k-mer: its canonical orientation)."""
    assert k % 2 == 1 and 33 <= k <= 63
    lut = np.full(256, 255, dtype=np.uint8)
    lut[np.frombuffer(b"ACGT", dtype=np.uint8)] = np.arange(4, dtype=np.uint8)
    codes = lut[genome].astype(np.uint64)
    if (codes > 3).any():
        raise ValueError("compact_dbg expects an ACGT genome")
    L = len(codes)
    nk = L - k + 1
    lo_len = k - 32
    w32 = _windows(codes, 32)
    wlo = _windows(codes, lo_len)
    rcodes = (np.uint64(3) - codes)[::-1].copy()
    r32 = _windows(rcodes, 32)
    rlo = _windows(rcodes, lo_len)
    hi_f = w32[:nk]
    lo_f = wlo[32:32 + nk]
    ridx = L - k - np.arange(nk)
    hi_r = r32[ridx]
    lo_r = rlo[ridx + 32]
    fwd = (hi_f < hi_r) | ((hi_f == hi_r) & (lo_f < lo_r))
    ch = np.where(fwd, hi_f, hi_r)
    cl = np.where(fwd, lo_f, lo_r)
    orient = (~fwd).astype(np.int64)
    perm = np.lexsort((cl, ch))
    newk = np.ones(nk, dtype=bool)
    newk[1:] = (ch[perm][1:] != ch[perm][:-1]) | (cl[perm][1:] != cl[perm][:-1])
    kid = np.empty(nk, dtype=np.int64)
    kid[perm] = np.cumsum(newk) - 1
    nkid = int(kid.max()) + 1
    node = 2 * kid + orient                      # oriented k-mer along the genome
    a, b = node[:-1], node[1:]
    fr = np.concatenate([a, b ^ 1])
    to = np.concatenate([b, a ^ 1])
    key = np.unique(fr * (2 * nkid) + to)
    outdeg = np.bincount(key // (2 * nkid), minlength=2 * nkid)
    indeg = np.bincount(key % (2 * nkid), minlength=2 * nkid)
    compactable = (outdeg[a] == 1) & (indeg[b] == 1) & (kid[:-1] != kid[1:])
    starts = np.concatenate([[0], np.nonzero(~compactable)[0] + 1])
    ends = np.concatenate([starts[1:] - 1, [nk - 1]])
    ks, ke = kid[starts], kid[ends]
    canon = np.where(starts == ends, orient[starts] == 0, ks <= ke)
    ukey = np.minimum(ks, ke)
    _, first_occ, inverse = np.unique(ukey, return_index=True, return_inverse=True)
    # number unitigs by first occurrence along the genome
    rank = np.empty(len(first_occ), dtype=np.int64)
    rank[np.argsort(first_occ, kind="stable")] = np.arange(len(first_occ))
    uid = rank[inverse] + 1
    order = np.argsort(rank)
    lines = []
    for u in order:
        occ = first_occ[u]
        s, e = int(starts[occ]), int(ends[occ])
        seq = genome[s:e + k]
        if not canon[occ]:
            seq = revcomp(seq)
        lines.append(f"S\t{rank[u] + 1}\t{seq.tobytes().decode()}")
    # links between consecutive occurrences, one representative per reverse-complement pair
    fa, fb = uid[:-1], uid[1:]
    sa, sb = canon[:-1].astype(np.int64), canon[1:].astype(np.int64)
    e1 = np.stack([fa, sa, fb, sb], axis=1)
    e2 = np.stack([fb, 1 - sb, fa, 1 - sa], axis=1)
    use2 = (e2[:, 0] < e1[:, 0]) | ((e2[:, 0] == e1[:, 0]) & ((e2[:, 1] > e1[:, 1]) | ((e2[:, 1] == e1[:, 1]) & ((e2[:, 2] < e1[:, 2]) | ((e2[:, 2] == e1[:, 2]) & (e2[:, 3] > e1[:, 3]))))))
    edges = np.where(use2[:, None], e2, e1)
    _, idx = np.unique(edges[:, 0] * (8 * len(first_occ) + 8) + edges[:, 1] * (4 * len(first_occ) + 4) + edges[:, 2] * 2 + edges[:, 3], return_index=True)
    ov = k - 1
    for i in np.sort(idx):
        x, xs, y, ys = (int(v) for v in edges[i])
        lines.append(f"L\t{x}\t{'+' if xs else '-'}\t{y}\t{'+' if ys else '-'}\t{ov}M")
    gfa = "\n".join(lines) + "\n"
    if not with_positions:
        return gfa
    # a base at genome position p lies in the occurrence that holds the k-mer starting at p
    # (the last k-1 bases: in the last occurrence)
    seg = np.searchsorted(starts, np.minimum(np.arange(L), nk - 1), side="right") - 1
    pos_offset = np.arange(L) - starts[seg]
    pos_bignode = uid[seg] * 2 + np.where(canon[seg], 0, 1)
    node_len = np.zeros(len(first_occ) + 1, dtype=np.int64)
    node_len[uid] = ends - starts + k
    return DbgGraph(gfa, node_len, pos_bignode.astype(np.int64), pos_offset.astype(np.int64))


def sample_genome_reads(genome: np.ndarray, n_reads: int, seed: int, length_fn, error_fn,
                        prefix: str = "read", dbg: DbgGraph | None = None) -> list:
    """Reads as windows of a linear genome on a random strand with errors
    (60 % substitution, 20 % insertion, 20 % deletion of the error budget).  With the
    genome's graph given, every unedited base carries its bigraph node and offset."""
    rng = np.random.default_rng(seed)
    reads = []
    for r in range(n_reads):
        length = int(min(length_fn(rng), len(genome) - 1))
        start = int(rng.integers(0, len(genome) - length + 1))
        gpos = np.arange(start, start + length)
        truth = genome[start:start + length]
        reverse = bool(rng.integers(0, 2))
        if reverse:
            truth = revcomp(truth)
            gpos = gpos[::-1]
        bases, src, exact = _apply_errors(rng, truth, float(error_fn(rng)))
        if dbg is None:
            bn = np.full(len(bases), -1, dtype=np.int64)
            bo = bn.copy()
        else:
            p = gpos[np.maximum(src, 0)]
            bn = dbg.pos_bignode[p]
            bo = dbg.pos_offset[p]
            if reverse:
                bo = dbg.node_len[bn // 2] - 1 - bo
                bn = bn ^ 1
            bn = np.where(exact & (src >= 0), bn, -1)
            bo = np.where(exact & (src >= 0), bo, -1)
        reads.append(Read(f"{prefix}{r}", bases.tobytes(), bn, bo, exact & (src >= 0)))
    return reads


def small_dbg_genome(seed: int = 0) -> np.ndarray:
    """100 kbp genome, 10 copies of a 2 kbp repeat at 1-3 % divergence, 20 tandem arrays."""
    return make_repeat_genome(100_000, 10, 2_000, 0.01, 0.03, 20, tandem_len=(200, 1000), seed=seed)


def mid_dbg_genome(seed: int = 0) -> np.ndarray:
    """1 Mbp genome, 20 copies of a 5 kbp repeat at 1-3 % divergence, 40 tandem arrays of period 2-50
    (the de Bruijn stress genome's shape at a tenth of its size)."""
    return make_repeat_genome(1_000_000, 20, 5_000, 0.01, 0.03, 40, seed=seed)


def stress_dbg_genome(seed: int = 0) -> np.ndarray:
    """10 Mbp genome, 200 copies of a 5 kbp repeat at 1-3 % divergence, tandem repeats of period 2-50."""
    return make_repeat_genome(10_000_000, 200, 5_000, 0.01, 0.03, 400, seed=seed)


def dbg_reads(genome: np.ndarray, n: int, length: int = 20_000, error: float = 0.12, seed: int = 1,
              dbg: DbgGraph | None = None) -> list:
    """Reads of ``length`` bp at ``error`` from the genome on random strands."""
    return sample_genome_reads(genome, n, seed, lambda rng: length, lambda rng: error, dbg=dbg)
