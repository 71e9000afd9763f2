"""Read-level alignment over the C ABI: GraphAligner's per-read flow with minimizer
seeding and both extensions of every seed on the GPU, GAF out.

``Aligner.align(names, seqs)`` returns the GAF text runComponentMappings would
write for those reads with the -x vg (or -x dbg) parameters (Aligner.cpp:440-592),
reads in input order.
"""
from __future__ import annotations

import ctypes
import dataclasses
import numpy as np

from . import _abi
from ._abi import ptr
from ._lib import check, lib


class HostGraphDesc(ctypes.Structure):
    _fields_ = [
        ("base", _abi.GraphDesc),
        ("node_ids", ctypes.POINTER(ctypes.c_int32)),
        ("node_offset", ctypes.POINTER(ctypes.c_uint32)),
        ("reverse", ctypes.POINTER(ctypes.c_uint8)),
        ("chain_number", ctypes.POINTER(ctypes.c_uint64)),
        ("chain_approx_pos", ctypes.POINTER(ctypes.c_uint64)),
        ("num_lookup", ctypes.c_uint32),
        ("lookup_ids", ctypes.POINTER(ctypes.c_int32)),
        ("original_size", ctypes.POINTER(ctypes.c_uint32)),
        ("lookup_offsets", ctypes.POINTER(ctypes.c_uint32)),
        ("lookup_nodes", ctypes.POINTER(ctypes.c_uint32)),
        ("names", ctypes.POINTER(ctypes.c_char_p)),
    ]

    @classmethod
    def from_graph(cls, g):
        keep = [np.ascontiguousarray(x, dtype=dt) for x, dt in (
            (g.node_ids, np.int32), (g.node_offset, np.uint32), (g.reverse, np.uint8), (g.chain_number, np.uint64),
            (g.chain_approx_pos, np.uint64), (g.lookup_ids, np.int32), (g.original_size, np.uint32),
            (g.lookup_offsets, np.uint32), (g.lookup_nodes, np.uint32))]
        # node names as one NUL-separated buffer and a pointer per name into it
        blob = ("\0".join(g.names) + "\0").encode()
        raw = np.frombuffer(blob, dtype=np.uint8)
        ends = np.flatnonzero(raw == 0)
        starts = np.concatenate(([0], ends[:-1] + 1)).astype(np.uint64)
        name_ptrs = starts + np.uint64(raw.ctypes.data)
        names = ctypes.cast(ctypes.c_void_p(name_ptrs.ctypes.data), ctypes.POINTER(ctypes.c_char_p))
        d = cls(_abi.GraphDesc.from_graph(g), ptr(keep[0], ctypes.c_int32), ptr(keep[1], ctypes.c_uint32),
                ptr(keep[2], ctypes.c_uint8), ptr(keep[3], ctypes.c_uint64), ptr(keep[4], ctypes.c_uint64),
                len(g.lookup_ids), ptr(keep[5], ctypes.c_int32), ptr(keep[6], ctypes.c_uint32),
                ptr(keep[7], ctypes.c_uint32), ptr(keep[8], ctypes.c_uint32), names)
        d._keep = (keep, blob, name_ptrs, d.base)
        return d


class AlignParams(ctypes.Structure):
    _fields_ = [
        ("extend", _abi.ExtendParams),
        ("minimizer_length", ctypes.c_uint32),
        ("minimizer_window", ctypes.c_uint32),
        ("minimizer_density", ctypes.c_double),
        ("minimizer_discard_fraction", ctypes.c_double),
        ("seed_extend_density", ctypes.c_double),
        ("min_cluster_size", ctypes.c_uint64),
        ("sloppy", ctypes.c_uint8),
        ("cigar_match_mismatch", ctypes.c_uint8),
        ("min_alignment_score", ctypes.c_int32),
        ("multimap_score_fraction", ctypes.c_double),
        ("multiseed_dp", ctypes.c_uint8),
    ]


class Seed(ctypes.Structure):
    """ga_seed: one SeedHit of MinimizerSeeder::getSeeds."""
    _fields_ = [("node_id", ctypes.c_int32), ("reverse", ctypes.c_uint32), ("node_offset", ctypes.c_uint64),
                ("seq_pos", ctypes.c_uint64), ("match_len", ctypes.c_uint32), ("raw_seed_goodness", ctypes.c_uint32),
                ("alignment_graph_node", ctypes.c_uint32), ("alignment_graph_offset", ctypes.c_uint32)]


class AlignStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("reads", "reads_with_seeds", "reads_aligned", "failed_reads", "bp_aligned",
                                                "rounds", "extensions", "cell_steps")] + \
               [(n, ctypes.c_double) for n in ("seed_ms", "extend_ms", "host_ms", "collect_ms", "staging_ms", "consume_ms", "finish_ms")] + \
              [(n, ctypes.c_uint64) for n in ("speculative_used", "speculative_discarded")] + \
              [(n, ctypes.c_double) for n in ("seed_lookup_ms", "seed_select_ms", "multiseed_kernel_ms")] + \
              [(n, ctypes.c_uint64) for n in ("multiseed_candidates", "multiseed_walks", "multiseed_traces", "multiseed_rounds")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class IndexInfo(ctypes.Structure):
    """ga_index_info: sizes of the minimizer index built by ga_aligner_create."""
    _fields_ = [(n, ctypes.c_uint64) for n in ("minimizer_length", "minimizer_window", "max_count", "num_keys", "num_positions",
                                                "table_capacity")] + [("build_ms", ctypes.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


def preset(name: str = "vg", bandwidth: int | None = None, tangle_effort: int | None = None, multiseed: bool = False) -> AlignParams:
    """AlignerMain.cpp:119-231 for the two presets (X-drop from the 0.66 clipping cutoff)."""
    from .extend import default_xdrop, xscore_error_cost
    if name == "vg":
        bw, cells, k, w, dens, ext_dens, discard = 10, 2**64 - 1, 15, 20, 10.0, -1.0, 0.001
    elif name == "dbg":
        bw, cells, k, w, dens, ext_dens, discard = 5, 10000, 19, 30, 5.0, 0.002, 0.0002
    else:
        raise ValueError(name)
    if bandwidth is not None:
        bw = bandwidth
    if tangle_effort is not None:
        cells = tangle_effort
    return AlignParams(_abi.ExtendParams(bw, default_xdrop(), cells, xscore_error_cost()), k, w, dens, discard,
                       ext_dens, 1, 1, 0, 0, 0.9, 1 if multiseed else 0)


class Aligner:
    def __init__(self, extender, graph, params: AlignParams):
        self.extender = extender
        self._desc = HostGraphDesc.from_graph(graph)
        self.params = params
        h = ctypes.c_void_p()
        check(lib().ga_aligner_create(extender.handle, ctypes.byref(self._desc), ctypes.byref(params), ctypes.byref(h)))
        self.handle = h

    def align(self, names, seqs) -> str:
        n = len(seqs)
        lens = np.fromiter((len(s) for s in seqs), dtype=np.uint32, count=n)
        offs = np.zeros(n, dtype=np.uint64)
        if n > 1:
            offs[1:] = np.cumsum(lens[:-1], dtype=np.uint64)
        blob = np.frombuffer(b"".join(bytes(s) for s in seqs) or b"\0", dtype=np.uint8).copy()
        cnames = (ctypes.c_char_p * max(1, n))(*[x.encode() for x in names])
        check(lib().ga_align_reads(self.handle, n, cnames, ptr(blob, ctypes.c_uint8), ptr(offs, ctypes.c_uint64), ptr(lens, ctypes.c_uint32)))
        text = ctypes.c_char_p()
        size = ctypes.c_uint64()
        check(lib().ga_aligner_gaf(self.handle, ctypes.byref(text), ctypes.byref(size)))
        return ctypes.string_at(text, size.value).decode()

    def seeds(self, seqs) -> list:
        """MinimizerSeeder::getSeeds per read (ga_aligner_get_seeds): a list of
        (node_id, node_offset, seq_pos, match_len, reverse, alignment_graph_node,
        alignment_graph_offset, raw_seed_goodness) tuples per read, in the reference's order."""
        n = len(seqs)
        lens = np.fromiter((len(s) for s in seqs), dtype=np.uint32, count=n)
        offs = np.zeros(n, dtype=np.uint64)
        if n > 1:
            offs[1:] = np.cumsum(lens[:-1], dtype=np.uint64)
        blob = np.frombuffer(b"".join(bytes(s) for s in seqs) or b"\0", dtype=np.uint8).copy()
        sp = ctypes.POINTER(Seed)()
        op = ctypes.POINTER(ctypes.c_uint64)()
        check(lib().ga_aligner_get_seeds(self.handle, n, ptr(blob, ctypes.c_uint8), ptr(offs, ctypes.c_uint64),
                                         ptr(lens, ctypes.c_uint32), ctypes.byref(sp), ctypes.byref(op)))
        out = []
        for i in range(n):
            out.append([(h.node_id, h.node_offset, h.seq_pos, h.match_len, h.reverse, h.alignment_graph_node,
                         h.alignment_graph_offset, h.raw_seed_goodness) for h in (sp[j] for j in range(op[i], op[i + 1]))])
        return out

    def index(self, arrays: bool = False):
        """The minimizer index built on the GPU (ga_aligner_index): its sizes and, with arrays,
        the distinct k-mers, each k-mer's first occurrence and the occurrences
        ((split node << 6) | offset, grouped by k-mer) as uint64 arrays."""
        info = IndexInfo()
        check(lib().ga_aligner_index(self.handle, ctypes.byref(info), None, None, None))
        if not arrays:
            return info.as_dict()
        keys = np.zeros(max(1, info.num_keys), dtype=np.uint64)
        start = np.zeros(info.num_keys + 1, dtype=np.uint64)
        pos = np.zeros(max(1, info.num_positions), dtype=np.uint64)
        check(lib().ga_aligner_index(self.handle, ctypes.byref(info), ptr(keys, ctypes.c_uint64), ptr(start, ctypes.c_uint64),
                                     ptr(pos, ctypes.c_uint64)))
        return info.as_dict(), keys[:info.num_keys], start, pos[:info.num_positions]

    def select_alignments(self, spans, min_alignment_score: int = 0, multimap_score_fraction: float = 0.9):
        """SelectAlignments on the device (ga_aligner_select_alignments): spans is, per read, a
        list of (alignmentStart, alignmentEnd, alignmentXScore); returns per read the kept flags."""
        first = np.zeros(len(spans) + 1, dtype=np.uint64)
        first[1:] = np.cumsum([len(x) for x in spans], dtype=np.uint64)
        flat = [a for x in spans for a in x] or [(0, 0, 0.0)]
        starts = np.array([a[0] for a in flat], dtype=np.uint64)
        ends = np.array([a[1] for a in flat], dtype=np.uint64)
        xs = np.array([a[2] for a in flat], dtype=np.float64)
        keep = np.zeros(len(flat), dtype=np.uint8)
        check(lib().ga_aligner_select_alignments(self.handle, len(spans), ptr(first, ctypes.c_uint64), ptr(starts, ctypes.c_uint64),
                                                 ptr(ends, ctypes.c_uint64), ptr(xs, ctypes.c_double), ctypes.c_int32(min_alignment_score),
                                                 ctypes.c_double(multimap_score_fraction), ptr(keep, ctypes.c_uint8)))
        return [list(keep[int(first[i]):int(first[i + 1])].astype(bool)) for i in range(len(spans))]

    def stats(self) -> dict:
        s = AlignStats()
        check(lib().ga_aligner_stats(self.handle, ctypes.byref(s)))
        return s.as_dict()

    def read_bp(self, n: int) -> np.ndarray:
        out = np.zeros(n, dtype=np.uint64)
        check(lib().ga_aligner_read_bp(self.handle, ptr(out, ctypes.c_uint64)))
        return out

    def close(self):
        if self.handle:
            lib().ga_aligner_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
