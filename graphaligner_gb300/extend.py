"""Host mirror of GraphAligner's seed-extension interface over the C ABI.

``Extender.extend`` is the batched form of
``GraphAlignerBitvectorBanded::getReverseTraceFromSeed(sequence, bigraphNodeId,
nodeOffset, Xdrop, state)`` (GraphAlignerBitvectorBanded.h:59-76): the same
arguments per extension, the same result (``OnewayTrace``: trace items in DP
order plus the score; a failed extension has score INT32_MAX,
GraphAlignerCommon.h:154-163), computed by the CUDA kernels in one batch.
A request that would make the reference throw ThreadReadAssertion::AssertionFailure
comes back with status GA_ASSERT, which the read-level code turns into the same
per-read drop the reference applies (Aligner.cpp:493-500).
"""
from __future__ import annotations

import ctypes
import dataclasses
import numpy as np

from . import _abi
from ._abi import ptr
from ._lib import check, lib

INT32_MAX = 2**31 - 1


def xscore_error_cost(precise_clipping: float = 0.66) -> int:
    """GraphAlignerCommon::Params::XscoreErrorCost (GraphAlignerCommon.h:94)."""
    return int(100 * (precise_clipping / (1.0 - precise_clipping) + 1.0))


def default_xdrop(precise_clipping: float = 0.66) -> int:
    """AlignerMain.cpp:220-231: X-drop so that a block of 50 mismatches ends an alignment."""
    x = 50.0
    if precise_clipping >= 0.501:
        x = max(x, 50 * (100 * (precise_clipping / (1.0 - precise_clipping) + 1.0)))
    return int(x)


@dataclasses.dataclass
class ExtendParams:
    bandwidth: int = 10
    xdrop: int = default_xdrop()
    max_cells_per_slice: int = 2**64 - 1
    xscore_error_cost: int = xscore_error_cost()

    def c(self):
        return _abi.ExtendParams(self.bandwidth, self.xdrop, self.max_cells_per_slice, self.xscore_error_cost)


@dataclasses.dataclass
class PackedBatch:
    """A batch in the C-ABI layout (host arrays)."""
    seq: np.ndarray
    seq_offset: np.ndarray
    seq_len: np.ndarray
    start_node: np.ndarray
    start_offset: np.ndarray
    trace_offset: np.ndarray
    trace_capacity: np.ndarray

    @property
    def num(self) -> int:
        return len(self.seq_len)

    @property
    def total_items(self) -> int:
        return int(self.trace_offset[-1] + self.trace_capacity[-1]) if self.num else 0

    def subset(self, idx) -> "PackedBatch":
        """The extensions at positions idx, repacked."""
        idx = np.asarray(idx, dtype=np.int64)
        lens = self.seq_len[idx]
        offs = np.zeros(len(idx), dtype=np.uint64)
        if len(idx) > 1:
            offs[1:] = np.cumsum(lens[:-1], dtype=np.uint64)
        parts = [self.seq[int(self.seq_offset[i]):int(self.seq_offset[i]) + int(self.seq_len[i])] for i in idx]
        seq = np.concatenate(parts) if parts else np.zeros(1, dtype=np.uint8)
        cap = trace_capacity_for(lens)
        toff = np.zeros(len(idx), dtype=np.uint64)
        if len(idx) > 1:
            toff[1:] = np.cumsum(cap[:-1].astype(np.uint64))
        return PackedBatch(seq, offs, lens.copy(), self.start_node[idx].copy(), self.start_offset[idx].copy(), toff, cap)

    def desc(self):
        return _abi.BatchDesc(self.num, ptr(self.seq, ctypes.c_uint8), ptr(self.seq_offset, ctypes.c_uint64),
                              ptr(self.seq_len, ctypes.c_uint32), ptr(self.start_node, ctypes.c_uint32),
                              ptr(self.start_offset, ctypes.c_uint32), ptr(self.trace_offset, ctypes.c_uint64),
                              ptr(self.trace_capacity, ctypes.c_uint32))


def trace_capacity_for(seq_len: np.ndarray) -> np.ndarray:
    """Room for a trace: one item per read row plus the horizontal (deletion) steps,
    which stay within a quarter of the read length at the error rates the
    workloads use (a trace that does not fit reports GA_CAPACITY)."""
    n = np.asarray(seq_len, dtype=np.uint64)
    return (n + n // 4 + 512).astype(np.uint32)


def pack_batch(graph, seqs, bignodes, offsets) -> PackedBatch:
    """Resolves (bigraphNodeId, nodeOffset) to split node + offset (AlignmentGraph::GetUnitigNode)
    and lays the sequences out contiguously."""
    n = len(seqs)
    lens = np.fromiter((len(s) for s in seqs), dtype=np.uint32, count=n)
    offs = np.zeros(n, dtype=np.uint64)
    if n > 1:
        offs[1:] = np.cumsum(lens[:-1], dtype=np.uint64)
    blob = np.frombuffer(b"".join(bytes(s) for s in seqs), dtype=np.uint8).copy() if n else np.zeros(1, np.uint8)
    sn = np.zeros(n, dtype=np.uint32)
    so = np.zeros(n, dtype=np.uint32)
    for i in range(n):
        sn[i], so[i] = graph.unitig_node(int(bignodes[i]), int(offsets[i]))
    cap = trace_capacity_for(lens)
    toff = np.zeros(n, dtype=np.uint64)
    if n > 1:
        toff[1:] = np.cumsum(cap[:-1].astype(np.uint64))
    return PackedBatch(blob, offs, lens, sn, so, toff, cap)


@dataclasses.dataclass
class BatchResult:
    status: np.ndarray
    score: np.ndarray
    trace_len: np.ndarray
    trace_items: np.ndarray
    trace_offset: np.ndarray
    cell_steps: np.ndarray

    def items(self, i: int) -> np.ndarray:
        o = int(self.trace_offset[i])
        return self.trace_items[o:o + int(self.trace_len[i])]

    def positions(self, i: int):
        """(node, nodeOffset, seqPos, nodeSwitch) per trace item, seqPos -1 above the read."""
        it = self.items(i)
        return ((it & 0xffffffff).astype(np.int64), ((it >> 32) & 63).astype(np.int64),
                (it >> 39).astype(np.int64) - 1, ((it >> 38) & 1).astype(np.int64))


def alloc_results(b: PackedBatch) -> BatchResult:
    n = b.num
    return BatchResult(np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n, np.uint32),
                       np.zeros(max(b.total_items, 1), np.uint64), b.trace_offset, np.zeros(n, np.uint64))


def results_desc(r: BatchResult):
    return _abi.Results(ptr(r.status, ctypes.c_int32), ptr(r.score, ctypes.c_int32), ptr(r.trace_len, ctypes.c_uint32),
                        ptr(r.trace_items, ctypes.c_uint64), ptr(r.cell_steps, ctypes.c_uint64))


@dataclasses.dataclass
class MultiseedBatch:
    """Reads and their multiseed DP seeds (prepareSeedsForMultiseeding: per read, (slice, split
    node) pairs in slice order), laid out for ga_multiseed_batch."""
    seq: np.ndarray
    seq_offset: np.ndarray
    seq_len: np.ndarray
    seed_offset: np.ndarray
    seed_slice: np.ndarray
    seed_node: np.ndarray
    trace_offset: np.ndarray
    trace_capacity: np.ndarray
    max_traces: int
    multimap_score_fraction: float = 0.9

    @property
    def num(self) -> int:
        return len(self.seq_len)

    @classmethod
    def pack(cls, seqs, seeds, max_traces: int = 64, items_per_bp: int = 4, multimap_score_fraction: float = 0.9):
        """seqs: read sequences; seeds: per read a list of (slice, split node)."""
        n = len(seqs)
        lens = np.fromiter((len(x) for x in seqs), dtype=np.uint32, count=n)
        offs = np.zeros(n, dtype=np.uint64)
        if n > 1:
            offs[1:] = np.cumsum(lens[:-1], dtype=np.uint64)
        blob = np.frombuffer(b"".join(bytes(x) for x in seqs) or b"\0", dtype=np.uint8).copy()
        soff = np.zeros(n + 1, dtype=np.uint64)
        soff[1:] = np.cumsum([len(x) for x in seeds], dtype=np.uint64)
        flat = [p for x in seeds for p in x] or [(0, 0)]
        sslice = np.array([p[0] for p in flat], dtype=np.uint32)
        snode = np.array([p[1] for p in flat], dtype=np.uint32)
        cap = lens.astype(np.uint64) * items_per_bp + 4096
        toff = np.zeros(n, dtype=np.uint64)
        if n > 1:
            toff[1:] = np.cumsum(cap[:-1])
        return cls(blob, offs, lens, soff, sslice, snode, toff, cap, max_traces, multimap_score_fraction)

    def desc(self):
        return _abi.MultiseedBatchDesc(self.num, ptr(self.seq, ctypes.c_uint8), ptr(self.seq_offset, ctypes.c_uint64),
                                       ptr(self.seq_len, ctypes.c_uint32), ptr(self.seed_offset, ctypes.c_uint64),
                                       ptr(self.seed_slice, ctypes.c_uint32), ptr(self.seed_node, ctypes.c_uint32),
                                       ptr(self.trace_offset, ctypes.c_uint64), ptr(self.trace_capacity, ctypes.c_uint64),
                                       self.max_traces, self.multimap_score_fraction)


@dataclasses.dataclass
class MultiseedResult:
    status: np.ndarray
    num_traces: np.ndarray
    trace_score: np.ndarray
    trace_start: np.ndarray
    trace_len: np.ndarray
    trace_items: np.ndarray
    cell_steps: np.ndarray
    trace_offset: np.ndarray
    max_traces: int
    items_needed: np.ndarray
    traces_needed: np.ndarray

    @classmethod
    def alloc(cls, b: MultiseedBatch):
        n, m = b.num, b.max_traces
        items = int(b.trace_offset[-1] + b.trace_capacity[-1]) if n else 1
        return cls(np.zeros(n, np.int32), np.zeros(n, np.uint32), np.zeros(n * m, np.int32), np.zeros(n * m, np.uint64),
                   np.zeros(n * m, np.uint32), np.zeros(max(items, 1), np.uint64), np.zeros(n, np.uint64), b.trace_offset, m,
                   np.zeros(n, np.uint64), np.zeros(n, np.uint32))

    def desc(self):
        return _abi.MultiseedResults(ptr(self.status, ctypes.c_int32), ptr(self.num_traces, ctypes.c_uint32),
                                     ptr(self.trace_score, ctypes.c_int32), ptr(self.trace_start, ctypes.c_uint64),
                                     ptr(self.trace_len, ctypes.c_uint32), ptr(self.trace_items, ctypes.c_uint64),
                                     ptr(self.cell_steps, ctypes.c_uint64), ptr(self.items_needed, ctypes.c_uint64),
                                     ptr(self.traces_needed, ctypes.c_uint32))

    def traces(self, i: int):
        """Read i's traces as (score, packed items), in the DP's order."""
        out = []
        for t in range(int(self.num_traces[i])):
            k = i * self.max_traces + t
            o = int(self.trace_offset[i] + self.trace_start[k])
            out.append((int(self.trace_score[k]), self.trace_items[o:o + int(self.trace_len[k])]))
        return out


@dataclasses.dataclass
class MultiseedExactResult:
    """ga_multiseed_batch_exact's output, copied out of the extender's buffers."""
    status: np.ndarray
    num_traces: np.ndarray
    trace_first: np.ndarray
    trace_score: np.ndarray
    trace_start: np.ndarray
    trace_len: np.ndarray
    trace_items: np.ndarray
    cell_steps: np.ndarray

    @classmethod
    def copy_of(cls, o, n: int):
        def arr(p, count, dtype):
            if count == 0 or not p:
                return np.zeros(0, dtype)
            return np.ctypeslib.as_array(p, shape=(count,)).astype(dtype, copy=True)
        t, i = int(o.total_traces), int(o.total_items)
        return cls(arr(o.status, n, np.int32), arr(o.num_traces, n, np.uint32), arr(o.trace_first, n, np.uint64),
                   arr(o.trace_score, t, np.int32), arr(o.trace_start, t, np.uint64), arr(o.trace_len, t, np.uint32),
                   arr(o.trace_items, i, np.uint64), arr(o.cell_steps, n, np.uint64))

    def traces(self, i: int):
        """Read i's traces as (score, packed items), in the DP's order."""
        out = []
        for t in range(int(self.num_traces[i])):
            k = int(self.trace_first[i]) + t
            o = int(self.trace_start[k])
            out.append((int(self.trace_score[k]), self.trace_items[o:o + int(self.trace_len[k])]))
        return out


class DeviceGraph:
    """AlignmentGraph arrays resident in HBM (ga_graph_upload)."""

    def __init__(self, graph, device: int = 0):
        self.graph = graph
        self._desc = graph.desc()
        h = ctypes.c_void_p()
        check(lib().ga_graph_upload(ctypes.byref(self._desc), device, ctypes.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            lib().ga_graph_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LaunchShape(ctypes.Structure):
    """ga_launch_shape: how the extension kernels are launched (one warp per extension; results
    never depend on it): warps per block, resident blocks per SM (0 = as many as fit), the
    first pass's frontier-table layout (0 shared memory, 1/2 global memory) and the arena
    chunk a warp takes at once, in KiB."""
    _fields_ = [
        ("warps_per_block", ctypes.c_uint32),
        ("blocks_per_sm", ctypes.c_uint32),
        ("first_layout", ctypes.c_uint32),
        ("chunk_kib", ctypes.c_uint32),
    ]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}

    def as_tuple(self):
        return tuple(getattr(self, n) for n, _ in self._fields_)


# launch shapes the autotuner tries: (warps_per_block, blocks_per_sm, first_layout, chunk_kib)
DEFAULT_CANDIDATES = [
    (4, 0, 0, 64), (2, 0, 0, 64), (1, 0, 0, 64), (4, 3, 0, 64), (4, 2, 0, 64),
    (4, 0, 0, 16), (4, 0, 0, 256), (4, 0, 1, 64),
]


class Extender:
    """Batched getReverseTraceFromSeed on the GPU."""

    def __init__(self, dgraph: DeviceGraph, arena_bytes: int = 0):
        self.dgraph = dgraph
        h = ctypes.c_void_p()
        check(lib().ga_extender_create(dgraph.handle, ctypes.c_uint64(arena_bytes), ctypes.byref(h)))
        self.handle = h

    def run(self, params: ExtendParams, batch: PackedBatch, out: BatchResult | None = None) -> BatchResult:
        r = out if out is not None else alloc_results(batch)
        p = params.c()
        d = batch.desc()
        rd = results_desc(r)
        check(lib().ga_extend_batch(self.handle, ctypes.byref(p), ctypes.byref(d), ctypes.byref(rd)))
        return r

    def extend(self, params: ExtendParams, seqs, bignodes, offsets) -> BatchResult:
        return self.run(params, pack_batch(self.dgraph.graph, seqs, bignodes, offsets))

    def multiseed(self, params: ExtendParams, batch: MultiseedBatch) -> MultiseedResult:
        """ga_multiseed_batch: the multiseed DP of every read of the batch."""
        r = MultiseedResult.alloc(batch)
        p = params.c()
        d = batch.desc()
        rd = r.desc()
        check(lib().ga_multiseed_batch(self.handle, ctypes.byref(p), ctypes.byref(d), ctypes.byref(rd)))
        return r

    def multiseed_exact(self, params: ExtendParams, batch: MultiseedBatch) -> MultiseedExactResult:
        """ga_multiseed_batch_exact: the same DP with every read's traces in room sized to them."""
        o = _abi.MultiseedOutput()
        p = params.c()
        d = batch.desc()
        check(lib().ga_multiseed_batch_exact(self.handle, ctypes.byref(p), ctypes.byref(d), ctypes.byref(o)))
        return MultiseedExactResult.copy_of(o, batch.num)

    def launch_shape(self) -> LaunchShape:
        sh = LaunchShape()
        check(lib().ga_extender_get_launch_shape(self.handle, ctypes.byref(sh)))
        return sh

    def set_launch_shape(self, warps_per_block=4, blocks_per_sm=0, first_layout=0, chunk_kib=64):
        sh = LaunchShape(warps_per_block, blocks_per_sm, first_layout, chunk_kib)
        check(lib().ga_extender_set_launch_shape(self.handle, ctypes.byref(sh)))

    def autotune(self, params: ExtendParams, batch: PackedBatch, candidates=None, sample_every: int = 4, repeats: int = 2) -> dict:
        """Times each launch shape on an evenly spaced sample of the batch (device time of the
        kernels, ``ga_extender_autotune``) and keeps the fastest.  The sample stays on the
        device; every candidate must give the same statuses and scores (GAError otherwise)."""
        idx = np.arange(0, batch.num, max(1, sample_every))
        sub = batch.subset(idx)
        cands = list(candidates or DEFAULT_CANDIDATES)
        shapes = (LaunchShape * len(cands))()
        for i, c in enumerate(cands):
            shapes[i] = LaunchShape(*c)
        ms = (ctypes.c_float * len(cands))()
        p = params.c()
        d = sub.desc()
        check(lib().ga_extender_autotune(self.handle, ctypes.byref(p), ctypes.byref(d), shapes,
                                         ctypes.c_uint32(len(cands)), ctypes.c_uint32(max(1, repeats)), ms))
        return {"chosen": self.launch_shape().as_dict(), "sample_extensions": int(len(idx)),
                "candidates_ms": [(round(float(ms[i]), 2), list(c)) for i, c in enumerate(cands)]}

    def last_times(self):
        f = ctypes.c_float()
        t = ctypes.c_float()
        check(lib().ga_extender_last_times(self.handle, ctypes.byref(f), ctypes.byref(t)))
        return f.value, t.value

    def last_arena_bytes(self) -> int:
        """DP-table bytes the first pass of the last call wrote to the arena."""
        b = ctypes.c_uint64()
        check(lib().ga_extender_last_arena_bytes(self.handle, ctypes.byref(b)))
        return int(b.value)

    def last_layout_counts(self):
        """Extensions run with each frontier-table layout (0, 1, 2) by the last call."""
        c = (ctypes.c_uint32 * 3)()
        check(lib().ga_extender_last_layout_counts(self.handle, c))
        return [int(v) for v in c]

    def last_launches(self) -> int:
        n = ctypes.c_uint32()
        check(lib().ga_extender_last_launches(self.handle, ctypes.byref(n)))
        return n.value

    def close(self):
        if self.handle:
            lib().ga_extender_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
