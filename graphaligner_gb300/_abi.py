"""ctypes mirrors of the structs in include/graphaligner_gb300.h."""
from __future__ import annotations

import ctypes
import numpy as np

_u8p = ctypes.POINTER(ctypes.c_uint8)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_i32p = ctypes.POINTER(ctypes.c_int32)


def ptr(a: np.ndarray | None, ctype):
    if a is None:
        return ctypes.cast(None, ctypes.POINTER(ctype))
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctype))


class GraphDesc(ctypes.Structure):
    _fields_ = [
        ("num_nodes", ctypes.c_uint32),
        ("first_ambiguous", ctypes.c_uint32),
        ("node_length", _u32p),
        ("seq2bit", _u64p),
        ("seq_ambiguous", _u64p),
        ("in_offsets", _u32p),
        ("in_neighbors", _u32p),
        ("out_offsets", _u32p),
        ("out_neighbors", _u32p),
        ("linearizable", _u8p),
        ("component", _u32p),
    ]

    @classmethod
    def from_graph(cls, g):
        keep = [np.ascontiguousarray(x, dtype=dt) for x, dt in (
            (g.node_length, np.uint32), (g.seq2bit, np.uint64), (g.seq_ambiguous, np.uint64),
            (g.in_offsets, np.uint32), (g.in_neighbors, np.uint32), (g.out_offsets, np.uint32),
            (g.out_neighbors, np.uint32), (g.linearizable, np.uint8), (g.component, np.uint32))]
        d = cls(g.num_nodes, g.first_ambiguous,
                ptr(keep[0], ctypes.c_uint32), ptr(keep[1], ctypes.c_uint64), ptr(keep[2], ctypes.c_uint64),
                ptr(keep[3], ctypes.c_uint32), ptr(keep[4], ctypes.c_uint32), ptr(keep[5], ctypes.c_uint32),
                ptr(keep[6], ctypes.c_uint32), ptr(keep[7], ctypes.c_uint8), ptr(keep[8], ctypes.c_uint32))
        d._keep = keep
        return d


class ExtendParams(ctypes.Structure):
    _fields_ = [
        ("bandwidth", ctypes.c_uint32),
        ("xdrop", ctypes.c_int32),
        ("max_cells_per_slice", ctypes.c_uint64),
        ("xscore_error_cost", ctypes.c_int32),
    ]


class BatchDesc(ctypes.Structure):
    _fields_ = [
        ("num", ctypes.c_uint32),
        ("seq", _u8p),
        ("seq_offset", _u64p),
        ("seq_len", _u32p),
        ("start_node", _u32p),
        ("start_offset", _u32p),
        ("trace_offset", _u64p),
        ("trace_capacity", _u32p),
    ]


class Results(ctypes.Structure):
    _fields_ = [
        ("status", _i32p),
        ("score", _i32p),
        ("trace_len", _u32p),
        ("trace_items", _u64p),
        ("cell_steps", _u64p),
    ]


GA_OK, GA_TRACE_FAILED, GA_ASSERT, GA_CAPACITY, GA_BAD_REQUEST = 0, 1, 2, 3, 4


class MultiseedBatchDesc(ctypes.Structure):
    _fields_ = [
        ("num", ctypes.c_uint32),
        ("seq", _u8p),
        ("seq_offset", _u64p),
        ("seq_len", _u32p),
        ("seed_offset", _u64p),
        ("seed_slice", _u32p),
        ("seed_node", _u32p),
        ("trace_offset", _u64p),
        ("trace_capacity", _u64p),
        ("max_traces", ctypes.c_uint32),
        ("multimap_score_fraction", ctypes.c_double),
    ]


class MultiseedResults(ctypes.Structure):
    _fields_ = [
        ("status", _i32p),
        ("num_traces", _u32p),
        ("trace_score", _i32p),
        ("trace_start", _u64p),
        ("trace_len", _u32p),
        ("trace_items", _u64p),
        ("cell_steps", _u64p),
        ("items_needed", _u64p),
        ("traces_needed", _u32p),
    ]


class MultiseedOutput(ctypes.Structure):
    _fields_ = [
        ("status", _i32p),
        ("num_traces", _u32p),
        ("trace_first", _u64p),
        ("trace_score", _i32p),
        ("trace_start", _u64p),
        ("trace_len", _u32p),
        ("trace_items", _u64p),
        ("cell_steps", _u64p),
        ("total_traces", ctypes.c_uint64),
        ("total_items", ctypes.c_uint64),
    ]
