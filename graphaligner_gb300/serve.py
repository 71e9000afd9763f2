"""Serving loop over the C ABI (ga_server_*): reads are submitted one at a time and
come back as GAF text with their latency, while the graph and minimizer table stay
resident on the GPU.

The worker thread behind it does continuous batching: reads that arrive while
others are on the GPU are admitted (up to a read count and an estimated band-memory
budget), seeded as a group, and join the next extension round, so one launch holds
extensions of reads at different stages of their seed loops.  Each read's GAF bytes
are those ``Aligner.align`` gives for it alone.
"""
from __future__ import annotations

import ctypes
import dataclasses

from ._lib import check, lib


class ServerParams(ctypes.Structure):
    _fields_ = [
        ("max_reads_in_flight", ctypes.c_uint32),
        ("max_band_bytes", ctypes.c_uint64),
        ("band_bytes_per_bp", ctypes.c_uint32),
        ("lanes", ctypes.c_uint32),
        ("long_read_bp", ctypes.c_uint32),
    ]


class _Result(ctypes.Structure):
    _fields_ = [
        ("ticket", ctypes.c_uint64),
        ("status", ctypes.c_int32),
        ("alignments", ctypes.c_uint32),
        ("bp_aligned", ctypes.c_uint64),
        ("gaf", ctypes.c_void_p),
        ("gaf_bytes", ctypes.c_uint64),
        ("queue_ms", ctypes.c_double),
        ("latency_ms", ctypes.c_double),
    ]


class _Stats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_uint64),
        ("completed", ctypes.c_uint64),
        ("rounds", ctypes.c_uint64),
        ("extensions", ctypes.c_uint64),
        ("admissions", ctypes.c_uint64),
        ("max_in_flight", ctypes.c_uint64),
        ("mixed_rounds", ctypes.c_uint64),
        ("busy_ms", ctypes.c_double),
    ]


@dataclasses.dataclass
class ServedRead:
    ticket: int
    status: int
    alignments: int
    bp_aligned: int
    gaf: str
    queue_ms: float
    latency_ms: float


class Server:
    """``Server(aligner).submit(name, seq) -> ticket``; ``poll()`` returns finished reads."""

    def __init__(self, aligner, max_reads_in_flight: int = 0, max_band_bytes: int = 0, band_bytes_per_bp: int = 0,
                 lanes: int = 0, long_read_bp: int = 0):
        self.aligner = aligner
        self.params = ServerParams(max_reads_in_flight, max_band_bytes, band_bytes_per_bp, lanes, long_read_bp)
        h = ctypes.c_void_p()
        check(lib().ga_server_create(aligner.handle, ctypes.byref(self.params), ctypes.byref(h)))
        self.handle = h
        self._buf = (_Result * 256)()

    def submit(self, name: str, seq: bytes) -> int:
        t = ctypes.c_uint64()
        check(lib().ga_server_submit(self.handle, name.encode(), seq, len(seq), ctypes.byref(t)))
        return t.value

    def poll(self, wait_ms: int = 0, max_results: int = 256) -> list:
        n = ctypes.c_uint32()
        check(lib().ga_server_poll(self.handle, self._buf, min(max_results, 256), ctypes.byref(n), wait_ms))
        out = []
        for i in range(n.value):
            r = self._buf[i]
            text = ctypes.string_at(r.gaf, r.gaf_bytes).decode() if r.gaf_bytes else ""
            check(lib().ga_server_release(self.handle, ctypes.c_uint64(r.ticket)))
            out.append(ServedRead(r.ticket, r.status, r.alignments, r.bp_aligned, text, r.queue_ms, r.latency_ms))
        return out

    def stats(self) -> dict:
        s = _Stats()
        check(lib().ga_server_stats_get(self.handle, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in _Stats._fields_}

    def close(self):
        if self.handle:
            check(lib().ga_server_free(self.handle))
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
