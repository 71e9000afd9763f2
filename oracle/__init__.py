"""ORACLE — test infrastructure, not product code.

CPU restatement of GraphAligner's seed-extension path (ga_oracle.cpp) and the
recipe that compiles the reference's own source into oracle/_ref/ga_ref
(Makefile + ref_driver.cpp + refshim/).  Only tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg use this package, and only as the checker or
the timed CPU baseline.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libga_oracle.so")
SRC = os.path.join(HERE, "ga_oracle.cpp")
REF_BIN = os.path.join(HERE, "_ref", "ga_ref")
# the GraphAligner checkout whose src/ the Makefile compiles (GA_REFERENCE overrides the default)
REFERENCE_ROOT = os.environ.get("GA_REFERENCE", "/root/reference")
REFERENCE_SRC = os.path.join(REFERENCE_ROOT, "src")

_lib = None


def build(reference: bool = True) -> str:
    """Compiles the restatement; also the reference driver when the reference source is present."""
    os.makedirs(BUILD, exist_ok=True)
    hdr = os.path.join(HERE, "..", "include", "graphaligner_gb300.h")
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(SRC), os.path.getmtime(hdr)):
        tmp = LIB + ".tmp"
        subprocess.run(["g++", "-std=c++17", "-O3", "-shared", "-fPIC", "-o", tmp, SRC, "-lpthread"], check=True)
        os.replace(tmp, LIB)
    if reference and os.path.isdir(REFERENCE_SRC):
        subprocess.run(["make", "-s", "-C", HERE, "-j8", f"GA_REFERENCE={REFERENCE_ROOT}"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(reference=False)
        _lib = ctypes.CDLL(LIB)
    return _lib


def extend(graph, params, batch, threads: int = 1):
    """Runs ora_extend_batch on a graphaligner_gb300.extend.PackedBatch; returns a BatchResult."""
    from graphaligner_gb300.extend import alloc_results, results_desc
    r = alloc_results(batch)
    d = graph.desc()
    p = params.c()
    b = batch.desc()
    rd = results_desc(r)
    rc = lib().ora_extend_batch(ctypes.byref(d), ctypes.byref(p), ctypes.byref(b), ctypes.byref(rd), int(threads))
    if rc != 0:
        raise RuntimeError(f"ora_extend_batch failed: {rc}")
    return r


def multiseed(graph, params, batch, threads: int = 1):
    """Runs ora_multiseed_batch on a graphaligner_gb300.extend.MultiseedBatch; returns a MultiseedResult."""
    from graphaligner_gb300.extend import MultiseedResult
    r = MultiseedResult.alloc(batch)
    d = graph.desc()
    p = params.c()
    b = batch.desc()
    rd = r.desc()
    rc = lib().ora_multiseed_batch(ctypes.byref(d), ctypes.byref(p), ctypes.byref(b), ctypes.byref(rd), int(threads))
    if rc != 0:
        raise RuntimeError(f"ora_multiseed_batch failed: {rc}")
    return r
