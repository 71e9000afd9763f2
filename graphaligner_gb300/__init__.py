"""GB300-native seed extension for GraphAligner.

The package holds the CUDA kernels of GraphAligner's seed-extension hot path
(banded Myers bit-vector DP over a genome graph with its component-ordered
frontier, X-drop and traceback; minimizer k-mer lookups) and the host code of the
read-level flow (seed loop, selection, GAF, serving loop) behind a C ABI
(include/graphaligner_gb300.h), with the Python mirror of the reference interface:
``extend.Extender`` (getReverseTraceFromSeed, batched), ``align.Aligner`` (the
per-read flow of the aligner) and ``serve.Server`` (continuous batching).
``graph.build_from_gfa`` builds an alignment graph from GFA text in native code;
``graph.load_gag`` reads one the reference built.
"""
from .build import build  # noqa: F401

__all__ = ["build"]
