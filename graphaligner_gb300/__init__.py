"""GB300-native seed extension for GraphAligner.

The package holds the CUDA kernels of GraphAligner's seed-extension hot path
(banded Myers bit-vector DP over a genome graph with its component-ordered
frontier, X-drop and traceback) behind a C ABI (include/graphaligner_gb300.h),
and the host-side mirror of the reference interface that drives it.
"""
from .build import build  # noqa: F401

__all__ = ["build"]
