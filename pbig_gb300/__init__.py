"""GB300-native pairwise box-intersection engine (the PBIG pair-detection path).

The CUDA kernels and the C ABI live in ``csrc/`` (built in-tree by
``pbig_gb300.build``); ``engine`` is the Python face of that ABI and ``gen``
the seeded workload generators.
"""
from .engine import Engine, PbigError, Scene, tune_shift  # noqa: F401
from .gen import RANGE  # noqa: F401

__all__ = ["Engine", "PbigError", "Scene", "tune_shift", "RANGE"]
