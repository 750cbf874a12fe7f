"""GB300-native (sm_103a) FFT-domain Bayesian AVO inversion -- CRAVA's hot path.

The compute lives in libcravagpu.so (CUDA, C-ABI in include/cravagpu.h);
this package builds and loads it and mirrors the reference's FFTGrid/Crava
calling surface for Python callers.
"""
from ._native import build, lib  # noqa: F401

__all__ = ["build", "lib"]
