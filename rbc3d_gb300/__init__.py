"""GB300 (sm_103a) implementation of RBC3D's Ewald-split boundary-integral
matvec behind a C ABI (include/rbc3d_gpu.h).

The compute path is ``librbc3d_gb300.so`` (CUDA C++, built in-tree by
``rbc3d_gb300.build``).  There is no CPU fallback: :func:`library` raises if
the shared library is missing or cannot be loaded.
"""
from __future__ import annotations

import os

from .abi import (FP32C, FP32D, FP32M, FP64, TERM_ALL, TERM_CORR, TERM_LINEAR, TERM_PME, TERM_REAL,
                  TERM_WALLS, TLIST_RAW, TLIST_RBC, TLIST_WALL, Context, Library, RBC3DError)

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "librbc3d_gb300.so")
_LIB = None


def library(build_if_missing: bool = False) -> Library:
    """Load the GPU library (prefix ``rbc3d_``).  Raises if it is absent."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise RuntimeError(f"{LIB_PATH} is not built; run `python -m rbc3d_gb300.build`")
            from . import build as _b
            _b.build()
        _LIB = Library(LIB_PATH, "rbc3d_")
    return _LIB


def context(params: dict) -> Context:
    """Create a GPU context (replaces PME_Init + table set-up of RBC3D)."""
    return Context(library(), params)


__all__ = ["library", "context", "Context", "Library", "RBC3DError", "FP64", "FP32C", "FP32M", "FP32D", "TLIST_RBC",
           "TLIST_WALL", "TLIST_RAW", "TERM_ALL", "TERM_REAL", "TERM_CORR", "TERM_LINEAR", "TERM_PME",
           "TERM_WALLS"]
