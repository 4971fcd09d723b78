"""GB300-native bidirectional wavefront aligner (gap-affine BiWFA, score + CIGAR).

The aligner is libbiwfa_gb300.so (C ABI in include/wfa_gpu.h); this package holds its
CUDA/C++ sources (csrc/), the build recipe (build.py) and a ctypes mirror of the C ABI.
"""
from ._capi import load as load_library  # noqa: F401
from .aligner import (BatchAligner, BatchResult, PairBatch, PinnedHost, ScorePredictor, WavefrontAligner,  # noqa: F401,E501
                      runs_to_cigar, runs_to_ops)

__all__ = ["load_library", "BatchAligner", "BatchResult", "PairBatch", "PinnedHost", "ScorePredictor", "WavefrontAligner",
           "runs_to_cigar", "runs_to_ops"]
