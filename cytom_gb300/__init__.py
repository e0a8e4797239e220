"""cytom_gb300 — GB300-native (sm_103a) evolving-graph engine with Cytom's operator surface.

The compute path is libcytom_gpu.so (hand-written CUDA kernels behind the C ABI of
include/cytom_gpu.h); this package only binds it. Importing the package does not
load the library; Engine() does, and raises when it has not been built.
"""
from . import _lib
from ._lib import (ALGO_BFS, ALGO_BFS_ASYNC, ALGO_CC, ALGO_CC_ASYNC, ALGO_PAGERANK, ALGO_PR_DELTA, ALGO_SSSP, ALGO_SSWP, ALGO_WPAGERANK, CytomError,
                   TRAVERSAL_COLUMN_FIRST, TRAVERSAL_HILBERT, TRAVERSAL_ROW_FIRST, UNWEIGHTED, WEIGHT_F32, WEIGHT_U32, load)
from .engine import (BFS, CC, SSSP, BFSAsync, CCAsync, SSWP, Engine, PageRank, PageRankDelta, Program, TileView, WeightedPageRank,
                     run_batch)

__all__ = [
    "Engine", "Program", "BFS", "CC", "BFSAsync", "CCAsync", "SSSP", "SSWP", "PageRankDelta", "PageRank", "WeightedPageRank", "TileView",
    "run_batch",
    "CytomError", "load", "UNWEIGHTED", "WEIGHT_U32", "WEIGHT_F32",
    "ALGO_BFS", "ALGO_CC", "ALGO_SSSP", "ALGO_PR_DELTA", "ALGO_PAGERANK", "ALGO_WPAGERANK", "ALGO_SSWP",
    "ALGO_BFS_ASYNC", "ALGO_CC_ASYNC", "TRAVERSAL_ROW_FIRST", "TRAVERSAL_COLUMN_FIRST", "TRAVERSAL_HILBERT",
]
