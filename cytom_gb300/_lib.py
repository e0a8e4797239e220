"""ctypes binding of libcytom_gpu.so (include/cytom_gpu.h).

The library is the only compute path: loading fails loudly when it is missing,
and there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libcytom_gpu.so"

CYTOM_OK = 0
ERRORS = {
    -1: "CYTOM_ERR_INVAL", -2: "CYTOM_ERR_OOM", -3: "CYTOM_ERR_RANGE", -4: "CYTOM_ERR_TIMEOUT",
    -5: "CYTOM_ERR_CUDA", -6: "CYTOM_ERR_UNIMPLEMENTED", -7: "CYTOM_ERR_IO",
}
PTR_HOST, PTR_DEVICE = 0, 1
UNWEIGHTED, WEIGHT_U32, WEIGHT_F32 = 0, 1, 2
ALGO_BFS, ALGO_CC, ALGO_SSSP, ALGO_PR_DELTA, ALGO_PAGERANK, ALGO_WPAGERANK, ALGO_SSWP = 0, 1, 2, 3, 4, 5, 6
ALGO_BFS_ASYNC, ALGO_CC_ASYNC = 7, 8
TRAVERSAL_ROW_FIRST, TRAVERSAL_COLUMN_FIRST, TRAVERSAL_HILBERT = 0, 1, 2
KERNEL_CLASSES = 8


class Config(C.Structure):
    _fields_ = [
        ("max_vertices", C.c_uint64),
        ("vertices_per_tile", C.c_uint64),
        ("weight_type", C.c_int32),
        ("enable_adaptive_scheduling", C.c_int32),
        ("edge_capacity_hint", C.c_uint64),
        ("stream", C.c_void_p),
        ("traversal", C.c_int32),
        ("use_dynamic_compaction", C.c_int32),
    ]


class RmatParams(C.Structure):
    _fields_ = [
        ("scale", C.c_uint32),
        ("a", C.c_double),
        ("b", C.c_double),
        ("c", C.c_double),
        ("seed", C.c_uint64),
        ("weight_seed", C.c_uint64),
        ("wmin", C.c_uint32),
        ("wmax", C.c_uint32),
    ]


class JobParams(C.Structure):
    _fields_ = [
        ("start_vertex", C.c_uint64),
        ("max_iterations", C.c_uint64),
        ("delta", C.c_double),
        ("alpha", C.c_double),
        ("tolerance", C.c_double),
        ("kahan", C.c_int32),
        ("reserved", C.c_int32),
    ]


class RunStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_uint64),
        ("count_edges", C.c_uint64),
        ("edges_scanned", C.c_uint64),
        ("active_vertices", C.c_uint64),
        ("converged", C.c_int32),
        ("reserved", C.c_int32),
        ("residual", C.c_double),
        ("elapsed_ms", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


class KernelStats(C.Structure):
    _fields_ = [
        ("name", (C.c_char * 24) * KERNEL_CLASSES),
        ("launches", C.c_uint64 * KERNEL_CLASSES),
        ("total_ms", C.c_double * KERNEL_CLASSES),
        ("algo_bytes", C.c_double * KERNEL_CLASSES),
    ]


class TuneReport(C.Structure):
    _fields_ = [("variants", C.c_int32), ("chosen", C.c_int32 * 2), ("edges_per_thread", C.c_int32 * 8),
                ("pipeline_depth", C.c_int32 * 8), ("blocks_per_sm", C.c_int32 * 8), ("reserved", C.c_int32),
                ("us", (C.c_double * 8) * 2), ("tuned_edges", C.c_uint64), ("sparse_div", C.c_int32 * 2),
                ("div_candidates", C.c_int32 * 6), ("dense_round_us", (C.c_double * 6) * 2),
                ("sparse_round_us", (C.c_double * 6) * 2)]

    def as_dict(self) -> dict:
        k = self.variants
        shapes = [{"edges_per_thread": self.edges_per_thread[v], "pipeline_depth": self.pipeline_depth[v],
                   "blocks_per_sm": self.blocks_per_sm[v], "kernel": "tiles" if v == 4 else "stream"}
                  for v in range(k)]
        return {"shapes": shapes, "chosen": {"bfs_cc": self.chosen[0], "sssp": self.chosen[1]},
                "round_us": {"bfs_cc": [self.us[0][v] for v in range(k)], "sssp": [self.us[1][v] for v in range(k)]},
                "tuned_edges": self.tuned_edges,
                "sparse_div": {"bfs_cc": self.sparse_div[0], "sssp": self.sparse_div[1]},
                "sparse_threshold_table": {
                    "div_candidates": list(self.div_candidates),
                    "bfs_cc": {"dense_us": list(self.dense_round_us[0]), "sparse_us": list(self.sparse_round_us[0])},
                    "sssp": {"dense_us": list(self.dense_round_us[1]), "sparse_us": list(self.sparse_round_us[1])}}}


class FaultInjection(C.Structure):
    _fields_ = [("fail_alloc_after", C.c_uint64), ("idle_poll_limit", C.c_uint32), ("phantom_jobs", C.c_uint32)]


# (name, restype, argtypes) of every exported entry point of include/cytom_gpu.h
SIGNATURES = [
    ("cytom_config_default", None, [C.POINTER(Config)]),
    ("cytom_create", C.c_int, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    ("cytom_destroy", C.c_int, [C.c_void_p]),
    ("cytom_last_error", C.c_char_p, [C.c_void_p]),
    ("cytom_geometry", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    ("cytom_rmat_default", None, [C.POINTER(RmatParams)]),
    ("cytom_rmat_generate", C.c_int, [C.c_void_p, C.POINTER(RmatParams), C.c_uint64, C.c_uint64,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    ("cytom_gridgraph_decode", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                                         C.c_int, C.POINTER(C.c_uint64)]),
    ("cytom_load_gridgraph", C.c_int, [C.c_void_p, C.c_char_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    ("cytom_insert_batch", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int]),
    ("cytom_compact", C.c_int, [C.c_void_p]),
    ("cytom_clear", C.c_int, [C.c_void_p]),
    ("cytom_count_edges", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    ("cytom_get_tiles", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("cytom_get_degrees", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("cytom_job_params_default", None, [C.POINTER(JobParams)]),
    ("cytom_job_create", C.c_int, [C.c_void_p, C.c_int, C.POINTER(JobParams), C.POINTER(C.c_int)]),
    ("cytom_job_destroy", C.c_int, [C.c_void_p, C.c_int]),
    ("cytom_job_reset", C.c_int, [C.c_void_p, C.c_int]),
    ("cytom_run", C.c_int, [C.c_void_p, C.c_int, C.POINTER(RunStats)]),
    ("cytom_run_many", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.c_int, C.POINTER(RunStats)]),
    ("cytom_run_many_async", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.c_int]),
    ("cytom_run_many_wait", C.c_int, [C.c_void_p, C.POINTER(RunStats)]),
    ("cytom_run_batch", C.c_int, [C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.c_int, C.POINTER(RunStats)]),
    ("cytom_batch_units", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    ("cytom_job_set_teleport", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    ("cytom_pagerank_adjoint", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                         C.c_int, C.POINTER(RunStats)]),
    ("cytom_set_edge_weights", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int]),
    ("cytom_delete_batch", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int,
                                     C.POINTER(C.c_uint64)]),
    ("cytom_delete_random", C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p, C.c_int,
                                      C.POINTER(C.c_uint64)]),
    ("cytom_get_result", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    ("cytom_get_result_f64", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    ("cytom_autotune", C.c_int, [C.c_void_p, C.POINTER(TuneReport)]),
    ("cytom_get_tune_report", C.c_int, [C.c_void_p, C.POINTER(TuneReport)]),
    ("cytom_set_profiling", C.c_int, [C.c_void_p, C.c_int]),
    ("cytom_get_kernel_stats", C.c_int, [C.c_void_p, C.POINTER(KernelStats)]),
    ("cytom_reset_kernel_stats", C.c_int, [C.c_void_p]),
    ("cytom_launch_count", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    ("cytom_sync", C.c_int, [C.c_void_p]),
    ("cytom_set_fault_injection", C.c_int, [C.c_void_p, C.POINTER(FaultInjection)]),
    ("cytom_persist_edges", C.c_int, [C.c_void_p, C.c_char_p]),
    ("cytom_read_edges", C.c_int, [C.c_void_p, C.c_char_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    ("cytom_write_results", C.c_int, [C.c_void_p, C.c_int, C.c_char_p]),
    ("cytom_tile_batch_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint64,
                                           C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.POINTER(C.c_uint64), C.c_void_p]),
]

_LIB = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads libcytom_gpu.so; raises if it has not been built."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
            " (there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


class CytomError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def check(lib: C.CDLL, ctx, rc: int) -> None:
    if rc != CYTOM_OK:
        msg = lib.cytom_last_error(ctx)
        raise CytomError(rc, msg.decode() if msg else "")
