"""Python host mirror of Cytom's operator surface over the C ABI.

Names follow the reference (oslab-swrc/cytom):
  Engine                 one graph: VertexStore + TileStore of execute<V,A,w>
                         (src/include/main/execute.h:534-620)
  Engine.insert_edges    MetaTileManager::insertEdge for a batch (meta-tile-manager.h:112-125)
  Engine.do_global_compaction   TileStore::doGlobalCompaction (tile-store.h:144-172)
  Engine.count_edges     TileStore::countEdges (tile-store.h:174-185)
  Engine.tile(x, y)      TileManager view: getCounts / getIdCounts / getTargets
                         (tile-manager.h:459-467)
  BFS / CC / SSSP / PageRankDelta / PageRank   vertex programs (examples/*.cc)
  Program.execute_algorithm   ContinuousAlgorithmExecutor::executeAlgorithm
                         (continuous-algorithm-executor.h:49-249)

Host arrays are numpy; device arrays may be any object with a CUDA data pointer
(``data_ptr()`` of a torch tensor, or an int address) and are passed as such.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L


def _ptr(a):
    """Returns (address, where) for a numpy array, torch tensor or raw int address."""
    if a is None:
        return None, L.PTR_HOST
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays must be C-contiguous")
        return a.ctypes.data, L.PTR_HOST
    if hasattr(a, "data_ptr") and hasattr(a, "is_cuda"):
        if not a.is_contiguous():
            raise ValueError("tensors must be contiguous")
        return a.data_ptr(), (L.PTR_DEVICE if a.is_cuda else L.PTR_HOST)
    if isinstance(a, int):
        return a, L.PTR_DEVICE
    raise TypeError(f"unsupported buffer type {type(a)}")


@dataclass
class TileView:
    """One tile in the reference's CSR terms (TileManager, tile-manager.h:585-591)."""
    x: int
    y: int
    edges: np.ndarray        # packed (src_local << 16 | tgt_local), CSR order
    weights: np.ndarray | None
    compact: bool            # compact counts_[vpt] storage vs sparse id_counts_

    @property
    def targets(self) -> np.ndarray:
        return (self.edges & 0xFFFF).astype(np.uint16)

    @property
    def sources(self) -> np.ndarray:
        return (self.edges >> 16).astype(np.uint16)

    def counts(self, vpt: int) -> np.ndarray:
        """counts_[vpt] (compact storage): out-edges per local source."""
        return np.bincount(self.sources, minlength=vpt)[:vpt]

    def id_counts(self) -> list[tuple[int, int]]:
        """id_counts_ (sparse storage): (count, id) runs of distinct sources."""
        ids, cnt = np.unique(self.sources, return_counts=True)
        return list(zip(cnt.tolist(), ids.tolist()))


class Engine:
    def __init__(self, max_vertices: int, vertices_per_tile: int = 65536,
                 weight_type: int = L.UNWEIGHTED, adaptive_scheduling: bool = True,
                 stream: int | None = None, lib=None, traversal: int = L.TRAVERSAL_ROW_FIRST,
                 dynamic_compaction: bool = False):
        self.lib = lib or L.load()
        cfg = L.Config()
        self.lib.cytom_config_default(C.byref(cfg))
        cfg.max_vertices = max_vertices
        cfg.vertices_per_tile = vertices_per_tile
        cfg.weight_type = weight_type
        cfg.enable_adaptive_scheduling = 1 if adaptive_scheduling else 0
        cfg.stream = stream
        cfg.traversal = traversal
        cfg.use_dynamic_compaction = 1 if dynamic_compaction else 0
        h = C.c_void_p()
        rc = self.lib.cytom_create(C.byref(cfg), C.byref(h))
        if rc != L.CYTOM_OK:
            raise L.CytomError(rc, "cytom_create failed")
        self.ctx = h
        v, vpt, t = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self._check(self.lib.cytom_geometry(self.ctx, C.byref(v), C.byref(vpt), C.byref(t)))
        self.n, self.vpt, self.tiles_per_dim = v.value, vpt.value, t.value
        self.weight_type = weight_type

    # -- lifecycle --
    def close(self):
        if getattr(self, "ctx", None):
            self.lib.cytom_destroy(self.ctx)
            self.ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        L.check(self.lib, self.ctx, rc)

    # -- edge sources --
    def generate_rmat(self, first: int, count: int, scale: int, seed: int = 2,
                      a: float | None = None, b: float | None = None, c: float | None = None,
                      weight_seed: int = 0, wmin: int = 1, wmax: int = 0, out=None):
        """RMATContext::getEdge(first .. first+count) (rmat-context.h:67-73). Returns host
        numpy arrays (src, tgt, w) unless `out` = (src, tgt, w) device buffers is given."""
        p = L.RmatParams()
        self.lib.cytom_rmat_default(C.byref(p))
        p.scale, p.seed, p.weight_seed, p.wmin, p.wmax = scale, seed, weight_seed, wmin, wmax
        if a is not None:
            p.a, p.b, p.c = a, b, c
        if out is None:
            src = np.empty(count, np.uint32)
            tgt = np.empty(count, np.uint32)
            w = np.empty(count, np.uint32) if wmax > 0 else None
            self._check(self.lib.cytom_rmat_generate(
                self.ctx, C.byref(p), first, count, src.ctypes.data, tgt.ctypes.data,
                w.ctypes.data if w is not None else None, L.PTR_HOST))
            return src, tgt, w
        s, _ = _ptr(out[0])
        t, _ = _ptr(out[1])
        wp, _ = _ptr(out[2]) if (len(out) > 2 and out[2] is not None) else (None, 0)
        self._check(self.lib.cytom_rmat_generate(self.ctx, C.byref(p), first, count, s, t, wp,
                                                 L.PTR_DEVICE))
        return out

    def decode_gridgraph(self, data: bytes):
        """GridGraph records (little-endian int32 pairs) -> (src, tgt) host arrays."""
        m = len(data) // 8
        src = np.empty(m, np.uint32)
        tgt = np.empty(m, np.uint32)
        buf = C.create_string_buffer(bytes(data), len(data))
        cnt = C.c_uint64()
        self._check(self.lib.cytom_gridgraph_decode(self.ctx, C.cast(buf, C.c_void_p), len(data),
                                                    src.ctypes.data, tgt.ctypes.data, L.PTR_HOST,
                                                    C.byref(cnt)))
        return src, tgt

    def load_gridgraph(self, path: str, batch: int = 1 << 20) -> int:
        cnt = C.c_uint64()
        self._check(self.lib.cytom_load_gridgraph(self.ctx, str(path).encode(), batch, C.byref(cnt)))
        return cnt.value

    # -- tile store --
    def insert_edges(self, src, tgt, w=None):
        sp, where = _ptr(src)
        tp, where2 = _ptr(tgt)
        wp, _ = _ptr(w)
        if where != where2:
            raise ValueError("src and tgt must live on the same side")
        n = len(src) if not isinstance(src, int) else None
        if n is None:
            raise ValueError("pass arrays or tensors, not raw addresses")
        self._check(self.lib.cytom_insert_batch(self.ctx, sp, tp, wp, n, where))

    def insert_edges_device(self, src_addr: int, tgt_addr: int, w_addr: int | None, count: int):
        self._check(self.lib.cytom_insert_batch(self.ctx, src_addr, tgt_addr, w_addr, count,
                                                L.PTR_DEVICE))

    def delete_edges(self, src, tgt) -> int:
        """Deletes stored edges (MetaTileManager::deleteEdge); returns how many were stored.

        Arrays may be numpy (host) or CUDA tensors (device)."""
        if isinstance(src, np.ndarray):
            src = np.ascontiguousarray(src, np.uint32)
        if isinstance(tgt, np.ndarray):
            tgt = np.ascontiguousarray(tgt, np.uint32)
        sp, where = _ptr(src)
        tp, where2 = _ptr(tgt)
        if where != where2:
            raise ValueError("src and tgt must live on the same side")
        if isinstance(src, int):
            raise ValueError("pass arrays or tensors, not raw addresses")
        cnt = C.c_uint64()
        self._check(self.lib.cytom_delete_batch(self.ctx, sp, tp, len(src), where, C.byref(cnt)))
        return cnt.value

    def delete_random(self, count: int, seed: int = 0):
        """Deletes `count` random stored edges (uniform tile, then uniform edge: the
        reference's deletion_percentage mode). Returns (deleted, src picks, tgt picks),
        UINT32_MAX where a pick hit an empty tile."""
        src = np.empty(count, np.uint32)
        tgt = np.empty(count, np.uint32)
        cnt = C.c_uint64()
        self._check(self.lib.cytom_delete_random(self.ctx, count, seed, src.ctypes.data, tgt.ctypes.data,
                                                 L.PTR_HOST, C.byref(cnt)))
        return cnt.value, src, tgt

    def set_edge_weights(self, src, tgt, w):
        """Overwrites the weights of stored edges (uint32 values or float32 bit patterns)."""
        src = np.ascontiguousarray(src, np.uint32)
        tgt = np.ascontiguousarray(tgt, np.uint32)
        w = np.ascontiguousarray(w)
        if w.dtype == np.float32:
            w = w.view(np.uint32)
        w = np.ascontiguousarray(w, np.uint32)
        self._check(self.lib.cytom_set_edge_weights(self.ctx, src.ctypes.data, tgt.ctypes.data, w.ctypes.data,
                                                    len(src), L.PTR_HOST))

    def persist_edges(self, path):
        """Start (or, with None, stop) logging inserted batches to `path` (EdgesWriter format)."""
        self._check(self.lib.cytom_persist_edges(self.ctx, None if path is None else str(path).encode()))

    def read_edges(self, path, batch: int = 1 << 20) -> int:
        """Insert the records of an edge log (EdgesWriter format); returns the record count."""
        cnt = C.c_uint64()
        self._check(self.lib.cytom_read_edges(self.ctx, str(path).encode(), batch, C.byref(cnt)))
        return cnt.value

    def run_many(self, programs) -> list[dict]:
        """Runs programs of this engine together (cytom_run_many): BFS / CC / SSSP / SSWP
        jobs run concurrently, each on a stream of its own; returns their statistics."""
        programs = list(programs)
        if not programs:
            return []
        n = len(programs)
        ids = (C.c_int * n)(*[p.job for p in programs])
        stats = (L.RunStats * n)()
        self._check(self.lib.cytom_run_many(self.ctx, ids, n, stats))
        return [stats[k].as_dict() for k in range(n)]

    def run_many_async(self, programs):
        """Queues programs of this engine side by side (cytom_run_many_async) and returns at
        once; the next batch may be inserted and compacted while they run. Collect the
        statistics with run_many_wait() before the next asynchronous launch."""
        programs = list(programs)
        ids = (C.c_int * len(programs))(*[p.job for p in programs])
        self._check(self.lib.cytom_run_many_async(self.ctx, ids, len(programs)))
        self._async_count = len(programs)

    def run_many_wait(self) -> list[dict]:
        n = getattr(self, "_async_count", 0)
        stats = (L.RunStats * max(n, 1))()
        self._check(self.lib.cytom_run_many_wait(self.ctx, stats))
        self._async_count = 0
        return [stats[k].as_dict() for k in range(n)]

    def autotune(self) -> dict:
        """Times the streaming-gather shapes on the current graph and keeps the fastest."""
        rep = L.TuneReport()
        self._check(self.lib.cytom_autotune(self.ctx, C.byref(rep)))
        return rep.as_dict()

    def tune_report(self) -> dict:
        rep = L.TuneReport()
        self._check(self.lib.cytom_get_tune_report(self.ctx, C.byref(rep)))
        return rep.as_dict()

    def do_global_compaction(self):
        self._check(self.lib.cytom_compact(self.ctx))

    def clear(self):
        """Drops every edge and zeroes the degrees (cytom_clear); buffers, tuned shapes and
        jobs stay, and every job restarts from scratch on its next run."""
        self._check(self.lib.cytom_clear(self.ctx))

    def count_edges(self) -> tuple[int, int]:
        a, b = C.c_uint64(), C.c_uint64()
        self._check(self.lib.cytom_count_edges(self.ctx, C.byref(a), C.byref(b)))
        return a.value, b.value

    def dump_tiles(self, weights: bool = False):
        """(tile_ptr, edges, weights|None, compact flags) of the compacted store."""
        e, _ = self.count_edges()
        ntiles = self.tiles_per_dim ** 2
        tp = np.empty(ntiles + 1, np.uint64)
        ed = np.empty(max(e, 1), np.uint32)
        wt = np.empty(max(e, 1), np.uint32) if weights else None
        cf = np.empty(ntiles, np.uint8)
        self._check(self.lib.cytom_get_tiles(self.ctx, tp.ctypes.data, ed.ctypes.data,
                                             wt.ctypes.data if wt is not None else None,
                                             cf.ctypes.data))
        return tp, ed[:e], (wt[:e] if wt is not None else None), cf

    def tile(self, x: int, y: int) -> TileView:
        tp, ed, wt, cf = self.dump_tiles(weights=self.weight_type != L.UNWEIGHTED)
        t = x * self.tiles_per_dim + y
        lo, hi = int(tp[t]), int(tp[t + 1])
        return TileView(x, y, ed[lo:hi].copy(), wt[lo:hi].copy() if wt is not None else None,
                        bool(cf[t]))

    def degrees(self):
        out = np.empty(self.n, np.uint32)
        inn = np.empty(self.n, np.uint32)
        self._check(self.lib.cytom_get_degrees(self.ctx, out.ctypes.data, inn.ctypes.data))
        return out, inn

    def launch_count(self) -> int:
        v = C.c_uint64()
        self._check(self.lib.cytom_launch_count(self.ctx, C.byref(v)))
        return v.value

    def set_profiling(self, on: bool):
        self._check(self.lib.cytom_set_profiling(self.ctx, 1 if on else 0))

    def kernel_stats(self) -> dict:
        ks = L.KernelStats()
        self._check(self.lib.cytom_get_kernel_stats(self.ctx, C.byref(ks)))
        out = {}
        for k in range(L.KERNEL_CLASSES):
            name = bytes(ks.name[k]).split(b"\0")[0].decode()
            out[name] = {"launches": ks.launches[k], "total_ms": ks.total_ms[k],
                         "algo_bytes": ks.algo_bytes[k]}
        return out

    def reset_kernel_stats(self):
        self._check(self.lib.cytom_reset_kernel_stats(self.ctx))

    def sync(self):
        self._check(self.lib.cytom_sync(self.ctx))

    def set_fault_injection(self, fail_alloc_after: int = 0, idle_poll_limit: int = 0, phantom_jobs: int = 0):
        """Test hook (cytom_set_fault_injection): the fail_alloc_after-th allocation from now
        on fails once; the batched executor's idle wait gives up after idle_poll_limit
        empty polls; phantom_jobs unfinished jobs without work keep its blocks waiting."""
        f = L.FaultInjection(fail_alloc_after, idle_poll_limit, phantom_jobs)
        self._check(self.lib.cytom_set_fault_injection(self.ctx, C.byref(f)))


class Program:
    """A vertex program bound to an Engine (one job with device-resident state)."""
    ALGO = -1
    result_dtype = np.uint32

    def __init__(self, engine: Engine, start_vertex: int = 1, max_iterations: int = 100,
                 delta: float = 0.01, alpha: float = 0.85, tolerance: float = 0.0,
                 kahan: bool = True):
        self.engine = engine
        p = L.JobParams()
        engine.lib.cytom_job_params_default(C.byref(p))
        p.start_vertex, p.max_iterations = start_vertex, max_iterations
        p.delta, p.alpha, p.tolerance, p.kahan = delta, alpha, tolerance, 1 if kahan else 0
        jid = C.c_int()
        engine._check(engine.lib.cytom_job_create(engine.ctx, self.ALGO, C.byref(p), C.byref(jid)))
        self.job = jid.value

    def execute_algorithm(self) -> dict:
        st = L.RunStats()
        self.engine._check(self.engine.lib.cytom_run(self.engine.ctx, self.job, C.byref(st)))
        return st.as_dict()

    def init_algorithm(self):
        """ContinuousAlgorithmExecutor::initAlgorithm: the next run starts from scratch."""
        self.engine._check(self.engine.lib.cytom_job_reset(self.engine.ctx, self.job))

    def result(self, out=None):
        if out is None:
            r = np.empty(self.engine.n, self.result_dtype)
            self.engine._check(self.engine.lib.cytom_get_result(self.engine.ctx, self.job,
                                                                r.ctypes.data, L.PTR_HOST))
            return r
        p, where = _ptr(out)
        self.engine._check(self.engine.lib.cytom_get_result(self.engine.ctx, self.job, p, where))
        return out

    def result64(self):
        """FP64 ranks (PageRank run in the FP64 plain form, kahan=False)."""
        r = np.empty(self.engine.n, np.float64)
        self.engine._check(self.engine.lib.cytom_get_result_f64(self.engine.ctx, self.job,
                                                                r.ctypes.data, L.PTR_HOST))
        return r

    def write_results(self, path):
        """ResultsWriter dump of this job's values (the reference's raw VertexType array)."""
        self.engine._check(self.engine.lib.cytom_write_results(self.engine.ctx, self.job, str(path).encode()))

    def destroy(self):
        self.engine._check(self.engine.lib.cytom_job_destroy(self.engine.ctx, self.job))


def run_batch(programs) -> list[dict]:
    """Runs the given programs (of one or more engines on one device) together in one
    persistent launch (cytom_run_batch); returns their run statistics in order."""
    programs = list(programs)
    if not programs:
        return []
    lib = programs[0].engine.lib
    n = len(programs)
    ctxs = (C.c_void_p * n)(*[p.engine.ctx for p in programs])
    ids = (C.c_int * n)(*[p.job for p in programs])
    stats = (L.RunStats * n)()
    rc = lib.cytom_run_batch(ctxs, ids, n, stats)
    programs[0].engine._check(rc)
    return [stats[k].as_dict() for k in range(n)]


class BFS(Program):
    """examples/bfs.cc: hop levels from start_vertex, UINT32_MAX = unreached."""
    ALGO = L.ALGO_BFS


class CC(Program):
    """examples/cc.cc: directed min-label propagation (label = least id reaching v)."""
    ALGO = L.ALGO_CC


class BFSAsync(Program):
    """examples/bfs-async.cc: BFS whose pull reads the freshest source values (next);
    the same levels as BFS, usually in fewer rounds."""
    ALGO = L.ALGO_BFS_ASYNC


class CCAsync(Program):
    """examples/cc-async.cc: CC whose pull reads the freshest source values (next)."""
    ALGO = L.ALGO_CC_ASYNC


class SSSP(Program):
    """examples/sssp.cc over uint32 weights: distances from start_vertex."""
    ALGO = L.ALGO_SSSP


class SSWP(Program):
    """examples/sswp.cc over uint32 weights: widest-path (bottleneck) value from
    start_vertex; 0 = unreached, UINT32_MAX at the start."""
    ALGO = L.ALGO_SSWP


class PageRankDelta(Program):
    """examples/pagerank-delta.cc: unnormalised delta PageRank, float ranks."""
    ALGO = L.ALGO_PR_DELTA
    result_dtype = np.float32


class PageRank(Program):
    """Normalised PageRank with dangling redistribution (FP32 + Kahan or FP64 plain)."""
    ALGO = L.ALGO_PAGERANK
    result_dtype = np.float32


class WeightedPageRank(Program):
    """PageRank over raw float edge weights normalised per source, teleport vector t
    (uniform unless set), differentiable through its adjoint."""
    ALGO = L.ALGO_WPAGERANK
    result_dtype = np.float32

    def set_teleport(self, t=None):
        if t is None:
            self.engine._check(self.engine.lib.cytom_job_set_teleport(self.engine.ctx, self.job, None, L.PTR_HOST))
            return
        t = np.ascontiguousarray(t, np.float64)
        self.engine._check(self.engine.lib.cytom_job_set_teleport(self.engine.ctx, self.job, t.ctypes.data,
                                                                  L.PTR_HOST))

    def adjoint(self, c):
        """dL/d(edge weights) in store order and dL/d(teleport) for L = c . r."""
        c = np.ascontiguousarray(c, np.float64)
        E = self.engine.count_edges()[0]
        gw = np.empty(E, np.float32)
        gt = np.empty(self.engine.n, np.float32)
        st = L.RunStats()
        self.engine._check(self.engine.lib.cytom_pagerank_adjoint(
            self.engine.ctx, self.job, c.ctypes.data, L.PTR_HOST, gw.ctypes.data, gt.ctypes.data, L.PTR_HOST,
            C.byref(st)))
        return gw, gt, st.as_dict()
