"""ctypes binding of the CPU oracle (oracle/cytom_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg, never by the cytom_gb300 package.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liborc.so"

BFS, CC, SSSP, SSWP = 0, 1, 2, 3
RMAT_A, RMAT_B, RMAT_C = float(np.float32(0.57)), float(np.float32(0.19)), float(np.float32(0.19))

_lib = None


def build() -> Path:
    r = subprocess.run(["make", "-C", str(HERE), "-s"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        u64, u32p, vp = C.c_uint64, C.POINTER(C.c_uint32), C.c_void_p
        L.orc_hash64.restype = u64
        L.orc_hash64.argtypes = [u64]
        L.orc_hash_double.restype = C.c_double
        L.orc_hash_double.argtypes = [u64]
        L.orc_rmat.restype = None
        L.orc_rmat.argtypes = [C.c_uint32, C.c_double, C.c_double, C.c_double, u64, u64, u64, vp, vp]
        L.orc_edge_weights.restype = None
        L.orc_edge_weights.argtypes = [u64, C.c_uint32, C.c_uint32, vp, vp, u64, vp]
        L.orc_gridgraph_decode.restype = C.c_int64
        L.orc_gridgraph_decode.argtypes = [vp, u64, u64, vp, vp]
        L.orc_store_create.restype = vp
        L.orc_store_create.argtypes = [u64, u64, C.c_int]
        L.orc_store_destroy.restype = None
        L.orc_store_destroy.argtypes = [vp]
        L.orc_store_insert.restype = C.c_int
        L.orc_store_insert.argtypes = [vp, vp, vp, vp, u64]
        L.orc_store_delete.restype = u64
        L.orc_store_delete.argtypes = [vp, vp, vp, u64]
        L.orc_store_pick_random.restype = None
        L.orc_store_pick_random.argtypes = [vp, u64, u64, vp, vp]
        L.orc_store_compact.restype = None
        L.orc_store_compact.argtypes = [vp]
        L.orc_store_count_edges.restype = u64
        L.orc_store_count_edges.argtypes = [vp]
        L.orc_store_count_tiles.restype = u64
        L.orc_store_count_tiles.argtypes = [vp]
        L.orc_store_dump.restype = None
        L.orc_store_dump.argtypes = [vp, vp, vp, vp, vp]
        L.orc_store_degrees.restype = None
        L.orc_store_degrees.argtypes = [vp, vp, vp]
        L.orc_run_minprop.restype = u64
        L.orc_run_minprop.argtypes = [vp, C.c_int, u64, u64, C.c_int, vp, C.POINTER(C.c_int),
                                      C.POINTER(u64)]
        L.orc_run_prdelta_ref.restype = u64
        L.orc_run_prdelta_ref.argtypes = [vp, u64, C.c_double, u64, vp, vp, C.POINTER(C.c_int),
                                          C.POINTER(u64)]
        L.orc_pagerank_unnorm_f64.restype = u64
        L.orc_pagerank_unnorm_f64.argtypes = [vp, C.c_double, C.c_double, u64, vp]
        L.orc_pagerank_norm_f64.restype = u64
        L.orc_pagerank_norm_f64.argtypes = [vp, C.c_double, C.c_double, u64, vp]
        L.orc_wpagerank_f64.restype = u64
        L.orc_wpagerank_f64.argtypes = [u64, u64, vp, vp, vp, vp, C.c_double, C.c_double, u64, vp]
        L.orc_wpagerank_adjoint_f64.restype = u64
        L.orc_wpagerank_adjoint_f64.argtypes = [u64, u64, vp, vp, vp, vp, C.c_double, C.c_double, u64,
                                                vp, vp, vp, vp, vp]
        _lib = L
    return _lib


def hash64(a: int) -> int:
    return lib().orc_hash64(a)


def rmat(scale: int, first: int, count: int, seed: int, a=RMAT_A, b=RMAT_B, c=RMAT_C):
    src = np.empty(count, np.uint32)
    tgt = np.empty(count, np.uint32)
    lib().orc_rmat(scale, a, b, c, seed, first, count, src.ctypes.data, tgt.ctypes.data)
    return src, tgt


def edge_weights(src, tgt, wseed: int, wmin: int = 1, wmax: int = 255):
    w = np.empty(len(src), np.uint32)
    lib().orc_edge_weights(wseed, wmin, wmax, src.ctypes.data, tgt.ctypes.data, len(src),
                           w.ctypes.data)
    return w


def gridgraph_decode(data: bytes, n: int):
    m = len(data) // 8
    src = np.empty(max(m, 1), np.uint32)
    tgt = np.empty(max(m, 1), np.uint32)
    buf = C.create_string_buffer(bytes(data), max(len(data), 1))
    r = lib().orc_gridgraph_decode(C.cast(buf, C.c_void_p), len(data), n, src.ctypes.data,
                                   tgt.ctypes.data)
    if r < 0:
        return None
    return src[:m], tgt[:m]


class Store:
    """The oracle's tile store (TileStore + TileManager + VertexStore degrees)."""

    def __init__(self, n: int, vpt: int, weighted: bool = False):
        self.n, self.vpt, self.weighted = n, vpt, weighted
        self.T = n // vpt
        self.h = lib().orc_store_create(n, vpt, 1 if weighted else 0)
        if not self.h:
            raise ValueError("bad store geometry")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_store_destroy(self.h)
            self.h = None

    def insert(self, src, tgt, w=None):
        src = np.ascontiguousarray(src, np.uint32)
        tgt = np.ascontiguousarray(tgt, np.uint32)
        wp = None
        if w is not None:
            w = np.ascontiguousarray(w, np.uint32)
            wp = w.ctypes.data
        rc = lib().orc_store_insert(self.h, src.ctypes.data, tgt.ctypes.data, wp, len(src))
        if rc != 0:
            raise ValueError("vertex id out of range")

    def compact(self):
        lib().orc_store_compact(self.h)

    def delete(self, src, tgt) -> int:
        src = np.ascontiguousarray(src, np.uint32)
        tgt = np.ascontiguousarray(tgt, np.uint32)
        return lib().orc_store_delete(self.h, src.ctypes.data, tgt.ctypes.data, len(src))

    def pick_random(self, count: int, seed: int):
        src = np.empty(count, np.uint32)
        tgt = np.empty(count, np.uint32)
        lib().orc_store_pick_random(self.h, count, seed, src.ctypes.data, tgt.ctypes.data)
        return src, tgt

    def count_edges(self) -> int:
        return lib().orc_store_count_edges(self.h)

    def dump(self):
        nt = self.T * self.T
        tp = np.empty(nt + 1, np.uint64)
        lib().orc_store_dump(self.h, tp.ctypes.data, None, None, None)
        e = int(tp[-1])
        ed = np.empty(max(e, 1), np.uint32)
        wt = np.empty(max(e, 1), np.uint32)
        cf = np.empty(nt, np.uint8)
        lib().orc_store_dump(self.h, tp.ctypes.data, ed.ctypes.data,
                             wt.ctypes.data if self.weighted else None, cf.ctypes.data)
        return tp, ed[:e], (wt[:e] if self.weighted else None), cf

    def degrees(self):
        o = np.empty(self.n, np.uint32)
        i = np.empty(self.n, np.uint32)
        lib().orc_store_degrees(self.h, o.ctypes.data, i.ctypes.data)
        return o, i

    def run_minprop(self, algo: int, start: int = 0, max_iter: int = 100, adaptive: bool = True):
        vals = np.empty(self.n, np.uint32)
        conv = C.c_int()
        ce = C.c_uint64()
        it = lib().orc_run_minprop(self.h, algo, start, max_iter, 1 if adaptive else 0,
                                   vals.ctypes.data, C.byref(conv), C.byref(ce))
        return vals, {"iterations": it, "converged": conv.value, "count_edges": ce.value}

    def run_prdelta_ref(self, max_iter: int = 100, delta: float = 0.01, batch: int = 256):
        rank = np.empty(self.n, np.float32)
        dl = np.empty(self.n, np.float32)
        conv = C.c_int()
        ce = C.c_uint64()
        it = lib().orc_run_prdelta_ref(self.h, max_iter, delta, batch, rank.ctypes.data,
                                       dl.ctypes.data, C.byref(conv), C.byref(ce))
        return rank, {"iterations": it, "converged": conv.value, "count_edges": ce.value}

    def pagerank_unnorm(self, alpha=0.85, tol=1e-13, max_iter=10000):
        r = np.empty(self.n, np.float64)
        it = lib().orc_pagerank_unnorm_f64(self.h, alpha, tol, max_iter, r.ctypes.data)
        return r, it

    def pagerank_norm(self, alpha=0.85, tol=1e-14, max_iter=10000):
        r = np.empty(self.n, np.float64)
        it = lib().orc_pagerank_norm_f64(self.h, alpha, tol, max_iter, r.ctypes.data)
        return r, it


def _vp(a):
    return None if a is None else a.ctypes.data


def wpagerank(n, src, tgt, w, t=None, alpha=0.85, tol=1e-15, max_iter=100000):
    """FP64 weighted PageRank over edge arrays (raw weights, normalised per source)."""
    src = np.ascontiguousarray(src, np.uint32)
    tgt = np.ascontiguousarray(tgt, np.uint32)
    w = np.ascontiguousarray(w, np.float64)
    t = None if t is None else np.ascontiguousarray(t, np.float64)
    r = np.empty(n, np.float64)
    it = lib().orc_wpagerank_f64(n, len(src), src.ctypes.data, tgt.ctypes.data, w.ctypes.data, _vp(t),
                                 alpha, tol, max_iter, r.ctypes.data)
    return r, it


def wpagerank_adjoint(n, src, tgt, w, r, c, t=None, alpha=0.85, tol=1e-15, max_iter=100000):
    """FP64 adjoint of L = c . r: (lambda, dL/dw per edge, dL/dt, iterations)."""
    src = np.ascontiguousarray(src, np.uint32)
    tgt = np.ascontiguousarray(tgt, np.uint32)
    w = np.ascontiguousarray(w, np.float64)
    t = None if t is None else np.ascontiguousarray(t, np.float64)
    r = np.ascontiguousarray(r, np.float64)
    c = np.ascontiguousarray(c, np.float64)
    lam = np.empty(n, np.float64)
    gw = np.empty(len(src), np.float64)
    gt = np.empty(n, np.float64)
    it = lib().orc_wpagerank_adjoint_f64(n, len(src), src.ctypes.data, tgt.ctypes.data, w.ctypes.data, _vp(t),
                                         alpha, tol, max_iter, r.ctypes.data, c.ctypes.data, lam.ctypes.data,
                                         gw.ctypes.data, gt.ctypes.data)
    return lam, gw, gt, it


def store_edges(store):
    """(src, tgt, w_bits) global arrays of a compacted store, in tile (store) order."""
    tp, ed, wt, _ = store.dump()
    T = store.n // store.vpt
    lv = store.vpt.bit_length() - 1
    tiles = np.repeat(np.arange(len(tp) - 1, dtype=np.uint64), np.diff(tp).astype(np.int64))
    x, y = tiles // T, tiles % T
    src = ((x << np.uint64(lv)) | (ed >> 16).astype(np.uint64)).astype(np.uint32)
    tgt = ((y << np.uint64(lv)) | (ed & 0xFFFF).astype(np.uint64)).astype(np.uint32)
    return src, tgt, wt


def unit_weights(src, tgt, wseed):
    """FP32 edge weights uniform in [0.1, 1.0], a function of (src, tgt) (duplicates agree)."""
    q = edge_weights(src, tgt, wseed, 0, (1 << 24) - 1).astype(np.float64)
    return (0.1 + 0.9 * q / float((1 << 24) - 1)).astype(np.float32)
