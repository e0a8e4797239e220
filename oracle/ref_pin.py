"""Runs the reference's own hot-path code (oracle/_ref/ref_driver, built by
oracle/ref/Makefile from the reference sources) on an edge list.

TEST INFRASTRUCTURE ONLY: the parity pin of the oracle and the CPU baseline.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
DRIVER = HERE / "_ref" / "ref_driver"


def build() -> bool:
    cmd = ["make", "-C", str(HERE / "ref"), "-s"]
    if os.environ.get("CYTOM_REFERENCE"):
        cmd.append(f"REF={os.environ['CYTOM_REFERENCE']}")
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.returncode == 0 and DRIVER.exists()


def available() -> bool:
    return DRIVER.exists() or build()


def _write_edges(path, src, tgt, w):
    with open(path, "wb") as f:
        f.write(struct.pack("<QI", len(src), 1 if w is not None else 0))
        f.write(np.ascontiguousarray(src, np.uint32).tobytes())
        f.write(np.ascontiguousarray(tgt, np.uint32).tobytes())
        if w is not None:
            f.write(np.ascontiguousarray(w, np.uint32).tobytes())


def run(mode, n, vpt, src, tgt, w=None, batch=0, executors=1, max_iter=100, delta=0.0, start=0,
        adaptive=True, timeout=3600):
    with tempfile.TemporaryDirectory() as d:
        ein, out = os.path.join(d, "e.bin"), os.path.join(d, "o.bin")
        _write_edges(ein, src, tgt, w)
        r = subprocess.run([str(DRIVER), mode, str(n), str(vpt), ein, out, str(batch), str(executors),
                            str(max_iter), repr(float(delta)), str(start), "1" if adaptive else "0"],
                           capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"reference driver failed ({r.returncode}): {r.stderr[-2000:]}")
        data = open(out, "rb").read()
    if mode == "compact":
        nt, e = struct.unpack_from("<QQ", data, 0)
        off = 16
        tp = np.frombuffer(data, np.uint64, nt + 1, off).copy()
        off += 8 * (nt + 1)
        cf = np.frombuffer(data, np.uint8, nt, off).copy()
        off += nt
        ed = np.frombuffer(data, np.uint32, e, off).copy()
        off += 4 * e
        wt = np.frombuffer(data, np.uint32, e, off).copy()
        off += 4 * e
        secs = struct.unpack_from("<d", data, off)[0]
        return {"tile_ptr": tp, "compact": cf, "edges": ed, "weights": wt, "seconds": secs}
    if mode == "istream":
        nb = struct.unpack_from("<Q", data, 0)[0]
        rec = np.frombuffer(data, np.float64, 4 * nb, 8).reshape(nb, 4)
        vals = np.frombuffer(data, np.uint32, 3 * n, 8 + 32 * nb).reshape(3, n)
        return {"count_edges": rec[:, 0].astype(np.int64), "insert_seconds": rec[:, 1], "run_seconds": rec[:, 2],
                "converged": rec[:, 3] != 0, "bfs": vals[0].copy(), "cc": vals[1].copy(), "sssp": vals[2].copy()}
    if mode == "stream":
        edges, run_s, ins_s, nb = struct.unpack_from("<dddd", data, 0)
        return {"count_edges": int(edges), "run_seconds": run_s, "insert_seconds": ins_s, "batches": int(nb)}
    cnt, conv, nn = struct.unpack_from("<QQQ", data, 0)
    vals = np.frombuffer(data, np.uint32, nn, 24).copy()
    secs = struct.unpack_from("<d", data, 24 + 4 * nn)[0]
    if mode == "prdelta":
        vals = vals.view(np.float32)
    return {"values": vals, "count_edges": cnt, "converged": bool(conv), "seconds": secs}
