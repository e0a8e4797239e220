"""Generates the golden fixtures in tests/golden/ by running the reference's own code.

Each fixture is a small RMAT graph streamed in batches into the reference's
TileStore (compactStorage after every batch) and the reference executor run on the
result, as compiled by oracle/ref/Makefile from the reference sources (with fixes
F1-F4). Run from the repository root where the reference sources are available:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as orc  # noqa: E402
from oracle import ref_pin  # noqa: E402

CASES = [
    # name, scale, vpt, edges, batch, seed, wseed
    ("rmat10_vpt64", 10, 64, 8 << 10, 2048, 11, 21),
    ("rmat12_vpt1024", 12, 1024, 16 << 12, 16384, 12, 22),
    ("rmat13_vpt8192", 13, 8192, 6 << 13, 16384, 13, 23),
]


def make(name, scale, vpt, m, batch, seed, wseed):
    n = 1 << scale
    s, t = orc.rmat(scale, 0, m, seed)
    w = orc.edge_weights(s, t, wseed)
    out = {"n": np.uint64(n), "vpt": np.uint64(vpt), "batch": np.uint64(batch), "src": s, "tgt": t, "w": w}
    c = ref_pin.run("compact", n, vpt, s, t, w, batch=batch)
    out.update(tile_ptr=c["tile_ptr"], edges=c["edges"], weights=c["weights"], compact=c["compact"])
    for mode in ("bfs", "cc", "sssp"):
        r = ref_pin.run(mode, n, vpt, s, t, w if mode == "sssp" else None, batch=batch, executors=2,
                        max_iter=100, start=0)
        out[f"{mode}_values"] = r["values"]
        out[f"{mode}_count_edges"] = np.uint64(r["count_edges"])
    r = ref_pin.run("prdelta", n, vpt, s, t, None, batch=batch, executors=1, max_iter=100, delta=0.01)
    out["prdelta_rank"] = r["values"]
    out["prdelta_count_edges"] = np.uint64(r["count_edges"])
    np.savez_compressed(Path(__file__).parent / f"{name}.npz", **out)
    print(name, "edges", len(c["edges"]))


if __name__ == "__main__":
    if not ref_pin.available():
        sys.exit("the reference build (oracle/ref/Makefile) is not available here")
    for case in CASES:
        make(*case)
