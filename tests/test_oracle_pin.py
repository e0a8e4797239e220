"""The oracle pinned against the reference itself.

1. Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py from the
   reference's own TileStore / ContinuousAlgorithmExecutor): the oracle reproduces
   them bit-exactly, including the FP32 PageRankDelta ranks.
2. Live: where the reference pin builds (oracle/ref/Makefile), further graphs,
   geometries and settings are compared against it directly.
"""
from pathlib import Path

import numpy as np
import pytest

GOLDEN = sorted((Path(__file__).parent / "golden").glob("*.npz"))


def oracle_store(orc, g, weighted):
    n, vpt, batch = int(g["n"]), int(g["vpt"]), int(g["batch"])
    st = orc.Store(n, vpt, weighted)
    s, t, w = g["src"], g["tgt"], g["w"]
    for lo in range(0, len(s), batch):
        sl = slice(lo, lo + batch)
        st.insert(s[sl], t[sl], w[sl] if weighted else None)
        st.compact()
    return st


@pytest.mark.parametrize("path", GOLDEN, ids=[p.stem for p in GOLDEN])
def test_oracle_matches_golden(orc, path):
    g = np.load(path)
    st = oracle_store(orc, g, True)
    tp, ed, wt, cf = st.dump()
    assert np.array_equal(tp, g["tile_ptr"])
    assert np.array_equal(ed, g["edges"])
    assert np.array_equal(wt, g["weights"])
    assert np.array_equal(cf, g["compact"])
    for mode, algo in (("bfs", orc.BFS), ("cc", orc.CC), ("sssp", orc.SSSP)):
        vals, info = st.run_minprop(algo, start=0, max_iter=100)
        assert np.array_equal(vals, g[f"{mode}_values"]), mode
        assert info["count_edges"] == int(g[f"{mode}_count_edges"]), mode
    st2 = oracle_store(orc, g, False)
    rank, info = st2.run_prdelta_ref(max_iter=100, delta=0.01)
    assert np.array_equal(rank.view(np.uint32), g["prdelta_rank"].view(np.uint32))
    assert info["count_edges"] == int(g["prdelta_count_edges"])


@pytest.fixture(scope="module")
def ref():
    from oracle import ref_pin
    if not ref_pin.available():
        pytest.skip("reference pin not buildable here (no reference sources)")
    return ref_pin


@pytest.mark.parametrize("scale,vpt,batches,seed", [(11, 32, 3, 1), (13, 512, 4, 2), (15, 4096, 2, 3),
                                                     (17, 65536, 2, 4)])
def test_live_compaction_and_minprop(orc, ref, scale, vpt, batches, seed):
    n = 1 << scale
    m = 8 << scale
    s, t = orc.rmat(scale, 0, m, seed)
    w = orc.edge_weights(s, t, seed)
    batch = m // batches
    st = orc.Store(n, vpt, True)
    for lo in range(0, m, batch):
        st.insert(s[lo:lo + batch], t[lo:lo + batch], w[lo:lo + batch])
        st.compact()
    r = ref.run("compact", n, vpt, s, t, w, batch=batch)
    tp, ed, wt, cf = st.dump()
    assert np.array_equal(tp, r["tile_ptr"]) and np.array_equal(ed, r["edges"])
    assert np.array_equal(wt, r["weights"]) and np.array_equal(cf, r["compact"])
    for mode, algo in (("bfs", orc.BFS), ("cc", orc.CC), ("sssp", orc.SSSP)):
        rr = ref.run(mode, n, vpt, s, t, w if mode == "sssp" else None, batch=batch, executors=4,
                     max_iter=100, start=0)
        vals, info = st.run_minprop(algo, start=0, max_iter=100)
        assert np.array_equal(vals, rr["values"]), mode
        assert info["count_edges"] == rr["count_edges"], mode


@pytest.mark.parametrize("mode,algo", [("bfs", 0), ("cc", 1), ("sssp", 2)])
def test_live_iteration_caps_and_no_adaptive(orc, ref, mode, algo):
    n, vpt = 1 << 12, 256
    s, t = orc.rmat(12, 0, 8 << 12, 9)
    w = orc.edge_weights(s, t, 9)
    st = orc.Store(n, vpt, True)
    st.insert(s, t, w)
    st.compact()
    for cap, adaptive in ((1, True), (2, True), (3, False), (100, False)):
        rr = ref.run(mode, n, vpt, s, t, w if mode == "sssp" else None, batch=len(s), executors=2,
                     max_iter=cap, start=0, adaptive=adaptive)
        vals, info = st.run_minprop(algo, start=0, max_iter=cap, adaptive=adaptive)
        assert np.array_equal(vals, rr["values"]), (cap, adaptive)
        assert info["count_edges"] == rr["count_edges"], (cap, adaptive)


@pytest.mark.parametrize("delta,iters", [(0.01, 100), (0.0, 40), (0.1, 100)])
def test_live_prdelta_bit_exact(orc, ref, delta, iters):
    n, vpt = 1 << 13, 1024
    s, t = orc.rmat(13, 0, 12 << 13, 5)
    batch = len(s) // 3
    st = orc.Store(n, vpt, False)
    for lo in range(0, len(s), batch):
        st.insert(s[lo:lo + batch], t[lo:lo + batch])
        st.compact()
    rr = ref.run("prdelta", n, vpt, s, t, None, batch=batch, executors=1, max_iter=iters, delta=delta)
    rank, info = st.run_prdelta_ref(max_iter=iters, delta=delta)
    assert np.array_equal(rank.view(np.uint32), rr["values"].view(np.uint32))
    assert info["count_edges"] == rr["count_edges"]


def test_live_corner_edge_quirk(orc, ref):
    # tile-manager.h:519-541 with vpt = 65536: a tile whose only edge is (65535, 65535)
    n, vpt = 1 << 17, 1 << 16
    s = np.array([65535, 65535, 65536 + 65535, 65536 + 5, 7], np.uint32)
    t = np.array([65536 + 65535, 65536 + 65535, 65535, 65535, 9], np.uint32)
    w = np.array([5, 5, 3, 4, 1], np.uint32)
    r = ref.run("compact", n, vpt, s, t, w, batch=len(s))
    st = orc.Store(n, vpt, True)
    st.insert(s, t, w)
    st.compact()
    tp, ed, wt, cf = st.dump()
    assert np.array_equal(tp, r["tile_ptr"]) and np.array_equal(ed, r["edges"])
    assert r["tile_ptr"][2] - r["tile_ptr"][1] == 0


def test_reference_incremental_stream_reaches_the_fixed_point(orc, ref):
    # The reference's own incremental path (edgeChanged(INSERT) per inserted edge, then
    # executeAlgorithm continuing from the vertex state; bitmap swap left out, fix F5),
    # which times the streaming CPU baseline, ends every stream at the oracle's
    # from-scratch fixed point.
    scale, vpt = 13, 2048
    n = 1 << scale
    s, t = orc.rmat(scale, 0, 12 * n, 31)
    w = orc.edge_weights(s, t, 37)
    r = ref.run("istream", n, vpt, s, t, w, batch=2 * n, executors=4, max_iter=100, start=0)
    assert len(r["count_edges"]) == 6 and r["converged"].all()
    st = orc.Store(n, vpt, True)
    st.insert(s, t, w)
    st.compact()
    for name, algo in (("bfs", orc.BFS), ("cc", orc.CC), ("sssp", orc.SSSP)):
        vals, _ = st.run_minprop(algo, start=0, max_iter=100)
        assert np.array_equal(r[name], vals), name
