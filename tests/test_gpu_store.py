"""GPU parity of the ingest path (RMAT, GridGraph decode, insert, compaction) against
the CPU oracle, through the C ABI. Integer and byte work: bit-exact."""
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scale,seed,first,count", [(4, 1, 0, 1000), (16, 1, 0, 1 << 20),
                                                     (22, 2, 5 << 20, 1 << 20), (26, 3, 123456, 1 << 18),
                                                     (30, 9, 0, 4096)])
def test_rmat_bit_exact(cg, orc, scale, seed, first, count):
    n = 1 << min(scale, 24)
    with cg.Engine(n, min(n, 65536)) as eng:
        gs, gt, _ = eng.generate_rmat(first, count, scale, seed=seed)
    s, t = orc.rmat(scale, first, count, seed)
    assert np.array_equal(gs, s) and np.array_equal(gt, t)


@pytest.mark.parametrize("abc", [(0.45, 0.15, 0.15), (0.25, 0.25, 0.25), (0.9, 0.05, 0.05)])
def test_rmat_custom_probabilities(cg, orc, abc):
    a, b, c = abc
    with cg.Engine(1 << 12, 1024) as eng:
        gs, gt, _ = eng.generate_rmat(0, 50000, 18, seed=4, a=a, b=b, c=c)
    s, t = orc.rmat(18, 0, 50000, 4, a=a, b=b, c=c)
    assert np.array_equal(gs, s) and np.array_equal(gt, t)


def test_rmat_weights(cg, orc):
    with cg.Engine(1 << 16, 4096, weight_type=cg.WEIGHT_U32) as eng:
        s, t, w = eng.generate_rmat(0, 100000, 16, seed=2, weight_seed=77, wmin=1, wmax=255)
    assert np.array_equal(w, orc.edge_weights(s, t, 77, 1, 255))
    assert w.min() >= 1 and w.max() <= 255


def test_gridgraph_decode_and_errors(cg, orc, tmp_path):
    rng = np.random.default_rng(1)
    pairs = rng.integers(0, 1 << 12, (5000, 2), dtype=np.int32)
    data = pairs.astype("<i4").tobytes()
    with cg.Engine(1 << 12, 1024) as eng:
        s, t = eng.decode_gridgraph(data)
        rs, rt = orc.gridgraph_decode(data, 1 << 12)
        assert np.array_equal(s, rs) and np.array_equal(t, rt)
        bad = data + struct.pack("<ll", -5, 3)
        with pytest.raises(cg.CytomError) as ei:
            eng.decode_gridgraph(bad)
        assert ei.value.code == -3
        f = tmp_path / "g.bin"
        f.write_bytes(data)
        assert eng.load_gridgraph(str(f), batch=1000) == 5000
        eng.do_global_compaction()
        st = orc.Store(1 << 12, 1024)
        st.insert(rs, rt)
        st.compact()
        tp, ed, _, cf = eng.dump_tiles()
        otp, oed, _, ocf = st.dump()
        assert np.array_equal(tp, otp) and np.array_equal(ed, oed) and np.array_equal(cf, ocf)


def _stream_compare(cg, orc, scale, vpt, nbatches, batch, seed, weighted):
    n = 1 << scale
    wt = cg.WEIGHT_U32 if weighted else cg.UNWEIGHTED
    st = orc.Store(n, vpt, weighted)
    with cg.Engine(n, vpt, weight_type=wt) as eng:
        for b in range(nbatches):
            s, t = orc.rmat(scale, b * batch, batch, seed)
            w = orc.edge_weights(s, t, seed + 100) if weighted else None
            eng.insert_edges(s, t, w)
            st.insert(s, t, w)
            eng.do_global_compaction()
            st.compact()
            tp, ed, gw, cf = eng.dump_tiles(weights=weighted)
            otp, oed, ow, ocf = st.dump()
            assert np.array_equal(tp, otp), f"tile_ptr differs after batch {b}"
            assert np.array_equal(ed, oed), f"edges differ after batch {b}"
            if weighted:
                assert np.array_equal(gw, ow), f"weights differ after batch {b}"
            assert np.array_equal(cf, ocf), f"storage flags differ after batch {b}"
        go, gi = eng.degrees()
        oo, oi = st.degrees()
        assert np.array_equal(go, oo) and np.array_equal(gi, oi)


@pytest.mark.parametrize("scale,vpt,nb,batch,weighted", [
    (10, 64, 4, 3000, False),
    (12, 1024, 5, 20000, True),
    (16, 4096, 16, 65536, False),      # the PR-delta streaming config's geometry
    (16, 65536, 3, 100000, True),      # one tile, vpt = 65536 (u16 local ids at full width)
    (18, 8192, 4, 262144, True),
])
def test_streaming_compaction_bit_exact(cg, orc, scale, vpt, nb, batch, weighted):
    _stream_compare(cg, orc, scale, vpt, nb, batch, seed=scale, weighted=weighted)


def test_compaction_corner_edge_and_keep_min(cg, orc):
    n, vpt = 1 << 17, 1 << 16
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as eng:
        st = orc.Store(n, vpt, True)
        # tile (0,1): only the local corner edge (65535, 65535) -> dropped
        # tile (1,0): the corner edge next to another edge -> kept
        # tile (0,0): (7,9) three times with different weights -> one copy, least weight
        src = np.array([65535, 65535, 65536 + 65535, 65536 + 5, 7, 7, 7], np.uint32)
        tgt = np.array([65536 + 65535, 65536 + 65535, 65535, 65535, 9, 9, 9], np.uint32)
        w = np.array([5, 5, 3, 4, 30, 10, 20], np.uint32)
        eng.insert_edges(src, tgt, w)
        st.insert(src, tgt, w)
        eng.do_global_compaction()
        st.compact()
        # a later, lighter copy of an existing edge lowers its weight
        eng.insert_edges(np.array([7], np.uint32), np.array([9], np.uint32), np.array([2], np.uint32))
        st.insert(np.array([7], np.uint32), np.array([9], np.uint32), np.array([2], np.uint32))
        eng.do_global_compaction()
        st.compact()
        tp, ed, gw, cf = eng.dump_tiles(weights=True)
        otp, oed, ow, ocf = st.dump()
        assert np.array_equal(tp, otp) and np.array_equal(ed, oed) and np.array_equal(gw, ow)
        assert tp[1] - tp[0] == 1  # tile (0,0): (7,9)
        assert gw[0] == 2          # lowered by the later copy
        assert tp[2] - tp[1] == 0  # tile (0,1): the lone corner edge was dropped
        assert tp[3] - tp[2] == 2  # tile (1,0): both kept


def test_insert_rejects_out_of_range_batch(cg):
    with cg.Engine(1 << 10, 256) as eng:
        eng.insert_edges(np.array([1, 2], np.uint32), np.array([3, 4], np.uint32))
        with pytest.raises(cg.CytomError) as ei:
            eng.insert_edges(np.array([1, 1024], np.uint32), np.array([3, 4], np.uint32))
        assert ei.value.code == -3
        assert eng.count_edges() == (0, 2)  # nothing of the bad batch went in
        o, _ = eng.degrees()
        assert o.sum() == 2


def test_empty_store_and_empty_batch(cg):
    with cg.Engine(1 << 8, 64) as eng:
        eng.insert_edges(np.zeros(0, np.uint32), np.zeros(0, np.uint32))
        eng.do_global_compaction()
        tp, ed, _, cf = eng.dump_tiles()
        assert tp.sum() == 0 and len(ed) == 0 and cf.sum() == 0


def test_device_resident_insert(cg, orc):
    torch = pytest.importorskip("torch")
    n, vpt = 1 << 14, 2048
    with cg.Engine(n, vpt) as eng:
        s = torch.empty(200000, dtype=torch.int32, device="cuda")
        t = torch.empty_like(s)
        eng.generate_rmat(0, 200000, 14, seed=5, out=(s, t, None))
        eng.insert_edges(s, t)
        eng.do_global_compaction()
        tp, ed, _, _ = eng.dump_tiles()
    hs, ht = orc.rmat(14, 0, 200000, 5)
    st = orc.Store(n, vpt)
    st.insert(hs, ht)
    st.compact()
    otp, oed, _, _ = st.dump()
    assert np.array_equal(tp, otp) and np.array_equal(ed, oed)


GOLDEN = sorted((__import__("pathlib").Path(__file__).parent / "golden").glob("*.npz"))


@pytest.mark.parametrize("path", GOLDEN, ids=[p.stem for p in GOLDEN])
def test_gpu_matches_reference_golden(cg, path):
    # fixtures made by the reference's own TileStore / executors (tests/golden/make_golden.py)
    g = np.load(path)
    n, vpt, batch = int(g["n"]), int(g["vpt"]), int(g["batch"])
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as eng:
        s, t, w = g["src"], g["tgt"], g["w"]
        for lo in range(0, len(s), batch):
            eng.insert_edges(s[lo:lo + batch].copy(), t[lo:lo + batch].copy(), w[lo:lo + batch].copy())
            eng.do_global_compaction()
        tp, ed, wt, cf = eng.dump_tiles(weights=True)
        assert np.array_equal(tp, g["tile_ptr"]) and np.array_equal(ed, g["edges"])
        assert np.array_equal(wt, g["weights"]) and np.array_equal(cf, g["compact"])
        for name in ("bfs", "cc", "sssp"):
            prog = {"bfs": cg.BFS, "cc": cg.CC, "sssp": cg.SSSP}[name](eng, start_vertex=0, max_iterations=100)
            st = prog.execute_algorithm()
            assert np.array_equal(prog.result(), g[f"{name}_values"]), name
            assert st["count_edges"] == int(g[f"{name}_count_edges"]), name


def test_dynamic_compaction(cg, orc):
    # use_dynamic_compaction (TileManager::insertEdge, tile-manager.h:117, 150-161): after an
    # insert, once some tile holds 4096 edges (then 8192, 16384, ...; stored + appended) the
    # store compacts by itself. RMAT-12 over 4 x 4 tiles puts about a third of the edges in
    # tile (0, 0), so 2,000-edge batches cross 4096 and 8192 there. The store then equals,
    # tile for tile, one compacted only when asked, and so do the runs over it.
    scale, vpt, nb, b = 12, 1024, 20, 2000
    n = 1 << scale
    s, t = orc.rmat(scale, 0, nb * b, 5)
    w = orc.edge_weights(s, t, 9)
    autos = 0
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32, dynamic_compaction=True) as ea, \
            cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as eb:
        for k in range(nb):
            sl = slice(k * b, (k + 1) * b)
            for e in (ea, eb):
                e.insert_edges(s[sl].copy(), t[sl].copy(), w[sl].copy())
            ca, pa = ea.count_edges()
            cb, pb = eb.count_edges()
            assert cb == 0 and pb == (k + 1) * b  # no compaction unless asked
            if pa == 0:
                autos += 1  # this insert compacted the store
        assert autos >= 2, autos
        for e in (ea, eb):
            e.do_global_compaction()
        ta, tb = ea.dump_tiles(weights=True), eb.dump_tiles(weights=True)
        for x, y in zip(ta, tb):
            assert np.array_equal(x, y)
        st = orc.Store(n, vpt, True)
        st.insert(s, t, w)
        st.compact()
        ot = st.dump()
        assert np.array_equal(ta[0], ot[0]) and np.array_equal(ta[1], ot[1])
        pa_, pb_ = cg.SSSP(ea, start_vertex=0, max_iterations=1000), cg.SSSP(eb, start_vertex=0, max_iterations=1000)
        pa_.execute_algorithm()
        pb_.execute_algorithm()
        assert np.array_equal(pa_.result(), pb_.result())
