"""CPU tests of the oracle: each restatement is checked against an independent
numpy / pure-Python restatement of the same reference code."""
import struct

import numpy as np
import pytest

M64 = (1 << 64) - 1


def py_hash64(a):
    # src/include/util/util.h:188-196, restated a second time in Python
    a = ((a + 0x7ed55d166bef7a1d) + (a << 12)) & M64
    a = ((a ^ 0xc761c23c510fa2dd) ^ (a >> 9)) & M64
    a = ((a + 0x165667b183a9c0e1) + (a << 59)) & M64
    a = ((a + 0xd3a2646cab3487e3) ^ (a << 49)) & M64
    a = ((a + 0xfd7046c5ef9ab54c) + (a << 3)) & M64
    a = ((a ^ 0xb55a4f090dd4a67b) ^ (a >> 32)) & M64
    return a


def py_rmat_edge(scale, index, seed, a, b, c):
    # rmat-context.h:39-73 followed literally (rMatIterative)
    h = py_hash64(seed)
    rs = py_hash64((2 * index * h) & M64)
    st = py_hash64(((2 * index + 1) * h) & M64)
    n = 1 << scale
    local_n, lrs = n, rs
    while local_n != 1:
        local_n //= 2
        lrs = (lrs + st) & M64
    s = t = 0
    while local_n != n:
        local_n *= 2
        lrs = (lrs - st) & M64
        r = float(py_hash64(lrs)) / float(M64)
        if r < a:
            pass
        elif r < a + b:
            t += local_n // 2
        elif r < a + b + c:
            s += local_n // 2
        else:
            s += local_n // 2
            t += local_n // 2
    return s, t


def test_hash_matches_python(orc):
    for v in [0, 1, 2, 3, 12345, 2**63, M64, 0xdeadbeefcafebabe]:
        assert orc.hash64(v) == py_hash64(v)


@pytest.mark.parametrize("scale,seed", [(4, 1), (10, 2), (16, 3), (22, 17)])
def test_rmat_matches_python(orc, scale, seed):
    first, count = 1000, 300
    s, t = orc.rmat(scale, first, count, seed)
    for k in range(count):
        assert (int(s[k]), int(t[k])) == py_rmat_edge(scale, first + k, seed, orc.RMAT_A,
                                                       orc.RMAT_B, orc.RMAT_C)


def test_rmat_quadrant_statistics(orc):
    # top-level quadrant frequencies follow a, b, c, d
    s, t = orc.rmat(20, 0, 1 << 18, seed=5)
    top_s, top_t = s >> 19, t >> 19
    fa = np.mean((top_s == 0) & (top_t == 0))
    fb = np.mean((top_s == 0) & (top_t == 1))
    fc = np.mean((top_s == 1) & (top_t == 0))
    assert abs(fa - 0.57) < 0.01 and abs(fb - 0.19) < 0.01 and abs(fc - 0.19) < 0.01
    assert s.max() < (1 << 20) and t.max() < (1 << 20)


def test_gridgraph_decode(orc):
    # writer of src/scripts/convert_graph.py:15-16: struct.pack("<l", ...) pairs
    pairs = [(0, 1), (5, 3), (1023, 7), (2, 2)]
    data = b"".join(struct.pack("<l", a) + struct.pack("<l", b) for a, b in pairs)
    s, t = orc.gridgraph_decode(data, 1024)
    assert s.tolist() == [p[0] for p in pairs] and t.tolist() == [p[1] for p in pairs]
    assert orc.gridgraph_decode(struct.pack("<ll", -1, 0), 1024) is None
    assert orc.gridgraph_decode(struct.pack("<ll", 0, 1024), 1024) is None
    # a trailing partial record is ignored (count = size / 8, jobs.h:64)
    s2, _ = orc.gridgraph_decode(data + b"\x01\x02\x03", 1024)
    assert len(s2) == 4


def np_compact(n, vpt, batches, weighted):
    """Independent numpy restatement of TileManager::compactStorage over a sequence
    of batches (each compacted after insertion)."""
    T = n // vpt
    tiles = {}
    flags = np.zeros(T * T, np.uint8)
    for src, tgt, w in batches:
        x, y = src // vpt, tgt // vpt
        for i in range(len(src)):
            tid = int(x[i] * T + y[i])
            loc = (int(src[i] % vpt) << 16) | int(tgt[i] % vpt)
            tiles.setdefault(tid, [[], []])[1].append((loc, int(w[i]) if weighted else 0))
        for tid, (csr, ovf) in tiles.items():
            allv = ovf + csr
            if not allv:
                continue
            allv.sort()
            srcs = {e >> 16 for e, _ in allv}
            flags[tid] = 1 if len(srcs) >= vpt // 2 else 0
            out, prev = [], 0xFFFFFFFF
            for e, wv in allv:
                if e == prev:
                    continue
                prev = e
                out.append((e, wv))
            tiles[tid] = [out, []]
    tp = np.zeros(T * T + 1, np.uint64)
    ed, wt = [], []
    for tid in range(T * T):
        tp[tid] = len(ed)
        for e, wv in tiles.get(tid, [[], []])[0]:
            ed.append(e)
            wt.append(wv)
    tp[-1] = len(ed)
    return tp, np.array(ed, np.uint32), np.array(wt, np.uint32), flags


@pytest.mark.parametrize("n,vpt,weighted", [(256, 64, False), (256, 32, True), (1024, 1024, True),
                                             (512, 16, False)])
def test_compaction_matches_numpy(orc, n, vpt, weighted):
    rng = np.random.default_rng(n + vpt)
    batches = []
    st = orc.Store(n, vpt, weighted)
    for b in range(3):
        m = 400 + 100 * b
        src = rng.integers(0, n, m, dtype=np.uint32)
        tgt = (rng.integers(0, n // 4, m, dtype=np.uint32) * 4 + rng.integers(0, 4, m)).astype(np.uint32) % n
        src[:50] = src[50:100]  # duplicates inside a batch
        tgt[:50] = tgt[50:100]
        w = rng.integers(1, 255, m, dtype=np.uint32)
        batches.append((src, tgt, w))
        st.insert(src, tgt, w if weighted else None)
        st.compact()
    tp, ed, wt, cf = st.dump()
    rtp, red, rwt, rcf = np_compact(n, vpt, batches, weighted)
    assert np.array_equal(tp, rtp)
    assert np.array_equal(ed, red)
    if weighted:
        assert np.array_equal(wt, rwt)
    assert np.array_equal(cf, rcf)


@pytest.mark.parametrize("weighted", [False, True])
def test_store_delete_matches_numpy(orc, weighted):
    # deletion after compaction of pending edges: the stored set minus the listed pairs
    # (duplicates deleted once, absent and out-of-range pairs skipped), degrees lowered by
    # the deleted edges, storage flags from the remaining distinct sources
    n, vpt = 512, 64
    rng = np.random.default_rng(7 + weighted)
    st = orc.Store(n, vpt, weighted)
    ref = orc.Store(n, vpt, weighted)
    for b in range(2):  # the second batch stays pending until the deletion compacts it
        src = rng.integers(0, n, 6000, dtype=np.uint32)
        tgt = rng.integers(0, n // 2, 6000, dtype=np.uint32)
        w = rng.integers(1, 255, 6000, dtype=np.uint32)
        for x in (st, ref):
            x.insert(src, tgt, w if weighted else None)
        if b == 0:
            st.compact()
    ref.compact()
    s1, t1, w1 = orc.store_edges(ref)
    o1, i1 = ref.degrees()
    k = rng.choice(len(s1), 900, replace=False)
    ds = np.concatenate([s1[k], s1[k[:60]], rng.integers(0, n, 300, dtype=np.uint32),
                         np.array([n + 3, 5], np.uint32)])
    dt = np.concatenate([t1[k], t1[k[:60]], rng.integers(0, n, 300, dtype=np.uint32),
                         np.array([1, n + 9], np.uint32)])
    removed = st.delete(ds, dt)
    gone = np.isin(s1.astype(np.uint64) << np.uint64(32) | t1, ds.astype(np.uint64) << np.uint64(32) | dt)
    assert removed == int(gone.sum()) and removed >= 900
    s2, t2, w2 = orc.store_edges(st)
    assert np.array_equal(s2, s1[~gone]) and np.array_equal(t2, t1[~gone])
    if weighted:
        assert np.array_equal(w2, w1[~gone])
    o2, i2 = st.degrees()
    assert np.array_equal(o2, o1 - np.bincount(s1[gone], minlength=n).astype(np.uint32))
    assert np.array_equal(i2, i1 - np.bincount(t1[gone], minlength=n).astype(np.uint32))
    tp, ed, _, cf = st.dump()
    T = n // vpt
    for ti in range(T * T):
        srcs = np.unique(ed[int(tp[ti]):int(tp[ti + 1])] >> 16)
        assert cf[ti] == (1 if len(srcs) >= vpt // 2 else 0), ti
    # a deleted pair inserted again is stored again
    st.insert(ds[:10], dt[:10], np.full(10, 7, np.uint32) if weighted else None)
    st.compact()
    assert st.count_edges() == len(s2) + len(np.unique(ds[:10].astype(np.uint64) << np.uint64(32) | dt[:10]))


def test_store_pick_random(orc):
    # picks are stored edges of the hashed tile (none for an empty tile), deterministic in
    # the seed, and roughly uniform over tiles
    n, vpt = 256, 64
    st = orc.Store(n, vpt)
    rng = np.random.default_rng(2)
    src = rng.integers(0, n // 2, 3000, dtype=np.uint32)  # tiles of source block >= 2 stay empty
    tgt = rng.integers(0, n, 3000, dtype=np.uint32)
    st.insert(src, tgt)
    s, t = st.pick_random(4000, 9)
    s2, t2 = st.pick_random(4000, 9)
    assert np.array_equal(s, s2) and np.array_equal(t, t2)
    none = s == 0xFFFFFFFF
    assert np.array_equal(none, t == 0xFFFFFFFF)
    stored = set(zip(src.tolist(), tgt.tolist()))
    assert all((a, b) in stored for a, b in zip(s[~none].tolist(), t[~none].tolist()))
    assert 0.4 < none.mean() < 0.6  # half of the 16 tiles are empty
    T = n // vpt
    counts = np.bincount((s[~none] // vpt) * T + t[~none] // vpt, minlength=T * T)[: T * T // 2]
    assert counts.min() > 0.6 * counts.mean()


def test_fillcsr_corner_edge_dropped(orc):
    # tile-manager.h:519-541: with vpt = 65536 an otherwise empty tile whose only edge is
    # local (65535, 65535) comes out empty; next to another edge it survives.
    n, vpt = 1 << 17, 1 << 16
    st = orc.Store(n, vpt)
    st.insert(np.array([65535, 65535], np.uint32), np.array([65535, 65535], np.uint32))
    st.insert(np.array([65536 + 65535, 65536 + 5], np.uint32), np.array([65535, 65535], np.uint32))
    st.compact()
    tp, ed, _, _ = st.dump()
    assert tp[1] - tp[0] == 0          # tile (0,0) lost its only edge
    assert tp[3] - tp[2] == 2          # tile (1,0) keeps both
    o, _ = st.degrees()
    assert o[65535] == 2               # degrees still count the dropped copies


def test_compact_flag_threshold(orc):
    n, vpt = 64, 16
    st = orc.Store(n, vpt)
    st.insert(np.arange(8, dtype=np.uint32), np.zeros(8, np.uint32))       # 8 sources in tile (0,0)
    st.insert(np.arange(7, dtype=np.uint32) + 16, np.zeros(7, np.uint32))  # 7 sources in tile (1,0)
    st.compact()
    _, _, _, cf = st.dump()
    assert cf[0] == 1 and cf[4] == 0


def np_fixed_point(n, src, tgt, w, algo, start):
    INF = np.iinfo(np.uint32).max
    val = np.full(n, INF, np.uint64)
    if algo == 1:
        val = np.arange(n, dtype=np.uint64)
    else:
        val[start] = 0
    while True:
        cand = val[src] + (1 if algo == 0 else (0 if algo == 1 else w.astype(np.uint64)))
        ok = val[src] != INF
        new = val.copy()
        np.minimum.at(new, tgt[ok], cand[ok])
        if np.array_equal(new, val):
            return val.astype(np.uint32)
        val = new


@pytest.mark.parametrize("algo", [0, 1, 2])
@pytest.mark.parametrize("vpt", [64, 256])
def test_minprop_fixed_points(orc, algo, vpt):
    n = 1024
    s, t = orc.rmat(10, 0, 6000, seed=3)
    w = orc.edge_weights(s, t, 9)
    st = orc.Store(n, vpt, weighted=True)
    st.insert(s, t, w)
    st.compact()
    got, info = st.run_minprop(algo, start=0, max_iter=1000)
    assert info["converged"] == 1
    assert np.array_equal(got, np_fixed_point(n, s.astype(np.int64), t.astype(np.int64), w, algo, 0))
    # adaptive scheduling off reaches the same fixed point
    got2, _ = st.run_minprop(algo, start=0, max_iter=1000, adaptive=False)
    assert np.array_equal(got, got2)


def test_pagerank_unnorm_matches_numpy(orc):
    n = 512
    s, t = orc.rmat(9, 0, 4000, seed=4)
    st = orc.Store(n, 128)
    st.insert(s, t)
    st.compact()
    r, it = st.pagerank_unnorm(tol=1e-15)
    tp, ed, _, _ = st.dump()
    deg, _ = st.degrees()
    T = 4
    xs, ys = [], []
    for tid in range(T * T):
        for e in ed[int(tp[tid]):int(tp[tid + 1])]:
            xs.append((tid // T) * 128 + (int(e) >> 16))
            ys.append((tid % T) * 128 + (int(e) & 0xFFFF))
    xs, ys = np.array(xs), np.array(ys)
    x = np.ones(n)
    for _ in range(2000):
        acc = np.zeros(n)
        np.add.at(acc, ys, x[xs] / deg[xs])
        x = 0.15 + 0.85 * acc
    assert np.allclose(r, x, rtol=1e-10, atol=1e-12)


def test_pagerank_norm_sums_to_one(orc):
    n = 1024
    s, t = orc.rmat(10, 0, 5000, seed=6)
    st = orc.Store(n, 256)
    st.insert(s, t)
    st.compact()
    r, _ = st.pagerank_norm()
    assert abs(r.sum() - 1.0) < 1e-10 and (r > 0).all()


def test_prdelta_ref_converges_toward_fixed_point(orc):
    n = 1024
    s, t = orc.rmat(10, 0, 8000, seed=8)
    st = orc.Store(n, 256)
    st.insert(s, t)
    st.compact()
    rank, info = st.run_prdelta_ref(max_iter=200, delta=0.0)
    r64, _ = st.pagerank_unnorm()
    rel = np.abs(rank - r64).sum() / r64.sum()
    assert rel < 1e-5, rel


def _wgraph(orc, scale, vpt, seed, wseed, ef=8):
    n = 1 << scale
    s, t = orc.rmat(scale, 0, ef * n, seed)
    w = orc.unit_weights(s, t, wseed)
    st = orc.Store(n, vpt, True)
    st.insert(s, t, w.view(np.uint32))
    st.compact()
    src, tgt, wb = orc.store_edges(st)
    return n, st, src, tgt, wb.view(np.float32).astype(np.float64)


def test_wpagerank_fixed_point_and_mass(orc):
    n, st, src, tgt, w = _wgraph(orc, 10, 256, 4, 7)
    assert ((w >= 0.1) & (w <= 1.0)).all()
    r, it = orc.wpagerank(n, src, tgt, w, tol=1e-15)
    assert abs(r.sum() - 1.0) < 1e-12
    # one more application of the map leaves r unchanged
    s = np.bincount(src, weights=w, minlength=n)
    acc = np.bincount(tgt, weights=w / s[src] * r[src], minlength=n)
    dang = r[s == 0].sum()
    r2 = 0.15 / n + 0.85 * (acc + dang / n)
    assert np.abs(r2 - r).sum() < 1e-13


def test_wpagerank_adjoint_matches_central_differences(orc):
    # the FP64 adjoint against FP64 central differences (eps 1e-3 on raw weights)
    n, st, src, tgt, w = _wgraph(orc, 10, 256, 4, 7)
    r, _ = orc.wpagerank(n, src, tgt, w, tol=1e-16)
    c = np.random.default_rng(5).standard_normal(n)
    lam, gw, gt, _ = orc.wpagerank_adjoint(n, src, tgt, w, r, c, tol=1e-16)
    rng = np.random.default_rng(9)
    scale_w = np.abs(gw).max()
    eps = 1e-3
    for e in rng.choice(len(src), 12, replace=False):
        wp, wm = w.copy(), w.copy()
        wp[e] += eps
        wm[e] -= eps
        fd = (c @ orc.wpagerank(n, src, tgt, wp, tol=1e-16)[0] - c @ orc.wpagerank(n, src, tgt, wm, tol=1e-16)[0]) / (2 * eps)
        assert abs(fd - gw[e]) <= 1e-4 * max(abs(fd), 1e-2 * scale_w), (e, fd, gw[e])
    # teleport: perturb one entry of the (unnormalised) teleport vector
    t0 = np.full(n, 1.0 / n)
    et = 1e-7
    for v in rng.choice(n, 6, replace=False):
        tp, tm = t0.copy(), t0.copy()
        tp[v] += et
        tm[v] -= et
        fd = (c @ orc.wpagerank(n, src, tgt, w, t=tp, tol=1e-16)[0] - c @ orc.wpagerank(n, src, tgt, w, t=tm, tol=1e-16)[0]) / (2 * et)
        assert abs(fd - gt[v]) <= 1e-4 * max(abs(fd), 1e-2 * np.abs(gt).max()), (v, fd, gt[v])


def _widest_path(n, src, tgt, w, start):
    # independent restatement: max-min relaxation to the fixed point (unique widest widths)
    val = np.zeros(n, np.uint64)
    val[start] = 0xFFFFFFFF
    while True:
        live = val[src] > 0
        cand = np.minimum(val[src[live]], w[live].astype(np.uint64))
        new = val.copy()
        np.maximum.at(new, tgt[live], cand)
        if np.array_equal(new, val):
            return val.astype(np.uint32)
        val = new


@pytest.mark.parametrize("scale,vpt", [(10, 256), (12, 1024)])
def test_sswp_oracle_matches_widest_path(orc, scale, vpt):
    n = 1 << scale
    s, t = orc.rmat(scale, 0, 8 * n, 3)
    w = orc.edge_weights(s, t, 4)
    st = orc.Store(n, vpt, True)
    st.insert(s, t, w)
    st.compact()
    for start in (0, 5):
        vals, info = st.run_minprop(orc.SSWP, start=start, max_iter=10000)
        assert info["converged"] == 1
        assert np.array_equal(vals, _widest_path(n, s, t, w, start))
