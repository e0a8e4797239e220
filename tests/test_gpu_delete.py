"""GPU tests of edge deletion (cytom_delete_batch) against the CPU oracle.

Store: after deletions (pending inserts compacted first, duplicate requests, pairs that are
not stored, out-of-range ids) the tiles, weights, storage flags and degrees equal the
oracle's bit for bit, and stay equal through later inserts and deletions down to an empty
store. Jobs: BFS / CC / SSSP / SSWP values after a deletion and a further run equal the
oracle's from-scratch fixed point on the new graph, bit for bit, whether the job restarted
(a tight deleted edge) or kept its values (none tight: the run has nothing to do);
PageRank (FP32-compensated, FP64) and PageRank-delta re-converge within the FP64-oracle
tolerance (relative L1 <= 1e-6, max relative <= 1e-5)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INF = 0xFFFFFFFF
L1_TOL, MAXREL_TOL = 1e-6, 1e-5


def same_store(eng, st, weighted):
    tp, ed, gw, cf = eng.dump_tiles(weights=weighted)
    otp, oed, ow, ocf = st.dump()
    assert np.array_equal(tp, otp), "tile_ptr"
    assert np.array_equal(ed, oed), "edges"
    if weighted:
        assert np.array_equal(gw, ow), "weights"
    assert np.array_equal(cf, ocf), "storage flags"
    for x, y in zip(eng.degrees(), st.degrees()):
        assert np.array_equal(x, y), "degrees"


@pytest.mark.parametrize("weighted", [True, False])
def test_delete_store_matches_oracle(cg, orc, weighted):
    scale, vpt = 12, 512
    n = 1 << scale
    rng = np.random.default_rng(3)
    st = orc.Store(n, vpt, weighted)
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32 if weighted else cg.UNWEIGHTED) as eng:
        def insert(first, count):
            s, t = orc.rmat(scale, first, count, 5)
            w = orc.edge_weights(s, t, 6) if weighted else None
            eng.insert_edges(s, t, w)
            st.insert(s, t, w)
            return s, t

        insert(0, 16 * n)
        eng.do_global_compaction()
        st.compact()
        s1, t1, _ = orc.store_edges(st)
        ps, pt = insert(16 * n, 2 * n)  # pending: the deletion compacts it first
        k = rng.choice(len(s1), len(s1) // 10, replace=False)
        ds = np.concatenate([s1[k], ps[:500], s1[k[:100]], rng.integers(0, n, 2000, dtype=np.uint32),
                             np.array([n + 3, 7], np.uint32)])
        dt = np.concatenate([t1[k], pt[:500], t1[k[:100]], rng.integers(0, n, 2000, dtype=np.uint32),
                             np.array([1, n + 11], np.uint32)])
        got = eng.delete_edges(ds, dt)
        assert got == st.delete(ds, dt) and got >= len(k)
        same_store(eng, st, weighted)
        # later inserts merge into the shrunken store; deleted pairs come back when inserted again
        insert(18 * n, 2 * n)
        eng.insert_edges(ds[:300].copy(), dt[:300].copy(), np.full(300, 9, np.uint32) if weighted else None)
        st.insert(ds[:300], dt[:300], np.full(300, 9, np.uint32) if weighted else None)
        eng.do_global_compaction()
        st.compact()
        same_store(eng, st, weighted)
        # device-side request arrays, then every edge of one tile row, then everything
        import torch
        s2, t2, _ = orc.store_edges(st)
        dev = torch.from_numpy(s2[::3].astype(np.int32)).cuda(), torch.from_numpy(t2[::3].astype(np.int32)).cuda()
        assert eng.delete_edges(*dev) == st.delete(s2[::3], t2[::3])
        same_store(eng, st, weighted)
        s3, t3, _ = orc.store_edges(st)
        row = s3 < vpt
        assert eng.delete_edges(s3[row], t3[row]) == st.delete(s3[row], t3[row]) == int(row.sum())
        same_store(eng, st, weighted)
        assert eng.delete_edges(s3, t3) == st.delete(s3, t3)
        assert eng.count_edges()[0] == 0
        same_store(eng, st, weighted)
        assert eng.delete_edges(s3[:10], t3[:10]) == 0


def test_delete_random_matches_oracle(cg, orc):
    # the deletion_percentage mode: hashed picks equal the oracle's, then the same store
    scale, vpt = 12, 256
    n = 1 << scale
    st = orc.Store(n, vpt, True)
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as eng:
        for b in range(3):
            s, t = orc.rmat(scale, b * 4 * n, 4 * n, 8)
            w = orc.edge_weights(s, t, 9)
            eng.insert_edges(s, t, w)
            st.insert(s, t, w)
            got, gs, gt = eng.delete_random(n // 2, seed=100 + b)  # a percentage of the batch
            os_, ot = st.pick_random(n // 2, 100 + b)
            assert np.array_equal(gs, os_) and np.array_equal(gt, ot)
            assert got == st.delete(os_, ot)
            same_store(eng, st, True)
        assert (gs == 0xFFFFFFFF).any()  # RMAT leaves tiles empty


def rel_errors(x, ref):
    x = np.asarray(x, np.float64)
    l1 = np.abs(x - ref).sum() / np.abs(ref).sum()
    mr = (np.abs(x - ref) / np.maximum(np.abs(ref), 1e-300)).max()
    return l1, mr


class Graph:
    """One evolving graph held twice: the engine with one job of each kind, and the oracle."""
    ALGO = {"bfs": 0, "cc": 1, "sssp": 2, "sswp": 3}

    def __init__(self, cg, orc, scale, vpt, seed):
        self.cg, self.orc = cg, orc
        self.n, self.scale, self.seed = 1 << scale, scale, seed
        self.eng = cg.Engine(self.n, vpt, weight_type=cg.WEIGHT_U32)
        self.st = orc.Store(self.n, vpt, True)
        self.pos = 0
        e = self.eng
        self.progs = {"bfs": cg.BFS(e, start_vertex=0, max_iterations=1000),
                      "cc": cg.CC(e, max_iterations=1000),
                      "sssp": cg.SSSP(e, start_vertex=0, max_iterations=1000),
                      "sswp": cg.SSWP(e, start_vertex=0, max_iterations=1000),
                      "pr32": cg.PageRank(e, max_iterations=500, tolerance=1e-10, kahan=True),
                      "pr64": cg.PageRank(e, max_iterations=500, tolerance=1e-12, kahan=False),
                      "prd": cg.PageRankDelta(e, delta=0.0, max_iterations=500, tolerance=1e-9)}

    def insert(self, count):
        s, t = self.orc.rmat(self.scale, self.pos, count, self.seed)
        w = self.orc.edge_weights(s, t, self.seed + 1)
        self.pos += count
        self.eng.insert_edges(s, t, w)
        self.st.insert(s, t, w)
        self.st.compact()
        return s, t

    def delete(self, s, t):
        got = self.eng.delete_edges(s, t)
        assert got == self.st.delete(s, t)
        return got

    def run_and_check(self, batched=False):
        progs = list(self.progs.values())
        stats = self.cg.run_batch(progs) if batched else [p.execute_algorithm() for p in progs]
        out = {}
        for (name, p), sa in zip(self.progs.items(), stats):
            out[name] = sa
            if name in self.ALGO:
                ref, _ = self.st.run_minprop(self.ALGO[name], start=0, max_iter=1000)
                assert np.array_equal(p.result(), ref), name
            elif name == "prd":
                ref, _ = self.st.pagerank_unnorm(tol=1e-14)
                l1, mr = rel_errors(p.result(), ref)
                assert l1 <= L1_TOL and mr <= MAXREL_TOL, (name, l1, mr)
            else:
                ref, _ = self.st.pagerank_norm(tol=1e-15)
                l1, mr = rel_errors(p.result64() if name == "pr64" else p.result(), ref)
                assert l1 <= L1_TOL and mr <= MAXREL_TOL, (name, l1, mr)
        return out


def test_delete_jobs_reach_new_fixed_point(cg, orc):
    g = Graph(cg, orc, 12, 1024, 21)
    try:
        g.insert(16 * g.n)
        g.run_and_check()
        rng = np.random.default_rng(4)
        # 5% of the stored edges (tight edges among them for every job)
        s, t, _ = orc.store_edges(g.st)
        k = rng.choice(len(s), len(s) // 20, replace=False)
        assert g.delete(s[k], t[k]) == len(k)
        g.run_and_check()
        # a pending batch, some of its edges deleted before any run, then the batched executor
        ps, pt = g.insert(g.n)
        assert g.delete(np.concatenate([ps[::4], s[:100]]), np.concatenate([pt[::4], t[:100]])) > 0
        g.run_and_check(batched=True)
        # deletions that empty the neighbourhood of the start vertex
        s, t, _ = orc.store_edges(g.st)
        m = (s == 0) | (t == 0)
        assert g.delete(s[m], t[m]) == int(m.sum())
        g.run_and_check()
    finally:
        g.eng.close()


def test_delete_non_tight_edges_keeps_values(cg, orc):
    # deleting edges that carry no value leaves BFS / SSSP with nothing to do; deleting a
    # tight edge restarts them; both end at the oracle's fixed point
    g = Graph(cg, orc, 12, 1024, 33)
    try:
        g.insert(16 * g.n)
        g.run_and_check()
        s, t, w = orc.store_edges(g.st)
        bfs = g.progs["bfs"].result().astype(np.uint64)
        sssp = g.progs["sssp"].result().astype(np.uint64)
        loose = ((bfs[s] == INF) | (bfs[s] + 1 != bfs[t])) & ((sssp[s] == INF) | (sssp[s] + w != sssp[t]))
        idx = np.flatnonzero(loose)[:2000]
        g.delete(s[idx], t[idx])
        st = g.run_and_check()
        for name in ("bfs", "sssp"):
            assert st[name]["iterations"] <= 1, (name, st[name])
        s, t, w = orc.store_edges(g.st)
        bfs = g.progs["bfs"].result().astype(np.uint64)
        tight = np.flatnonzero((bfs[s] != INF) & (bfs[s] + 1 == bfs[t]) & (bfs[t] >= 2))[:50]
        g.delete(s[tight], t[tight])
        st = g.run_and_check()
        assert st["bfs"]["iterations"] > 1, st["bfs"]
    finally:
        g.eng.close()
