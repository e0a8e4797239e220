"""GPU tests of the batched persistent executor (cytom_run_batch).

Mixed programs (BFS from two sources, CC, SSSP, SSWP, PageRank FP32-compensated and FP64,
PageRank-delta) over graph snapshots of uneven size run in ONE launch. Every job must
end exactly where the one-job executor (cytom_run) ends: BFS / CC / SSSP / SSWP values, round
counts and processed-edge counts bit-exact (and equal to the CPU oracle's fixed point);
PageRank within the FP64-oracle tolerance (relative L1 <= 1e-6, max relative <= 1e-5)
-- on a fresh run and after further insert batches (incremental runs)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L1_TOL, MAXREL_TOL = 1e-6, 1e-5


def rel_errors(x, ref):
    x = np.asarray(x, np.float64)
    l1 = np.abs(x - ref).sum() / np.abs(ref).sum()
    mr = (np.abs(x - ref) / np.maximum(np.abs(ref), 1e-300)).max()
    return l1, mr


class Snap:
    """One snapshot held three times: batched engine, one-job engine, CPU oracle."""

    def __init__(self, cg, orc, scale, vpt, seed):
        self.n = 1 << scale
        self.scale, self.seed = scale, seed
        self.a = cg.Engine(self.n, vpt, weight_type=cg.WEIGHT_U32)
        self.b = cg.Engine(self.n, vpt, weight_type=cg.WEIGHT_U32)
        self.st = orc.Store(self.n, vpt, True)
        self.pos = 0
        self.progs = {}
        for name, mk in (("bfs0", lambda e: cg.BFS(e, start_vertex=0, max_iterations=1000)),
                         ("bfs1", lambda e: cg.BFS(e, start_vertex=1, max_iterations=1000)),
                         ("cc", lambda e: cg.CC(e, max_iterations=1000)),
                         ("sssp", lambda e: cg.SSSP(e, start_vertex=0, max_iterations=1000)),
                         ("sswp", lambda e: cg.SSWP(e, start_vertex=0, max_iterations=1000)),
                         ("pr32", lambda e: cg.PageRank(e, max_iterations=500, tolerance=1e-10, kahan=True)),
                         ("pr64", lambda e: cg.PageRank(e, max_iterations=500, tolerance=1e-12, kahan=False)),
                         ("prd", lambda e: cg.PageRankDelta(e, delta=0.0, max_iterations=500, tolerance=1e-9))):
            self.progs[name] = (mk(self.a), mk(self.b))

    def insert(self, orc, count):
        s, t = orc.rmat(self.scale, self.pos, count, self.seed)
        w = orc.edge_weights(s, t, self.seed + 100)
        self.pos += count
        for e in (self.a, self.b):
            e.insert_edges(s.copy(), t.copy(), w.copy())
        self.st.insert(s, t, w)
        self.st.compact()

    def close(self):
        self.a.close()
        self.b.close()


def check_round(cg, orc, snaps):
    batched = [p[0] for s in snaps for p in s.progs.values()]
    bstats = cg.run_batch(batched)
    k = 0
    for s in snaps:
        for name, (pa, pb) in s.progs.items():
            sa = bstats[k]
            k += 1
            sb = pb.execute_algorithm()
            if name.startswith(("bfs", "cc", "sssp", "sswp")):
                algo = {"bfs": 0, "cc": 1, "sss": 2, "ssw": 3}[name[:3]]
                start = 1 if name == "bfs1" else 0
                ref, info = s.st.run_minprop(algo, start=start, max_iter=1000)
                ra, rb = pa.result(), pb.result()
                assert np.array_equal(ra, rb), (s.scale, name)
                assert np.array_equal(ra, ref), (s.scale, name)
                for key in ("iterations", "count_edges", "active_vertices", "converged"):
                    assert sa[key] == sb[key], (s.scale, name, key, sa, sb)
            elif name == "prd":
                ref, _ = s.st.pagerank_unnorm(tol=1e-14)
                l1, mr = rel_errors(pa.result(), ref)
                assert l1 <= L1_TOL and mr <= MAXREL_TOL, (s.scale, name, l1, mr, sa)
                l1b, mrb = rel_errors(pa.result(), pb.result().astype(np.float64))
                assert mrb <= MAXREL_TOL, (s.scale, name, l1b, mrb)
            else:
                ref, _ = s.st.pagerank_norm(tol=1e-15)
                got = pa.result64() if name == "pr64" else pa.result()
                l1, mr = rel_errors(got, ref)
                assert l1 <= L1_TOL and mr <= MAXREL_TOL, (s.scale, name, l1, mr, sa)
                if name == "pr64":
                    assert np.allclose(pa.result64(), pb.result64(), rtol=1e-10, atol=0), (s.scale, name)


def test_batch_matches_one_job_runs(cg, orc):
    # four snapshots of uneven size (scales 9..12), 7 jobs each: 28 jobs in one launch
    snaps = [Snap(cg, orc, scale, vpt, seed) for scale, vpt, seed in
             ((9, 128, 10), (10, 256, 11), (11, 512, 12), (12, 1024, 13))]
    try:
        for s in snaps:
            s.insert(orc, 16 << s.scale)
        check_round(cg, orc, snaps)
        # incremental: two further batches of 5% of the edges, a batched run after each
        for _ in range(2):
            for s in snaps:
                s.insert(orc, (16 << s.scale) // 20)
            check_round(cg, orc, snaps)
    finally:
        for s in snaps:
            s.close()


def test_batch_iteration_cap_and_empty_graph(cg, orc):
    # a capped run stops after the same round as the one-job executor; a snapshot without
    # edges finishes after its seeding round
    n, vpt = 1 << 11, 256
    s, t = orc.rmat(11, 0, 16 * n, 21)
    w = orc.edge_weights(s, t, 22)
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as ea, \
            cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as eb, \
            cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as empty:
        for e in (ea, eb):
            e.insert_edges(s.copy(), t.copy(), w.copy())
        pa = [cg.SSSP(ea, start_vertex=0, max_iterations=2), cg.BFS(ea, start_vertex=0, max_iterations=1),
              cg.CC(ea, max_iterations=3)]
        pb = [cg.SSSP(eb, start_vertex=0, max_iterations=2), cg.BFS(eb, start_vertex=0, max_iterations=1),
              cg.CC(eb, max_iterations=3)]
        pe = [cg.BFS(empty, start_vertex=5, max_iterations=100), cg.PageRank(empty, max_iterations=50, tolerance=1e-9)]
        stats = cg.run_batch(pa + pe)
        for x, y, sa in zip(pa, pb, stats):
            sb = y.execute_algorithm()
            assert np.array_equal(x.result(), y.result())
            assert sa["iterations"] == sb["iterations"] and sa["count_edges"] == sb["count_edges"], (sa, sb)
        r = pe[0].result()
        assert r[5] == 0 and (np.delete(r, 5) == 0xFFFFFFFF).all()
        pr = pe[1].result()
        assert np.allclose(pr, 1.0 / n, rtol=1e-6)


def test_batch_rejects_bad_calls(cg):
    with cg.Engine(1 << 10, 256, weight_type=cg.WEIGHT_U32) as e:
        p = cg.BFS(e, start_vertex=0)
        with pytest.raises(cg.CytomError):
            cg.run_batch([p, p])  # the same job twice


@pytest.mark.parametrize("kahan", [True, False])
def test_paired_pagerank_jobs_share_passes(cg, orc, kahan):
    # PageRank jobs of one snapshot and form run as pairs in the batched executor (one
    # pass per round for both): each job ends where it ends alone -- same rounds, values
    # equal up to the order of the FP64 dangling-mass atomics, and within the tolerance of
    # the FP64 oracle -- also when the two jobs differ in damping and tolerance, when an
    # odd job is left over, fresh and after a further batch
    import os
    scale, vpt = 13, 1024
    n = 1 << scale
    s, t = orc.rmat(scale, 0, 16 * n, 41)
    st = orc.Store(n, vpt)
    st.insert(s, t)
    st.compact()
    specs = [(0.85, 1e-10), (0.85, 1e-10), (0.80, 1e-9)]
    rtol = 1e-6 if kahan else 1e-12
    with cg.Engine(n, vpt) as ea, cg.Engine(n, vpt) as eb:
        ea.insert_edges(s.copy(), t.copy())
        eb.insert_edges(s.copy(), t.copy())
        pa = [cg.PageRank(ea, max_iterations=500, alpha=alpha, tolerance=tol, kahan=kahan) for alpha, tol in specs]
        pb = [cg.PageRank(eb, max_iterations=500, alpha=alpha, tolerance=tol, kahan=kahan) for alpha, tol in specs]
        for rnd in range(2):
            sa = cg.run_batch(pa)  # paired: jobs 0 and 1; job 2 on its own passes
            os.environ["CYTOM_BATCH_PAIR"] = "0"
            try:
                sb = cg.run_batch(pb)
            finally:
                del os.environ["CYTOM_BATCH_PAIR"]
            for x, y, xs, ys in zip(pa, pb, sa, sb):
                assert xs["iterations"] == ys["iterations"], (rnd, xs, ys)
                gx = x.result64() if not kahan else x.result().astype(np.float64)
                gy = y.result64() if not kahan else y.result().astype(np.float64)
                assert np.allclose(gx, gy, rtol=rtol, atol=0), (rnd, np.abs(gx - gy).max())
            ref, _ = st.pagerank_norm(tol=1e-15)
            got = pa[0].result64() if not kahan else pa[0].result()
            l1, mr = rel_errors(got, ref)
            assert l1 <= L1_TOL and mr <= MAXREL_TOL, (rnd, l1, mr)
            s2, t2 = orc.rmat(scale, 16 * n + rnd * 4096, 4096, 41)
            for e in (ea, eb):
                e.insert_edges(s2.copy(), t2.copy())
            st.insert(s2, t2)
            st.compact()
