"""GPU parity at the configured workload geometries (not scaled down).

- PageRank-delta stream: RMAT-16 (65,536 vertices), seed 1, 65,536-edge batches x 16 in
  generation order into a store with 4,096 vertices per tile, an update after each batch
  to an FP64 L1 residual of 1e-7 of the rank sum. After EVERY batch the FP32 ranks are
  within relative L1 1e-6 and max relative 1e-5 of the FP64 fixed point of that
  snapshot (the CPU oracle's unnormalised PageRank over the stored edges with
  multiplicity degrees, the reference's PageRankDelta model,
  examples/pagerank-delta.cc:127-174).
- Batching: 64 jobs -- per snapshot BFS from 0 and 1, CC twice, SSSP from 0 and 1,
  PageRank twice (FP32 compensated, L1 tolerance 1e-8) -- over 8 RMAT snapshots of
  scales 14..21 (edge factor 16, seeds 10..17, weights 1..255), each receiving 4 further
  batches of 5 % of its edges between job rounds, every round ONE persistent launch
  (cytom_run_batch). Integer results equal the CPU oracle's fixed point bit for bit
  after every round; PageRank is within 1e-6 / 1e-5 of the oracle's FP64 PageRank.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L1_TOL, MAXREL_TOL = 1e-6, 1e-5


def rel_errors(x, ref):
    x = np.asarray(x, np.float64)
    l1 = np.abs(x - ref).sum() / np.abs(ref).sum()
    mr = (np.abs(x - ref) / np.maximum(np.abs(ref), 1e-300)).max()
    return l1, mr


def test_prdelta_stream_rmat16_every_batch(cg, orc):
    scale, vpt, B, nb = 16, 4096, 65536, 16
    n = 1 << scale
    with cg.Engine(n, vpt) as eng:
        s, t, _ = eng.generate_rmat(0, B * nb, scale, seed=1)
        rs, rt = orc.rmat(scale, 0, 4096, 1)
        assert np.array_equal(s[:4096], rs) and np.array_equal(t[:4096], rt)
        st = orc.Store(n, vpt)
        p = cg.PageRankDelta(eng, delta=0.0, max_iterations=1000, tolerance=1e-7)
        worst = (0.0, 0.0)
        for b in range(nb):
            sl = slice(b * B, (b + 1) * B)
            eng.insert_edges(s[sl].copy(), t[sl].copy())
            st.insert(s[sl], t[sl])
            st.compact()
            stats = p.execute_algorithm()
            assert stats["converged"] == 1, (b, stats)
            ref, _ = st.pagerank_unnorm(tol=1e-14)
            l1, mr = rel_errors(p.result(), ref)
            worst = (max(worst[0], l1), max(worst[1], mr))
            assert l1 <= L1_TOL and mr <= MAXREL_TOL, (b, l1, mr, stats)


def test_batching_64_jobs_configured(cg, orc):
    scales, seeds, rounds = list(range(14, 22)), list(range(10, 18)), 4
    snaps = []
    try:
        for scale, seed in zip(scales, seeds):
            n = 1 << scale
            vpt = min(65536, n >> 2)  # 65,536 would give the smallest snapshots no tile (config.cc:18-19)
            m = 16 << scale
            b = m // 20
            eng = cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32)
            s, t, w = eng.generate_rmat(0, m + rounds * b, scale, seed=seed, weight_seed=seed + 1000,
                                        wmin=1, wmax=255)
            st = orc.Store(n, vpt, True)
            progs = [cg.BFS(eng, start_vertex=0, max_iterations=100), cg.BFS(eng, start_vertex=1, max_iterations=100),
                     cg.CC(eng, max_iterations=100), cg.CC(eng, max_iterations=100),
                     cg.SSSP(eng, start_vertex=0, max_iterations=100),
                     cg.SSSP(eng, start_vertex=1, max_iterations=100),
                     cg.PageRank(eng, max_iterations=100, tolerance=1e-8, kahan=True),
                     cg.PageRank(eng, max_iterations=100, tolerance=1e-8, kahan=True)]
            snaps.append(dict(eng=eng, st=st, s=s, t=t, w=w, m=m, b=b, progs=progs))
        for r in range(rounds + 1):
            for sn in snaps:
                lo, hi = (0, sn["m"]) if r == 0 else (sn["m"] + (r - 1) * sn["b"], sn["m"] + r * sn["b"])
                sl = slice(lo, hi)
                sn["eng"].insert_edges(sn["s"][sl].copy(), sn["t"][sl].copy(), sn["w"][sl].copy())
                sn["st"].insert(sn["s"][sl], sn["t"][sl], sn["w"][sl])
                sn["st"].compact()
            allp = [p for sn in snaps for p in sn["progs"]]
            assert len(allp) == 64
            out = cg.run_batch(allp)
            assert all(x["converged"] == 1 for x in out), r
            for sn in snaps:
                st, ps = sn["st"], sn["progs"]
                bfs0, _ = st.run_minprop(orc.BFS, start=0, max_iter=100)
                bfs1, _ = st.run_minprop(orc.BFS, start=1, max_iter=100)
                cc, _ = st.run_minprop(orc.CC, start=0, max_iter=100)
                d0, _ = st.run_minprop(orc.SSSP, start=0, max_iter=100)
                d1, _ = st.run_minprop(orc.SSSP, start=1, max_iter=100)
                for p, ref in zip(ps[:6], (bfs0, bfs1, cc, cc, d0, d1)):
                    assert np.array_equal(p.result(), ref), (r, sn["eng"].n, type(p).__name__)
                pr, _ = st.pagerank_norm(tol=1e-15)
                for p in ps[6:]:
                    l1, mr = rel_errors(p.result(), pr)
                    assert l1 <= L1_TOL and mr <= MAXREL_TOL, (r, sn["eng"].n, l1, mr)
    finally:
        for sn in snaps:
            sn["eng"].close()
