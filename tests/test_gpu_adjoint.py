"""GPU tests of weighted PageRank (CYTOM_ALGO_WPAGERANK) and its adjoint.

Forward: FP32-compensated and FP64 forms against the FP64 CPU oracle (relative L1 <= 1e-6,
max relative <= 1e-5 for FP32; relative L1 <= 1e-10 for FP64), uniform and personalised
teleport. Adjoint of L = c . r: dL/d(edge weights) (store order) and dL/d(teleport)
against the FP64 CPU adjoint and against FP64 central differences (eps 1e-3 on raw
weights, GPU FP64 forward solves), within 1e-4 relative to the largest gradient entry."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-4


def wgraph(cg, orc, scale, vpt, seed, wseed, ef=16):
    n = 1 << scale
    s, t = orc.rmat(scale, 0, ef * n, seed)
    w = orc.unit_weights(s, t, wseed)
    eng = cg.Engine(n, vpt, weight_type=cg.WEIGHT_F32)
    eng.insert_edges(s, t, w.view(np.uint32))
    eng.do_global_compaction()
    st = orc.Store(n, vpt, True)
    st.insert(s, t, w.view(np.uint32))
    st.compact()
    src, tgt, wb = orc.store_edges(st)
    return n, eng, src, tgt, wb.view(np.float32).astype(np.float64)


def rel(x, ref):
    x = np.asarray(x, np.float64)
    return np.abs(x - ref).sum() / np.abs(ref).sum(), (np.abs(x - ref) / np.abs(ref)).max()


@pytest.mark.parametrize("personalised", [False, True])
def test_weighted_pagerank_matches_fp64(cg, orc, personalised):
    n, eng, src, tgt, w = wgraph(cg, orc, 12, 1024, 4, 7)
    with eng:
        t = None
        if personalised:
            t = np.random.default_rng(3).random(n) + 0.05
            t /= t.sum()
        ref, _ = orc.wpagerank(n, src, tgt, w, t=t, tol=1e-15)
        p32 = cg.WeightedPageRank(eng, max_iterations=1000, tolerance=1e-10, kahan=True)
        p64 = cg.WeightedPageRank(eng, max_iterations=1000, tolerance=1e-14, kahan=False)
        for p in (p32, p64):
            if t is not None:
                p.set_teleport(t)
            p.execute_algorithm()
        l1, mr = rel(p32.result(), ref)
        assert l1 <= 1e-6 and mr <= 1e-5, (l1, mr)
        l1, mr = rel(p64.result64(), ref)
        assert l1 <= 1e-10, (l1, mr)


def test_adjoint_matches_cpu_adjoint_and_central_differences(cg, orc):
    n, eng, src, tgt, w = wgraph(cg, orc, 12, 1024, 4, 7)
    with eng:
        c = np.random.default_rng(5).standard_normal(n)
        r_ref, _ = orc.wpagerank(n, src, tgt, w, tol=1e-16)
        _, gw_ref, gt_ref, _ = orc.wpagerank_adjoint(n, src, tgt, w, r_ref, c, tol=1e-16)
        for kahan, tol in ((True, 1e-10), (False, 1e-14)):
            p = cg.WeightedPageRank(eng, max_iterations=2000, tolerance=tol, kahan=kahan)
            p.execute_algorithm()
            gw, gt, st = p.adjoint(c)
            assert st["converged"] == 1, st
            ew = np.abs(gw - gw_ref).max() / np.abs(gw_ref).max()
            et = np.abs(gt - gt_ref).max() / np.abs(gt_ref).max()
            assert ew <= GRAD_TOL and et <= GRAD_TOL, (kahan, ew, et)
            p.destroy()
        # FP64 central differences on the GPU (eps 1e-3 on raw weights)
        pf = cg.WeightedPageRank(eng, max_iterations=5000, tolerance=1e-15, kahan=False)
        pf.execute_algorithm()
        scale = np.abs(gw_ref).max()
        eps = 1e-3
        for e in np.random.default_rng(11).choice(len(src), 16, replace=False):
            vals = []
            for d in (eps, -eps):
                eng.set_edge_weights(src[e:e + 1], tgt[e:e + 1], np.array([w[e] + d], np.float32))
                pf.execute_algorithm()
                vals.append(c @ pf.result64())
            eng.set_edge_weights(src[e:e + 1], tgt[e:e + 1], np.array([w[e]], np.float32))
            # the perturbed weight is w + d rounded to FP32: divide by the step actually taken
            step = float(np.float32(w[e] + eps)) - float(np.float32(w[e] - eps))
            fd = (vals[0] - vals[1]) / step
            assert abs(fd - gw_ref[e]) <= GRAD_TOL * max(abs(fd), 1e-2 * scale), (e, fd, gw_ref[e])


def test_set_edge_weights(cg, orc):
    n, eng, src, tgt, w = wgraph(cg, orc, 10, 256, 2, 3, ef=8)
    with eng:
        idx = np.arange(0, len(src), 7)
        neww = (w[idx] * 2.0).astype(np.float32)
        eng.set_edge_weights(src[idx], tgt[idx], neww)
        tp, ed, wt, _ = eng.dump_tiles(weights=True)
        got = wt.view(np.float32)
        exp = w.astype(np.float32).copy()
        exp[idx] = neww
        assert np.array_equal(got, exp)
        # an edge that is not stored is an error
        present = set(tgt[src == 0].tolist())
        v = next(v for v in range(n) if v not in present)
        with pytest.raises(cg.CytomError):
            eng.set_edge_weights(np.array([0], np.uint32), np.array([v], np.uint32), np.array([1.0], np.float32))


def test_adjoint_odd_edge_count(cg, orc):
    # an odd number of stored edges (scratch regions after E floats must stay aligned)
    n, vpt = 64, 32
    src = np.array([0, 1, 2, 2, 5, 40, 41], np.uint32)
    tgt = np.array([1, 2, 0, 33, 40, 41, 5], np.uint32)
    w = np.array([0.5, 0.25, 1.0, 0.75, 0.3, 0.9, 0.6], np.float32)
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_F32) as eng:
        eng.insert_edges(src, tgt, w.view(np.uint32))
        eng.do_global_compaction()
        assert eng.count_edges()[0] % 2 == 1
        st = orc.Store(n, vpt, True)
        st.insert(src, tgt, w.view(np.uint32))
        st.compact()
        s2, t2, wb = orc.store_edges(st)
        w2 = wb.view(np.float32).astype(np.float64)
        c = np.random.default_rng(1).standard_normal(n)
        r_ref, _ = orc.wpagerank(n, s2, t2, w2, tol=1e-16)
        _, gw_ref, gt_ref, _ = orc.wpagerank_adjoint(n, s2, t2, w2, r_ref, c, tol=1e-16)
        p = cg.WeightedPageRank(eng, max_iterations=2000, tolerance=1e-14, kahan=False)
        p.execute_algorithm()
        gw, gt, _ = p.adjoint(c)
        assert np.abs(gw - gw_ref).max() <= GRAD_TOL * np.abs(gw_ref).max()
        assert np.abs(gt - gt_ref).max() <= GRAD_TOL * np.abs(gt_ref).max()
