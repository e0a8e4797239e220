"""GPU PageRank-delta and normalised PageRank against FP64 oracles.

Tolerances (FP32 values): relative L1 <= 1e-6 and max relative error <= 1e-5 against
the FP64 fixed point; the FP64 plain form within 1e-10 relative L1."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L1_TOL, MAXREL_TOL = 1e-6, 1e-5


def rel_errors(x, ref):
    x = np.asarray(x, np.float64)
    l1 = np.abs(x - ref).sum() / np.abs(ref).sum()
    mr = (np.abs(x - ref) / np.maximum(np.abs(ref), 1e-300)).max()
    return l1, mr


def graph(cg, orc, scale, vpt, m, seed, batches=1):
    n = 1 << scale
    eng = cg.Engine(n, vpt)
    st = orc.Store(n, vpt)
    s, t = orc.rmat(scale, 0, m, seed)
    b = m // batches
    for lo in range(0, m, b):
        eng.insert_edges(s[lo:lo + b].copy(), t[lo:lo + b].copy())
        st.insert(s[lo:lo + b], t[lo:lo + b])
        st.compact()
    eng.do_global_compaction()
    return eng, st


@pytest.mark.parametrize("scale,vpt", [(12, 1024), (16, 4096)])
def test_prdelta_matches_fp64_fixed_point(cg, orc, scale, vpt):
    eng, st = graph(cg, orc, scale, vpt, 16 << scale, seed=scale)
    with eng:
        p = cg.PageRankDelta(eng, delta=0.0, max_iterations=400, tolerance=1e-9)
        stats = p.execute_algorithm()
        ref, _ = st.pagerank_unnorm(tol=1e-14)
        l1, mr = rel_errors(p.result(), ref)
        assert l1 <= L1_TOL and mr <= MAXREL_TOL, (l1, mr, stats)


def test_prdelta_streaming_tracks_each_snapshot(cg, orc):
    # 16 batches in generation order, an update after each (the PR-delta streaming setup)
    scale, vpt, nb = 14, 4096, 8
    n, m = 1 << scale, 16 << 14
    s, t = orc.rmat(scale, 0, m, 1)
    st = orc.Store(n, vpt)
    with cg.Engine(n, vpt) as eng:
        p = cg.PageRankDelta(eng, delta=0.0, max_iterations=400, tolerance=1e-9)
        b = m // nb
        for lo in range(0, m, b):
            eng.insert_edges(s[lo:lo + b].copy(), t[lo:lo + b].copy())
            st.insert(s[lo:lo + b], t[lo:lo + b])
            st.compact()
            p.execute_algorithm()
            ref, _ = st.pagerank_unnorm(tol=1e-14)
            l1, mr = rel_errors(p.result(), ref)
            assert l1 <= L1_TOL and mr <= MAXREL_TOL, (lo, l1, mr)


def test_prdelta_reference_threshold_close_to_reference_order(cg, orc):
    # delta = 0.01 (the reference default): activation thresholds make the result
    # approximate; the engine and the reference-order oracle take the same rounds
    scale, vpt = 13, 1024
    eng, st = graph(cg, orc, scale, vpt, 12 << scale, seed=5)
    with eng:
        p = cg.PageRankDelta(eng, delta=0.01, max_iterations=100)
        p.execute_algorithm()
        ref, _ = st.run_prdelta_ref(max_iter=100, delta=0.01)
        l1, _ = rel_errors(p.result(), ref.astype(np.float64))
        assert l1 < 1e-3, l1


@pytest.mark.parametrize("kahan", [True, False])
def test_pagerank_normalised(cg, orc, kahan):
    scale, vpt = 15, 4096
    eng, st = graph(cg, orc, scale, vpt, 16 << scale, seed=7)
    with eng:
        p = cg.PageRank(eng, max_iterations=500, tolerance=1e-10, kahan=kahan)
        stats = p.execute_algorithm()
        ref, _ = st.pagerank_norm(tol=1e-15)
        got = p.result() if kahan else p.result64()
        l1, mr = rel_errors(got, ref)
        if kahan:
            assert l1 <= L1_TOL and mr <= MAXREL_TOL, (l1, mr, stats)
        else:
            assert l1 <= 1e-10, (l1, mr, stats)
        assert abs(np.asarray(got, np.float64).sum() - 1.0) < 1e-5


@pytest.mark.parametrize("kahan", [True, False])
def test_incremental_csc_matches_full_build(cg, orc, kahan):
    # A context whose PageRank job runs after every batch merges the compaction's kept
    # edges into its CSC (no re-sort) once the CSC holds 2 M edges; a context that runs
    # PageRank only at the end sorts once. Fresh jobs on the two end in the same round with the same ranks up to the
    # order of the FP64 dangling-mass atomics (a wrong or missing in-edge moves its
    # target's rank by far more) -- after six batches with duplicates (within and across
    # batches), after a deletion (a full rebuild on both) and after one more batch merged
    # on top of the rebuilt CSC -- and the FP32 form stays within the tolerance of the
    # FP64 oracle.
    scale, vpt = 17, 4096
    n = 1 << scale
    st = orc.Store(n, vpt)

    def fresh_pair(ea, eb):
        fa = cg.PageRank(ea, max_iterations=300, tolerance=1e-10, kahan=kahan)
        fb = cg.PageRank(eb, max_iterations=300, tolerance=1e-10, kahan=kahan)
        sa, sb = fa.execute_algorithm(), fb.execute_algorithm()
        assert sa["iterations"] == sb["iterations"]
        ra = fa.result().astype(np.float64) if kahan else fa.result64()
        rb = fb.result().astype(np.float64) if kahan else fb.result64()
        assert np.allclose(ra, rb, rtol=1e-6 if kahan else 1e-12, atol=0), np.abs(ra - rb).max()
        fa.destroy()
        fb.destroy()
        return ra

    with cg.Engine(n, vpt) as ea, cg.Engine(n, vpt) as eb, cg.Engine(n, vpt) as ec:
        pa = cg.PageRank(ea, max_iterations=300, tolerance=1e-10, kahan=kahan)
        for b in range(6):
            s, t = orc.rmat(scale, b * 4 * n, 4 * n, 77)  # past 2 M stored edges after the fifth
            s = np.concatenate([s, s[:100]])  # duplicates inside the batch
            t = np.concatenate([t, t[:100]])
            for e in (ea, eb, ec):
                e.insert_edges(s.copy(), t.copy())
                e.do_global_compaction()
            st.insert(s, t)
            st.compact()
            pa.execute_algorithm()
        r = fresh_pair(ea, eb)
        ref, _ = st.pagerank_norm(tol=1e-15)
        l1, mr = rel_errors(r, ref)
        assert l1 <= L1_TOL and mr <= MAXREL_TOL, (l1, mr)
        ds, dt = orc.rmat(scale, 0, 500, 77)
        for e in (ea, eb, ec):
            e.delete_edges(ds.copy(), dt.copy())
        pa.execute_algorithm()
        fresh_pair(ea, eb)
        s, t = orc.rmat(scale, 24 * n, 4 * n, 78)
        for e in (ea, eb, ec):
            e.insert_edges(s.copy(), t.copy())
            e.do_global_compaction()
        pa.execute_algorithm()
        # ea merged the last batch into the CSC rebuilt after the deletion; ec, which ran
        # no PageRank before, sorts once
        fresh_pair(ea, ec)
