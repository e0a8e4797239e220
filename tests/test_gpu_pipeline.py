"""GPU tests of the pipelined streaming path: cytom_run_many_async queues a batch's jobs
and returns; the next batch is inserted and merged while they run, and the merged
snapshot is installed (jobs seeded, lowered weights applied) only after they finish.

Every batch's results equal the oracle's fixed points on that batch's snapshot, bit for
bit, and the round and processed-edge counts equal those of synchronous runs; calls that
read or change job state in between wait for the queued runs; lowered weights of stored
edges reach the merged store exactly as in the synchronous path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALGOS = [0, 1, 2, 3]


def make(cg, e):
    return [cg.BFS(e, start_vertex=0, max_iterations=1000), cg.CC(e, max_iterations=1000),
            cg.SSSP(e, start_vertex=0, max_iterations=1000), cg.SSWP(e, start_vertex=0, max_iterations=1000)]


@pytest.mark.parametrize("scale,vpt,batch", [(13, 1024, 4 << 13), (16, 65536, 1 << 16)])
def test_pipelined_batches_match_synchronous_runs(cg, orc, scale, vpt, batch):
    # engine A: insert + compaction of batch b overlap the queued jobs of batch b-1;
    # engine B: the same stream, synchronous. Same rounds and counts every batch, and the
    # oracle's fixed points at the end (and on B after every batch).
    n = 1 << scale
    st = orc.Store(n, vpt, weighted=True)
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as ea, cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as eb:
        pa, pb = make(cg, ea), make(cg, eb)
        prev_b = None
        for b in range(6):
            s, t = orc.rmat(scale, b * batch, batch, 5)
            w = orc.edge_weights(s, t, 6)
            ea.insert_edges(s.copy(), t.copy(), w.copy())
            ea.do_global_compaction()  # overlaps the previous batch's queued jobs
            if b:
                sa = ea.run_many_wait()
                for k in range(4):
                    assert sa[k]["iterations"] == prev_b[k]["iterations"], (b - 1, k)
                    assert sa[k]["count_edges"] == prev_b[k]["count_edges"], (b - 1, k)
            ea.run_many_async(pa)
            eb.insert_edges(s.copy(), t.copy(), w.copy())
            prev_b = eb.run_many(pb)
            st.insert(s, t, w)
            st.compact()
            for k, algo in enumerate(ALGOS):
                assert np.array_equal(pb[k].result(), st.run_minprop(algo, start=0, max_iter=1000)[0]), (b, k)
        last = ea.run_many_wait()
        for k, algo in enumerate(ALGOS):
            assert last[k]["iterations"] == prev_b[k]["iterations"]
            assert last[k]["count_edges"] == prev_b[k]["count_edges"]
            assert np.array_equal(pa[k].result(), st.run_minprop(algo, start=0, max_iter=1000)[0]), k


def test_reading_results_waits_for_queued_runs(cg, orc):
    scale, vpt = 12, 1024
    n = 1 << scale
    s, t = orc.rmat(scale, 0, 16 * n, 3)
    w = orc.edge_weights(s, t, 4)
    st = orc.Store(n, vpt, weighted=True)
    st.insert(s, t, w)
    st.compact()
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as e:
        progs = make(cg, e)
        e.insert_edges(s, t, w)
        e.run_many_async(progs)
        for p, algo in zip(progs, ALGOS):  # no wait: get_result waits for the runs itself
            assert np.array_equal(p.result(), st.run_minprop(algo, start=0, max_iter=1000)[0]), algo
        assert all(x["converged"] == 1 for x in e.run_many_wait())


def test_pipelined_weight_lowering_and_state_calls(cg, orc):
    # a batch that lowers weights of stored edges while the previous jobs are queued; a
    # deletion and a second asynchronous launch without collecting are handled
    scale, vpt = 12, 512
    n = 1 << scale
    rng = np.random.default_rng(2)
    st = orc.Store(n, vpt, weighted=True)
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as e:
        progs = make(cg, e)
        s, t = orc.rmat(scale, 0, 16 * n, 9)
        w = rng.integers(100, 255, len(s), dtype=np.uint32)
        e.insert_edges(s, t, w)
        st.insert(s, t, w)
        st.compact()
        e.run_many_async(progs)
        with pytest.raises(cg.CytomError):
            e.run_many_async(progs)  # the previous launch is not collected yet
        k = rng.choice(len(s), 5000, replace=False)
        w2 = rng.integers(1, 99, len(k), dtype=np.uint32)  # lower: the stored copies change
        e.insert_edges(s[k].copy(), t[k].copy(), w2)
        e.do_global_compaction()
        st.insert(s[k], t[k], w2)
        st.compact()
        e.run_many_wait()
        tp, ed, gw, cf = e.dump_tiles(weights=True)
        otp, oed, ow, ocf = st.dump()
        assert np.array_equal(ed, oed) and np.array_equal(gw, ow) and np.array_equal(cf, ocf)
        e.run_many_async(progs)
        s3, t3, _ = orc.store_edges(st)
        d = rng.choice(len(s3), 2000, replace=False)
        assert e.delete_edges(s3[d], t3[d]) == st.delete(s3[d], t3[d])  # waits for the queued runs
        e.run_many_wait()
        out = e.run_many(progs)
        for p, algo in zip(progs, ALGOS):
            ref, _ = st.run_minprop(algo, start=0, max_iter=1000)
            assert np.array_equal(p.result(), ref), algo
        assert all(x["converged"] == 1 for x in out)
