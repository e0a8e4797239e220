"""Failure paths of the C ABI, made to run without a GPU fault.

The reference aborts on every failure (util::die, src/lib/util/util.cc:21-32); the
engine returns a status instead and keeps the context usable. The failures are made on
the host (cytom_set_fault_injection):
- an allocation that fails (CYTOM_ERR_OOM) while a job, a batch or a context is set up;
- the batched executor's bounded idle wait running out: a phantom unfinished job that
  has no work keeps the blocks polling until the (shortened) limit, then the launch
  ends with CYTOM_ERR_TIMEOUT; nothing traps, the context stays usable and the jobs
  restart from scratch;
- GridGraph files: a trailing partial record (the reference reads size / 8 records,
  src/include/core/jobs.h:53-64), a missing file (CYTOM_ERR_IO) and an out-of-range id
  (CYTOM_ERR_RANGE).
"""
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_allocation_failure_returns_oom_and_context_survives(cg, orc):
    scale, vpt = 11, 512
    n = 1 << scale
    s, t = orc.rmat(scale, 0, 8 * n, 3)
    with cg.Engine(n, vpt) as eng:
        eng.insert_edges(s, t)
        eng.do_global_compaction()
        # the next allocation (the job's loop state) fails
        eng.set_fault_injection(fail_alloc_after=1)
        with pytest.raises(cg.CytomError) as ei:
            cg.BFS(eng, start_vertex=0, max_iterations=1000)
        assert ei.value.code == -2
        # the injection fired once: the same call now succeeds and computes the right answer
        bfs = cg.BFS(eng, start_vertex=0, max_iterations=1000)
        bfs.execute_algorithm()
        st = orc.Store(n, vpt)
        st.insert(s, t)
        st.compact()
        ref, _ = st.run_minprop(orc.BFS, start=0, max_iter=1000)
        assert np.array_equal(bfs.result(), ref)
        # a host batch needs a staging buffer: that allocation fails, nothing is inserted
        s2, t2 = orc.rmat(scale, 8 * n, n, 3)
        before = eng.count_edges()
        eng.set_fault_injection(fail_alloc_after=1)
        with pytest.raises(cg.CytomError) as ei:
            eng.insert_edges(s2, t2)
        assert ei.value.code == -2
        assert eng.count_edges() == before
        eng.insert_edges(s2, t2)
        st.insert(s2, t2)
        st.compact()
        bfs.execute_algorithm()
        ref, _ = st.run_minprop(orc.BFS, start=0, max_iter=1000)
        assert np.array_equal(bfs.result(), ref)
    # every allocation of a context's creation, one at a time: each fails cleanly
    for k in range(1, 9):
        cg.load()
        probe = cg.Engine(1 << 10, 256)
        probe.set_fault_injection(fail_alloc_after=k)
        try:
            e2 = cg.Engine(1 << 10, 256)
        except cg.CytomError as err:
            assert err.code == -2
        else:
            e2.close()
        probe.set_fault_injection(fail_alloc_after=0)
        probe.close()


def test_batched_idle_wait_gives_up_with_timeout(cg, orc):
    scale, vpt = 12, 1024
    n = 1 << scale
    s, t = orc.rmat(scale, 0, 8 * n, 9)
    w = orc.edge_weights(s, t, 19)
    st = orc.Store(n, vpt, True)
    st.insert(s, t, w)
    st.compact()
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as eng:
        eng.insert_edges(s, t, w)
        progs = [cg.BFS(eng, start_vertex=0, max_iterations=1000), cg.CC(eng, max_iterations=1000),
                 cg.SSSP(eng, start_vertex=0, max_iterations=1000)]
        # a phantom job that never finishes: every block ends up polling, gives up after
        # 2000 empty polls and the launch returns
        eng.set_fault_injection(idle_poll_limit=2000, phantom_jobs=1)
        with pytest.raises(cg.CytomError) as ei:
            cg.run_batch(progs)
        assert ei.value.code == -4
        eng.set_fault_injection()
        out = cg.run_batch(progs)
        assert all(x["converged"] == 1 for x in out)
        for p, algo in zip(progs, (orc.BFS, orc.CC, orc.SSSP)):
            ref, _ = st.run_minprop(algo, start=0, max_iter=1000)
            assert np.array_equal(p.result(), ref), algo


def test_gridgraph_partial_record_missing_file_and_range(cg, orc, tmp_path):
    n = 1 << 12
    rng = np.random.default_rng(4)
    src = rng.integers(0, n, 5000, dtype=np.int64)
    tgt = rng.integers(0, n, 5000, dtype=np.int64)
    data = b"".join(struct.pack("<ii", int(a), int(b)) for a, b in zip(src, tgt))
    f = tmp_path / "g.bin"
    f.write_bytes(data + b"\x07\x00\x00")  # 3 bytes of a partial record after 5000 records
    with cg.Engine(n, 1024) as eng:
        assert eng.load_gridgraph(str(f), batch=1024) == 5000
        eng.do_global_compaction()
        st = orc.Store(n, 1024)
        st.insert(src.astype(np.uint32), tgt.astype(np.uint32))
        st.compact()
        tp, ed, _, _ = eng.dump_tiles()
        otp, oed, _, _ = st.dump()
        assert np.array_equal(tp, otp) and np.array_equal(ed, oed)
        with pytest.raises(cg.CytomError) as ei:
            eng.load_gridgraph(str(tmp_path / "missing.bin"))
        assert ei.value.code == -7
        bad = tmp_path / "bad.bin"
        bad.write_bytes(struct.pack("<iiii", 1, 2, n, 3))  # id n is out of range
        before = eng.count_edges()
        with pytest.raises(cg.CytomError) as ei:
            eng.load_gridgraph(str(bad))
        assert ei.value.code == -3
        assert eng.count_edges() == before
