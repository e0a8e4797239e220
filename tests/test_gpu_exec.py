"""GPU parity of the BFS / CC / SSSP / SSWP executors against the CPU oracle.

Fresh runs: values, round count and the reference's processed-edge count equal the
oracle's Jacobi run round for round. Streaming runs: after every batch the
incremental result equals the oracle's from-scratch fixed point. Bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALGOS = [("BFS", 0), ("CC", 1), ("SSSP", 2), ("SSWP", 3)]


def build(cg, orc, scale, vpt, m, seed, adaptive=True):
    n = 1 << scale
    s, t = orc.rmat(scale, 0, m, seed)
    w = orc.edge_weights(s, t, seed + 1)
    eng = cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32, adaptive_scheduling=adaptive)
    eng.insert_edges(s, t, w)
    eng.do_global_compaction()
    st = orc.Store(n, vpt, weighted=True)
    st.insert(s, t, w)
    st.compact()
    return eng, st


@pytest.mark.parametrize("name,algo", ALGOS)
@pytest.mark.parametrize("scale,vpt,ef,start", [(10, 64, 8, 0), (12, 256, 16, 1), (14, 4096, 16, 0),
                                                (16, 65536, 8, 3), (17, 2048, 16, 0)])
def test_fresh_run_round_by_round(cg, orc, name, algo, scale, vpt, ef, start):
    eng, st = build(cg, orc, scale, vpt, ef << scale, seed=scale + 31)
    with eng:
        prog = getattr(cg, name)(eng, start_vertex=start, max_iterations=1000)
        stats = prog.execute_algorithm()
        got = prog.result()
        ref, rinfo = st.run_minprop(algo, start=start, max_iter=1000)
        assert np.array_equal(got, ref)
        assert stats["iterations"] == rinfo["iterations"]
        assert stats["count_edges"] == rinfo["count_edges"]
        assert stats["converged"] == 1


@pytest.mark.parametrize("name,algo", ALGOS)
def test_iteration_cap_matches_reference_state(cg, orc, name, algo):
    # with a cap below convergence the state after k rounds still matches (Jacobi rounds)
    eng, st = build(cg, orc, 14, 1024, 16 << 14, seed=5)
    with eng:
        for cap in (1, 2, 3):
            prog = getattr(cg, name)(eng, start_vertex=0, max_iterations=cap)
            stats = prog.execute_algorithm()
            ref, rinfo = st.run_minprop(algo, start=0, max_iter=cap)
            assert np.array_equal(prog.result(), ref), cap
            assert stats["iterations"] == rinfo["iterations"]
            assert stats["count_edges"] == rinfo["count_edges"]


@pytest.mark.parametrize("name,algo", ALGOS)
def test_adaptive_scheduling_off(cg, orc, name, algo):
    eng, st = build(cg, orc, 12, 512, 16 << 12, seed=9, adaptive=False)
    with eng:
        prog = getattr(cg, name)(eng, start_vertex=0, max_iterations=1000)
        stats = prog.execute_algorithm()
        ref, rinfo = st.run_minprop(algo, start=0, max_iter=1000, adaptive=False)
        assert np.array_equal(prog.result(), ref)
        assert stats["iterations"] == rinfo["iterations"]
        assert stats["count_edges"] == rinfo["count_edges"]


@pytest.mark.parametrize("scale,vpt,nb,batch", [(12, 512, 6, 8192), (16, 4096, 8, 65536),
                                                (18, 65536, 4, 1 << 18)])
def test_streaming_incremental_equals_from_scratch(cg, orc, scale, vpt, nb, batch):
    n = 1 << scale
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as eng:
        progs = [cg.BFS(eng, start_vertex=0, max_iterations=1000), cg.CC(eng, max_iterations=1000),
                 cg.SSSP(eng, start_vertex=0, max_iterations=1000), cg.SSWP(eng, start_vertex=0, max_iterations=1000)]
        st = orc.Store(n, vpt, weighted=True)
        for b in range(nb):
            s, t = orc.rmat(scale, b * batch, batch, seed=scale)
            w = orc.edge_weights(s, t, 99)
            eng.insert_edges(s, t, w)
            eng.do_global_compaction()
            st.insert(s, t, w)
            st.compact()
            for prog, (_, algo) in zip(progs, ALGOS):
                stats = prog.execute_algorithm()
                assert stats["converged"] == 1
                ref, _ = st.run_minprop(algo, start=0, max_iter=1000)
                assert np.array_equal(prog.result(), ref), (b, algo)


def test_isolated_start_vertex(cg):
    with cg.Engine(1 << 10, 256, weight_type=cg.WEIGHT_U32) as eng:
        eng.insert_edges(np.array([1, 2], np.uint32), np.array([2, 3], np.uint32),
                         np.array([4, 5], np.uint32))
        p = cg.BFS(eng, start_vertex=7)
        st = p.execute_algorithm()
        r = p.result()
        assert r[7] == 0 and (np.delete(r, 7) == 0xFFFFFFFF).all()
        assert st["iterations"] == 1
        q = cg.SSSP(eng, start_vertex=1)
        q.execute_algorithm()
        d = q.result()
        assert d[1] == 0 and d[2] == 4 and d[3] == 9
        r = cg.SSWP(eng, start_vertex=1)
        r.execute_algorithm()
        wv = r.result()
        assert wv[1] == 0xFFFFFFFF and wv[2] == 4 and wv[3] == 4 and wv[0] == 0


def test_start_vertex_out_of_range(cg):
    with cg.Engine(1 << 10, 256) as eng:
        with pytest.raises(cg.CytomError) as ei:
            cg.BFS(eng, start_vertex=1 << 10)
        assert ei.value.code == -3


def test_graph_and_host_loop_agree(cg, orc, monkeypatch):
    # profiling mode drives the loop from the host; results and counters must agree
    eng, st = build(cg, orc, 14, 2048, 16 << 14, seed=12)
    with eng:
        a = cg.CC(eng, max_iterations=1000)
        sa = a.execute_algorithm()
        eng.set_profiling(True)
        b = cg.CC(eng, max_iterations=1000)
        sb = b.execute_algorithm()
        eng.set_profiling(False)
        assert np.array_equal(a.result(), b.result())
        for k in ("iterations", "count_edges", "edges_scanned", "active_vertices"):
            assert sa[k] == sb[k], k
        ks = eng.kernel_stats()
        assert ks["gather"]["launches"] + ks["gather_sparse"]["launches"] == sb["iterations"]


@pytest.mark.parametrize("mode", ["simple", "stream"])
def test_gather_variants_agree(cg, orc, mode, tmp_path):
    # both gather kernels run in a subprocess with CYTOM_GATHER set, on the same graph
    import json
    import os
    import subprocess
    import sys
    code = f"""
import sys, json, numpy as np
sys.path.insert(0, {str(tmp_path.parents[0])!r})
sys.path.insert(0, {str(__import__('pathlib').Path(__file__).resolve().parents[1])!r})
import cytom_gb300 as cg
from oracle import oracle as orc
n = 1 << 16
s, t = orc.rmat(16, 0, 16 << 16, 21)
w = orc.edge_weights(s, t, 3)
st = orc.Store(n, 4096, True); st.insert(s, t, w); st.compact()
out = {{}}
with cg.Engine(n, 4096, weight_type=cg.WEIGHT_U32) as eng:
    eng.insert_edges(s, t, w); eng.do_global_compaction()
    for name, algo in (("BFS", 0), ("CC", 1), ("SSSP", 2)):
        p = getattr(cg, name)(eng, start_vertex=0, max_iterations=1000)
        stt = p.execute_algorithm()
        ref, info = st.run_minprop(algo, start=0, max_iter=1000)
        out[name] = [bool(np.array_equal(p.result(), ref)), stt["iterations"] == info["iterations"],
                     stt["count_edges"] == info["count_edges"]]
print(json.dumps(out))
"""
    env = dict(os.environ, CYTOM_GATHER=mode)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    for name, checks in res.items():
        assert all(checks), (mode, name, checks)


@pytest.mark.parametrize("sparse,div", [("0", None), ("1", None), ("1", "2"), ("1", "64")])
def test_sparse_and_dense_rounds_agree(cg, orc, sparse, div, tmp_path):
    # incremental runs on a growing graph, with sparse (directory) rounds allowed or not,
    # at the tuned threshold and at fixed thresholds the tuner may choose from (a sparse
    # round while at most 1/div of the frontier words are non-zero)
    import json
    import os
    import subprocess
    import sys
    code = f"""
import sys, json, numpy as np
sys.path.insert(0, {str(__import__('pathlib').Path(__file__).resolve().parents[1])!r})
import cytom_gb300 as cg
from oracle import oracle as orc
scale, vpt = 17, 8192
n = 1 << scale
ok = []
with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as eng:
    progs = [cg.BFS(eng, start_vertex=0, max_iterations=1000), cg.CC(eng, max_iterations=1000),
             cg.SSSP(eng, start_vertex=0, max_iterations=1000), cg.SSWP(eng, start_vertex=0, max_iterations=1000)]
    st = orc.Store(n, vpt, True)
    for b in range(6):
        s, t = orc.rmat(scale, b * 200000, 200000, 3)
        w = orc.edge_weights(s, t, 8)
        eng.insert_edges(s, t, w); st.insert(s, t, w); st.compact()
        for prog, algo in zip(progs, (0, 1, 2, 3)):
            stt = prog.execute_algorithm()
            ref, info = st.run_minprop(algo, start=0, max_iter=1000)
            ok.append(bool(np.array_equal(prog.result(), ref)) and stt["converged"] == 1)
    fresh = cg.SSSP(eng, start_vertex=0, max_iterations=1000)
    stt = fresh.execute_algorithm()
    ref, info = st.run_minprop(2, start=0, max_iter=1000)
    ok.append(bool(np.array_equal(fresh.result(), ref)) and stt["iterations"] == info["iterations"]
              and stt["count_edges"] == info["count_edges"])
print(json.dumps(ok))
"""
    env = dict(os.environ, CYTOM_SPARSE=sparse)
    if div:
        env["CYTOM_SPARSE_DIV"] = div
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    ok = json.loads(r.stdout.strip().splitlines()[-1])
    assert all(ok), (sparse, div, ok)


@pytest.mark.parametrize("variant", ["0", "1", "2", "3", "4"])
def test_stream_shapes_agree(cg, orc, variant):
    # every dense-round kernel and shape the autotuner may pick gives the oracle's values,
    # round counts and processed-edge counts (dense rounds only; single- and multi-row
    # stages; variant 4, the column-ordered tiles kernel, with its shared-memory slice
    # covering all targets (4096), half of them (65536) and with small columns (1024);
    # below 1024 vertices per tile it falls back to the stream)
    import json
    import os
    import subprocess
    import sys
    code = f"""
import sys, json, numpy as np
sys.path.insert(0, {str(__import__('pathlib').Path(__file__).resolve().parents[1])!r})
import cytom_gb300 as cg
from oracle import oracle as orc
ok = []
for scale, vpt, adaptive in ((16, 4096, True), (15, 256, True), (17, 65536, True), (18, 1024, True),
                             (16, 4096, False)):
    n = 1 << scale
    s, t = orc.rmat(scale, 0, 16 * n, 5)
    w = orc.edge_weights(s, t, 6)
    st = orc.Store(n, vpt, True)
    st.insert(s, t, w); st.compact()
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32, adaptive_scheduling=adaptive) as eng:
        eng.insert_edges(s, t, w)
        for prog, algo in ((cg.BFS, 0), (cg.CC, 1), (cg.SSSP, 2), (cg.SSWP, 3)):
            p = prog(eng, start_vertex=0, max_iterations=1000)
            stt = p.execute_algorithm()
            ref, info = st.run_minprop(algo, start=0, max_iter=1000, adaptive=adaptive)
            ok.append(bool(np.array_equal(p.result(), ref)) and stt["iterations"] == info["iterations"]
                      and stt["count_edges"] == info["count_edges"])
        # a further batch: incremental runs on a grown store (the stage list is rebuilt)
        s2, t2 = orc.rmat(scale, 16 * n, 2 * n, 5)
        w2 = orc.edge_weights(s2, t2, 6)
        progs = [cg.BFS(eng, start_vertex=0, max_iterations=1000), cg.CC(eng, max_iterations=1000)]
        for p in progs:
            p.execute_algorithm()
        eng.insert_edges(s2, t2, w2)
        st.insert(s2, t2, w2); st.compact()
        for p, algo in zip(progs, (0, 1)):
            p.execute_algorithm()
            ref, _ = st.run_minprop(algo, start=0, max_iter=1000, adaptive=adaptive)
            ok.append(bool(np.array_equal(p.result(), ref)))
print(json.dumps(ok))
"""
    env = dict(os.environ, CYTOM_SG_VARIANT=variant, CYTOM_SPARSE="0", CYTOM_AUTOTUNE="0")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    ok = json.loads(r.stdout.strip().splitlines()[-1])
    assert all(ok), (variant, ok)


def test_autotune_report(cg, orc):
    scale, vpt = 17, 8192
    n = 1 << scale
    s, t = orc.rmat(scale, 0, 16 * n, 9)
    w = orc.edge_weights(s, t, 10)
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as eng:
        eng.insert_edges(s, t, w)
        rep = eng.autotune()
        assert rep["tuned_edges"] == eng.count_edges()[0]
        k = len(rep["shapes"])
        assert k >= 2 and all(x > 0 for x in rep["round_us"]["bfs_cc"]) and all(x > 0 for x in rep["round_us"]["sssp"])
        best = rep["chosen"]["sssp"]
        assert rep["round_us"]["sssp"][best] == min(rep["round_us"]["sssp"])
        # the sparse-round threshold: one of the candidates (1024 = sparse rounds lost
        # at every tried density), with both round kinds timed at every density
        cands = rep["sparse_threshold_table"]["div_candidates"]
        for cls in ("bfs_cc", "sssp"):
            assert rep["sparse_div"][cls] in cands + [1024], rep["sparse_div"]
            tab = rep["sparse_threshold_table"][cls]
            assert all(x > 0 for x in tab["dense_us"]) and all(x > 0 for x in tab["sparse_us"])
        st = orc.Store(n, vpt, True)
        st.insert(s, t, w)
        st.compact()
        for prog, algo in ((cg.BFS, 0), (cg.CC, 1), (cg.SSSP, 2)):
            p = prog(eng, start_vertex=0, max_iterations=1000)
            stt = p.execute_algorithm()
            ref, info = st.run_minprop(algo, start=0, max_iter=1000)
            assert np.array_equal(p.result(), ref)
            assert stt["iterations"] == info["iterations"] and stt["count_edges"] == info["count_edges"]
        # incremental runs after further batches use the tuned threshold on small frontiers
        progs = [cg.BFS(eng, start_vertex=0, max_iterations=1000), cg.SSSP(eng, start_vertex=0, max_iterations=1000)]
        for p in progs:
            p.execute_algorithm()
        for b in range(3):
            s2, t2 = orc.rmat(scale, 16 * n + b * 20000, 20000, 9)
            w2 = orc.edge_weights(s2, t2, 10)
            eng.insert_edges(s2, t2, w2)
            st.insert(s2, t2, w2)
            st.compact()
            for p, algo in zip(progs, (0, 2)):
                p.execute_algorithm()
                ref, _ = st.run_minprop(algo, start=0, max_iter=1000)
                assert np.array_equal(p.result(), ref), (b, algo)


@pytest.mark.parametrize("name,algo", [("BFSAsync", 0), ("CCAsync", 1)])
@pytest.mark.parametrize("scale,vpt", [(12, 256), (16, 4096), (18, 65536)])
def test_async_programs_reach_the_fixed_point(cg, orc, name, algo, scale, vpt):
    # examples/bfs-async.cc / cc-async.cc: the pull reads next[src]; the values equal the
    # synchronous fixed point, in no more rounds than the synchronous program, fresh, after
    # further batches, and in the batched executor
    n = 1 << scale
    s, t = orc.rmat(scale, 0, 8 << scale, scale + 3)
    w = orc.edge_weights(s, t, 1)
    st = orc.Store(n, vpt, weighted=True)
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as eng:
        eng.insert_edges(s, t, w)
        st.insert(s, t, w)
        st.compact()
        pa = getattr(cg, name)(eng, start_vertex=0, max_iterations=1000)
        pb = getattr(cg, name)(eng, start_vertex=0, max_iterations=1000)
        sa = pa.execute_algorithm()
        ref, rinfo = st.run_minprop(algo, start=0, max_iter=1000)
        assert np.array_equal(pa.result(), ref)
        assert sa["converged"] == 1 and 1 <= sa["iterations"] <= rinfo["iterations"]
        cg.run_batch([pb])
        assert np.array_equal(pb.result(), ref)
        for b in range(2):
            s2, t2 = orc.rmat(scale, (8 << scale) + b * n, n, scale + 3)
            w2 = orc.edge_weights(s2, t2, 1)
            eng.insert_edges(s2, t2, w2)
            st.insert(s2, t2, w2)
            st.compact()
            pa.execute_algorithm()
            cg.run_batch([pb])
            ref, _ = st.run_minprop(algo, start=0, max_iter=1000)
            assert np.array_equal(pa.result(), ref), b
            assert np.array_equal(pb.result(), ref), b


def test_run_many_concurrent_jobs(cg, orc):
    # cytom_run_many: BFS / CC / SSSP / SSWP (and the asynchronous programs) of one context
    # run side by side on their own streams; every batch ends at the oracle's fixed points,
    # with the same round and processed-edge counts as one-at-a-time runs
    scale, vpt = 14, 2048
    n = 1 << scale
    st = orc.Store(n, vpt, weighted=True)
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as ea, cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as eb:
        mk = lambda e: [cg.BFS(e, start_vertex=0, max_iterations=1000), cg.CC(e, max_iterations=1000),
                        cg.SSSP(e, start_vertex=0, max_iterations=1000), cg.SSWP(e, start_vertex=0, max_iterations=1000),
                        cg.BFSAsync(e, start_vertex=0, max_iterations=1000)]
        pa, pb = mk(ea), mk(eb)
        algos = [0, 1, 2, 3, 0]
        for b in range(4):
            s, t = orc.rmat(scale, b * 4 * n, 4 * n, 17)
            w = orc.edge_weights(s, t, 18)
            for e in (ea, eb):
                e.insert_edges(s.copy(), t.copy(), w.copy())
            st.insert(s, t, w)
            st.compact()
            sa = ea.run_many(pa)
            sb = [p.execute_algorithm() for p in pb]
            for k, algo in enumerate(algos):
                ref, _ = st.run_minprop(algo, start=0, max_iter=1000)
                assert np.array_equal(pa[k].result(), ref), (b, k)
                assert np.array_equal(pb[k].result(), ref), (b, k)
                if k < 4:  # the synchronous programs: identical rounds and counts
                    assert sa[k]["iterations"] == sb[k]["iterations"], (b, k)
                    assert sa[k]["count_edges"] == sb[k]["count_edges"], (b, k)
        # a list with a PageRank job runs one after another; a job listed twice is an error
        pr = cg.PageRank(ea, max_iterations=100, tolerance=1e-9)
        out = ea.run_many([pa[0], pr])
        assert len(out) == 2 and out[1]["iterations"] > 0
        with pytest.raises(cg.CytomError):
            ea.run_many([pa[0], pa[0]])


def test_traversal_orders_agree(cg, orc):
    # the column-ordered dense round (variant 4) visits the tiles in each of the
    # reference's traversal orders (row-first, column-first, Hilbert): the same values,
    # rounds, processed-edge counts and scanned edges as the oracle / each other
    import json
    import os
    import subprocess
    import sys
    code = f"""
import sys, json, numpy as np
sys.path.insert(0, {str(__import__('pathlib').Path(__file__).resolve().parents[1])!r})
import cytom_gb300 as cg
from oracle import oracle as orc
out = []
for scale, vpt in ((16, 4096), (17, 1024)):
    n = 1 << scale
    s, t = orc.rmat(scale, 0, 16 * n, 13)
    w = orc.edge_weights(s, t, 14)
    st = orc.Store(n, vpt, True)
    st.insert(s, t, w); st.compact()
    scans = []
    for order in (cg.TRAVERSAL_ROW_FIRST, cg.TRAVERSAL_COLUMN_FIRST, cg.TRAVERSAL_HILBERT):
        with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32, traversal=order) as eng:
            eng.insert_edges(s, t, w)
            sc = []
            for prog, algo in ((cg.BFS, 0), (cg.CC, 1), (cg.SSSP, 2), (cg.SSWP, 3)):
                p = prog(eng, start_vertex=0, max_iterations=1000)
                stt = p.execute_algorithm()
                ref, info = st.run_minprop(algo, start=0, max_iter=1000)
                out.append(bool(np.array_equal(p.result(), ref)) and stt["iterations"] == info["iterations"]
                           and stt["count_edges"] == info["count_edges"])
                sc.append(stt["edges_scanned"])
            scans.append(sc)
    out.append(scans[0] == scans[1] == scans[2])
print(json.dumps(out))
"""
    env = dict(os.environ, CYTOM_SG_VARIANT="4", CYTOM_SPARSE="0", CYTOM_AUTOTUNE="0")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    ok = json.loads(r.stdout.strip().splitlines()[-1])
    assert all(ok), ok


def test_engine_rejects_unknown_traversal(cg):
    with pytest.raises(cg.CytomError) as ei:
        cg.Engine(1 << 12, 1024, traversal=7)
    assert ei.value.code == -1
