"""GPU tests of the reference's on-disk formats: the edge log (EdgesWriter records
edge_compact_t / edge_compact_weighted_t, arrival order, duplicates kept) written by
cytom_persist_edges and read back by cytom_read_edges into an identical store, and the
ResultsWriter dumps (raw VertexType arrays) written by cytom_write_results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLT_MAX = np.finfo(np.float32).max


@pytest.mark.parametrize("wtype", ["u32", "none", "f32"])
def test_edge_log_round_trip(cg, orc, tmp_path, wtype):
    scale, vpt = 12, 512
    n = 1 << scale
    kind = {"u32": cg.WEIGHT_U32, "none": cg.UNWEIGHTED, "f32": cg.WEIGHT_F32}[wtype]
    log = tmp_path / "edges_0"
    batches = []
    with cg.Engine(n, vpt, weight_type=kind) as a:
        a.persist_edges(log)
        for b in range(3):
            s, t = orc.rmat(scale, b * 20000, 20000, 7)
            if wtype == "u32":
                w = orc.edge_weights(s, t, 8)
            elif wtype == "f32":
                w = orc.unit_weights(s, t, 8).view(np.uint32)
            else:
                w = None
            a.insert_edges(s, t, w)
            batches.append((s, t, w))
        a.persist_edges(None)
        a.do_global_compaction()
        ref_tiles = a.dump_tiles(weights=kind != cg.UNWEIGHTED)
        ref_deg = a.degrees()
    # the file: the batches' records in arrival order
    raw = np.fromfile(log, dtype=np.uint32)
    rec = 2 if wtype == "none" else 3
    assert raw.size == rec * sum(len(s) for s, _, _ in batches)
    raw = raw.reshape(-1, rec)
    assert np.array_equal(raw[:, 0], np.concatenate([s for s, _, _ in batches]))
    assert np.array_equal(raw[:, 1], np.concatenate([t for _, t, _ in batches]))
    if wtype == "u32":
        assert np.array_equal(raw[:, 2].view(np.float32), np.concatenate([w for _, _, w in batches]).astype(np.float32))
    elif wtype == "f32":
        assert np.array_equal(raw[:, 2], np.concatenate([w for _, _, w in batches]))
    # read back into a fresh store: the same tiles and degrees
    with cg.Engine(n, vpt, weight_type=kind) as b:
        assert b.read_edges(log, batch=7000) == raw.shape[0]
        b.do_global_compaction()
        got = b.dump_tiles(weights=kind != cg.UNWEIGHTED)
        for x, y in zip(got, ref_tiles):
            if x is None:
                assert y is None
            else:
                assert np.array_equal(x, y)
        for x, y in zip(b.degrees(), ref_deg):
            assert np.array_equal(x, y)


def test_results_dumps(cg, orc, tmp_path):
    scale, vpt = 12, 1024
    n = 1 << scale
    s, t = orc.rmat(scale, 0, 16 * n, 3)
    w = orc.edge_weights(s, t, 4)
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as e:
        e.insert_edges(s, t, w)
        progs = {"bfs": cg.BFS(e, start_vertex=0), "cc": cg.CC(e), "sssp": cg.SSSP(e, start_vertex=0),
                 "sswp": cg.SSWP(e, start_vertex=0), "pr": cg.PageRank(e, tolerance=1e-9),
                 "prd": cg.PageRankDelta(e, delta=0.0, tolerance=1e-9, max_iterations=300)}
        for name, p in progs.items():
            p.execute_algorithm()
            path = tmp_path / f"results_{name}"
            p.write_results(path)
            got = p.result()
            if name in ("bfs", "cc"):
                assert np.array_equal(np.fromfile(path, np.uint32), got)
            elif name in ("sssp", "sswp"):
                f = np.fromfile(path, np.float32)
                exp = np.where(got == 0xFFFFFFFF, FLT_MAX, got.astype(np.float32)).astype(np.float32)
                assert np.array_equal(f, exp), name
            elif name == "pr":
                assert np.array_equal(np.fromfile(path, np.float32), got)
            else:
                f = np.fromfile(path, np.float32).reshape(n, 3)  # {delta_sum, rank, delta}
                assert np.array_equal(f[:, 1], got)
                assert np.allclose(f[:, 0] * 0.85, f[:, 2], rtol=1e-6, atol=0)
