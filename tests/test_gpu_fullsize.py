"""GPU tests at the configured full sizes, through properties that do not depend on size.

- Streaming RMAT-22 (4,194,304 vertices, 64 batches of 1,048,576 edges, weights 1..255,
  the pipelined path of the benchmark): the store holds exactly the distinct inserted
  pairs, in tile order, each with its weight; degrees count every inserted edge; BFS
  levels and SSSP distances satisfy their fixed-point equations over the stored edges
  (unique solutions, positive increments); CC labels equal an independent min-label
  fixed point; the incremental BFS / CC / SSSP results equal fresh runs on the final
  snapshot.
- PageRank on RMAT-26 (67,108,864 vertices, 1,073,741,824 edges): the FP64 form within
  relative L1 1e-8 of an independent FP64 power iteration (torch), and FP32-compensated
  within relative L1 1e-6 and max relative 1e-5 of both.
- Weighted PageRank on RMAT-20 and its adjoint: gradients within 1e-4 of the FP64 CPU
  adjoint and of FP64 central differences.
The checks are computed with torch on the device (an independent implementation)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INF = 0xFFFFFFFF


def stored_edges(torch, eng, T, lvpt, weights):
    """Global (src, tgt[, w]) of the compacted store, in store order, as device tensors."""
    tp, ed, wt, _ = eng.dump_tiles(weights=weights)
    dev = torch.device("cuda")
    counts = torch.from_numpy(np.diff(tp.astype(np.int64))).to(dev)
    tiles = torch.repeat_interleave(torch.arange(len(counts), device=dev, dtype=torch.int64), counts)
    e = torch.from_numpy(ed.astype(np.int64)).to(dev)
    src = ((tiles // T) << lvpt) | (e >> 16)
    tgt = ((tiles % T) << lvpt) | (e & 0xFFFF)
    w = torch.from_numpy(wt.astype(np.int64)).to(dev) if weights else None
    return src, tgt, w


def relax_min(torch, n, src, tgt, cand_u, init):
    """min(init[v], min over edges u->v of cand_u[edge]) for every v."""
    out = init.clone()
    return out.scatter_reduce(0, tgt, cand_u, reduce="amin", include_self=True)


def test_streaming_rmat22_full_size(cg):
    torch = pytest.importorskip("torch")
    scale, vpt, B, nb = 22, 65536, 1 << 20, 64
    n, T, lvpt = 1 << scale, (1 << scale) // 65536, 16
    dev = torch.device("cuda")
    s = torch.empty(B * nb, dtype=torch.int32, device=dev)
    t = torch.empty_like(s)
    w = torch.empty_like(s)
    with cg.Engine(1 << 14, 4096, weight_type=cg.WEIGHT_U32) as gen:
        gen.generate_rmat(0, B * nb, scale, seed=2, weight_seed=1002, wmin=1, wmax=255, out=(s, t, w))
    torch.cuda.synchronize()
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as e:
        progs = [cg.BFS(e, start_vertex=0, max_iterations=1000), cg.CC(e, max_iterations=1000),
                 cg.SSSP(e, start_vertex=0, max_iterations=1000)]
        for k in range(nb):
            e.insert_edges_device(s.data_ptr() + 4 * k * B, t.data_ptr() + 4 * k * B, w.data_ptr() + 4 * k * B, B)
            e.do_global_compaction()
            if k:
                assert all(x["converged"] == 1 for x in e.run_many_wait()), k
            e.run_many_async(progs)
        assert all(x["converged"] == 1 for x in e.run_many_wait())
        lvl, lab, dist = [torch.from_numpy(p.result().astype(np.int64)).to(dev) for p in progs]
        fresh = [cg.BFS(e, start_vertex=0, max_iterations=1000), cg.CC(e, max_iterations=1000),
                 cg.SSSP(e, start_vertex=0, max_iterations=1000)]
        e.run_many(fresh)
        for p, got in zip(fresh, (lvl, lab, dist)):
            assert torch.equal(torch.from_numpy(p.result().astype(np.int64)).to(dev), got)
        S, Tg, W = stored_edges(torch, e, T, lvpt, True)
        out_deg, in_deg = e.degrees()
    # the store: the distinct inserted pairs in tile order, with their weights
    keys_in = ((s.to(torch.int64) & INF) << 32) | (t.to(torch.int64) & INF)
    ksorted, kidx = torch.sort(keys_in, stable=True)
    firsts = torch.ones_like(ksorted, dtype=torch.bool)
    firsts[1:] = ksorted[1:] != ksorted[:-1]
    uniq, first = ksorted[firsts], kidx[firsts]  # each pair's first insertion
    keys_st = (S << 32) | Tg
    order = torch.argsort(keys_st)
    assert len(keys_st) == len(uniq)
    assert torch.equal(keys_st[order], uniq)
    assert torch.equal(W[order], w.to(torch.int64)[first])
    tile_of = (S >> lvpt) * T + (Tg >> lvpt)
    assert bool((tile_of[1:] >= tile_of[:-1]).all())
    # degrees count every inserted edge
    assert np.array_equal(out_deg, np.bincount(s.cpu().numpy().view(np.uint32), minlength=n))
    assert np.array_equal(in_deg, np.bincount(t.cpu().numpy().view(np.uint32), minlength=n))
    # BFS: L[v] = min(init, min_in L[u] + 1), init 0 at the start, unreached = INF
    init = torch.full((n,), INF, dtype=torch.int64, device=dev)
    init[0] = 0
    reach = lvl[S] != INF
    assert torch.equal(relax_min(torch, n, S[reach], Tg[reach], lvl[S[reach]] + 1, init), lvl)
    # SSSP: D[v] = min(init, min_in D[u] + w), weights >= 1
    reach = dist[S] != INF
    assert torch.equal(relax_min(torch, n, S[reach], Tg[reach], dist[S[reach]] + W[reach], init), dist)
    # CC (directed min-label propagation, examples/cc.cc:81-91): label[v] = the least id
    # of any vertex that reaches v. Independent fixed point: start from the ids and
    # lower every target to its sources' labels until nothing changes.
    ref = torch.arange(n, device=dev, dtype=torch.int64)
    for _ in range(100000):
        nxt = ref.scatter_reduce(0, Tg, ref[S], reduce="amin", include_self=True)
        if torch.equal(nxt, ref):
            break
        ref = nxt
    else:
        raise AssertionError("the CC check did not reach its fixed point")
    assert torch.equal(lab, ref)


def torch_pagerank_f64(torch, n, S, Tg, alpha=0.85, tol=1e-13, max_iter=1000):
    """Normalised PageRank with dangling mass spread uniformly, FP64, over the stored
    (distinct) edges with distinct out-degrees: the model of CYTOM_ALGO_PAGERANK, written
    independently with torch (gather + index_add) on the device."""
    deg = torch.bincount(S, minlength=n).to(torch.float64)
    dangling = deg == 0
    inv = torch.where(dangling, torch.zeros_like(deg), 1.0 / torch.clamp(deg, min=1.0))
    r = torch.full((n,), 1.0 / n, dtype=torch.float64, device=S.device)
    for it in range(max_iter):
        acc = torch.zeros_like(r).index_add_(0, Tg, (r * inv)[S])
        rn = (1 - alpha) / n + alpha * (acc + r[dangling].sum() / n)
        diff = float((rn - r).abs().sum())
        r = rn
        if diff <= tol:
            return r, it + 1
    raise AssertionError("torch PageRank did not converge")


def test_pagerank_rmat26_full_size(cg):
    torch = pytest.importorskip("torch")
    scale = 26
    n, m = 1 << scale, 16 << scale
    dev = torch.device("cuda")
    with cg.Engine(n, 65536) as e:
        s = torch.empty(m, dtype=torch.int32, device=dev)
        t = torch.empty_like(s)
        e.generate_rmat(0, m, scale, seed=3, out=(s, t, None))
        e.insert_edges_device(s.data_ptr(), t.data_ptr(), None, m)
        del s, t
        e.do_global_compaction()
        p32 = cg.PageRank(e, max_iterations=200, tolerance=1e-9, kahan=True)
        p64 = cg.PageRank(e, max_iterations=200, tolerance=1e-9, kahan=False)
        st32, st64 = p32.execute_algorithm(), p64.execute_algorithm()
        assert st32["converged"] == 1 and st64["converged"] == 1
        r32 = p32.result().astype(np.float64)
        r64 = p64.result64()
        S, Tg, _ = stored_edges(torch, e, n // 65536, 16, False)
    torch.cuda.empty_cache()
    ref, _ = torch_pagerank_f64(torch, n, S, Tg)
    del S, Tg
    ref = ref.cpu().numpy()
    assert abs(r64.sum() - 1.0) < 1e-9
    # the FP64 plain form against the independent FP64 solve (both at residual <= 1e-9:
    # at most about alpha / (1 - alpha) * 1e-9 apart)
    l1_64 = np.abs(r64 - ref).sum() / np.abs(ref).sum()
    assert l1_64 <= 1e-8, l1_64
    l1 = np.abs(r32 - ref).sum() / np.abs(ref).sum()
    mr = (np.abs(r32 - ref) / ref).max()
    assert l1 <= 1e-6 and mr <= 1e-5, (l1, mr)
    l1 = np.abs(r32 - r64).sum() / np.abs(r64).sum()
    mr = (np.abs(r32 - r64) / r64).max()
    assert l1 <= 1e-6 and mr <= 1e-5, (l1, mr)


def test_adjoint_rmat20_full_size(cg, orc):
    scale, vpt = 20, 65536
    n, m = 1 << scale, 16 << 20
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_F32) as e:
        s, t, q = e.generate_rmat(0, m, scale, seed=4, weight_seed=1004, wmin=0, wmax=(1 << 24) - 1)
        w = (0.1 + 0.9 * q.astype(np.float64) / float((1 << 24) - 1)).astype(np.float32)
        e.insert_edges(s, t, w.view(np.uint32))
        e.do_global_compaction()
        st = orc.Store(n, vpt, True)
        st.insert(s, t, w.view(np.uint32))
        st.compact()
        src, tgt, wb = orc.store_edges(st)
        wd = wb.view(np.float32).astype(np.float64)
        c = np.random.default_rng(5).standard_normal(n)
        fwd = cg.WeightedPageRank(e, max_iterations=1000, tolerance=1e-8, kahan=True)
        fwd.execute_algorithm()
        gw, gt, ast = fwd.adjoint(c)
        assert ast["converged"] == 1
        r_ref, _ = orc.wpagerank(n, src, tgt, wd, tol=1e-13)
        _, gw_ref, gt_ref, _ = orc.wpagerank_adjoint(n, src, tgt, wd, r_ref, c, tol=1e-13)
        assert np.abs(gw - gw_ref).max() <= 1e-4 * np.abs(gw_ref).max()
        assert np.abs(gt - gt_ref).max() <= 1e-4 * np.abs(gt_ref).max()
        # FP64 central differences on the GPU (eps 1e-3 on raw weights), 8 random edges
        pf = cg.WeightedPageRank(e, max_iterations=5000, tolerance=1e-15, kahan=False)
        scale_g = np.abs(gw_ref).max()
        for k in np.random.default_rng(11).choice(len(src), 8, replace=False):
            vals = []
            for d in (1e-3, -1e-3):
                e.set_edge_weights(src[k:k + 1], tgt[k:k + 1], np.array([wd[k] + d], np.float32))
                pf.execute_algorithm()
                vals.append(c @ pf.result64())
            e.set_edge_weights(src[k:k + 1], tgt[k:k + 1], np.array([wd[k]], np.float32))
            step = float(np.float32(wd[k] + 1e-3)) - float(np.float32(wd[k] - 1e-3))
            fd = (vals[0] - vals[1]) / step
            assert abs(fd - gw_ref[k]) <= 1e-4 * max(abs(fd), 1e-2 * scale_g), (k, fd, gw_ref[k])
