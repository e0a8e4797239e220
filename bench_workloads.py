"""Secondary benchmark workloads of bench.py (--workload prdelta | precision | batching | adjoint).

prdelta: RMAT scale 16 (65,536 vertices, 1,048,576 edges, graph500 a,b,c, seed 1,
    duplicates and self-loops kept) streamed in 16 batches of 65,536 edges in
    generation order; after each batch the store is compacted and PageRank-delta
    (alpha 0.85, FP32 ranks, delta 0) runs until the FP64 L1 residual <= 1e-7 of the
    rank sum. One step = one batch. Errors are measured against the FP64 fixed point
    of the final snapshot (CPU oracle).
precision: RMAT scale 26 (67,108,864 vertices, 1,073,741,824 edges, seed 3); normalised
    PageRank (alpha 0.85) in FP32 with compensated sums and in FP64 plain, both run to
    an FP64-measured L1 residual of 1e-9. Errors of the FP32 form
    are against the FP64 form (validated against the CPU FP64 oracle at smaller scales
    by tests/test_gpu_pagerank.py). One step = one full PageRank solve.
"""
from __future__ import annotations

import json
import os
import time

import numpy as np

METRIC = "GTEPS & HBM GB/s per executor, M edges/s ingest; batched/FP32 vs plain at tol"


def _line(args, world, value, ms_per_step, config, extra):
    d = {"metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
         "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
         "vs_baseline": None, "dtype": "f32", "data": "synthetic RMAT (graph500 a,b,c), generated",
         "config": config}
    d.update(extra)
    return d


def run_prdelta(args, rank, world, local):
    import torch
    import cytom_gb300 as cg
    from oracle import oracle as orc
    from oracle import ref_pin
    scale, vpt, B, nb = 16, 4096, 65536, 16
    n = 1 << scale
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    src, tgt = orc.rmat(scale, 0, B * nb, 1)
    hs = torch.from_numpy(src.view(np.int32)).pin_memory()
    ht = torch.from_numpy(tgt.view(np.int32)).pin_memory()
    eng = cg.Engine(n, vpt, stream=stream.cuda_stream)
    p = cg.PageRankDelta(eng, delta=0.0, max_iterations=1000, tolerance=1e-7)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nb)]
    edges = rounds = 0
    ms = 0.0
    for b in range(nb):
        a, c = ev[b]
        a.record(stream)
        eng.insert_edges(hs[b * B:(b + 1) * B].numpy().view(np.uint32), ht[b * B:(b + 1) * B].numpy().view(np.uint32))
        st = p.execute_algorithm()
        c.record(stream)
        torch.cuda.synchronize()
        if b >= min(args.warmup, nb - 1):
            ms += a.elapsed_time(c)
            edges += st["count_edges"]
            rounds += st["iterations"]
    timed = nb - min(args.warmup, nb - 1)
    got = p.result().astype(np.float64)
    store = orc.Store(n, vpt)
    store.insert(src, tgt)
    store.compact()
    ref, _ = store.pagerank_unnorm(tol=1e-14)
    l1 = float(np.abs(got - ref).sum() / np.abs(ref).sum())
    mr = float((np.abs(got - ref) / ref).max())
    cpu = None
    if rank == 0 and not args.no_cpu and ref_pin.available():
        r = ref_pin.run("prdelta", n, vpt, src, tgt, None, batch=B, executors=1, max_iter=100, delta=0.0)
        cpu = {"value": r["count_edges"] / r["seconds"] / 1e9, "unit": "GTEPS", "cores": 1, "kind": "reference",
               "sample": "the reference PageRankDelta (1 executor, delta 0, 100 iterations) on the final snapshot"}
    eng.close()
    if rank == 0:
        print(json.dumps(_line(args, world, edges / (ms / 1e3) / 1e9, ms / timed,
                               {"workload": "PageRank-delta stream: RMAT-16, 16 batches of 65,536 edges, "
                                            "update after each to FP64 L1 residual 1e-7",
                                "vertices": n, "vertices_per_tile": vpt},
                               {"l1_vs_fp64": l1, "max_rel_vs_fp64": mr, "rounds_per_update": rounds / timed,
                                "cpu_baseline": cpu,
                                "e2e": {"value": edges / (ms / 1e3) / 1e9, "unit": "GTEPS",
                                        "h2d_bytes_per_step": B * 8, "d2h_bytes_per_step": 160}})), flush=True)


def run_precision(args, rank, world, local):
    import torch
    import cytom_gb300 as cg
    scale = args.precision_scale
    vpt = 65536
    n = 1 << scale
    m = 16 << scale
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    eng = cg.Engine(n, vpt, stream=stream.cuda_stream)
    chunk = 1 << 28
    s = torch.empty(min(chunk, m), dtype=torch.int32, device="cuda")
    t = torch.empty_like(s)
    t0 = time.time()
    for lo in range(0, m, chunk):
        cnt = min(chunk, m - lo)
        eng.generate_rmat(lo, cnt, scale, seed=3, out=(s[:cnt], t[:cnt], None))
        eng.insert_edges(s[:cnt], t[:cnt])
        eng.do_global_compaction()
    del s, t
    build_s = time.time() - t0
    res = {}
    for kahan in (False, True):
        tol = 1e-9  # both forms stop at the same FP64-measured L1 residual
        prog = cg.PageRank(eng, max_iterations=1000, tolerance=tol, kahan=kahan)
        prog.execute_algorithm()  # warm-up solve (builds the CSC)
        times, stats = [], None
        for _ in range(max(args.steps, 1)):
            prog.init_algorithm()
            a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            stats = prog.execute_algorithm()
            c.record(stream)
            torch.cuda.synchronize()
            times.append(a.elapsed_time(c))
        res[kahan] = {"ms": float(np.median(times)), "stats": stats,
                      "result": prog.result64() if not kahan else prog.result().astype(np.float64)}
        prog.destroy()
    ref = res[False]["result"]
    got = res[True]["result"]
    l1 = float(np.abs(got - ref).sum() / np.abs(ref).sum())
    mr = float((np.abs(got - ref) / ref).max())
    E = eng.count_edges()[0]
    fp32 = res[True]
    fp64 = res[False]
    value = E * fp32["stats"]["iterations"] / (fp32["ms"] / 1e3) / 1e9
    eng.close()
    if rank == 0:
        print(json.dumps(_line(args, world, value, fp32["ms"],
                               {"workload": f"PageRank precision: RMAT-{scale}, FP32-compensated vs FP64 plain",
                                "vertices": n, "distinct_edges": E},
                               {"fp32_ms": fp32["ms"], "fp64_ms": fp64["ms"], "fp32_over_fp64_speedup": fp64["ms"] / fp32["ms"],
                                "fp32_iterations": fp32["stats"]["iterations"], "fp64_iterations": fp64["stats"]["iterations"],
                                "fp64_final_l1_residual": fp64["stats"]["residual"],
                                "fp32_final_l1_residual": fp32["stats"]["residual"],
                                "fp32_l1_vs_fp64": l1, "fp32_max_rel_vs_fp64": mr, "graph_build_s": build_s,
                                "e2e": None, "cpu_baseline": None})), flush=True)


def run_batching(args, rank, world, local):
    """64 jobs over 8 snapshots (RMAT scales 14..21, edge factor 16, seeds 10..17, uint32
    weights uniform in [1, 255]): 16 each of BFS (sources 0, 1), CC, SSSP (sources 0, 1)
    and PageRank (FP32 compensated, FP64 L1 tolerance 1e-8), 8 per snapshot. A job round
    runs every job; the first round computes from scratch, then each snapshot receives
    4 further insert batches of 5% of its edges with a job round after each. The batched
    arm runs each job round as ONE persistent launch (cytom_run_batch); the plain arm
    runs each job by itself (cytom_run: one CUDA-graph launch per BFS/CC/SSSP run, a
    host-driven round loop per PageRank run). Inserts and compactions are untimed and
    identical in both arms; a job round is timed from the first call to the readback of
    the last job's statistics. BFS/CC/SSSP results of the two arms are compared bit for
    bit after every round."""
    import torch
    import cytom_gb300 as cg
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    scales, seeds, rounds = list(range(14, 22)), list(range(10, 18)), 4
    gen = cg.Engine(1 << 14, 4096, weight_type=cg.WEIGHT_U32, stream=stream.cuda_stream)
    inputs = []
    for scale, seed in zip(scales, seeds):
        m = 16 << scale
        b = m // 20
        total = m + rounds * b
        t3 = [torch.empty(total, dtype=torch.int32, device=dev) for _ in range(3)]
        gen.generate_rmat(0, total, scale, seed=seed, weight_seed=seed + 1000, wmin=1, wmax=255, out=tuple(t3))
        inputs.append((scale, m, b, t3))
    gen.close()

    def make_arm():
        engs, progs = [], []
        for scale, m, b, (s, t, w) in inputs:
            n = 1 << scale
            e = cg.Engine(n, min(65536, n >> 2), weight_type=cg.WEIGHT_U32, stream=stream.cuda_stream)
            e.insert_edges_device(s.data_ptr(), t.data_ptr(), w.data_ptr(), m)
            e.do_global_compaction()
            engs.append(e)
            progs += [cg.BFS(e, start_vertex=0, max_iterations=100), cg.BFS(e, start_vertex=1, max_iterations=100),
                      cg.CC(e, max_iterations=100), cg.CC(e, max_iterations=100),
                      cg.SSSP(e, start_vertex=0, max_iterations=100), cg.SSSP(e, start_vertex=1, max_iterations=100),
                      cg.PageRank(e, max_iterations=100, tolerance=1e-8, kahan=True),
                      cg.PageRank(e, max_iterations=100, tolerance=1e-8, kahan=True)]
        return engs, progs

    def insert_round(engs, r):
        for e, (scale, m, b, (s, t, w)) in zip(engs, inputs):
            off = 4 * (m + r * b)
            e.insert_edges_device(s.data_ptr() + off, t.data_ptr() + off, w.data_ptr() + off, b)
            e.do_global_compaction()

    per_kind = [0.0] * 8  # plain arm: wall time by job slot of a snapshot

    def run_arm(batched, check_against=None):
        engs, progs = make_arm()
        for k in range(8):
            per_kind[k] = 0.0
        torch.cuda.synchronize()
        times, results, stats_all = [], [], []
        for r in range(rounds + 1):
            if r:
                insert_round(engs, r - 1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if batched:
                st = cg.run_batch(progs)
            else:
                st = []
                for k, p in enumerate(progs):
                    t1 = time.perf_counter()
                    st.append(p.execute_algorithm())
                    per_kind[k % 8] += time.perf_counter() - t1
            times.append(time.perf_counter() - t0)
            stats_all.append(st)
            results.append([p.result() for p in progs if not isinstance(p, cg.PageRank)])
        launches = sum(e.launch_count() for e in engs)
        for e in engs:
            e.close()
        return times, results, stats_all, launches

    # warm-up pass of each arm (allocations, graph builds), then the timed passes
    for _ in range(max(1, min(args.warmup, 1))):
        run_arm(False)
        run_arm(True)
    tp, rp, sp, lp = run_arm(False)
    plain_kind = list(per_kind)
    tb, rb, sb, lb = run_arm(True)
    exact = all(np.array_equal(x, y) for ra, rb_ in zip(rp, rb) for x, y in zip(ra, rb_))
    njobs = len(sb[0])
    minprop = [k for k in range(njobs) if k % 8 < 6]  # BFS, CC, SSSP jobs of each snapshot
    counts_equal = all(sa[k]["iterations"] == sb_[k]["iterations"] and sa[k]["count_edges"] == sb_[k]["count_edges"]
                       for sa, sb_ in zip(sp, sb) for k in minprop)
    jobs_b = njobs * (rounds + 1) / sum(tb)
    jobs_p = njobs * (rounds + 1) / sum(tp)
    edges_b = sum(x["count_edges"] for st in sb for x in st)
    if rank == 0:
        line = _line(args, world, jobs_b, 1e3 * sum(tb) / (rounds + 1),
                     {"workload": "batching: 64 jobs (16 each of BFS, CC, SSSP, PageRank) over 8 RMAT snapshots "
                                  "(scales 14..21, edge factor 16, seeds 10..17), 4 rounds of +5% inserts",
                      "jobs": njobs, "job_rounds": rounds + 1, "snapshot_scales": scales,
                      "vertices_per_tile": "min(65536, vertices / 4)"},
                     {"unit": "jobs/s", "dtype": "u32 (BFS/CC/SSSP), f32 (PageRank)",
                      "batched_jobs_per_s": jobs_b, "plain_jobs_per_s": jobs_p,
                      "batched_over_plain": jobs_b / jobs_p,
                      "round_ms_batched": [1e3 * x for x in tb], "round_ms_plain": [1e3 * x for x in tp],
                      "integer_results_bit_exact": bool(exact), "rounds_and_counts_equal": bool(counts_equal),
                      "batched_gteps": edges_b / sum(tb) / 1e9,
                      "batched_device_ms_per_round": [st[0]["elapsed_ms"] for st in sb],
                      "pagerank_rounds_per_run": [[st[k]["iterations"] for k in range(njobs) if k % 8 == 6] for st in sb],
                      "plain_ms_by_job_kind": dict(zip(["bfs0", "bfs1", "cc", "cc2", "sssp0", "sssp1", "pr", "pr2"],
                                                       [1e3 * x for x in plain_kind])),
                      "gpu_launches_batched_pass": lb, "gpu_launches_plain_pass": lp,
                      "e2e": None, "cpu_baseline": None})
        line["unit"] = "jobs/s"
        print(json.dumps(line), flush=True)


def run_adjoint(args, rank, world, local):
    """Weighted PageRank on RMAT scale 20 (1,048,576 vertices, 16,777,216 edges, seed 4),
    FP32 edge weights uniform in [0.1, 1.0] (a hash of (src, tgt)) normalised per source,
    damping 0.85, FP32-compensated forward to L1 residual 1e-8; L = c . r with c ~ N(0,1)
    (seed 5); the adjoint gives dL/d(edge weights) and dL/d(teleport). One step = one
    forward + adjoint. Checks: FP64 central differences (eps 1e-3 on raw weights, GPU FP64
    forward solves) on 64 random edges, and the FP64 CPU adjoint (oracle) on every edge."""
    import torch
    import cytom_gb300 as cg
    from oracle import oracle as orc
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    scale, seed = 20, 4
    n, m = 1 << scale, 16 << 20
    eng = cg.Engine(n, 65536, weight_type=cg.WEIGHT_F32, stream=stream.cuda_stream)
    s, t, q = eng.generate_rmat(0, m, scale, seed=seed, weight_seed=seed + 1000, wmin=0, wmax=(1 << 24) - 1)
    w = (0.1 + 0.9 * q.astype(np.float64) / float((1 << 24) - 1)).astype(np.float32)
    eng.insert_edges(s, t, w.view(np.uint32))
    eng.do_global_compaction()
    E = eng.count_edges()[0]
    c = np.random.default_rng(5).standard_normal(n)
    fwd = cg.WeightedPageRank(eng, max_iterations=1000, tolerance=1e-8, kahan=True)
    times, fst, ast = [], None, None
    for k in range(max(args.warmup, 1) + max(args.steps, 1)):
        fwd.init_algorithm()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fst = fwd.execute_algorithm()
        gw, gt, ast = fwd.adjoint(c)
        if k >= max(args.warmup, 1):
            times.append((time.perf_counter() - t0, fst["elapsed_ms"], ast["elapsed_ms"]))
    wall = float(np.median([x[0] for x in times]))
    fwd_ms = float(np.median([x[1] for x in times]))
    adj_ms = float(np.median([x[2] for x in times]))
    edges = fst["iterations"] * E + ast["iterations"] * E
    # FP64 central differences on the GPU
    tp, ed, wb, _ = eng.dump_tiles(weights=True)
    T = n // 65536
    tiles = np.repeat(np.arange(len(tp) - 1, dtype=np.uint64), np.diff(tp).astype(np.int64))
    src = (((tiles // T) << np.uint64(16)) | (ed >> 16).astype(np.uint64)).astype(np.uint32)
    tgt = (((tiles % T) << np.uint64(16)) | (ed & 0xFFFF).astype(np.uint64)).astype(np.uint32)
    wst = wb.view(np.float32)
    f64 = cg.WeightedPageRank(eng, max_iterations=5000, tolerance=1e-15, kahan=False)
    f64.execute_algorithm()
    eps = 1e-3
    gmax = float(np.abs(gw).max())
    fd_err = 0.0
    t_fd = time.perf_counter()
    for e in np.random.default_rng(6).choice(E, 64, replace=False):
        vals = []
        for d in (eps, -eps):
            eng.set_edge_weights(src[e:e + 1], tgt[e:e + 1], np.array([wst[e] + d], np.float32))
            f64.execute_algorithm()
            vals.append(float(c @ f64.result64()))
        eng.set_edge_weights(src[e:e + 1], tgt[e:e + 1], wst[e:e + 1].copy())
        step = float(np.float32(wst[e] + eps)) - float(np.float32(wst[e] - eps))
        fd = (vals[0] - vals[1]) / step
        fd_err = max(fd_err, abs(fd - float(gw[e])) / max(abs(fd), 1e-2 * gmax))
    t_fd = time.perf_counter() - t_fd
    # FP64 CPU adjoint (oracle) on every edge: the CPU baseline as well
    t_cpu = time.perf_counter()
    r_ref, it_f = orc.wpagerank(n, src, tgt, wst.astype(np.float64), tol=1e-8)
    _, gw_ref, gt_ref, it_a = orc.wpagerank_adjoint(n, src, tgt, wst.astype(np.float64), r_ref, c, tol=1e-8)
    t_cpu = time.perf_counter() - t_cpu
    r_ref14, _ = orc.wpagerank(n, src, tgt, wst.astype(np.float64), tol=1e-14)
    _, gw_ref14, gt_ref14, _ = orc.wpagerank_adjoint(n, src, tgt, wst.astype(np.float64), r_ref14, c, tol=1e-14)
    ew = float(np.abs(gw - gw_ref14).max() / np.abs(gw_ref14).max())
    et = float(np.abs(gt - gt_ref14).max() / np.abs(gt_ref14).max())
    r32 = fwd.result().astype(np.float64)
    l1 = float(np.abs(r32 - r_ref14).sum() / np.abs(r_ref14).sum())
    eng.close()
    if rank == 0:
        print(json.dumps(_line(args, world, edges / wall / 1e9, 1e3 * wall,
                               {"workload": "differentiation: weighted PageRank RMAT-20 (16,777,216 edges, seed 4), "
                                            "forward to L1 1e-8 + adjoint, c ~ N(0,1) seed 5",
                                "vertices": n, "distinct_edges": E},
                               {"unit": "GTEPS (forward + adjoint rounds x stored edges per second)",
                                "forward_ms": fwd_ms, "adjoint_ms": adj_ms, "forward_rounds": fst["iterations"],
                                "adjoint_rounds": ast["iterations"],
                                "forward_gteps": fst["iterations"] * E / (fwd_ms / 1e3) / 1e9,
                                "adjoint_gteps": ast["iterations"] * E / (adj_ms / 1e3) / 1e9,
                                "grad_w_vs_central_diff_max_rel": fd_err, "central_diff_edges": 64,
                                "central_diff_eps": eps, "central_diff_seconds": t_fd,
                                "grad_w_vs_fp64_cpu_adjoint_max_rel": ew, "grad_t_vs_fp64_cpu_adjoint_max_rel": et,
                                "forward_l1_vs_fp64": l1,
                                "cpu_baseline": {"value": (it_f + it_a) * E / t_cpu / 1e9, "unit": "GTEPS", "cores": 1,
                                                 "kind": "port",
                                                 "sample": "the FP64 CPU forward (L1 1e-8) + adjoint on the same graph"},
                                "e2e": {"value": edges / wall / 1e9, "unit": "GTEPS", "h2d_bytes_per_step": n * 8,
                                        "d2h_bytes_per_step": E * 4 + n * 4 + 2 * 56}})), flush=True)


def run_workload(args, rank, world, local):
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "secondary workloads are measured by the cytom arm; "
                              "the reference arm runs the default streaming workload"}))
        return
    if args.workload == "prdelta":
        run_prdelta(args, rank, world, local)
    elif args.workload == "batching":
        run_batching(args, rank, world, local)
    elif args.workload == "adjoint":
        run_adjoint(args, rank, world, local)
    else:
        run_precision(args, rank, world, local)
