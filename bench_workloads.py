"""Secondary benchmark workloads of bench.py (--workload prdelta | precision).

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


def run_workload(args, rank, world, local):
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "secondary workloads are measured by the cytom arm; "
                              "the reference arm runs the default streaming workload"}))
        return
    if args.workload == "prdelta":
        run_prdelta(args, rank, world, local)
    else:
        run_precision(args, rank, world, local)
