"""Benchmark: streaming RMAT scale 22 on the tile store, BFS / CC / SSSP re-run
incrementally after every batch.

Workload (the GPU-sized streaming configuration): 4,194,304 vertices, RMAT graph500
parameters, seed 2, uint32 weights uniform in [1, 255] (a pure function of
(src, tgt)), batches of 1,048,576 edges inserted in generation order; after each
batch the tile store is compacted and BFS (source 0), CC (min label) and SSSP
(source 0) continue from their previous state to the new fixed point. One step =
one batch: insert + compact + the three runs. 64 batches make the full 67,108,864-
edge stream; the default run uses W = 3 warm-up batches and K = 61 timed batches.

Metric: GTEPS by the reference's counting rule (edges of tiles with an active
source, summed over rounds and algorithms, algorithm-executor.h:424-426) per second
of device time, plus ingest M edges/s. `value` times device-resident inputs;
`e2e` feeds every batch from pinned host memory through the public C ABI and reads
the per-run statistics back.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GTEPS & HBM GB/s per executor, M edges/s ingest; batched/FP32 vs plain at tol"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=61)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="cytom", choices=["cytom", "reference"])
    ap.add_argument("--workload", default="streaming",
                    choices=["streaming", "prdelta", "precision", "batching", "adjoint"],
                    help="streaming: RMAT-22 BFS/CC/SSSP stream (default); prdelta: RMAT-16 PageRank-delta "
                         "stream; precision: RMAT-26 PageRank FP32-compensated vs FP64; batching: 64 jobs over "
                         "8 snapshots, one persistent launch per job round vs one job per launch; adjoint: weighted "
                         "PageRank RMAT-20 forward + adjoint with gradient checks")
    ap.add_argument("--scale", type=int, default=22)
    ap.add_argument("--batch", type=int, default=1 << 20)
    ap.add_argument("--vpt", type=int, default=65536)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--max-iter", type=int, default=100)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile-steps", type=int, default=4)
    ap.add_argument("--precision-scale", type=int, default=26)
    ap.add_argument("--profile-only", action="store_true",
                    help="run preload, warm-up and --profile-steps batches with every launch timed and "
                         "its algorithmic bytes recorded (host-driven rounds), print the per-class totals "
                         "and exit: pairs with an ncu capture of the same command")
    ap.add_argument("--programs", default="bfs,cc,sssp",
                    help="vertex programs run after every batch (profiling cases use a subset)")
    ap.add_argument("--preload", type=int, default=0,
                    help="insert this many batches as one batch before the warm-up (profiling cases)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_over_ranks(ms: float, edges: float, dev, world: int):
    """Replicas: the slowest rank's time and the edges of all ranks (one all-reduce each;
    NCCL on GPUs, gloo for the CPU tests)."""
    if world <= 1:
        return float(ms), float(edges)
    import torch
    t = torch.tensor([ms], device=dev, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    e = torch.tensor([edges], device=dev, dtype=torch.float64)
    torch.distributed.all_reduce(e)
    return float(t.item()), float(e.item())


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, path: Path, index: int):
        self.path, self.index, self.proc = path, index, None

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        self.fh.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(args, batches: int = 8) -> dict:
    """The reference's own hot-path code (oracle/_ref, built from its sources; all host
    threads as executors and appliers) on a bounded sample of the same workload: the
    first `batches` batches of the stream, each inserted and compacted, then BFS / CC /
    SSSP run on the snapshot (from scratch: the reference's incremental re-runs stop
    after one round, so they are not used), counted by the reference's own rule.
    Falls back to the single-thread oracle port when the reference cannot be built."""
    from oracle import oracle as orc
    from oracle import ref_pin
    n = 1 << args.scale
    cores = os.cpu_count() or 1
    s, t = orc.rmat(args.scale, 0, batches * args.batch, args.seed)
    w = orc.edge_weights(s, t, args.seed + 1000)
    if ref_pin.available():
        r = ref_pin.run("stream", n, args.vpt, s, t, w, batch=args.batch, executors=min(cores, 255),
                        max_iter=args.max_iter, start=0)
        return {"value": r["count_edges"] / r["run_seconds"] / 1e9, "unit": "GTEPS", "cores": min(cores, 255),
                "kind": "reference",
                "sample": f"first {r['batches']} batches of the stream; after each, BFS/CC/SSSP run on the "
                          f"snapshot by the reference executor ({min(cores, 255)} executors + appliers)",
                "ingest_medges_per_s": batches * args.batch / r["insert_seconds"] / 1e6}
    st = orc.Store(n, args.vpt, weighted=True)
    total_edges, total_t = 0, 0.0
    for b in range(batches):
        sl = slice(b * args.batch, (b + 1) * args.batch)
        st.insert(s[sl], t[sl], w[sl])
        st.compact()
        t0 = time.perf_counter()
        for algo in (orc.BFS, orc.CC, orc.SSSP):
            _, info = st.run_minprop(algo, start=0, max_iter=args.max_iter)
            total_edges += info["count_edges"]
        total_t += time.perf_counter() - t0
    return {"value": total_edges / total_t / 1e9, "unit": "GTEPS", "cores": 1, "kind": "port",
            "sample": f"first {batches} batches of the stream; BFS/CC/SSSP from scratch after each "
                      f"(single-thread oracle port)"}


def run_reference(args, rank):
    if rank != 0:
        return
    t0 = time.time()
    cb = cpu_baseline(args, batches=max(2, min(16, (args.steps + args.warmup) // 8)))
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "GTEPS",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic RMAT (graph500 a,b,c), generated",
            "config": {"workload": f"streaming RMAT-{args.scale}, {args.batch}-edge batches, "
                                   "compaction + BFS/CC/SSSP after each batch",
                       "vertices_per_tile": args.vpt},
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "ingest_medges_per_s": cb.get("ingest_medges_per_s"),
            "e2e": {"value": cb["value"], "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.time() - t0}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.workload != "streaming":
        from bench_workloads import run_workload
        run_workload(args, rank, world, local)
        return
    if args.impl == "reference":
        run_reference(args, rank)
        return
    import numpy as np
    import torch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    import cytom_gb300 as cg

    n = 1 << args.scale
    B = args.batch
    nsteps = args.preload + args.warmup + args.steps
    stream = torch.cuda.Stream(device=dev)
    out_dir = ROOT / "gpurun_out"
    out_dir.mkdir(exist_ok=True)

    def make_engine():
        eng = cg.Engine(n, args.vpt, weight_type=cg.WEIGHT_U32, stream=stream.cuda_stream)
        make = {"bfs": lambda: cg.BFS(eng, start_vertex=0, max_iterations=args.max_iter),
                "cc": lambda: cg.CC(eng, max_iterations=args.max_iter),
                "sssp": lambda: cg.SSSP(eng, start_vertex=0, max_iterations=args.max_iter)}
        progs = [make[name]() for name in args.programs.split(",")]
        return eng, progs

    # device-resident inputs for every step (generated by the library's RMAT kernel)
    eng, progs = make_engine()
    d_src = torch.empty(nsteps * B, dtype=torch.int32, device=dev)
    d_tgt = torch.empty_like(d_src)
    d_w = torch.empty_like(d_src)
    with torch.cuda.stream(stream):
        eng.generate_rmat(0, nsteps * B, args.scale, seed=args.seed, weight_seed=args.seed + 1000,
                          wmin=1, wmax=255, out=(d_src, d_tgt, d_w))
    stream.synchronize()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > L2 (126 MB)
    with torch.cuda.stream(stream):
        flush.zero_()  # first launch outside the timed steps (the fill kernel may be JIT-compiled)

    def step(e, ps, k, srcs):
        s, t, w = srcs
        e.insert_edges_device(s.data_ptr() + 4 * k * B, t.data_ptr() + 4 * k * B,
                              w.data_ptr() + 4 * k * B, B)
        e.do_global_compaction()
        return e.run_many(ps)

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
    if args.profile_only:
        eng.set_profiling(True)
    if args.preload:
        eng.insert_edges_device(d_src.data_ptr(), d_tgt.data_ptr(), d_w.data_ptr(), args.preload * B)
        eng.do_global_compaction()
    for k in range(args.preload, args.preload + args.warmup):
        step(eng, progs, k, (d_src, d_tgt, d_w))
    if args.profile_only:
        for k in range(args.preload + args.warmup, nsteps):
            step(eng, progs, k, (d_src, d_tgt, d_w))
        if rank == 0:
            print(json.dumps({"profile_only": True, "config": {"scale": args.scale, "batch": B,
                                                               "steps": nsteps, "programs": args.programs},
                              "kernel_stats": {k: v for k, v in eng.kernel_stats().items() if v["launches"]}}),
                  flush=True)
        eng.close()
        return
    # streaming-gather shapes tuned once on the warmed-up graph (outside the timed steps)
    tune = eng.autotune() if os.environ.get("CYTOM_AUTOTUNE", "1") != "0" else eng.tune_report()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(out_dir / f"clocks_rank{rank}.csv", local)
    clocks.start()
    launches0 = eng.launch_count()
    teps_edges, scanned, ingest_ms, total_ms = 0, 0, 0.0, 0.0
    per_algo = [0] * len(progs)
    per_algo_ms = [0.0] * len(progs)

    def account(stats):
        nonlocal teps_edges, scanned
        for i, s in enumerate(stats):
            teps_edges += s["count_edges"]
            scanned += s["edges_scanned"]
            per_algo[i] += s["count_edges"]
            per_algo_ms[i] += s["elapsed_ms"]

    # Pipelined: batch k's jobs run (cytom_run_many_async) while batch k+1 is inserted,
    # sorted and merged into the alternate buffers; the compaction waits for them only
    # where it installs the merged snapshot. The timed region runs from the first insert
    # to the last batch's job statistics, L2 flushes included.
    pipelined = os.environ.get("CYTOM_PIPELINE", "1") != "0"
    first = args.preload + args.warmup
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(first, nsteps):
        with torch.cuda.stream(stream):
            flush.zero_()
        a, b, c = ev[k]
        a.record(stream)
        eng.insert_edges_device(d_src.data_ptr() + 4 * k * B, d_tgt.data_ptr() + 4 * k * B,
                                d_w.data_ptr() + 4 * k * B, B)
        eng.do_global_compaction()
        b.record(stream)
        if pipelined:
            if k > first:
                account(eng.run_many_wait())  # the previous batch's jobs
            eng.run_many_async(progs)  # the programs side by side, as the reference's jobs
        else:
            account(eng.run_many(progs))
        c.record(stream)
    if pipelined:
        account(eng.run_many_wait())
    t_end.record(stream)
    torch.cuda.synchronize()
    launches = eng.launch_count() - launches0
    clk = clocks.stop()
    total_ms = t_start.elapsed_time(t_end)
    for k in range(args.preload + args.warmup, nsteps):
        a, b, c = ev[k]
        ingest_ms += a.elapsed_time(b)
    if world > 1:
        torch.distributed.barrier()
    total_ms, teps_all = reduce_over_ranks(total_ms, teps_edges, dev, world)
    value = teps_all / (total_ms / 1e3) / 1e9
    ingest_meps = world * args.steps * B / (ingest_ms / 1e3) / 1e6  # pipelined: replaced below
    final_edges = eng.count_edges()[0]

    # ---- roofline pass: the gather kernel timed per launch with CUDA events on the
    # engine's stream (profiling mode drives the loop from the host), on the next
    # batches of the same stream
    eng.reset_kernel_stats()
    eng.set_profiling(True)
    prof_stats = []
    extra = min(args.profile_steps, 64)
    src_h, tgt_h, w_h = eng.generate_rmat(nsteps * B, extra * B, args.scale, seed=args.seed,
                                          weight_seed=args.seed + 1000, wmin=1, wmax=255)
    for k in range(extra):
        with torch.cuda.stream(stream):
            flush.zero_()
        sl = slice(k * B, (k + 1) * B)
        eng.insert_edges(src_h[sl].copy(), tgt_h[sl].copy(), w_h[sl].copy())
        eng.do_global_compaction()
        prof_stats.append([(i, p.execute_algorithm()) for i, p in enumerate(progs)])
    ks = eng.kernel_stats()
    eng.set_profiling(False)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    prog_names = args.programs.split(",")
    # Executor gather, both round kinds: the library attributes to every gather launch
    # its algorithmic bytes (scanned edges + weights, one value per active source, a
    # read and a reduction per changed target, the frontier bitmap or, in a sparse
    # round, the listed frontier words and their directory entries).
    def _variant(k):
        v = ks[k]
        if not v["launches"] or v["total_ms"] <= 0:
            return None
        gbs = v["algo_bytes"] / (v["total_ms"] / 1e3) / 1e9
        return {"launches": v["launches"], "avg_launch_us": v["total_ms"] * 1e3 / v["launches"],
                "bytes_per_launch": v["algo_bytes"] / v["launches"], "achieved_gbs": gbs,
                "frac": gbs / hbm_peak}
    variants = {"dense_stream": _variant("gather"), "sparse_directory": _variant("gather_sparse")}
    if pipelined:
        # insert + sort + merge device time per batch in the profiling pass: with the jobs
        # overlapped, the timed steps' insert-to-compaction time includes waiting for them
        ing = sum(ks[k]["total_ms"] for k in ("insert", "sort", "merge") if k in ks)
        if ing > 0 and extra:
            ingest_meps = world * B / (ing / extra / 1e3) / 1e6
    g_ms = ks["gather"]["total_ms"] + ks["gather_sparse"]["total_ms"]
    g_launches = ks["gather"]["launches"] + ks["gather_sparse"]["launches"]
    g_bytes = ks["gather"]["algo_bytes"] + ks["gather_sparse"]["algo_bytes"]
    achieved = g_bytes / (g_ms / 1e3) / 1e9 if g_ms > 0 else None
    run_profile = {}
    for i, name in enumerate(prog_names):
        runs = [st for r in prof_stats for (k, st) in r if k == i]
        rounds = sum(st["iterations"] for st in runs)
        if runs and rounds:
            run_profile[name] = {"rounds_per_run": rounds / len(runs),
                                 "active_vertices_per_round": sum(st["active_vertices"] for st in runs) / rounds,
                                 "edges_scanned_per_round": sum(st["edges_scanned"] for st in runs) / rounds}
    # DRAM traffic per launch: the ncu-measured DRAM bytes per algorithmic byte of each
    # round kind (profiles/gather_traffic_rmat22.md) times this run's algorithmic bytes
    traffic = None
    tfile = ROOT / "profiles" / "gather_traffic.json"
    if tfile.exists() and g_launches:
        try:
            ratio = json.loads(tfile.read_text())["dram_per_algorithmic_byte"]
            traffic = (ratio["dense_stream"] * ks["gather"]["algo_bytes"]
                       + ratio["sparse_directory"] * ks["gather_sparse"]["algo_bytes"]) / g_launches
        except Exception:
            traffic = None

    # ---- end to end: a fresh engine fed from pinned host memory through the C ABI
    e2e = None
    if not args.no_e2e:
        eng2, progs2 = make_engine()
        hs = torch.empty(nsteps * B, dtype=torch.int32, pin_memory=True)
        ht = torch.empty_like(hs)
        hw = torch.empty_like(hs)
        hs.copy_(d_src.cpu())
        ht.copy_(d_tgt.cpu())
        hw.copy_(d_w.cpu())
        hsn, htn, hwn = hs.numpy().view(np.uint32), ht.numpy().view(np.uint32), hw.numpy().view(np.uint32)
        if args.preload:
            sl = slice(0, args.preload * B)
            eng2.insert_edges(hsn[sl], htn[sl], hwn[sl])
            eng2.do_global_compaction()
        for k in range(args.preload, args.preload + args.warmup):
            sl = slice(k * B, (k + 1) * B)
            eng2.insert_edges(hsn[sl], htn[sl], hwn[sl])
            eng2.do_global_compaction()
            eng2.run_many(progs2)
        if os.environ.get("CYTOM_AUTOTUNE", "1") != "0":
            eng2.autotune()
        torch.cuda.synchronize()
        e_edges, e_ms = 0, 0.0
        e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e_start.record(stream)
        for k in range(args.preload + args.warmup, nsteps):
            with torch.cuda.stream(stream):
                flush.zero_()
            sl = slice(k * B, (k + 1) * B)
            eng2.insert_edges(hsn[sl], htn[sl], hwn[sl])  # H2D from pinned host buffers
            eng2.do_global_compaction()
            if pipelined:
                if k > args.preload + args.warmup:
                    e_edges += sum(s["count_edges"] for s in eng2.run_many_wait())  # statistics read back (D2H)
                eng2.run_many_async(progs2)
            else:
                e_edges += sum(s["count_edges"] for s in eng2.run_many(progs2))
        if pipelined:
            e_edges += sum(s["count_edges"] for s in eng2.run_many_wait())
        e_end.record(stream)
        torch.cuda.synchronize()
        e_ms = e_start.elapsed_time(e_end)
        e2e = {"value": world * e_edges / (e_ms / 1e3) / 1e9, "unit": "GTEPS",
               "h2d_bytes_per_step": B * 12, "d2h_bytes_per_step": 3 * 160 + 16}
        eng2.close()

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(args)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic RMAT (graph500 a,b,c), generated on the device",
            "config": {"workload": f"streaming RMAT-{args.scale}: {args.batch}-edge batches, compaction "
                                   f"+ incremental BFS/CC/SSSP after each batch",
                       "vertices": n, "vertices_per_tile": args.vpt, "batch_edges": B,
                       "max_iterations": args.max_iter, "parallelism": "replicas" if world > 1 else "1 GPU",
                       "l2": "flushed (256 MiB write) before every timed step",
                       "jobs": "BFS, CC and SSSP run side by side after each batch (cytom_run_many_async); "
                               "the next batch's insert and merge overlap them" if pipelined else
                               "BFS, CC and SSSP run side by side after each batch (cytom_run_many)"},
            "ingest_medges_per_s": ingest_meps,
            # each job's edges over its own device time, measured while the jobs share the GPU
            "gteps_per_algorithm": {nm: per_algo[i] / (per_algo_ms[i] / 1e3) / 1e9 if per_algo_ms[i] else None
                                    for i, nm in enumerate(args.programs.split(","))},
            "edges_scanned_per_s": scanned / (total_ms / 1e3),
            "final_edges": final_edges,
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": (achieved / hbm_peak) if achieved else None, "traffic": traffic,
                         "kernel": "executor gather (gather_stream_kernel dense rounds + "
                                   "gather_sparse_kernel/gather_sparse_chunks sparse rounds)",
                         "launches": g_launches,
                         "avg_launch_us": (g_ms * 1e3 / g_launches) if g_launches else None,
                         "bytes_per_launch": (g_bytes / g_launches) if g_launches else None,
                         "variants": variants,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
            "kernel_time_ms": {k: v["total_ms"] for k, v in ks.items() if v["launches"]},
            "run_profile": run_profile,
            "autotune": tune,
            "clocks": clk,
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    eng.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
