"""Benchmark: streaming RMAT scale 22 on the tile store, BFS / CC / SSSP re-run
incrementally after every batch -- plus the other configured workloads as keys of the
same JSON line.

Headline workload: 4,194,304 vertices, RMAT graph500 parameters, seed 2, uint32 weights
uniform in [1, 255] (a pure function of (src, tgt)), 64 batches of 1,048,576 edges
inserted in generation order; after each batch the tile store is compacted and BFS
(source 0), CC (min label) and SSSP (source 0) continue from their previous state to the
new fixed point. One step = the whole 64-batch stream (67,108,864 edges) on a cleared
context: every batch inserted, compacted and run. Inputs are generated on the device
before the timed steps.

Metric: GTEPS by the reference's counting rule (edges of tiles with an active source,
summed over rounds and algorithms, algorithm-executor.h:424-426) per second of device
time, ingest included, plus ingest M edges/s. `value` times device-resident inputs;
`e2e` feeds every batch from pinned host memory through the public C ABI and reads the
per-run statistics back.

The other configured workloads run after the headline in the same process and appear
under "workloads" (bench_workloads.py): the RMAT-16 PageRank-delta stream, the RMAT-26
FP32-vs-FP64 PageRank, the 64-job batched executor and the RMAT-20 PageRank adjoint.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GTEPS & HBM GB/s per executor, M edges/s ingest; batched/FP32 vs plain at tol"


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="cytom", choices=["cytom", "reference"])
    ap.add_argument("--workload", default="streaming",
                    choices=["streaming", "prdelta", "precision", "batching", "adjoint"],
                    help="streaming: RMAT-22 BFS/CC/SSSP stream with every other workload as keys (default); "
                         "the others print one workload alone: prdelta: RMAT-16 PageRank-delta stream; precision: "
                         "RMAT-26 PageRank FP32-compensated vs FP64; batching: 64 jobs over 8 snapshots, one "
                         "persistent launch per job round vs one job per launch; adjoint: weighted PageRank RMAT-20 "
                         "forward + adjoint with gradient checks")
    ap.add_argument("--scale", type=int, default=22)
    ap.add_argument("--batch", type=int, default=1 << 20)
    ap.add_argument("--batches", type=int, default=64, help="batches of one stream (one step)")
    ap.add_argument("--vpt", type=int, default=65536)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--max-iter", type=int, default=100)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-workloads", action="store_true", help="headline stream only")
    ap.add_argument("--profile-steps", type=int, default=63,
                    help="batches at the end of the stream timed launch by launch for the roofline "
                         "(default: every batch after the first)")
    ap.add_argument("--precision-scale", type=int, default=26)
    ap.add_argument("--profile-only", action="store_true",
                    help="run --batches batches once with every launch timed and its algorithmic bytes recorded "
                         "(host-driven rounds), print the per-class totals and exit: pairs with an ncu capture "
                         "of the same command")
    ap.add_argument("--programs", default="bfs,cc,sssp",
                    help="vertex programs run after every batch (profiling cases use a subset)")
    ap.add_argument("--preload", type=int, default=0,
                    help="with --profile-only: insert this many batches as one batch first")
    ap.add_argument("--traversal", default="row", choices=["row", "column", "hilbert"],
                    help="tile visiting order of the column-ordered dense round (the reference's --traversal)")
    return ap.parse_args(argv)


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
    """nvidia-smi sampling during the timed region (samples kept in a temporary file)."""

    def __init__(self, index: int):
        self.index, self.proc = index, None
        self.path = Path(tempfile.mkstemp(prefix="cytom_clocks_", suffix=".csv")[1])

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
        try:
            self.path.unlink()
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def stream_config(args, pipelined: bool = True) -> dict:
    """The headline workload, named identically by both arms."""
    return {"workload": f"streaming RMAT-{args.scale}: {args.batches} batches of {args.batch} edges, compaction "
                        f"+ incremental BFS/CC/SSSP after each batch; one step = the whole stream",
            "vertices": 1 << args.scale, "vertices_per_tile": args.vpt, "batch_edges": args.batch,
            "batches_per_step": args.batches, "max_iterations": args.max_iter,
            "parallelism": "replicas" if dist_env()[1] > 1 else "1 GPU",
            "l2": "inputs (805 MB per stream) and store larger than L2; flushed (256 MiB write) before every step"}


def cpu_stream_baseline(args, batches: int, warm: int) -> dict:
    """The reference's own hot-path code (oracle/_ref, built from its sources; all host
    threads as executors and appliers) on a bounded sample of the same stream: the first
    `batches` batches, each inserted and compacted, then BFS / CC / SSSP continue
    incrementally -- the reference's edgeChanged(INSERT) seeding and executeAlgorithm
    (with its active-bitmap swap left out, which otherwise stops every incremental run
    after one round). The first `warm` batches are untimed; value = processed edges of
    the others (the reference's counting rule) over their insert + compaction + run time.
    Falls back to the single-thread oracle port (from-scratch runs) when the reference
    cannot be built."""
    from oracle import oracle as orc
    from oracle import ref_pin
    n = 1 << args.scale
    cores = os.cpu_count() or 1
    s, t = orc.rmat(args.scale, 0, batches * args.batch, args.seed)
    w = orc.edge_weights(s, t, args.seed + 1000)
    if ref_pin.available():
        ex = min(cores, 255)
        r = ref_pin.run("istream", n, args.vpt, s, t, w, batch=args.batch, executors=ex, max_iter=args.max_iter,
                        start=0)
        ce, ins, run = r["count_edges"][warm:], r["insert_seconds"][warm:], r["run_seconds"][warm:]
        secs = float(ins.sum() + run.sum())
        return {"value": float(ce.sum()) / secs / 1e9, "unit": "GTEPS", "cores": ex, "kind": "reference",
                "sample": f"batches {warm + 1}-{batches} of the stream (after {warm} untimed), BFS/CC/SSSP "
                          f"incremental after each, insert + compaction + runs timed, {ex} executors + appliers",
                "run_only_gteps": float(ce.sum()) / float(run.sum()) / 1e9,
                "ingest_medges_per_s": (batches - warm) * args.batch / float(ins.sum()) / 1e6 * 3,
                "seconds": secs}
    st = orc.Store(n, args.vpt, weighted=True)
    total_edges, total_t = 0, 0.0
    for b in range(batches):
        sl = slice(b * args.batch, (b + 1) * args.batch)
        t0 = time.perf_counter()
        st.insert(s[sl], t[sl], w[sl])
        st.compact()
        for algo in (orc.BFS, orc.CC, orc.SSSP):
            _, info = st.run_minprop(algo, start=0, max_iter=args.max_iter)
            if b >= warm:
                total_edges += info["count_edges"]
        if b >= warm:
            total_t += time.perf_counter() - t0
    return {"value": total_edges / total_t / 1e9, "unit": "GTEPS", "cores": 1, "kind": "port",
            "sample": f"batches {warm + 1}-{batches} of the stream; BFS/CC/SSSP from scratch after each "
                      f"(single-thread oracle port)", "seconds": total_t}


def run_reference(args, rank):
    """The reference arm: the reference's CPU path on the host cores, same config."""
    if rank != 0:
        return
    t0 = time.time()
    batches = max(2, min(args.batches, args.warmup + args.steps))
    warm = min(args.warmup, batches - 1)
    cb = cpu_stream_baseline(args, batches, warm)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "GTEPS",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * cb["seconds"] / max(1, batches - warm) * args.batches,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic RMAT (graph500 a,b,c), generated", "config": stream_config(args),
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "run_only_gteps": cb.get("run_only_gteps"), "ingest_medges_per_s": cb.get("ingest_medges_per_s"),
            "e2e": {"value": cb["value"], "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "ms_per_step extrapolates the sampled batches' mean time to a whole stream",
            "wall_s": time.time() - t0}
    print(json.dumps(line), flush=True)



def dense_kernel_names(tune) -> str:
    """The dense gather kernels the tuned jobs run (gather_stream_kernel or gather_tiles_kernel)."""
    try:
        kinds = sorted({tune["shapes"][k]["kernel"] for k in tune["chosen"].values()})
    except (TypeError, KeyError, IndexError):
        kinds = ["stream"]
    return " + ".join(f"gather_{k}_kernel" for k in kinds)

def main(argv=None):
    args = parse(argv)
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
    B, NB = args.batch, args.batches
    stream = torch.cuda.Stream(device=dev)
    prog_names = args.programs.split(",")

    def make_engine():
        order = {"row": cg.TRAVERSAL_ROW_FIRST, "column": cg.TRAVERSAL_COLUMN_FIRST,
                 "hilbert": cg.TRAVERSAL_HILBERT}[args.traversal]
        eng = cg.Engine(n, args.vpt, weight_type=cg.WEIGHT_U32, stream=stream.cuda_stream, traversal=order)
        make = {"bfs": lambda: cg.BFS(eng, start_vertex=0, max_iterations=args.max_iter),
                "cc": lambda: cg.CC(eng, max_iterations=args.max_iter),
                "sssp": lambda: cg.SSSP(eng, start_vertex=0, max_iterations=args.max_iter)}
        return eng, [make[name]() for name in prog_names]

    # device-resident inputs of one stream (generated by the library's RMAT kernel)
    eng, progs = make_engine()
    total_edges_in = (args.preload + NB) * B
    d_src = torch.empty(total_edges_in, dtype=torch.int32, device=dev)
    d_tgt = torch.empty_like(d_src)
    d_w = torch.empty_like(d_src)
    with torch.cuda.stream(stream):
        eng.generate_rmat(0, len(d_src), args.scale, seed=args.seed, weight_seed=args.seed + 1000,
                          wmin=1, wmax=255, out=(d_src, d_tgt, d_w))
    stream.synchronize()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > L2 (126 MB)
    with torch.cuda.stream(stream):
        flush.zero_()  # first launch outside the timed steps (the fill kernel may be JIT-compiled)

    def ins(e, k):
        e.insert_edges_device(d_src.data_ptr() + 4 * k * B, d_tgt.data_ptr() + 4 * k * B,
                              d_w.data_ptr() + 4 * k * B, B)

    if args.profile_only:
        eng.set_profiling(True)
        if args.preload:
            eng.insert_edges_device(d_src.data_ptr(), d_tgt.data_ptr(), d_w.data_ptr(), args.preload * B)
            eng.do_global_compaction()
        for k in range(args.preload, args.preload + NB):
            ins(eng, k)
            eng.do_global_compaction()
            eng.run_many(progs)
        if rank == 0:
            print(json.dumps({"profile_only": True, "config": {"scale": args.scale, "batch": B,
                                                               "batches": NB, "preload": args.preload,
                                                               "programs": args.programs},
                              "kernel_stats": {k: v for k, v in eng.kernel_stats().items() if v["launches"]}}),
                  flush=True)
        eng.close()
        return

    def run_stream(e, ps, from_host=None):
        """One step: the whole stream on a cleared context, pipelined -- batch k's jobs run
        (cytom_run_many_async) while batch k+1 is inserted, sorted and merged into the
        alternate buffers; the compaction waits for them only where it installs the merged
        snapshot. Returns the run statistics of every batch."""
        e.clear()
        out = []
        for k in range(NB):
            if from_host is None:
                ins(e, k)
            else:
                hs, ht, hw = from_host
                sl = slice(k * B, (k + 1) * B)
                e.insert_edges(hs[sl], ht[sl], hw[sl])  # H2D from pinned host buffers
            e.do_global_compaction()
            if k:
                out.append(e.run_many_wait())  # the previous batch's statistics (D2H)
            e.run_many_async(ps)
        out.append(e.run_many_wait())
        return out

    # warm-up: the first step grows every buffer; the kernel shapes are tuned once on the
    # full graph it leaves (outside the timed steps) and kept by the context
    tune = None
    for w_ in range(max(1, args.warmup)):
        run_stream(eng, progs)
        if w_ == 0:
            tune = eng.autotune() if os.environ.get("CYTOM_AUTOTUNE", "1") != "0" else eng.tune_report()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    # the timed regions run with Python's cyclic garbage collector paused (as timeit
    # does): a full collection of the interpreter's heap is tens of milliseconds of host
    # time that would otherwise land in a random step
    gc.collect()
    gc.disable()
    clocks = Clocks(local)
    clocks.start()
    launches0 = eng.launch_count()
    teps_edges, scanned = 0, 0
    per_algo = [0] * len(progs)
    per_algo_ms = [0.0] * len(progs)
    t_marks = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    t_marks[0].record(stream)
    for k_ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        for stats in run_stream(eng, progs):
            for i, s in enumerate(stats):
                teps_edges += s["count_edges"]
                scanned += s["edges_scanned"]
                per_algo[i] += s["count_edges"]
                per_algo_ms[i] += s["elapsed_ms"]
        t_marks[k_ + 1].record(stream)
    torch.cuda.synchronize()
    gc.enable()
    launches = eng.launch_count() - launches0
    clk = clocks.stop()
    total_ms = t_marks[0].elapsed_time(t_marks[-1])
    step_ms = [round(t_marks[k_].elapsed_time(t_marks[k_ + 1]), 2) for k_ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    total_ms, teps_all = reduce_over_ranks(total_ms, teps_edges, dev, world)
    value = teps_all / (total_ms / 1e3) / 1e9
    final_edges = eng.count_edges()[0]

    # ---- roofline pass: the last batches of the stream, every launch timed with CUDA
    # events on the engine's stream (profiling mode drives the loop from the host)
    prof_k = max(0, min(args.profile_steps, NB - 1))
    eng.clear()
    for k in range(NB - prof_k):
        ins(eng, k)
        eng.do_global_compaction()
        eng.run_many(progs)
    eng.reset_kernel_stats()
    eng.set_profiling(True)
    prof_stats = []
    for k in range(NB - prof_k, NB):
        with torch.cuda.stream(stream):
            flush.zero_()
        ins(eng, k)
        eng.do_global_compaction()
        prof_stats.append([(i, p.execute_algorithm()) for i, p in enumerate(progs)])
    ks = eng.kernel_stats()
    # the dense kernel on the full graph: fresh BFS / CC / SSSP runs (their first rounds
    # are dense), each launch timed the same way
    eng.reset_kernel_stats()
    fresh = [cg.BFS(eng, start_vertex=0, max_iterations=args.max_iter), cg.CC(eng, max_iterations=args.max_iter),
             cg.SSSP(eng, start_vertex=0, max_iterations=args.max_iter)]
    for p_ in fresh:
        p_.execute_algorithm()
    ks_fresh = eng.kernel_stats()
    for p_ in fresh:
        p_.destroy()
    eng.set_profiling(False)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "MEASURED_PEAKS.json hbm_gbs (measured)" if "hbm_gbs" in peaks else "fallback 6800 GB/s"

    def _variant(k, stats=None):
        v = (stats or ks)[k]
        if not v["launches"] or v["total_ms"] <= 0:
            return None
        gbs = v["algo_bytes"] / (v["total_ms"] / 1e3) / 1e9
        return {"launches": v["launches"], "avg_launch_us": v["total_ms"] * 1e3 / v["launches"],
                "bytes_per_launch": v["algo_bytes"] / v["launches"], "achieved_gbs": gbs,
                "frac": gbs / hbm_peak}

    variants = {"dense": _variant("gather"), "sparse": _variant("gather_sparse"),
                "dense_fresh_runs": _variant("gather", ks_fresh), "sparse_fresh_runs": _variant("gather_sparse", ks_fresh)}
    ing = sum(ks[k]["total_ms"] for k in ("insert", "sort", "merge") if k in ks)
    ingest_meps = world * B / (ing / prof_k / 1e3) / 1e6 if (ing > 0 and prof_k) else None
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
    # round kind (a capture of this workload, committed beside the kernel summaries)
    # times this run's algorithmic bytes
    traffic = None
    tfile = ROOT / "profiles" / "gather_traffic.json"
    if tfile.exists() and g_launches:
        try:
            ratio = json.loads(tfile.read_text())["dram_per_algorithmic_byte"]
            traffic = (ratio["dense"] * ks["gather"]["algo_bytes"]
                       + ratio["sparse"] * ks["gather_sparse"]["algo_bytes"]) / g_launches
        except Exception:
            traffic = None

    # ---- end to end: the same context (its tuned shapes and thresholds) fed from pinned
    # host memory through the C ABI, every step from a cleared store
    e2e = None
    if not args.no_e2e:
        eng2, progs2 = eng, progs
        hs = torch.empty(NB * B, dtype=torch.int32, pin_memory=True)
        ht = torch.empty_like(hs)
        hw = torch.empty_like(hs)
        hs.copy_(d_src[:NB * B].cpu())
        ht.copy_(d_tgt[:NB * B].cpu())
        hw.copy_(d_w[:NB * B].cpu())
        host = (hs.numpy().view(np.uint32), ht.numpy().view(np.uint32), hw.numpy().view(np.uint32))
        for w_ in range(max(1, args.warmup)):
            run_stream(eng2, progs2, host)
        torch.cuda.synchronize()
        e_edges = 0
        gc.collect()
        gc.disable()
        e_clocks = Clocks(local)
        e_clocks.start()
        e_marks = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
        e_marks[0].record(stream)
        for k_ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            e_edges += sum(s["count_edges"] for stats in run_stream(eng2, progs2, host) for s in stats)
            e_marks[k_ + 1].record(stream)
        torch.cuda.synchronize()
        gc.enable()
        e_clk = e_clocks.stop()
        e_ms = e_marks[0].elapsed_time(e_marks[-1])
        e_step_ms = [round(e_marks[k_].elapsed_time(e_marks[k_ + 1]), 2) for k_ in range(args.steps)]
        e_ms, e_all = reduce_over_ranks(e_ms, e_edges, dev, world)
        e2e = {"value": e_all / (e_ms / 1e3) / 1e9, "unit": "GTEPS",
               "h2d_bytes_per_step": NB * B * 12, "d2h_bytes_per_step": NB * len(progs) * 56,
               "ms_per_step": e_ms / args.steps, "step_ms": e_step_ms, "clocks": e_clk}
    eng.close()
    del d_src, d_tgt, d_w, flush
    torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_stream_baseline(args, batches=8, warm=2)

    line = None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic RMAT (graph500 a,b,c), generated on the device",
            "config": stream_config(args),
            "ingest_medges_per_s": ingest_meps,
            # each job's edges over its own device time, measured while the jobs share the GPU
            "gteps_per_algorithm": {nm: per_algo[i] / (per_algo_ms[i] / 1e3) / 1e9 if per_algo_ms[i] else None
                                    for i, nm in enumerate(prog_names)},
            "edges_scanned_per_s": scanned / (total_ms / 1e3),
            "counting_note": "value counts whole tile rows with an active source (the reference's rule); "
                             "edges_scanned_per_s counts the edges the kernels read",
            "final_edges": final_edges,
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": (achieved / hbm_peak) if achieved else None, "traffic": traffic,
                         "kernel": "executor gather, dense + sparse rounds (" + dense_kernel_names(tune)
                                   + " / gather_sparse_kernel + gather_sparse_chunks)",
                         "launches": g_launches,
                         "avg_launch_us": (g_ms * 1e3 / g_launches) if g_launches else None,
                         "bytes_per_launch": (g_bytes / g_launches) if g_launches else None,
                         "variants": variants, "peak_source": peak_src,
                         "measured_on": f"batches {NB - prof_k + 1}-{NB} of the stream, launches timed one by one; "
                                        "*_fresh_runs: fresh BFS / CC / SSSP runs on the final graph"},
            "kernel_time_ms": {k: v["total_ms"] for k, v in ks.items() if v["launches"]},
            "run_profile": run_profile,
            "autotune": tune,
            "clocks": clk,
            "step_ms": step_ms,
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
    if world == 1 and not args.no_workloads:
        from bench_workloads import all_workloads
        wl = all_workloads(args, rank, world, local)
        if line is not None:
            line["workloads"] = wl
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
