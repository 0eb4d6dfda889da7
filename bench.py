"""Benchmark: TLR-GEMM updates/s, batched vs plain per-tile, on one GB300.

Workload (one "step"): every Schur update of panel 0 of a TLR Cholesky,
C_ij <- C_ij - A_i0 A_j0^T for 1 <= j < i < 64, i.e. 1953 HCORE_dgemm
recompressions at once: 65536 seeded uniform points in [0,1]^2, Morton
sorted, nb = 1024, kernel exp(-|x-y|^2/0.01), tiles compressed to acc 1e-8
(relative to each tile's largest singular value), maxrank 128, FP64.  The
update itself uses the reference's absolute rule sigma_i < 1e-8.

Arms:
  default           the batched GPU plan (hcore_gb300, C ABI), graph-captured
  --impl reference  the reference's CPU algorithm (the oracle's LAPACK
                    restatement, oracle/) on all host cores, same workload

Output: one JSON line (see the keys below).  Multi-GPU: launched under
torchrun, each rank takes a rank-balanced share of the update list
(longest processing time first on a per-update cost model; independent
updates, no collective on the data path: weak scaling) and builds only the
tiles its share reads; value = all ranks' updates / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TLR-GEMM updates/s batched vs plain per-tile on 1 GB300 at rel err <= acc"
# DRAM bytes (read + write) per algorithmic byte of each phase's kernels:
# dram__bytes_read.sum + dram__bytes_write.sum from ncu captures of the
# 300-update case (a working set beyond L2), divided by the algorithmic bytes.
# QR: every panel and trailing-update launch of one execute of the blocked QR
# (406 MB against 353 MB); stack: one 300-update launch.  The full phase's
# traffic is this ratio times its own algorithmic bytes.
DRAM_PER_ALG_BYTE = {"stack": 0.46, "qr": 1.15, "svd": None, "rebuild": None}
WORKLOAD = dict(workload="TLR Cholesky panel-0 Schur updates (HCORE_dgemm recompression)",
                points=65536, dim=2, nb=1024, tiles_per_dim=64, kernel="exp(-|x-y|^2/0.01)",
                acc=1e-8, maxrank=128, tile_compression="relative sigma >= acc*sigma_max",
                update_truncation="absolute sigma_i < acc (reference rule)")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="panel", choices=["panel", "precision", "dense", "predictor", "tlr",
                                                         "compress", "zgemm", "fp64peak", "panelstep"],
                   help="panel: the headline (1953 Schur updates of a 65,536-point TLR panel); "
                        "precision: acc sweep on the same updates; "
                        "dense: batched dsyrk/dgemmcd tile updates; predictor: "
                        "learned rank predictor on 3D exponential-kernel Cholesky sweeps; "
                        "tlr: batched POTRF + TRSM, the steps either side of the update; "
                        "compress: the GPU tile compressor on the panel workload's tiles; "
                        "zgemm: the complex update through HCORE_zgemm; "
                        "fp64peak: the FP64 probe forms with sampled clocks; "
                        "panelstep: a whole TLR Cholesky panel step through the panel API")
    p.add_argument("--max-updates", type=int, default=None, help="truncate the update list")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-sub", action="store_true",
                   help="panel workload: skip the precision and dense sub-runs")
    p.add_argument("--no-single", action="store_true",
                   help="panel workload: skip the single drop-in call (profiling runs)")
    p.add_argument("--no-autotune", action="store_true",
                   help="panel workload: use the built-in launch shapes instead of autotuning")
    p.add_argument("--dfma-rebuild", action="store_true",
                   help="panel workload: the FP64 reflector kernel for every rebuild instead of "
                        "the tensor-core rebuild (A/B runs)")
    p.add_argument("--per-tile-sample", type=int, default=48)
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--probe-seconds", type=float, default=2.0,
                   help="fp64peak workload: seconds per probe form")
    p.add_argument("--probe-forms", default=None,
                   help="fp64peak workload: only these forms, 'name:chains,...'")
    p.add_argument("--compress-tiles", type=int, default=None,
                   help="compress workload: only the first N tiles (a small profiling case)")
    p.add_argument("--sweep-shape", default=None,
                   help="predictor workload at a reduced shape 'block_tiles,nb,sweeps' (a quick check)")
    return p.parse_args()


def dist_init():
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def all_sum_ints(vec, world: int):
    """Set-up reduction of an integer vector over ranks (tile ranks before
    the partition); not on the timed path."""
    import numpy as np
    import torch

    if world == 1:
        return np.asarray(vec)
    import torch.distributed as dist

    on_gpu = torch.cuda.is_available() and dist.get_backend() == "nccl"
    t = torch.as_tensor(np.asarray(vec, dtype=np.int64), device="cuda" if on_gpu else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().numpy()


def panel_for_rank(args, rank, world, dev):
    """The panel workload of this rank: the whole panel at N=1; at N>1 a
    rank-balanced share (longest processing time first on the per-update
    cost model) holding only the tiles the share reads.  Returns (panel,
    cost imbalance of the partition or None)."""
    from hcore_gb300 import panel as pnl

    if world > 1:
        panel, _, imbalance = pnl.build_panel_share(
            rank, world, lambda v: all_sum_ints(v, world), device=str(dev),
            max_updates=args.max_updates, workers=max(1, (os.cpu_count() or 1) // world))
        return panel, imbalance
    return pnl.build_panel(device=str(dev), max_updates=args.max_updates), None


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        # the raw samples go to $HCORE_BENCH_OUT (default: the temp folder)
        out = os.environ.get("HCORE_BENCH_OUT") or tempfile.gettempdir()
        self.path = os.path.join(out, f"clocks_rank{index}.csv")

    def start(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}",
                                          f"--query-gpu={self.FIELDS}", "--format=csv,noheader",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        sm, mx, reasons, pw = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1].split()[0]))
                mx.append(float(parts[2].split()[0]))
                pw.append(float(parts[3].split()[0]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "power_w_max": max(pw) if pw else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def build_tasks(hc, panel, updates, out_U, out_V, out_off, host=None, acc=None, src=None):
    """LrTask list for the updates (device arenas, or pinned host copies).
    `src` = (U, V) arenas to read instead of the panel's (e.g. FP32 copies)."""
    nb = panel.nb
    U = host["U"] if host else (src[0] if src else panel.U)
    V = host["V"] if host else (src[1] if src else panel.V)
    oU = host["oU"] if host else out_U
    oV = host["oV"] if host else out_V
    esz = U.element_size()
    acc = panel.acc if acc is None else acc
    bU, bV, boU, boV = U.data_ptr(), V.data_ptr(), oU.data_ptr(), oV.data_ptr()
    tasks = []
    for u, (i, j) in enumerate(updates):
        sa, sb, sc = panel.index[(i, 0)], panel.index[(j, 0)], panel.index[(i, j)]
        a, b, c = int(panel.rank[sa]), int(panel.rank[sb]), int(panel.rank[sc])
        tasks.append(hc.LrTask(
            M=nb, a=a, b=b, c=c, rk=0, maxrk=panel.maxrank, ld_newv=0,
            storage_maxrank=panel.maxrank, alpha=-1.0, beta=1.0, acc=acc,
            AU=bU + esz * int(panel.offset[sa]), AV=bV + esz * int(panel.offset[sa]), lda=nb,
            BU=bU + esz * int(panel.offset[sb]), BV=bV + esz * int(panel.offset[sb]), ldb=nb,
            Bdense=None,
            CU=bU + esz * int(panel.offset[sc]), CV=bV + esz * int(panel.offset[sc]), ldc=nb,
            CUo=boU + esz * int(out_off[u]), CVo=boV + esz * int(out_off[u]), ldco=nb))
    return tasks


def input_bytes(panel, updates):
    tot = 0
    for (i, j) in updates:
        a = int(panel.rank[panel.index[(i, 0)]])
        b = int(panel.rank[panel.index[(j, 0)]])
        c = int(panel.rank[panel.index[(i, j)]])
        tot += 2 * panel.nb * (a + b + c) * 8
    return tot


def run_gb300(args):
    import numpy as np
    import torch

    import hcore_gb300 as hc
    from hcore_gb300 import build as hbuild
    from hcore_gb300 import panel as pnl

    rank, world, local = dist_init()
    if not os.path.exists(hbuild.LIB):
        hbuild.build()
    L = hc.lib()
    dev = torch.device("cuda", local)
    t0 = time.time()
    panel, imbalance = panel_for_rank(args, rank, world, dev)
    gen_s = time.time() - t0
    updates = panel.updates
    n = len(updates)
    nb, maxrank = panel.nb, panel.maxrank
    # out-of-place outputs: maxrank columns per update, so steps repeat on
    # the same inputs
    out_off = np.arange(n + 1, dtype=np.int64) * nb * maxrank
    out_U = torch.empty(int(out_off[-1]) + 1, dtype=torch.float64, device=dev)
    out_V = torch.empty_like(out_U)
    tasks = build_tasks(hc, panel, updates, out_U, out_V, out_off)
    stream = torch.cuda.current_stream(dev)
    # the plan's launch shapes, picked by the library's autotuner on this batch
    # (set-up, outside the timed region)
    t0 = time.time()
    flags = hc.DFMA_REBUILD if args.dfma_rebuild else 0
    if args.no_autotune:   # the library's built-in launch shapes (profiling runs)
        tuning, tuned_ms = hc.make_tuning(), None
    else:
        tuning, tuned_ms = hc.autotune(tasks, flags=flags, reps=3, stream=stream.cuda_stream)
    tune_s = time.time() - t0
    batch = hc.Batch(tasks, flags=flags, tuning=tuning)
    batch.execute(stream.cuda_stream)
    ranks, status = batch.results(stream.cuda_stream)
    if (status != 0).any():
        bad = {int(s): int((status == s).sum()) for s in set(status.tolist()) if s}
        raise SystemExit(f"tasks failed: {bad}")

    # capture the four launches in one CUDA graph
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream(dev)
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        with torch.cuda.graph(graph, stream=side):
            batch.execute(side.cuda_stream)
    stream.wait_stream(side)
    torch.cuda.synchronize(dev)

    for _ in range(args.warmup):
        graph.replay()
    torch.cuda.synchronize(dev)
    clocks = Clocks(local)
    barrier(world)
    torch.cuda.synchronize(dev)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        graph.replay()
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    barrier(world)
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    ms_max = max_over_ranks(ms, world)
    total_updates = sum_over_ranks(n, world)
    value = total_updates / (ms_max / 1e3)

    # reference flop model of what this rank did (ranks from the first run)
    flops_model, phase_model = 0, {"stack": 0, "qr": 0, "svd": 0, "rebuild": 0}
    for u, (i, j) in enumerate(updates):
        a = int(panel.rank[panel.index[(i, 0)]])
        b = int(panel.rank[panel.index[(j, 0)]])
        c = int(panel.rank[panel.index[(i, j)]])
        r = int(ranks[u])
        flops_model += pnl.update_flops(nb, a, b, c, r)
        for key, v in pnl.phase_flops(nb, a, b, c, r).items():
            phase_model[key] += v

    result = {"metric": METRIC, "value": value, "unit": "updates/s", "n_gpus": world,
              "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max,
              "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
              "data": "synthetic (seeded points, covariance tiles compressed on the host cores)",
              "config": dict(WORKLOAD, updates_per_step=int(total_updates), parallelism=f"dp{world}",
                             **({"shard": "longest processing time first on the per-update "
                                          "cost model", "shard_cost_imbalance": imbalance}
                                if world > 1 else {}),
                             l2="inputs+outputs+workspace larger than L2 (no flush needed)",
                             graph=f"{batch.launches} kernel launches ({tuning.stream_groups} stream "
                                   f"groups: stack, QR, one SVD launch per rank bucket, one "
                                   f"rebuild launch per padded-k class) captured in one CUDA "
                                   f"graph",
                             rebuild="FP64 reflector kernel" if args.dfma_rebuild else
                                     "tensor cores (exact bf16 digit products) for a + c <= 64"),
              "gpu_launches": batch.launches * args.steps,
              "tuning": dict(tuning.as_dict(), autotune_ms_per_execute=tuned_ms,
                             autotune_s=round(tune_s, 2)),
              "gflops_model": flops_model / (ms / 1e3) / 1e9,
              "clocks": clk}
    if rank != 0:
        barrier(world)
        return

    # ---- per-phase timing: each phase's launches captured in a CUDA graph of
    # their own (as the step runs them: direct launches over dozens of group
    # and bucket streams are falsely serialised), replayed back to back in
    # phase order with events between ----
    phases = [("stack", 1), ("qr", 2), ("svd", 4), ("rebuild", 8)]
    reps = 3
    ph_graphs = []
    for nm, bit in phases:
        g = torch.cuda.CUDAGraph()
        side.wait_stream(stream)
        with torch.cuda.stream(side):
            with torch.cuda.graph(g, stream=side):
                batch.execute_phases(bit, side.cuda_stream)
        stream.wait_stream(side)
        ph_graphs.append(g)
    torch.cuda.synchronize(dev)
    for g in ph_graphs:   # upload / warm
        g.replay()
    torch.cuda.synchronize(dev)
    ph_ms = {nm: 0.0 for nm, _ in phases}
    for _ in range(reps):
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(len(phases) + 1)]
        torch.cuda.synchronize(dev)
        evs[0].record(stream)
        for q, g in enumerate(ph_graphs):
            g.replay()
            evs[q + 1].record(stream)
        torch.cuda.synchronize(dev)
        for q, (nm, _) in enumerate(phases):
            ph_ms[nm] += evs[q].elapsed_time(evs[q + 1]) / reps
    dom = max(ph_ms, key=ph_ms.get)
    result["phase_tflops_model"] = {nm: phase_model[nm] / (ph_ms[nm] / 1e3) / 1e12 for nm in ph_ms}
    ceiling = fp64_ceiling(L, torch, dev, local)
    peak = ceiling["tflops"]
    # algorithmic bytes of each phase (see DRAM_PER_ALG_BYTE)
    alg_bytes = {"stack": 0, "qr": 0, "svd": 0, "rebuild": 0}
    for u, (i, j) in enumerate(updates):
        a = int(panel.rank[panel.index[(i, 0)]])
        b = int(panel.rank[panel.index[(j, 0)]])
        c = int(panel.rank[panel.index[(i, j)]])
        kk, r = a + c, int(ranks[u])
        alg_bytes["stack"] += 8 * nb * (2 * a + 2 * b + 2 * c) + 8 * 2 * nb * kk
        alg_bytes["qr"] += 2 * 2 * nb * kk * 8
        alg_bytes["rebuild"] += 2 * nb * kk * 8 + 2 * nb * r * 8
    achieved = phase_model[dom] / (ph_ms[dom] / 1e3) / 1e12
    result["phases_ms"] = ph_ms
    sw = batch.sweeps(stream.cuda_stream)
    kk = np.array([t.a + t.c for t in tasks])
    result["jacobi_sweeps"] = {"mean": float(sw.mean()), "max": int(sw.max()),
                               "k_mean": float(kk.mean()), "k_max": int(kk.max())}
    ratio = DRAM_PER_ALG_BYTE.get(dom)
    result["roofline"] = {"bound": "fp64", "kernel": dom, "achieved": achieved, "peak": peak,
                          "unit": "TFLOP/s", "frac": achieved / peak,
                          "traffic": (ratio * alg_bytes[dom]) if ratio else None,
                          "traffic_basis": "ncu DRAM bytes per algorithmic byte of this phase's "
                                           "kernels in the 300-update case (working set beyond "
                                           "L2), times this phase's algorithmic bytes "
                                           f"({alg_bytes[dom]:.3e})",
                          "peak_source": "FP64 issue-rate probe timed live (DMMA and DFMA "
                                         "share the FP64 pipe at 1.06-1.10 TFLOP/s on GB300; "
                                         "MEASURED_PEAKS.json has no FP64 figure)",
                          "peak_probe": ceiling,
                          "flops_basis": "reference flop model (flop_counts.c) of that phase",
                          "note": "FP64-equivalent: for a + c <= 64 the QR is blocked and its "
                                  "trailing updates, and the rebuild, run as exact digit "
                                  "products on the tensor cores; the model counts the "
                                  "unblocked FP64 flops, so frac can exceed what the FP64 "
                                  "pipe alone delivers"}

    # ---- the rebuild on the tensor cores: tensor work executed and the FP64
    # rate it stands in for ----
    if not args.dfma_rebuild:
        ks_r = [(t.a + t.c, int(r)) for t, r in zip(tasks, ranks)]
        tflop = tc_rebuild_tensor_flops(nb, ks_r)
        bf16_peak = measured_peak("bf16_tflops")
        t_s = ph_ms["rebuild"] / 1e3
        result["rebuild_tensor_cores"] = {
            "kernel": "rebuild_tc_kernel / rebuild_tc_wide_kernel (tcgen05.mma kind::f16, bf16 "
                      "digit slices, FP32 accumulators in tensor memory)",
            "updates_on_tensor_cores": sum(1 for k_, _ in ks_r if k_ <= 64),
            "tensor_flop_executed": tflop, "tensor_tflops": tflop / t_s / 1e12,
            "bf16_peak_tflops": bf16_peak,
            "frac_of_bf16_peak": (tflop / t_s / 1e12 / bf16_peak) if bf16_peak else None,
            "fp64_equivalent_tflops": phase_model["rebuild"] / t_s / 1e12,
            "fp64_equivalent_frac_of_fp64_peak": phase_model["rebuild"] / t_s / 1e12 / peak,
            "note": "the FP64 reflector products (reference flop model) ran as exact digit "
                    "products on the tensor cores at this FP64-equivalent rate; the tensor work "
                    "counts every MMA as issued (padding rows and zero slices included)"}

    # ---- accuracy on a sample of the timed updates vs the oracle and the
    # exact dense update (rel err <= acc is the metric's condition) ----
    result["accuracy"] = accuracy_all(panel, updates, ranks, out_U, out_V, out_off)

    # ---- plain per-tile loop: one plan per update, device pointers ----
    k = min(args.per_tile_sample, n)
    singles = [hc.Batch([t]) for t in tasks[:k]]
    for s in singles[:2]:
        s.execute(stream.cuda_stream)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for s in singles:
        s.execute(stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    pt_ms = e0.elapsed_time(e1)
    result["per_tile"] = {"value": k / (pt_ms / 1e3), "unit": "updates/s", "sample": k,
                          "how": "one single-update plan launched per tile on one stream"}
    result["batched_vs_per_tile"] = value / result["per_tile"]["value"]
    for s in singles:
        s.close()

    # ---- one plain drop-in call (the single-update configuration) ----
    if not args.no_single:
        result["config1"] = config1_call(hc)

    # ---- the precision sweep and the dense-C step, each oracle-checked ----
    sub_steps = max(3, args.steps // 4)
    if not args.no_sub:
        runs = precision_runs(hc, torch, panel, updates, dev, stream, args.warmup, sub_steps)
        result["precision"] = [
            {"acc": r["acc"], "arithmetic": r["arithmetic"], "updates_per_s": r["updates_per_s"],
             "ms_per_step": r["ms_per_step"], "mean_rank": r["mean_rank"], "all_ok": r["all_ok"],
             **{k: r["accuracy"][k] for k in ("checked", "rank_equal_to_oracle", "gate",
                                               "within_oracle_error", "max_rel_fro_diff_vs_oracle",
                                               "panel_rel_fro_err_vs_dense")}}
            for r in runs]
    if not args.no_sub and world == 1:     # the dense step reads all 63 panel tiles
        d = dense_run(hc, torch, panel, dev, stream, args.warmup, sub_steps, world)
        result["dense"] = {"value": d["value"], "unit": d["unit"], "ms_per_step": d["ms_per_step"],
                           "workload": d["config"]["workload"], "tflops": d["roofline"]["achieved"],
                           "frac_of_fp64_peak": d["roofline"]["frac"],
                           "max_rel_err_vs_oracle": d["accuracy"]["max_rel_err_vs_oracle_sequential_dsyrk"],
                           "tiles_checked": d["accuracy"]["tiles_checked"]}

    # ---- e2e: the same plan over pinned host buffers (zero-copy C2C) ----
    if not args.no_e2e:
        result["e2e"] = e2e_pinned(hc, panel, updates, stream, dev, args, tuning=tuning)
    batch.close()

    # ---- CPU baseline: the reference algorithm on the host cores ----
    if not args.no_cpu:
        result["cpu_baseline"] = cpu_baseline(panel, updates, args.cpu_seconds)
    result["generation_s"] = gen_s
    print(json.dumps(result))
    sys.stdout.flush()
    barrier(world)


def accuracy_sample(panel, updates, ranks, out_U, out_V, out_off, count, acc=None, slack=1e-14):
    """Rank and product of `count` evenly spread updates against the oracle's
    LAPACK restatement (FP64, same acc), and relative Frobenius error against
    the exact dense update beta*C + alpha*A*B^T.  `slack` is the relative
    error allowed on top of the oracle's own (1e-14 for FP64 paths)."""
    import numpy as np

    from oracle import oracle as O

    port = O.Port()
    nb = panel.nb
    U = panel.U
    V = panel.V
    acc = panel.acc if acc is None else acc

    def fac(s):
        o0, o1 = int(panel.offset[s]), int(panel.offset[s + 1])
        r = (o1 - o0) // nb
        return (np.asfortranarray(U[o0:o1].cpu().numpy().reshape(r, nb).T),
                np.asfortranarray(V[o0:o1].cpu().numpy().reshape(r, nb).T), r)

    picks = np.unique(np.linspace(0, len(updates) - 1, count).astype(int))
    worst_oracle, rank_ok, gate_ok = 0.0, 0, 0
    e2_gpu = e2_ref = d2 = 0.0
    worst_tile = worst_tile_ref = 0.0
    for u in picks:
        i, j = updates[u]
        AU, AV, a = fac(panel.index[(i, 0)])
        BU, BV, b = fac(panel.index[(j, 0)])
        CU, CV, c = fac(panel.index[(i, j)])
        r = int(ranks[u])
        o = int(out_off[u])
        gU = np.asfortranarray(out_U[o:o + nb * r].double().cpu().numpy().reshape(r, nb).T)
        gV = np.asfortranarray(out_V[o:o + nb * r].double().cpu().numpy().reshape(r, nb).T)
        ref = port.gemm(nb, -1.0, AU, AV, a, BU, BV, b, 1.0, CU, CV, c, maxrk=panel.maxrank,
                        acc=acc, variant=2)
        D = O.dense_update(-1.0, AU, AV, BU, BV, 1.0, CU, CV)
        P = gU @ gV.T
        Pr = ref["CU"] @ ref["CV"].T
        eg, er, nd = np.linalg.norm(P - D), np.linalg.norm(Pr - D), np.linalg.norm(D)
        rank_ok += int(r == ref["rank"])
        # the reference's own truncation error is the bar (absolute threshold)
        gate_ok += int(eg <= 1.01 * er + slack * nd)
        e2_gpu += eg * eg
        e2_ref += er * er
        d2 += nd * nd
        worst_tile = max(worst_tile, eg / nd)
        worst_tile_ref = max(worst_tile_ref, er / nd)
        worst_oracle = max(worst_oracle, O.rel_fro(P, Pr))
    return {"sample": int(len(picks)), "rank_equal_to_oracle": int(rank_ok),
            "within_oracle_error": int(gate_ok),
            "panel_rel_fro_err_vs_dense": float(np.sqrt(e2_gpu / d2)),
            "oracle_panel_rel_fro_err_vs_dense": float(np.sqrt(e2_ref / d2)),
            "max_tile_rel_fro_err_vs_dense": worst_tile,
            "oracle_max_tile_rel_fro_err_vs_dense": worst_tile_ref,
            "max_rel_fro_diff_vs_oracle": worst_oracle,
            "note": "per-tile errors above acc come from the reference's absolute threshold on "
                    "tiles whose entries are themselves near acc; the oracle shows the same"}


def _lr_norm(X, Y) -> float:
    """||X Y^T||_F without forming the product: QR of both factors, then the
    small core (backward stable, so a difference far below the terms'
    magnitude is still resolved to about eps times that magnitude)."""
    import numpy as np

    if X.shape[1] == 0:
        return 0.0
    rx = np.linalg.qr(X, mode="r")
    ry = np.linalg.qr(Y, mode="r")
    return float(np.linalg.norm(rx @ ry.T))


def _accuracy_worker(args):
    """Oracle check of a chunk of updates (spawned process, one BLAS thread):
    the oracle's LAPACK restatement of the reference on the same inputs, and
    the exact update D = C - A B^T in low-rank form.  Returns per update
    (index, oracle rank, ||P - P_oracle||, ||P_oracle||, ||P - D||,
    ||P_oracle - D||, ||D||), P being the GPU's product."""
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    sys.path.insert(0, ROOT)
    import numpy as np

    from oracle import oracle as O

    folder, items, nb, acc, maxrk = args
    U = np.load(os.path.join(folder, "U.npy"), mmap_mode="r")
    V = np.load(os.path.join(folder, "V.npy"), mmap_mode="r")
    off = np.load(os.path.join(folder, "off.npy"))
    gU_all = np.load(os.path.join(folder, "gU.npy"), mmap_mode="r")
    gV_all = np.load(os.path.join(folder, "gV.npy"), mmap_mode="r")
    goff = np.load(os.path.join(folder, "goff.npy"))
    port = O.Port()
    port.set_threads(1)

    def fac(s_):
        o0, o1 = int(off[s_]), int(off[s_ + 1])
        r = (o1 - o0) // nb
        return (np.asfortranarray(U[o0:o1].reshape(r, nb).T),
                np.asfortranarray(V[o0:o1].reshape(r, nb).T), r)

    out = []
    for u, sa, sb, sc in items:
        AU, AV, a = fac(sa)
        BU, BV, b = fac(sb)
        CU, CV, c = fac(sc)
        o0, o1 = int(goff[u]), int(goff[u + 1])
        r = (o1 - o0) // nb
        gU = np.asarray(gU_all[o0:o1]).reshape(r, nb).T
        gV = np.asarray(gV_all[o0:o1]).reshape(r, nb).T
        ref = port.gemm(nb, -1.0, AU, AV, a, BU, BV, b, 1.0, CU, CV, c, maxrk=maxrk, acc=acc,
                        variant=2)
        rU, rV = ref["CU"], ref["CV"]
        AF = AU @ (AV.T @ BV)                          # D = [CU | AF] [CV | -BU]^T
        d_or = _lr_norm(np.hstack([gU, rU]), np.hstack([gV, -rV]))
        n_or = _lr_norm(rU, rV)
        eg = _lr_norm(np.hstack([gU, CU, AF]), np.hstack([gV, -CV, BU]))
        er = _lr_norm(np.hstack([rU, CU, AF]), np.hstack([rV, -CV, BU]))
        nd = _lr_norm(np.hstack([CU, AF]), np.hstack([CV, -BU]))
        nin = _lr_norm(CU, CV) + _lr_norm(AF, BU)     # ||C|| + ||A B^T||
        out.append((u, int(ref["rank"]), d_or, n_or, eg, er, nd, nin))
    return out


def accuracy_all(panel, updates, ranks, out_U, out_V, out_off, acc=None, slack=1e-14,
                 slack_of_inputs=False):
    """Every update of the step against the oracle (rank, product) and against
    the exact dense update, on all host cores.  The gate per update is the
    reference's own truncation error: ||P - D|| <= 1.01 ||P_oracle - D|| +
    slack ||D|| (`slack` 1e-14 for FP64 paths).  With FP32 arithmetic the
    rounding scales with the inputs, not with a result that cancels, so
    `slack_of_inputs` takes slack (||C|| + ||A B^T||) instead, plus FP32's
    absolute floor nb * FLT_MIN (far-field tiles of the panel have norms near
    1e-42, where FP32 values are subnormal)."""
    import multiprocessing as mp

    import numpy as np
    import torch

    nb = panel.nb
    acc = panel.acc if acc is None else acc
    n = len(updates)
    goff = np.zeros(n + 1, dtype=np.int64)
    goff[1:] = np.cumsum(np.asarray(ranks, dtype=np.int64) * nb)
    segs_U = [out_U[int(out_off[u]):int(out_off[u]) + nb * int(ranks[u])] for u in range(n)]
    segs_V = [out_V[int(out_off[u]):int(out_off[u]) + nb * int(ranks[u])] for u in range(n)]
    gU = torch.cat(segs_U).double().cpu().numpy()
    gV = torch.cat(segs_V).double().cpu().numpy()
    items = [(u, panel.index[(i, 0)], panel.index[(j, 0)], panel.index[(i, j)])
             for u, (i, j) in enumerate(updates)]
    cores = os.cpu_count() or 1
    t0 = time.time()
    with tempfile.TemporaryDirectory() as folder:
        np.save(os.path.join(folder, "U.npy"), panel.U.double().cpu().numpy())
        np.save(os.path.join(folder, "V.npy"), panel.V.double().cpu().numpy())
        np.save(os.path.join(folder, "off.npy"), panel.offset)
        np.save(os.path.join(folder, "gU.npy"), gU)
        np.save(os.path.join(folder, "gV.npy"), gV)
        np.save(os.path.join(folder, "goff.npy"), goff)
        os.environ.update(OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")
        chunks = [c for c in (items[w::cores] for w in range(cores)) if c]
        with mp.get_context("spawn").Pool(len(chunks)) as pool:
            res = pool.map(_accuracy_worker, [(folder, ch, nb, acc, panel.maxrank)
                                              for ch in chunks])
    rows = sorted(r for part in res for r in part)
    rk_ref = np.array([r[1] for r in rows])
    d_or, n_or, eg, er, nd, nin = (np.array([r[q] for r in rows]) for q in range(2, 8))
    rank_ok = int((rk_ref == np.asarray(ranks)).sum())
    # FP32 arithmetic also has an absolute floor: below its smallest normal
    # number (1.2e-38) values are subnormal and lose relative precision
    floor = np.finfo(np.float32).tiny * nb if slack_of_inputs else 0.0
    gate = eg <= 1.01 * er + slack * (nin if slack_of_inputs else nd) + floor
    rel_or = d_or / np.maximum(n_or, 1e-300)
    return {"checked": n, "rank_equal_to_oracle": rank_ok, "within_oracle_error": int(gate.sum()),
            "gate": f"||P - D|| <= 1.01 ||P_oracle - D|| + {slack:g} "
                    + ("(||C|| + ||A B^T||) + nb * FLT_MIN" if slack_of_inputs else "||D||"),
            "panel_rel_fro_err_vs_dense": float(np.sqrt((eg ** 2).sum() / (nd ** 2).sum())),
            "oracle_panel_rel_fro_err_vs_dense": float(np.sqrt((er ** 2).sum() / (nd ** 2).sum())),
            "max_tile_rel_fro_err_vs_dense": float((eg / nd).max()),
            "oracle_max_tile_rel_fro_err_vs_dense": float((er / nd).max()),
            "max_rel_fro_diff_vs_oracle": float(rel_or.max()),
            "check_s": round(time.time() - t0, 1), "cores": cores,
            "how": "every update of the step: the oracle (LAPACK restatement of the reference) "
                   "on the same inputs, and the exact update C - A B^T, norms of the low-rank "
                   "differences by QR of the stacked factors (no dense product formed)",
            "note": "per-tile errors above acc come from the reference's absolute threshold on "
                    "tiles whose entries are themselves near acc; the oracle shows the same"}


def config1_call(hc, reps=40, warmup=5):
    """One plain HCORE_dgemm call on host arrays, as a HiCMA tile codelet makes
    it (src/compute/hcore_dgemm.c:703; call pattern of the reference's test,
    testing/testing_dgemm.c:347-359): nb = 512, A, B, C each U diag(sigma) V^T
    with Haar 512 x 32 factors and sigma_i = 10^(-8i/32), ranks 32, acc 1e-8,
    maxrk 64, C += A B^T.  Each call is timed on the host clock around the C
    call: host->device copies, the four phases, the copy back and the sync.
    The same call of the oracle (the reference's LAPACK sequence restated) is
    timed on one host core beside it, and its rank and product are the
    check."""
    import ctypes as C

    import numpy as np

    from oracle import oracle as O

    L = hc.lib()
    rng = np.random.default_rng(512)
    M, k0, maxrk, acc = 512, 32, 64, 1e-8
    AU, AV = O.graded_lowrank(rng, M, k0)
    BU, BV = O.graded_lowrank(rng, M, k0)
    CU, CV = O.graded_lowrank(rng, M, k0)
    CU0 = np.zeros((M, maxrk), order="F")
    CV0 = np.zeros((M, maxrk), order="F")
    CU0[:, :k0], CV0[:, :k0] = CU, CV
    CUw, CVw = CU0.copy(order="F"), CV0.copy(order="F")
    ra, rb, rc = (np.array([float(k0)]) for _ in range(3))
    fc = hc.FlopCounter()
    dp = C.POINTER(C.c_double)
    pt = lambda x: x.ctypes.data_as(dp)  # noqa: E731
    times = []
    for it in range(warmup + reps):
        np.copyto(CUw, CU0)
        np.copyto(CVw, CV0)
        rc[0] = float(k0)
        t0 = time.perf_counter()
        L.HCORE_dgemm(111, 112, M, M, 1.0, pt(AU), pt(AV), pt(ra), M, pt(BU), pt(BV), pt(rb), M,
                      1.0, pt(CUw), pt(CVw), pt(rc), M, 0, maxrk, acc, None, C.byref(fc))
        t1 = time.perf_counter()
        if it >= warmup:
            times.append((t1 - t0) * 1e3)
    r = int(rc[0])
    port = O.Port()
    port.set_threads(1)
    ptimes = []
    for it in range(3 + 10):
        t0 = time.perf_counter()
        ref = port.gemm(M, 1.0, AU, AV, k0, BU, BV, k0, 1.0, CU, CV, k0, maxrk=maxrk, acc=acc)
        if it >= 3:
            ptimes.append((time.perf_counter() - t0) * 1e3)
    diff = O.rel_fro(CUw[:, :r] @ CVw[:, :r].T, ref["CU"] @ ref["CV"].T)
    med = statistics.median(times)
    # where the call's time goes: the same update as a one-task plan with the
    # drop-in's launch shape, its four phases timed with CUDA events
    import torch

    from hcore_gb300 import devmem

    dv = [devmem.to_device(x) for x in (AU, AV, BU, BV, CU, CV)]
    oU, oV = (torch.zeros((maxrk, M), dtype=torch.float64, device="cuda") for _ in range(2))
    task = hc.LrTask(M=M, a=k0, b=k0, c=k0, rk=0, maxrk=maxrk, ld_newv=maxrk, storage_maxrank=0,
                     alpha=1.0, beta=1.0, acc=acc, AU=dv[0].data_ptr(), AV=dv[1].data_ptr(),
                     lda=M, BU=dv[2].data_ptr(), BV=dv[3].data_ptr(), ldb=M, Bdense=None,
                     CU=dv[4].data_ptr(), CV=dv[5].data_ptr(), ldc=M, CUo=oU.data_ptr(),
                     CVo=oV.data_ptr(), ldco=M)
    one = hc.Batch([task], tuning=hc.make_tuning(stream_groups=1, svd_lanes=[4, 4, 4], qr_warps=8))
    st = torch.cuda.current_stream()
    ph = {"stack": 1, "qr": 2, "svd": 4, "rebuild": 8}
    acc_ms = {nm: [] for nm in ph}
    for it in range(8):
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        torch.cuda.synchronize()
        evs[0].record(st)
        for q, bit in enumerate(ph.values()):
            one.execute_phases(bit, st.cuda_stream)
            evs[q + 1].record(st)
        torch.cuda.synchronize()
        if it >= 3:
            for q, nm in enumerate(ph):
                acc_ms[nm].append(evs[q].elapsed_time(evs[q + 1]))
    one.close()
    phases = {nm: round(statistics.median(v), 4) for nm, v in acc_ms.items()}
    # the SVD phase of this one update against the lanes per column pair
    svd_by_lanes = {}
    for g in (2, 4, 8, 16):
        one = hc.Batch([task], tuning=hc.make_tuning(stream_groups=1, svd_lanes=[g, g, g],
                                                     qr_warps=8))
        ts = []
        for it in range(6):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            one.execute_phases(3, st.cuda_stream)
            e0.record(st)
            one.execute_phases(4, st.cuda_stream)
            e1.record(st)
            torch.cuda.synchronize()
            if it >= 2:
                ts.append(e0.elapsed_time(e1))
        one.close()
        svd_by_lanes[g] = round(statistics.median(ts), 4)
    return {"ms_per_call": med, "ms_min": min(times), "calls_per_s": 1e3 / med, "calls": reps,
            "rank": r, "oracle_rank": int(ref["rank"]), "rel_fro_diff_vs_oracle": diff,
            "phases_ms": phases,
            "svd_ms_by_lanes_per_pair": svd_by_lanes,
            "phases_how": "the same update as a one-task plan (device pointers, the drop-in's "
                          "launch shape), phases timed back to back with CUDA events",
            "cpu_1core_ms_per_call": statistics.median(ptimes),
            "cpu_1core_kind": "port (the oracle's LAPACK restatement of the reference, one "
                              "host core, one OpenBLAS thread)",
            "reference_1core_ms_per_call_x86": 2.51,
            "reference_1core_note": "the reference library itself on one x86 core (Xeon, "
                                    "2.7 GHz, OpenBLAS, one thread), measured when the "
                                    "workload was specified; not re-timed on this host",
            "how": "HCORE_dgemm drop-in on host arrays, median over calls after warm-up, "
                   "host clock around the call (copies, kernels and the sync included)",
            "config": "nb 512, ranks 32/32/32, sigma_i = 10^(-8i/32), acc 1e-8, maxrk 64"}


def e2e_pinned(hc, panel, updates, stream, dev, args, tuning=None):
    """The same workload through the C ABI with every factor in pinned HOST
    memory: each execute copies the unique input tiles host->device (the
    plan's HCORE_GPU_STAGE_INPUTS segments: a panel tile shared by many
    updates crosses the link once) and the rebuild kernel writes the new
    factors straight into the host output buffers.  All transfers are inside
    the timed region."""
    import numpy as np
    import torch

    n = len(updates)
    nb, maxrank = panel.nb, panel.maxrank
    out_off = np.arange(n + 1, dtype=np.int64) * nb * maxrank
    host = {"U": panel.U.cpu().pin_memory(), "V": panel.V.cpu().pin_memory(),
            "oU": torch.empty(int(out_off[-1]) + 1, dtype=torch.float64).pin_memory(),
            "oV": torch.empty(int(out_off[-1]) + 1, dtype=torch.float64).pin_memory()}
    tasks = build_tasks(hc, panel, updates, None, None, out_off, host=host)
    batch = hc.Batch(tasks, flags=hc.STAGE_INPUTS, tuning=tuning)
    batch.execute(stream.cuda_stream)
    ranks, status = batch.results(stream.cuda_stream)
    # the execute (its host->device copies included) captured once, replayed per step
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream(dev)
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        with torch.cuda.graph(graph, stream=side):
            batch.execute(side.cuda_stream)
    stream.wait_stream(side)
    for _ in range(max(args.warmup, 1)):
        graph.replay()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = max(args.steps // 2, 1)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(steps):
        graph.replay()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / steps
    out_bytes = int(sum(2 * nb * int(r) * 8 for r in ranks))
    staged, zero_copy = batch.staged_bytes, batch.zero_copy_bytes
    batch.close()
    return {"value": n / (ms / 1e3), "unit": "updates/s", "h2d_bytes_per_step": int(staged + zero_copy),
            "d2h_bytes_per_step": out_bytes, "ms_per_step": ms,
            "h2d_copied_bytes": int(staged), "h2d_read_in_place_bytes": int(zero_copy),
            "how": "plan over pinned host factors (HCORE_GPU_STAGE_INPUTS), its execute captured "
                   "in a CUDA graph and replayed per step: panel tiles shared by many updates "
                   "copied host->device each step, each update's own C tile read in place by "
                   "the stack kernel over NVLink-C2C, new factors written to host memory by the "
                   "rebuild kernel",
            "all_ok": bool((status == 0).all())}


# ---------------------------------------------------------------------------
# CPU side: the reference algorithm (oracle/, LAPACK restatement)
# ---------------------------------------------------------------------------

def _cpu_worker(args):
    """One host core's share of the CPU baseline: the oracle's restatement of
    the reference over the share's updates, the loop itself in C
    (port_dgemm_list), repeated until the time bound."""
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    sys.path.insert(0, ROOT)
    import numpy as np

    from oracle import oracle as O

    folder, items, nb, acc, maxrk, deadline = args
    U = np.load(os.path.join(folder, "U.npy"), mmap_mode="r")
    V = np.load(os.path.join(folder, "V.npy"), mmap_mode="r")
    off = np.load(os.path.join(folder, "off.npy"))
    port = O.Port()
    port.set_threads(1)
    sa, sb, sc = (np.array([it[q] for it in items], dtype=np.int32) for q in range(3))
    done = 0
    t0 = time.time()
    while True:
        bad = port.gemm_list(nb, U, V, off, sa, sb, sc, alpha=-1.0, beta=1.0, maxrk=maxrk,
                             acc=acc, variant=2)
        if bad:
            raise RuntimeError(f"{bad} updates failed in the CPU baseline")
        done += len(items)
        if deadline <= 0 or time.time() - t0 > deadline:
            return done, time.time() - t0


def cpu_run(panel, updates, seconds):
    """Time the reference algorithm over the update list on all host cores
    (one single-threaded process per core, factors memory-mapped from a
    scratch folder); returns (updates/s, cores, updates done)."""
    import multiprocessing as mp
    import tempfile

    import numpy as np

    cores = os.cpu_count() or 1
    slots = [(panel.index[(i, 0)], panel.index[(j, 0)], panel.index[(i, j)]) for i, j in updates]
    with tempfile.TemporaryDirectory() as folder:
        np.save(os.path.join(folder, "U.npy"), panel.U.cpu().numpy())
        np.save(os.path.join(folder, "V.npy"), panel.V.cpu().numpy())
        np.save(os.path.join(folder, "off.npy"), panel.offset)
        os.environ.update(OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")
        ctx = mp.get_context("spawn")
        chunks = [slots[w::cores] for w in range(cores)]
        chunks = [c for c in chunks if c]
        with ctx.Pool(len(chunks)) as pool:
            pool.map(_cpu_worker, [(folder, ch[:1], panel.nb, panel.acc, panel.maxrank, 0)
                                   for ch in chunks])
            t0 = time.time()
            res = pool.map(_cpu_worker, [(folder, ch, panel.nb, panel.acc, panel.maxrank, seconds)
                                         for ch in chunks])
            wall = time.time() - t0
    done = sum(d for d, _ in res)
    return done / wall, len(chunks), done, wall


def cpu_baseline(panel, updates, seconds):
    v, cores, done, wall = cpu_run(panel, updates, seconds)
    return {"value": v, "unit": "updates/s", "cores": cores, "kind": "port",
            "sample": f"{done} updates in {wall:.1f} s, the step's {len(updates)} updates dealt "
                      f"round-robin to one single-threaded process per core and repeated until "
                      f"the time bound, OpenBLAS LAPACK (oracle/hcore_port.c, the loop over "
                      f"updates in C)"}


def run_reference(args):
    import torch

    rank, world, local = dist_init()
    if rank != 0:
        barrier(world)
        return
    from hcore_gb300 import panel as pnl

    dev = "cuda" if torch.cuda.is_available() else "cpu"
    panel = pnl.build_panel(device=dev, max_updates=args.max_updates)
    updates = panel.updates
    vals = []
    per_step = max(args.cpu_seconds / max(args.steps, 1), 2.0)
    for s in range(args.warmup + args.steps):
        v, cores, done, _ = cpu_run(panel, updates, per_step)
        if s >= args.warmup:
            vals.append(v)
    v = statistics.median(vals)
    kind = "port"
    line = {"metric": METRIC, "value": v, "unit": "updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": len(updates) / v * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": dict(WORKLOAD, updates_per_step=len(updates), parallelism="cpu"),
            "cpu_baseline": {"value": v, "unit": "updates/s", "cores": cores, "kind": kind,
                             "sample": f"bounded sample per step (~{per_step:.0f} s) of the "
                                       f"{len(updates)}-update panel, all host cores; the "
                                       "oracle's restatement of the reference (the same LAPACK "
                                       "calls in the same order) runs, since the reference "
                                       "library is built only where its sources are"},
            "e2e": {"value": v, "unit": "updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    sys.stdout.flush()
    barrier(world)


def timed_plan(hc, batch, torch, dev, stream, warmup, steps):
    """Graph-capture one plan's execute and time `steps` replays (ms/step)."""
    batch.execute(stream.cuda_stream)
    torch.cuda.synchronize(dev)
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream(dev)
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        with torch.cuda.graph(graph, stream=side):
            batch.execute(side.cuda_stream)
    stream.wait_stream(side)
    for _ in range(warmup):
        graph.replay()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        graph.replay()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    return e0.elapsed_time(e1) / steps


PRECISION_RUNS = ((1e-4, "F64", "MIXED_FACTORS", "fp64 QR/SVD, fp32 factors+rebuild"),
                  (1e-6, "F64", "MIXED_FACTORS", "fp64 QR/SVD, fp32 factors+rebuild"),
                  (1e-8, "F64", None, "fp64"),
                  (1e-4, "F32", None, "fp32 end to end (HCORE_sgemm)"))


def precision_runs(hc, torch, panel, updates, dev, stream, warmup, steps):
    """The panel's updates at each accuracy of the sweep: FP32 factor products
    and rebuild at 1e-4 / 1e-6 (QR, SVD, truncation FP64), FP64 at 1e-8, and
    HCORE_sgemm semantics (FP32 end to end) at 1e-4.  Each run is graph-timed
    and every update is checked against the FP64 oracle at the same acc."""
    import numpy as np

    n, nb, maxrank = len(updates), panel.nb, panel.maxrank
    out_off = np.arange(n + 1, dtype=np.int64) * nb * maxrank
    runs = []
    for acc, prec_name, flag_name, label in PRECISION_RUNS:
        precision = getattr(hc, prec_name)
        flags = getattr(hc, flag_name) if flag_name else 0
        dt = torch.float64 if precision == hc.F64 else torch.float32
        src = (panel.U, panel.V) if dt == torch.float64 else (panel.U.float(), panel.V.float())
        oU = torch.empty(int(out_off[-1]) + 1, dtype=dt, device=dev)
        oV = torch.empty_like(oU)
        tasks = build_tasks(hc, panel, updates, oU, oV, out_off, acc=acc, src=src)
        batch = hc.Batch(tasks, precision=precision, flags=flags)
        ms = timed_plan(hc, batch, torch, dev, stream, warmup, steps)
        ranks, status = batch.results(stream.cuda_stream)
        fp64 = precision == hc.F64 and not flags
        accs = accuracy_all(panel, updates, ranks, oU, oV, out_off, acc=acc,
                            slack=1e-14 if fp64 else 2e-6, slack_of_inputs=not fp64)
        runs.append({"acc": acc, "arithmetic": label, "updates_per_s": n / (ms / 1e3),
                     "ms_per_step": ms, "mean_rank": float(np.mean(ranks)),
                     "all_ok": bool((status == 0).all()), "accuracy": accs})
        batch.close()
        del oU, oV, src
    return runs


def run_precision(args):
    """Precision sweep on the panel's tiles (precision_runs), one JSON line."""
    import torch

    import hcore_gb300 as hc
    from hcore_gb300 import build as hbuild

    rank, world, local = dist_init()
    if not os.path.exists(hbuild.LIB):
        hbuild.build()
    hc.lib()
    dev = torch.device("cuda", local)
    panel, _ = panel_for_rank(args, rank, world, dev)
    updates = panel.updates
    stream = torch.cuda.current_stream(dev)
    runs = precision_runs(hc, torch, panel, updates, dev, stream, args.warmup, args.steps)
    if rank == 0:
        line = {"metric": "TLR-GEMM updates/s per accuracy (precision sweep)", "value": runs[0]["updates_per_s"],
                "unit": "updates/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64/f32",
                "data": "synthetic (the panel workload's tiles)",
                "config": dict(WORKLOAD, workload="precision sweep on the panel-0 Schur updates",
                               updates_per_step=len(updates)), "runs": runs}
        print(json.dumps(line))
        sys.stdout.flush()
    barrier(world)


def run_dense(args):
    """Batched dense-C updates (HCORE_dsyrk / HCORE_dgemmcd semantics): the 64
    diagonal 1024 x 1024 covariance tiles each take 63 syrk updates
    D_i -= U (V^T V) U^T from the panel's low-rank tiles (ranks 7..35), and 62
    dense off-diagonal tiles C_{i,i-1} take a gemmcd update
    C -= Au (Av^T Bv) Bu^T, all in one plan.  Every step applies all tasks
    again to the current tiles."""
    import numpy as np
    import torch

    import hcore_gb300 as hc
    from hcore_gb300 import build as hbuild
    from hcore_gb300 import panel as pnl
    from oracle import oracle as O

    rank, world, local = dist_init()
    if not os.path.exists(hbuild.LIB):
        hbuild.build()
    hc.lib()
    dev = torch.device("cuda", local)
    panel = pnl.build_panel(device=str(dev), max_updates=1)   # the 63 panel tiles
    stream = torch.cuda.current_stream(dev)
    line = dense_run(hc, torch, panel, dev, stream, args.warmup, args.steps, world)
    if rank == 0:
        print(json.dumps(line))
        sys.stdout.flush()
    barrier(world)


def dense_run(hc, torch, panel, dev, stream, warmup, steps, world=1):
    """The dense-C step on the panel's 63 low-rank tiles (see run_dense);
    returns its JSON line."""
    import numpy as np

    from hcore_gb300 import panel as pnl
    from oracle import oracle as O

    nb, T = panel.nb, panel.ntiles
    P = torch.from_numpy(pnl.morton_points(WORKLOAD["points"], 2, 0)).to(dev)

    def ktile(i, j):
        X, Y = P[i * nb:(i + 1) * nb], P[j * nb:(j + 1) * nb]
        d2 = (X * X).sum(1)[:, None] + (Y * Y).sum(1)[None, :] - 2.0 * X @ Y.T
        return torch.exp(-torch.clamp(d2, min=0.0) / 0.01)

    # column-major tiles: tensor (nb, nb) row-major = transposed storage
    diag = [ktile(i, i).T.contiguous() for i in range(T)]
    offd = [ktile(i, i - 1).T.contiguous() for i in range(2, T)]
    diag0 = [d.clone() for d in diag]
    offd0 = [d.clone() for d in offd]

    def fac(j):
        s_ = panel.index[(j, 0)]
        o = int(panel.offset[s_])
        return panel.U.data_ptr() + 8 * o, panel.V.data_ptr() + 8 * o, int(panel.rank[s_])

    # flops: the reference's model (three GEMMs per task over the full tile)
    # and what the kernels execute (a syrk skips the 64 x 64 blocks strictly
    # above the diagonal, whose result is zero)
    tpd = (nb + 63) // 64
    lower = tpd * (tpd + 1) / 2 / (tpd * tpd)
    tasks, flops, flops_exec = [], 0, 0
    for i in range(T):
        for j in range(1, T):
            u, v, r = fac(j)
            tasks.append(hc.DenseTask(kind=0, M=nb, a=r, b=0, alpha=-1.0, Au=u, Av=v, lda=nb,
                                      Bu=None, Bv=None, ldb=nb, CD=diag[i].data_ptr(), ldcd=nb))
            flops += 2 * r * r * nb + 2 * nb * r * r + 2 * nb * nb * r
            flops_exec += 2 * r * r * nb + 2 * nb * r * r + 2 * nb * nb * r * lower
    for t, i in enumerate(range(2, T)):
        ua, va, ra = fac(i)
        ub, vb, rb = fac(i - 1)
        tasks.append(hc.DenseTask(kind=1, M=nb, a=ra, b=rb, alpha=-1.0, Au=ua, Av=va, lda=nb,
                                  Bu=ub, Bv=vb, ldb=nb, CD=offd[t].data_ptr(), ldcd=nb))
        f = 2 * ra * rb * nb + 2 * nb * min(ra, rb) * max(ra, rb) + 2 * nb * nb * min(ra, rb)
        flops += f
        flops_exec += f
    plan = hc.DensePlan(tasks)
    # correctness on a sample: tiles 0 and 63 and one off-diagonal tile after one step
    plan.execute(stream.cuda_stream)
    torch.cuda.synchronize(dev)
    port = O.Port()
    errs = []
    for i in (0, T - 1):
        ref = np.asfortranarray(diag0[i].cpu().numpy().T)
        for j in range(1, T):
            s_ = panel.index[(j, 0)]
            o0, o1 = int(panel.offset[s_]), int(panel.offset[s_ + 1])
            r = int(panel.rank[s_])
            U_ = np.asfortranarray(panel.U[o0:o1].cpu().numpy().reshape(r, nb).T)
            V_ = np.asfortranarray(panel.V[o0:o1].cpu().numpy().reshape(r, nb).T)
            ref, _ = port.dsyrk(nb, r, -1.0, U_, V_, ref)
        got = diag[i].cpu().numpy().T
        errs.append(float(np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-300)))
    # timed steps
    for _ in range(warmup):
        plan.execute(stream.cuda_stream)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        plan.execute(stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / steps
    peak = fp64_peak(hc.lib(), torch, dev)
    tiles_bytes = (len(diag) + len(offd)) * nb * nb * 8 * 2
    line = {"metric": "dense-C tile updates/s (HCORE_dsyrk + HCORE_dgemmcd batched)",
            "value": len(tasks) / (ms / 1e3), "unit": "tile-updates/s", "n_gpus": world,
            "steps": steps, "warmup": warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (covariance tiles of the panel workload)",
            "config": {"workload": "64 diagonal 1024^2 tiles x 63 syrk updates + 62 gemmcd updates",
                       "syrk_tasks": T * (T - 1), "gemmcd_tasks": len(offd), "nb": nb},
            "gflops_model": flops / (ms / 1e3) / 1e9,
            "roofline": {"bound": "fp64", "achieved": flops_exec / (ms / 1e3) / 1e12, "peak": peak,
                         "unit": "TFLOP/s", "frac": flops_exec / (ms / 1e3) / 1e12 / peak,
                         "flops_basis": "flops the kernels execute: the reference's three GEMMs "
                                        "per task, syrk tiles without the 64x64 blocks strictly "
                                        "above the diagonal (gflops_model counts full tiles)",
                         "tile_bytes_per_step": tiles_bytes},
            "accuracy": {"max_rel_err_vs_oracle_sequential_dsyrk": max(errs),
                         "tiles_checked": [0, T - 1]}}
    plan.close()
    del diag, offd, diag0, offd0
    return line


SWEEPS = dict(workload="learned rank predictor: 16 panel sweeps of a TLR Cholesky factorization",
          points=262144, dim=3, nb=2048, tiles_per_dim=128, block_tiles=64,
          kernel="exp(-|x-y|/0.1) (Matern 1/2)", nugget=1e-2, acc=1e-7, maxrank=256, maxrk=512,
          sweeps=16,
          tile_compression="relative sigma >= 1e-7*sigma_max, capped at maxrank",
          update_truncation="absolute sigma_i < acc (reference rule); new rank above the "
                            "tile storage maxrank (256) reported as STORAGE and the tile kept",
          sweep="POTRF of the dense diagonal tile and TRSM of the panel's V factors (library "
                "kernels, outside the compared step), HCORE_dsyrk of the diagonal tiles (batched dense plan), "
                "HCORE_dgemm Schur updates (batched plan: the timed, compared step)",
          region="leading 64 x 64 tiles (the first 131072 of the 262144 Morton-sorted points); "
                 "their factorization does not depend on the rest of the matrix")


def _time_execute(batch, torch, stream):
    """Warm execute, then the plan's execute captured in a CUDA graph and one
    timed replay (ms), as the panel plan is timed."""
    batch.execute(stream.cuda_stream)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        with torch.cuda.graph(graph, stream=side):
            batch.execute(side.cuda_stream)
    stream.wait_stream(side)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    graph.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def _panel_logs(hc, torch, dev, pnl, P):
    """Recompression logs of the panel workload (2D squared-exponential,
    nb 1024): features and new ranks of its Schur updates at acc 1e-8 (FP64),
    1e-6 and 1e-4 (FP32 factor products) and 1e-4 (FP32 end to end)."""
    import numpy as np

    panel = pnl.build_panel(device=str(dev))
    nb = panel.nb
    cen, diam = P.cluster_geometry(pnl.morton_points(WORKLOAD["points"], 2, 0), nb)
    norm = [float(panel.V[int(panel.offset[s]):int(panel.offset[s + 1])].norm()) for s in range(len(panel.tiles))]
    ups = panel.updates
    sa = [panel.index[(i, 0)] for i, j in ups]
    sb = [panel.index[(j, 0)] for i, j in ups]
    sc = [panel.index[(i, j)] for i, j in ups]
    out_off = np.arange(len(ups) + 1, dtype=np.int64) * nb * panel.maxrank
    F, R = [], []
    for acc, prec, flags in ((1e-8, hc.F64, 0), (1e-6, hc.F64, hc.MIXED_FACTORS),
                             (1e-4, hc.F64, hc.MIXED_FACTORS), (1e-4, hc.F32, 0)):
        dt = torch.float64 if prec == hc.F64 else torch.float32
        src = (panel.U, panel.V) if prec == hc.F64 else (panel.U.float(), panel.V.float())
        oU = torch.empty(int(out_off[-1]) + 1, dtype=dt, device=dev)
        oV = torch.empty_like(oU)
        b = hc.Batch(build_tasks(hc, panel, ups, oU, oV, out_off, acc=acc, src=src),
                     precision=prec, flags=flags)
        b.execute()
        r, st = b.results()
        b.close()
        ok = st == 0
        f = P.features(panel.rank[sa], panel.rank[sb], panel.rank[sc], [norm[x] for x in sa],
                       [norm[x] for x in sb], [norm[x] for x in sc],
                       [np.linalg.norm(cen[i] - cen[j]) for i, j in ups],
                       [(diam[i] + diam[j]) / 2 for i, j in ups], acc)
        F.append(f[ok])
        R.append(r[ok])
        del oU, oV
    return np.concatenate(F), np.concatenate(R)


def _compact(store, torch, keys=None):
    """Copy the listed tiles (default: all) into one fresh arena of exact
    ranks; arenas no tile refers to any more are released."""
    import numpy as np

    keys = list(store.tiles) if keys is None else list(keys)
    if not keys:
        return
    ranks = np.array([store.tiles[t][3] for t in keys], dtype=np.int64)
    off = np.zeros(len(keys) + 1, dtype=np.int64)
    off[1:] = np.cumsum(ranks * store.nb)
    dev = next(iter(store.tiles.values()))[0].device
    U = torch.empty(int(off[-1]) + 1, dtype=torch.float64, device=dev)
    V = torch.empty_like(U)
    for q, t in enumerate(keys):
        u, v, o, r = store.tiles[t]
        n = r * store.nb
        U[int(off[q]):int(off[q]) + n] = u[o:o + n]
        V[int(off[q]):int(off[q]) + n] = v[o:o + n]
    for q, t in enumerate(keys):
        store.tiles[t] = (U, V, int(off[q]), int(ranks[q]))


def run_predictor(args):
    """Config 5: the learned rank predictor against pad-to-maxrank and the
    per-tile launch loop, in the first 16 panel sweeps of a TLR Cholesky
    factorization of a 3D exponential-kernel covariance matrix (nb 2048,
    maxrank 256, acc 1e-7).  Both batched arms run the same kernels, so
    every rank is the SVD's; the predictor only sizes the Schur updates'
    output slots (and the rebuild grid); updates above their predicted
    capacity are rebuilt from the workspace into exact-size slots.  The
    network is trained on the GPU (library kernels) on the panel workload's
    logs (2D, nb 1024, acc 1e-8 .. 1e-4), then fine-tuned after every sweep
    on the ranks this factorization produced so far."""
    import copy

    import numpy as np
    import torch

    import hcore_gb300 as hc
    from hcore_gb300 import build as hbuild
    from hcore_gb300 import panel as pnl
    from hcore_gb300 import predictor as P
    from oracle import oracle as O

    rank, world, local = dist_init()
    if not os.path.exists(hbuild.LIB):
        hbuild.build()
    hc.lib()
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    t0 = time.time()
    F2, R2 = _panel_logs(hc, torch, dev, pnl, P)
    t_logs = time.time() - t0

    nb, B, S = SWEEPS["nb"], SWEEPS["block_tiles"], SWEEPS["sweeps"]
    if args.sweep_shape:
        B, nb, S = (int(x) for x in args.sweep_shape.split(","))
    MAXR, MAXRK, ACC = SWEEPS["maxrank"], SWEEPS["maxrk"], SWEEPS["acc"]
    pts = pnl.morton_points(SWEEPS["points"], SWEEPS["dim"], 0)[:B * nb]
    t0 = time.time()
    tiles = [(i, j) for i in range(B) for j in range(i)]
    store0 = pnl.TileStore.build(pts, nb, tiles, "exp", 0.1, 1e-7, MAXR, seed=0, device=str(dev))
    Pd = torch.from_numpy(pts).to(dev)

    def dense_tile(i):   # column-major storage of the symmetric diagonal tile (+ nugget)
        X = Pd[i * nb:(i + 1) * nb]
        d2 = (X * X).sum(1)[:, None] + (X * X).sum(1)[None, :] - 2.0 * X @ X.T
        K = torch.exp(-torch.sqrt(torch.clamp(d2, min=0.0)) / 0.1)
        return (K + SWEEPS["nugget"] * torch.eye(nb, dtype=K.dtype, device=K.device)).contiguous()

    D0 = [dense_tile(i) for i in range(B)]
    t_tiles = time.time() - t0
    cen, diam = P.cluster_geometry(pts, nb)

    def ev():
        return torch.cuda.Event(enable_timing=True)

    def feats(store, ups, k):
        return P.features([store.tiles[(i, k)][3] for i, j in ups], [store.tiles[(j, k)][3] for i, j in ups],
                          [store.tiles[(i, j)][3] for i, j in ups], [store.norm[(i, k)] for i, j in ups],
                          [store.norm[(j, k)] for i, j in ups], [store.norm[(i, j)] for i, j in ups],
                          [np.linalg.norm(cen[i] - cen[j]) for i, j in ups],
                          [(diam[i] + diam[j]) / 2 for i, j in ups], ACC)

    def maker(store, ups, k):
        def make(u, storage, oU, oV):
            i, j = ups[u]
            au, av, a = store.ptrs((i, k))
            bu, bv, b = store.ptrs((j, k))
            cu, cv, c = store.ptrs((i, j))
            return hc.LrTask(M=nb, a=a, b=b, c=c, rk=0, maxrk=MAXRK, ld_newv=0,
                             storage_maxrank=storage, alpha=-1.0, beta=1.0, acc=ACC, AU=au, AV=av,
                             lda=nb, BU=bu, BV=bv, ldb=nb, Bdense=None, CU=cu, CV=cv, ldc=nb,
                             CUo=oU, CVo=oV, ldco=nb)
        return make

    def gemm_step(store, ups, k, caps, tuning):
        """The batched Schur updates of one sweep with output capacities caps:
        warm execute, timed execute, rebuild of capacity overflows (timed)."""
        n = len(ups)
        make = maker(store, ups, k)
        # memory torch no longer uses goes back to the driver before the
        # plan allocates its own workspace (large sweeps of the full matrix)
        torch.cuda.empty_cache()
        off = P.slot_offsets(caps, nb)
        oU = torch.empty(int(off[-1]) + 1, dtype=torch.float64, device=dev)
        oV = torch.empty_like(oU)
        tasks = [make(u, int(caps[u]), oU.data_ptr() + 8 * int(off[u]), oV.data_ptr() + 8 * int(off[u]))
                 for u in range(n)]
        b = hc.Batch(tasks, tuning=tuning)
        ms = _time_execute(b, torch, stream)
        r, st = b.results(stream.cuda_stream)
        where = {u: (oU, oV, int(off[u])) for u in range(n)}
        # STORAGE: above the predicted capacity (rebuilt at its rank) or above
        # the tiles' maxrank (rebuilt truncated to maxrank, as HCORE_dgemm
        # with rk = maxrank; the same updates in both arms)
        over = np.nonzero(st == 5)[0]
        n_over = int(((r[over] <= MAXR) & (caps[over] < MAXR)).sum())
        n_trunc = int((r[over] > MAXR).sum())
        arena = 2 * oU.numel() * 8
        ms_over = 0.0
        if len(over):
            off2 = P.slot_offsets(np.minimum(r[over], MAXR), nb)
            xU = torch.empty(int(off2[-1]) + 1, dtype=torch.float64, device=dev)
            xV = torch.empty_like(xU)
            e0, e1 = ev(), ev()
            e0.record(stream)
            b.rebuild(over, [xU.data_ptr() + 8 * int(off2[q]) for q in range(len(over))],
                      [xV.data_ptr() + 8 * int(off2[q]) for q in range(len(over))], [nb] * len(over),
                      max_rank=[MAXR] * len(over), stream=stream.cuda_stream)
            e1.record(stream)
            r, st = b.results(stream.cuda_stream)
            ms_over = e0.elapsed_time(e1)
            for q, u in enumerate(over):
                where[u] = (xU, xV, int(off2[q]))
            arena += 2 * xU.numel() * 8
        ws = b.workspace_bytes
        b.close()
        return ms, ms_over, r, st, where, n_over, n_trunc, arena, ws

    net = P.RankPredictor(seed=5)
    t0 = time.time()
    base_loss = net.fit(F2, R2, epochs=150, batch=256, lr=2e-3, seed=1)
    t_train = time.time() - t0
    policy0 = P.CapacityPolicy.fit(net.predict(F2), R2, target_overflow=0.02)
    net_state0 = net.state()

    arms, sample_out, extra = {}, {}, {}
    tuning = None
    for arm in ("pad", "predictor"):
        net.load(net_state0)
        policy = policy0
        store = copy.copy(store0)
        store.tiles, store.norm = dict(store0.tiles), dict(store0.norm)
        D = [d.clone() for d in D0]
        logF, logR = [F2], [R2]
        tot = dict(ms_gemm=0.0, ms_predict=0.0, ms_rebuild=0.0, ms_potrf_trsm=0.0, ms_syrk=0.0,
                   updates=0, ok=0, truncated=0, overflow=0, arena_bytes_max=0, arena_bytes_sum=0,
                   ws_bytes_max=0, per_sweep=[])
        for k in range(S):
            # HCORE_dpotrf + HCORE_dtrsm of panel k (the library's kernels):
            # D[k] = L L^T in place (D[k] holds the lower triangle, column-major),
            # then V <- L^-1 V for every tile (i, k), i > k, as one TRSM whose
            # right-hand sides are all the panel's V columns (copied first: the
            # factors may be shared with the other arm's starting store)
            e0, e1 = ev(), ev()
            e0.record(stream)
            info = hc.potrf_batched([hc.PotrfTask(uplo=ord("L"), n=nb, A=D[k].data_ptr(), lda=nb)],
                                    stream=stream.cuda_stream)
            if int(info[0]) != 0:
                raise SystemExit(f"POTRF of diagonal tile {k} failed (info {int(info[0])})")
            col = [(i, k) for i in range(k + 1, B)]
            if col:
                Vs = torch.cat([store.tiles[t][1][store.tiles[t][2]:store.tiles[t][2] + nb * store.tiles[t][3]]
                                .view(store.tiles[t][3], nb) for t in col], 0)
                hc.trsm_batched([hc.TrsmTask(side=141, uplo=122, trans=111, diag=131, M=nb,
                                             N=Vs.shape[0], alpha=1.0, A=D[k].data_ptr(), lda=nb,
                                             B=Vs.data_ptr(), ldb=nb)], stream=stream.cuda_stream)
                Us = torch.cat([store.tiles[t][0][store.tiles[t][2]:store.tiles[t][2] + nb * store.tiles[t][3]]
                                for t in col])
                Vflat = Vs.reshape(-1)
                o = 0
                for t in col:
                    r_ = store.tiles[t][3]
                    store.tiles[t] = (Us, Vflat, o, r_)
                    o += nb * r_
            e1.record(stream)
            torch.cuda.synchronize()
            tot["ms_potrf_trsm"] += e0.elapsed_time(e1)
            for t in col:
                U_, V_, o_, r_ = store.tiles[t]
                store.norm[t] = float(V_[o_:o_ + nb * r_].norm())
            # HCORE_dsyrk of the trailing diagonal tiles (batched dense plan)
            if col:
                dts = []
                for j in range(k + 1, B):
                    au, av, a = store.ptrs((j, k))
                    dts.append(hc.DenseTask(kind=0, M=nb, a=a, b=0, alpha=-1.0, Au=au, Av=av, lda=nb,
                                            Bu=None, Bv=None, ldb=nb, CD=D[j].data_ptr(), ldcd=nb))
                dp = hc.DensePlan(dts)
                e0, e1 = ev(), ev()
                e0.record(stream)
                dp.execute(stream.cuda_stream)
                e1.record(stream)
                torch.cuda.synchronize()
                tot["ms_syrk"] += e0.elapsed_time(e1)
                dp.close()
            # HCORE_dgemm Schur updates of the trailing low-rank tiles
            ups = [(i, j) for j in range(k + 1, B) for i in range(j + 1, B)]
            n = len(ups)
            if n == 0:
                continue
            F = feats(store, ups, k)
            ms_pred = 0.0
            if arm == "pad":
                caps = np.full(n, MAXR, dtype=np.int64)
            else:
                Xd = net._x(F)
                e0, e1 = ev(), ev()
                e0.record(stream)
                y = net.net.predict(Xd, stream=stream.cuda_stream)
                e1.record(stream)
                torch.cuda.synchronize()
                ms_pred = e0.elapsed_time(e1)
                caps = policy(P.rank_from_output(y.cpu().numpy()), MAXR)
            if tuning is None:
                # the plans' launch shapes: the library autotuner on sweep 0's batch
                # (set-up, outside the timed region; used by both arms and all sweeps)
                make_t = maker(store, ups, k)
                # at most 2000 evenly spread updates of the batch (the whole
                # 64-tile sweep; a sample of the 8001 of the full-size one)
                sub = sorted(set(np.linspace(0, n - 1, min(n, 2000)).astype(int).tolist()))
                tU = torch.empty(len(sub) * nb * MAXR + 1, dtype=torch.float64, device=dev)
                tV = torch.empty_like(tU)
                t0 = time.time()
                tuning, tuned_ms = hc.autotune(
                    [make_t(u, MAXR, tU.data_ptr() + 8 * q * nb * MAXR, tV.data_ptr() + 8 * q * nb * MAXR)
                     for q, u in enumerate(sub)], reps=1)
                extra["tuning"] = dict(tuning.as_dict(), autotune_s=round(time.time() - t0, 1),
                                       sample_updates=len(sub), sample_ms=round(tuned_ms, 1))
                del tU, tV
            ms, ms_over, r, st, where, nover, ntrunc, arena, ws = gemm_step(store, ups, k, caps, tuning)
            ok = st == 0
            if k == 0:
                samp = list(range(0, n, max(1, n // 24)))[:24]
                sample_out[arm] = {u: (where[u], int(r[u])) for u in samp if ok[u]}
                if arm == "pad":
                    # plain per-tile launch loop and the oracle, on sweep 0's inputs
                    make0 = maker(store, ups, 0)
                    per_ms = 0.0
                    for u in samp:
                        oU1 = torch.empty(nb * MAXR + 1, dtype=torch.float64, device=dev)
                        oV1 = torch.empty_like(oU1)
                        b1 = hc.Batch([make0(u, MAXR, oU1.data_ptr(), oV1.data_ptr())])
                        per_ms += _time_execute(b1, torch, stream)
                        b1.close()
                    extra["per_tile"] = {"updates_per_s": len(samp) / (per_ms / 1e3), "sample": len(samp)}
                    accs = []
                    for u in samp[:4]:
                        i, j = ups[u]
                        AU, AV = store.factors((i, 0))
                        BU, BV = store.factors((j, 0))
                        CU, CV = store.factors((i, j))
                        ref = O.Port().gemm(nb, -1.0, AU, AV, AU.shape[1], BU, BV, BU.shape[1], 1.0,
                                            CU, CV, CU.shape[1], maxrk=MAXRK, acc=ACC)
                        if not ok[u] or ref["status"] != 0:
                            continue
                        (U_, V_, o_), r_ = where[u], int(r[u])
                        Pg = (U_[o_:o_ + nb * r_].view(r_, nb).T @ V_[o_:o_ + nb * r_].view(r_, nb)).cpu().numpy()
                        accs.append(dict(rank=r_, oracle_rank=int(ref["rank"]),
                                         rel_fro_vs_oracle=float(O.rel_fro(Pg, ref["CU"] @ ref["CV"].T))))
                    extra["accuracy_vs_oracle"] = accs
            for u in np.nonzero(ok)[0]:
                U_, V_, o_ = where[u]
                store.tiles[ups[u]] = (U_, V_, o_, int(r[u]))
                store.norm[ups[u]] = float(V_[o_:o_ + nb * int(r[u])].norm())
            tot["ms_gemm"] += ms
            tot["ms_predict"] += ms_pred
            tot["ms_rebuild"] += ms_over
            tot["updates"] += n
            tot["ok"] += int(ok.sum())
            tot["truncated"] += ntrunc
            tot["overflow"] += nover
            tot["arena_bytes_max"] = max(tot["arena_bytes_max"], arena)
            tot["arena_bytes_sum"] += arena
            tot["ws_bytes_max"] = max(tot["ws_bytes_max"], ws)
            tot["per_sweep"].append(dict(k=k, updates=n, gemm_ms=round(ms + ms_over + ms_pred, 3),
                                         overflow=nover, truncated=ntrunc, mean_rank=round(float(r[ok].mean()), 2) if ok.any() else 0.0,
                                         max_rank=int(r[ok].max()) if ok.any() else 0,
                                         arena_gb=round(arena / 1e9, 3)))
            if arm == "predictor":
                # online: fine-tune on every rank produced so far (fixed standardisation)
                logF.append(F[ok])
                logR.append(r[ok])
                Xall = net._x(np.concatenate(logF))
                Tall = torch.from_numpy(P.rank_target(np.concatenate(logR))).cuda()
                net.net.train(Xall, Tall, epochs=8, batch=256, lr=1e-3, seed=100 + k)
                recent_F, recent_R = np.concatenate(logF[-2:]), np.concatenate(logR[-2:])
                policy = P.CapacityPolicy.fit(net.predict(recent_F), recent_R, target_overflow=0.02)
            del where
            _compact(store, torch)
        arms[arm] = tot
        del D

    # equal results: sampled sweep-0 products of both arms
    max_diff, same = 0.0, True
    for u, ((U_, V_, o), r) in sample_out["pad"].items():
        if u not in sample_out["predictor"]:
            same = False
            continue
        (U2, V2, o2), r2 = sample_out["predictor"][u]
        if r2 != r:
            same = False
            continue
        n_ = nb * r
        P1 = U_[o:o + n_].view(r, nb).T @ V_[o:o + n_].view(r, nb)
        P2 = U2[o2:o2 + n_].view(r, nb).T @ V2[o2:o2 + n_].view(r, nb)
        max_diff = max(max_diff, float((P1 - P2).norm() / P1.norm()))

    def gemm_ups(t):
        return t["ok"] / ((t["ms_gemm"] + t["ms_rebuild"] + t["ms_predict"]) / 1e3)

    pad, prd = arms["pad"], arms["predictor"]
    line = {"metric": "TLR Cholesky sweep Schur updates/s (3D kernel, nb 2048): predictor-sized vs pad-to-maxrank vs per-tile",
            "value": gemm_ups(prd), "unit": "updates/s", "n_gpus": world, "steps": 1,
            "warmup": 1, "ms_per_step": prd["ms_gemm"] + prd["ms_rebuild"] + prd["ms_predict"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded 3D points, tiles compressed on the host cores)",
            "config": dict(SWEEPS, block_tiles=B, nb=nb, sweeps=S,
                           region=(f"the whole matrix: {B} x {B} tiles, all {B * nb} points"
                                   if B * nb >= SWEEPS["points"] else
                                   f"leading {B} x {B} tiles (the first {B * nb} of the "
                                   f"{SWEEPS['points']} Morton-sorted points); their "
                                   "factorization does not depend on the rest of the matrix")),
            "pad_to_maxrank": {"updates_per_s": gemm_ups(pad),
                               **{k: v for k, v in pad.items() if k != "per_sweep"}},
            "predictor": {k: v for k, v in prd.items() if k != "per_sweep"},
            "per_sweep": {"pad": pad["per_sweep"], "predictor": prd["per_sweep"]},
            "per_tile": extra.get("per_tile"),
            "output_memory_ratio_max": prd["arena_bytes_max"] / pad["arena_bytes_max"],
            "output_memory_ratio_sum": prd["arena_bytes_sum"] / pad["arena_bytes_sum"],
            "overflow_rate": prd["overflow"] / max(prd["updates"], 1),
            "same_results": {"ok_counts_equal": pad["ok"] == prd["ok"], "sample_ranks_equal": same,
                             "max_rel_fro_diff_sweep0_sample": max_diff},
            "accuracy_vs_oracle": extra.get("accuracy_vs_oracle"),
            "tuning": extra.get("tuning"),
            "training": {"samples": int(len(R2)), "epochs": 150, "loss_first": float(base_loss[0]),
                         "loss_last": float(base_loss[-1]), "train_s": t_train,
                         "policy_margin_initial": policy0.margin},
            "setup_s": {"logs": t_logs, "tiles": t_tiles},
            "timing": "each sweep's batched plan executed once (warm), then captured in a CUDA "
                      "graph and replayed once, timed; the predictor arm adds its inference "
                      "kernel and the rebuild of overflows"}
    if rank == 0:
        print(json.dumps(line))
        sys.stdout.flush()
    barrier(world)


def fp64_peak(L, torch, dev) -> float:
    """FP64 ceiling in TFLOP/s, measured now (hcore_gpu_fp64_peak: the DMMA
    m16n8k16 probe; DMMA and DFMA share the FP64 pipe on this GPU)."""
    return float(L.hcore_gpu_fp64_peak(torch.cuda.current_stream(dev).cuda_stream))


def measured_peak(key):
    """A peak from MEASURED_PEAKS.json beside this file (None when absent)."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)),
                               "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)[key])
    except Exception:
        return None


def tc_rebuild_tensor_flops(nb, ks_r):
    """Tensor FLOP one execute issues in the tensor-core rebuild, mirroring
    the kernel's MMA loops (hc_rebuild_tc.cu): per (update, side) with k <=
    64, padded KP = 16/32/48/64 and rp = r rounded up to 16, the Gram passes
    (M/128 chunks, 8 K steps) and the output tiles (M/128, KP/16 K steps),
    each an M=128 MMA per digit slice i and piece of planes i..7 whose N is
    (planes in the piece) x (plane width)."""
    def pieces(width):
        per = 256 // width
        out = []
        for i in range(7):
            d0 = i
            while d0 < 8:
                d1 = min(d0 + per, 8)
                out.append((d1 - d0) * width)
                d0 = d1
        return out
    total = 0
    nch = (nb + 127) // 128
    for k, r in ks_r:
        if k > 64 or r <= 0:
            continue
        KP = 16 if k <= 16 else 32 if k <= 32 else 48 if k <= 48 else 64
        rp = (r + 15) // 16 * 16
        gram = nch * 8 * sum(2 * 128 * n * 16 for n in pieces(KP))
        outp = nch * (KP // 16) * sum(2 * 128 * n * 16 for n in pieces(rp))
        total += 2 * (gram + outp)
    return float(total)


def fp64_ceiling(L, torch, dev, index, seconds=1.5) -> dict:
    """The best FP64 probe form (DMMA m16n8k4, 2 chains: 1.10 TFLOP/s at
    2070 MHz, the same pipe and rate as DFMA) timed for about `seconds` with
    nvidia-smi sampling SM clock, power and throttle reasons meanwhile."""
    import ctypes as C

    stream = torch.cuda.current_stream(dev).cuda_stream
    tf, ms = C.c_double(), C.c_double()
    L.hcore_gpu_fp64_probe(2, 2, 8, 256, stream, C.byref(tf), C.byref(ms))
    iters = max(256, int(256 * seconds * 1e3 / max(ms.value, 1e-3)))
    clocks = Clocks(index)
    clocks.start()
    time.sleep(0.3)
    rc = L.hcore_gpu_fp64_probe(2, 2, 8, iters, stream, C.byref(tf), C.byref(ms))
    clk = clocks.stop()
    if rc != 0:
        raise SystemExit(f"FP64 probe failed: {rc}")
    return {"tflops": tf.value, "form": "DMMA m16n8k4 f64, 2 chains, 8 CTAs x 128 threads per SM",
            "ms": ms.value, "clocks": clk}


def run_tlr(args):
    """The steps either side of the Schur update in a TLR Cholesky, on the
    panel workload's tiles: HCORE_dpotrf of the 64 diagonal 1024 x 1024
    covariance tiles (a nugget of 1 on the diagonal keeps them well
    conditioned) in one batched call, then HCORE_dtrsm V <- L_k^-1 V of the
    panel's 63 V factors (all their columns as right-hand sides) against
    each of the 64 factors, one batched call.  One panel step = one POTRF +
    one panel TRSM; a timed step runs all 64 of them."""
    import numpy as np
    import torch

    import hcore_gb300 as hc
    from hcore_gb300 import build as hbuild
    from hcore_gb300 import panel as pnl
    from oracle import oracle as O

    rank, world, local = dist_init()
    if not os.path.exists(hbuild.LIB):
        hbuild.build()
    hc.lib()
    dev = torch.device("cuda", local)
    panel = pnl.build_panel(device=str(dev), max_updates=1)
    nb, T = panel.nb, panel.ntiles
    P = torch.from_numpy(pnl.morton_points(WORKLOAD["points"], 2, 0)).to(dev)

    def ktile(i):
        X = P[i * nb:(i + 1) * nb]
        d2 = (X * X).sum(1)[:, None] + (X * X).sum(1)[None, :] - 2.0 * X @ X.T
        return torch.exp(-torch.clamp(d2, min=0.0) / 0.01) + torch.eye(nb, dtype=torch.float64, device=dev)

    D0 = torch.stack([ktile(i) for i in range(T)])          # symmetric: storage order is moot
    D = D0.clone()
    # the panel's V factors, all columns: column-major nb x R (tensor R x nb)
    V0 = torch.cat([panel.V[int(panel.offset[panel.index[(j, 0)]]):int(panel.offset[panel.index[(j, 0)] + 1])]
                    .view(-1, nb) for j in range(1, T)], 0)
    R = V0.shape[0]
    Vs0 = V0.unsqueeze(0).expand(T, R, nb).contiguous()
    Vs = Vs0.clone()
    ptasks = [hc.PotrfTask(uplo=ord("L"), n=nb, A=D[k].data_ptr(), lda=nb) for k in range(T)]
    ttasks = [hc.TrsmTask(side=141, uplo=122, trans=111, diag=131, M=nb, N=R, alpha=1.0,
                          A=D[k].data_ptr(), lda=nb, B=Vs[k].data_ptr(), ldb=nb) for k in range(T)]
    stream = torch.cuda.current_stream(dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def step():
        D.copy_(D0)
        Vs.copy_(Vs0)
        e0, e1, e2 = ev(), ev(), ev()
        e0.record(stream)
        info = hc.potrf_batched(ptasks, stream=stream.cuda_stream)
        e1.record(stream)
        hc.trsm_batched(ttasks, stream=stream.cuda_stream)
        e2.record(stream)
        torch.cuda.synchronize(dev)
        assert not info.any(), info
        return e0.elapsed_time(e1), e1.elapsed_time(e2)

    step()
    # correctness: tiles 0 and 63 against the oracle
    port = O.Port()
    errs = {}
    for k in (0, T - 1):
        A = np.asfortranarray(D0[k].cpu().numpy())
        Lr, info, _ = port.dpotrf(ord("L"), nb, A)
        Lg = D[k].cpu().numpy().T
        errs[f"potrf_{k}"] = float(np.abs(np.tril(Lg) - np.tril(Lr)).max() / np.abs(np.tril(Lr)).max())
        Vr, _ = port.dtrsm(141, 122, 111, 131, nb, R, 1.0, np.asfortranarray(np.tril(Lr)),
                           np.asfortranarray(V0.cpu().numpy().T))
        Vg = Vs[k].cpu().numpy().T
        errs[f"trsm_{k}"] = float(np.abs(Vg - Vr).max() / np.abs(Vr).max())
    for _ in range(args.warmup):
        step()
    tp, tt = [], []
    for _ in range(args.steps):
        a, b = step()
        tp.append(a)
        tt.append(b)
    ms_p, ms_t = float(np.mean(tp)), float(np.mean(tt))
    ms = ms_p + ms_t
    # library comparison (cuSOLVER / cuBLAS through torch), same work; reported
    # as null where torch's linear-algebra library does not load
    try:
        Lt = torch.linalg.cholesky(D0)
        torch.cuda.synchronize(dev)
        e0, e1, e2 = ev(), ev(), ev()
        e0.record(stream)
        torch.linalg.cholesky_ex(D0)
        e1.record(stream)
        torch.linalg.solve_triangular(Lt, Vs0.transpose(1, 2), upper=False)
        e2.record(stream)
        torch.cuda.synchronize(dev)
        lib_p, lib_t = round(e0.elapsed_time(e1), 3), round(e1.elapsed_time(e2), 3)
        del Lt
    except RuntimeError:
        lib_p = lib_t = None
    # CPU: the oracle (OpenBLAS through the reference's calls) on one panel step
    cores = os.cpu_count() or 1
    port.set_threads(cores)
    A0 = np.asfortranarray(D0[0].cpu().numpy())
    Vh = np.asfortranarray(V0.cpu().numpy().T)
    t0 = time.time()
    Lr, _, _ = port.dpotrf(ord("L"), nb, A0)
    port.dtrsm(141, 122, 111, 131, nb, R, 1.0, Lr, Vh)
    cpu_s = time.time() - t0
    port.set_threads(1)
    fl_p, fl_t = nb ** 3 / 3, float(nb) * nb * R
    flops = T * (fl_p + fl_t)
    peak = fp64_peak(hc.lib(), torch, dev)
    line = {"metric": "TLR Cholesky panel steps/s (HCORE_dpotrf + HCORE_dtrsm, batched)",
            "value": T / (ms / 1e3), "unit": "panel-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (covariance tiles of the panel workload, nugget 1)",
            "config": {"workload": f"{T} x (POTRF of a {nb}^2 diagonal tile + TRSM of the "
                                   f"panel's {T - 1} V factors, {R} columns)",
                       "nb": nb, "tiles": T, "rhs_per_panel": R},
            "phases_ms": {"potrf": round(ms_p, 3), "trsm": round(ms_t, 3)},
            "roofline": {"bound": "fp64", "achieved": flops / (ms / 1e3) / 1e12, "peak": peak,
                         "unit": "TFLOP/s", "frac": flops / (ms / 1e3) / 1e12 / peak,
                         "flops_basis": "n^3/3 per POTRF, n^2 R per TRSM (FMA = 2 flops)",
                         "potrf_tflops": T * fl_p / (ms_p / 1e3) / 1e12,
                         "trsm_tflops": T * fl_t / (ms_t / 1e3) / 1e12},
            "library_comparison_ms": {"potrf_cusolver_batched": lib_p,
                                      "trsm_cublas_batched": lib_t},
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "panel-steps/s", "cores": cores,
                             "kind": "port", "sample": "one panel step (POTRF + TRSM) through "
                                                       "OpenBLAS as the reference calls it"},
            "accuracy": {"max_rel_err_vs_oracle": errs}}
    if rank == 0:
        print(json.dumps(line))
        sys.stdout.flush()
    barrier(world)


def run_panelstep(args):
    """One whole panel step of the TLR Cholesky of the headline matrix through
    the library's panel API (hcore_gpu_tlr_panel_step): POTRF of the 1024^2
    diagonal tile 0 (kernel + nugget 1, as the tile-steps workload), TRSM of
    the 63 panel V factors, SYRK of the 63 later diagonal tiles and the 1953
    recompressed Schur updates (acc 1e-8, maxrk 128), tiles stored with 128
    columns each.  Every timed step restores the matrix first (device copies,
    outside the timed region) and times the API call on the host clock (plan
    creation and its workspace allocation included)."""
    import ctypes as C

    import numpy as np
    import torch

    import hcore_gb300 as hc
    from hcore_gb300 import build as hbuild
    from hcore_gb300 import panel as pnl
    from oracle import oracle as O

    rank, world, local = dist_init()
    if not os.path.exists(hbuild.LIB):
        hbuild.build()
    L = hc.lib()
    dev = torch.device("cuda", local)
    panel = pnl.build_panel(device=str(dev))          # every tile of the lower triangle
    nb, T, store = panel.nb, panel.ntiles, panel.maxrank
    P = torch.from_numpy(pnl.morton_points(WORKLOAD["points"], 2, 0)).to(dev)

    def ktile(i):
        X = P[i * nb:(i + 1) * nb]
        d2 = (X * X).sum(1)[:, None] + (X * X).sum(1)[None, :] - 2.0 * X @ X.T
        return torch.exp(-torch.clamp(d2, min=0.0) / 0.01) + torch.eye(nb, dtype=torch.float64,
                                                                         device=dev)

    D0 = torch.stack([ktile(i) for i in range(T)])
    D = D0.clone()
    tiles = [t for t in panel.tiles]
    slot = {t: q for q, t in enumerate(tiles)}
    S0U = torch.zeros((len(tiles), store, nb), dtype=torch.float64, device=dev)
    S0V = torch.zeros_like(S0U)
    rank0 = np.zeros(T * T, dtype=np.int32)
    for t in tiles:
        s_ = panel.index[t]
        o0, o1 = int(panel.offset[s_]), int(panel.offset[s_ + 1])
        r = int(panel.rank[s_])
        S0U[slot[t], :r] = panel.U[o0:o1].view(r, nb)
        S0V[slot[t], :r] = panel.V[o0:o1].view(r, nb)
        rank0[t[0] + t[1] * T] = r
    SU, SV = S0U.clone(), S0V.clone()
    Dp = (C.c_void_p * T)(*[D[i].data_ptr() for i in range(T)])
    Up = (C.c_void_p * (T * T))()
    Vp = (C.c_void_p * (T * T))()
    for t in tiles:
        Up[t[0] + t[1] * T] = SU[slot[t]].data_ptr()
        Vp[t[0] + t[1] * T] = SV[slot[t]].data_ptr()
    rk = (C.c_int * (T * T))()
    mat = hc.TlrMatrix(nt=T, nb=nb, D=C.cast(Dp, C.c_void_p), ldd=nb, U=C.cast(Up, C.c_void_p),
                       V=C.cast(Vp, C.c_void_p), rank=C.cast(rk, C.c_void_p), maxrank=store)
    status = (C.c_int * (T * T))()

    def restore():
        D.copy_(D0)
        SU.copy_(S0U)
        SV.copy_(S0V)
        C.memmove(rk, rank0.ctypes.data, rank0.nbytes)
        torch.cuda.synchronize(dev)

    def call():
        info = C.c_int(-1)
        t0 = time.perf_counter()
        rc = L.hcore_gpu_tlr_panel_step(C.byref(mat), 0, panel.acc, store, C.byref(info), status,
                                        None)
        dt = (time.perf_counter() - t0) * 1e3
        if rc != 0:
            raise SystemExit(f"panel step failed ({rc}): {hc.last_error()}")
        return dt

    times = []
    for it in range(args.warmup + args.steps):
        restore()
        dt = call()
        if it >= args.warmup:
            times.append(dt)
    ms = statistics.median(times)
    # oracle: the same panel step on host copies of the initial state
    port = O.Port()
    hD = [np.asfortranarray(D0[i].cpu().numpy().T) for i in range(T)]
    hU, hV, hr = {}, {}, {}
    for t in tiles:
        r = int(rank0[t[0] + t[1] * T])
        hr[t] = r
        hU[t] = np.asfortranarray(S0U[slot[t], :r].cpu().numpy().T)
        hV[t] = np.asfortranarray(S0V[slot[t], :r].cpu().numpy().T)
    t0 = time.time()
    info_ref, st_ref = O.tlr_panel_step(port, hD, hU, hV, hr, 0, panel.acc, store, store)
    cpu_s = time.time() - t0
    ups = [t for t in tiles if t[1] > 0]
    rank_eq = sum(int(rk[i + j * T]) == hr[(i, j)] for (i, j) in ups)
    picks = [ups[q] for q in np.unique(np.linspace(0, len(ups) - 1, 48).astype(int))]
    worst = 0.0
    for (i, j) in picks:
        r = int(rk[i + j * T])
        gU = SU[slot[(i, j)], :r].cpu().numpy().T
        gV = SV[slot[(i, j)], :r].cpu().numpy().T
        d = _lr_norm(np.hstack([gU, hU[(i, j)]]), np.hstack([gV, -hV[(i, j)]]))
        worst = max(worst, d / max(_lr_norm(hU[(i, j)], hV[(i, j)]), 1e-300))
    dmax = max(float(np.abs(D[i].cpu().numpy().T - hD[i]).max() / np.abs(hD[i]).max())
               for i in (1, T - 1))
    l0 = float(np.abs(np.tril(D[0].cpu().numpy().T) - np.tril(hD[0])).max() /
               np.abs(np.tril(hD[0])).max())
    line = {"metric": "TLR Cholesky panel steps/s through hcore_gpu_tlr_panel_step",
            "value": 1e3 / ms, "unit": "panel-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (the panel workload's tiles; diagonal tiles with a nugget of 1)",
            "config": {"workload": "panel 0 of the 64 x 64-tile TLR Cholesky: POTRF + 63 TRSM + "
                                   "63 SYRK + 1953 recompressed Schur updates",
                       "nb": nb, "tiles": T, "storage_columns": store, "acc": panel.acc},
            "ms_min": min(times),
            "accuracy": {"schur_updates": len(ups), "rank_equal_to_oracle": int(rank_eq),
                         "sample_products": len(picks),
                         "max_rel_fro_diff_vs_oracle": worst,
                         "potrf_rel_err": l0, "syrk_tiles_rel_err": dmax},
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "panel-steps/s", "cores": 1,
                             "kind": "port", "sample": "the same panel step through the "
                                                       "oracle's restatement, one host core"}}
    if rank == 0:
        print(json.dumps(line))
        sys.stdout.flush()
    barrier(world)


def run_compress(args):
    """Tile compression on the GPU (hcore_gpu_compress_batched): all 2016
    off-diagonal 1024 x 1024 tiles of the panel workload's covariance matrix,
    relative threshold 1e-8 sigma_max, maxrank 128 (the panel workload's own
    compression).  A step compresses every tile once, from tiles resident in
    HBM."""
    import numpy as np
    import torch

    import hcore_gb300 as hc
    from hcore_gb300 import build as hbuild
    from hcore_gb300 import panel as pnl
    from oracle import oracle as O

    rank, world, local = dist_init()
    if not os.path.exists(hbuild.LIB):
        hbuild.build()
    hc.lib()
    dev = torch.device("cuda", local)
    nb, T, acc, maxrank = 1024, WORKLOAD["points"] // 1024, 1e-8, 128
    Pt = pnl.morton_points(WORKLOAD["points"], 2, 0)
    P = torch.from_numpy(Pt).to(dev)

    def ktile(i, j):   # column-major tile (i, j): tensor row c = column c
        X, Y = P[i * nb:(i + 1) * nb], P[j * nb:(j + 1) * nb]
        d2 = (X * X).sum(1)[:, None] + (Y * Y).sum(1)[None, :] - 2.0 * X @ Y.T
        return torch.exp(-torch.clamp(d2, min=0.0) / 0.01).T.contiguous()

    pairs = [(i, j) for i in range(1, T) for j in range(i)][:args.compress_tiles]
    n = len(pairs)
    D = torch.empty(n, nb, nb, dtype=torch.float64, device=dev)
    for q, (i, j) in enumerate(pairs):
        D[q] = ktile(i, j)
    U = torch.empty(n, maxrank, nb, dtype=torch.float64, device=dev)
    V = torch.empty_like(U)
    tasks = [hc.CompressTask(M=nb, D=D[q].data_ptr(), ldd=nb, acc=acc, relative=1,
                             maxrank=maxrank, U=U[q].data_ptr(), V=V[q].data_ptr(), ldo=nb)
             for q in range(n)]
    stream = torch.cuda.current_stream(dev)
    ranks, status = hc.compress_batched(tasks, stream=stream.cuda_stream)
    for _ in range(max(args.warmup - 1, 0)):
        hc.compress_batched(tasks, stream=stream.cuda_stream)
    torch.cuda.synchronize(dev)
    ms = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ranks, status = hc.compress_batched(tasks, stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms.append(e0.elapsed_time(e1))
    ms_step = float(np.mean(ms))
    # accuracy on a sample against the oracle (full SVD, the reference's rule
    # with the relative threshold)
    port = O.Port()
    samp = list(range(0, n, max(1, n // 12)))[:12]
    eq, diffs, margins = 0, [], []
    for q in samp:
        Dq = np.asfortranarray(D[q].cpu().numpy().T)
        rr, Ur, Vr, sig = port.dcompress(Dq, acc, maxrank, relative=True)
        r = int(ranks[q])
        eq += int(r == rr)
        margins.append(float(np.min(np.abs(sig - acc * sig[0])) / (acc * sig[0])))
        if r == rr and r > 0:
            Ug = U[q, :r].cpu().numpy().T
            Vg = V[q, :r].cpu().numpy().T
            diffs.append(float(np.linalg.norm(Ug @ Vg.T - Ur @ Vr.T) / np.linalg.norm(Ur @ Vr.T)))
    # CPU: the reference's compressor (full dgesvd, restated) on a sample with
    # every host core through OpenBLAS threads, and the host path the panel
    # workload uses (randomized range finder, one process per core)
    cores = os.cpu_count() or 1
    port.set_threads(cores)
    t0 = time.time()
    for q in samp[:4]:
        port.dcompress(np.asfortranarray(D[q].cpu().numpy().T), acc, maxrank, relative=True)
    cpu_exact = 4 / (time.time() - t0)
    port.set_threads(1)
    host_pairs = pairs[: 4 * cores]
    t0 = time.time()
    pnl.compress_tiles(Pt, nb, host_pairs, "sqexp", 0.01, acc, maxrank)
    cpu_rand = len(host_pairs) / (time.time() - t0)
    # flops executed by the pivoted QR (dot, update and norm per trailing
    # element and step: 6 flops) over the ranges it found, which are at least
    # the ranks; reported on the ranks (a lower bound)
    flops = float(sum(6.0 * nb * nb * int(r) for r in ranks))
    peak = fp64_peak(hc.lib(), torch, dev)
    line = {"metric": "TLR tiles compressed/s (GPU tile compressor, batched)",
            "value": n / (ms_step / 1e3), "unit": "tiles/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (covariance tiles of the panel workload, generated on the GPU)",
            "config": {"workload": f"{n} off-diagonal {nb}^2 tiles, sigma >= {acc:g} sigma_max, "
                                   f"maxrank {maxrank}", "nb": nb, "tiles": n},
            "ranks": {"mean": float(ranks.mean()), "max": int(ranks.max()),
                      "status_nonzero": int((status != 0).sum())},
            "roofline": {"bound": "fp64", "achieved": flops / (ms_step / 1e3) / 1e12, "peak": peak,
                         "unit": "TFLOP/s", "frac": flops / (ms_step / 1e3) / 1e12 / peak,
                         "flops_basis": "6 nb^2 flops per tile and pivoted-QR step, counted "
                                        "over the final ranks (a lower bound: the QR runs "
                                        "past the rank to 1e-3 of the threshold)"},
            "accuracy": {"sample": len(samp), "rank_equal_to_oracle": eq,
                         "max_rel_fro_diff_vs_oracle": max(diffs) if diffs else None,
                         "min_threshold_margin": min(margins)},
            "cpu_baseline": {"value": cpu_exact, "unit": "tiles/s", "cores": cores, "kind": "port",
                             "sample": "4 tiles, the reference tests' compressor (full dgesvd) "
                                       "restated, OpenBLAS on all cores"},
            "host_randomized_tiles_per_s": cpu_rand}
    if rank == 0:
        print(json.dumps(line))
        sys.stdout.flush()
    barrier(world)


def run_zgemm(args):
    """Complex updates (HCORE_zgemm semantics) on the GPU.  Workload: 256
    independent updates of the "nb=512, ranks 32" shape in complex
    arithmetic (seeded complex factors, sigma_i = 10^(-8i/32) folded into U,
    acc 1e-8, maxrk 64, alpha = beta = 1), host arrays in and out.  A step is
    one hcore_gpu_zgemm_batched call over all of them, run by the native
    complex kernels (complex Householder QR, complex one-sided Jacobi, complex
    rebuild); only complex factors cross the host link.  The same batch
    through the order-2M real embedding and the single-call drop-in
    (HCORE_zgemm) are timed beside it."""
    import numpy as np
    import torch

    import hcore_gb300 as hc
    from hcore_gb300 import build as hbuild
    from oracle import oracle as O

    rank, world, local = dist_init()
    if not os.path.exists(hbuild.LIB):
        hbuild.build()
    hc.lib()
    M, a, acc, maxrk, n = 512, 32, 1e-8, 64, 256
    rng = np.random.default_rng(2024)

    def clr(k):
        U, _ = np.linalg.qr(rng.standard_normal((M, k)) + 1j * rng.standard_normal((M, k)))
        V, _ = np.linalg.qr(rng.standard_normal((M, k)) + 1j * rng.standard_normal((M, k)))
        return np.asfortranarray(U * 10.0 ** (-8.0 * np.arange(k) / k)), np.asfortranarray(V)

    ups = [clr(a) + clr(a) + clr(a) for _ in range(n)]   # AU, AV, BU, BV, CU, CV
    outU = [np.zeros((M, maxrk), dtype=np.complex128, order="F") for _ in range(n)]
    outV = [np.zeros((M, maxrk), dtype=np.complex128, order="F") for _ in range(n)]
    one = hc.DComplex(1.0, 0.0)
    tasks = [hc.ZlrTask(M=M, a=a, b=a, c=a, rk=0, maxrk=maxrk, alpha=one, beta=one, acc=acc,
                        AU=u[0].ctypes.data, AV=u[1].ctypes.data, lda=M, BU=u[2].ctypes.data,
                        BV=u[3].ctypes.data, ldb=M, CU=oU.ctypes.data, CV=oV.ctypes.data, ldc=M)
             for u, oU, oV in zip(ups, outU, outV)]

    def reset():
        for u, oU, oV in zip(ups, outU, outV):
            oU[:, :a] = u[4]
            oV[:, :a] = u[5]

    for _ in range(max(args.warmup, 1)):
        reset()
        ranks, status = hc.zgemm_batched(tasks)
    ts = []
    for _ in range(args.steps):
        reset()
        t0 = time.perf_counter()
        ranks, status = hc.zgemm_batched(tasks)
        ts.append(time.perf_counter() - t0)
    ms = 1e3 * float(np.median(ts))
    # the same batch through the order-2M real embedding, for comparison
    os.environ["HCORE_GPU_ZGEMM_EMBED"] = "1"
    te = []
    for it in range(max(args.steps // 2, 2) + 1):
        reset()
        t0 = time.perf_counter()
        hc.zgemm_batched(tasks)
        if it:
            te.append(time.perf_counter() - t0)
    del os.environ["HCORE_GPU_ZGEMM_EMBED"]
    ms_embed = 1e3 * float(np.median(te))
    reset()
    ranks, status = hc.zgemm_batched(tasks)
    # accuracy on a sample against the restated reference
    port = O.Port()
    eq, diffs = 0, []
    for q in range(0, n, 32):
        u = ups[q]
        ref = port.zgemm(M, 1.0, u[0], u[1], a, u[2], u[3], a, 1.0, u[4], u[5], a, maxrk=maxrk,
                         acc=acc)
        r = int(ranks[q])
        eq += int(r == ref["rank"])
        Pr = ref["CU"] @ ref["CV"].T
        diffs.append(float(np.linalg.norm(outU[q][:, :r] @ outV[q][:, :r].T - Pr) / np.linalg.norm(Pr)))
    # the single-call drop-in, for its latency
    u = ups[0]
    hc.hcore_zgemm(M, 1.0, u[0], u[1], a, u[2], u[3], a, 1.0, u[4], u[5], a, maxrk=maxrk, acc=acc)
    t0 = time.perf_counter()
    for _ in range(3):
        hc.hcore_zgemm(M, 1.0, u[0], u[1], a, u[2], u[3], a, 1.0, u[4], u[5], a, maxrk=maxrk,
                       acc=acc)
    single_ms = 1e3 * (time.perf_counter() - t0) / 3
    # CPU: the restated reference (complex LAPACK), one process per core
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    nc = 0
    while time.perf_counter() - t0 < min(args.cpu_seconds, 4.0) or nc == 0:
        port.zgemm(M, 1.0, u[0], u[1], a, u[2], u[3], a, 1.0, u[4], u[5], a, maxrk=maxrk, acc=acc)
        nc += 1
    cpu1 = nc / (time.perf_counter() - t0)
    line = {"metric": "complex TLR-GEMM updates/s (HCORE_zgemm semantics, batched)",
            "value": n / (ms / 1e3), "unit": "updates/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic (seeded complex factors)",
            "config": {"workload": f"{n} complex updates nb=512, ranks 32, sigma 10^(-8i/32), "
                                   "acc 1e-8, maxrk 64", "nb": M, "ranks": a, "updates": n},
            "ranks": {"mean": float(np.mean(ranks)), "status_nonzero": int((status != 0).sum())},
            "accuracy": {"sample": len(diffs), "rank_equal_to_oracle": eq,
                         "max_rel_fro_diff_vs_oracle": max(diffs)},
            "e2e": {"value": n / (ms / 1e3), "unit": "updates/s",
                    "h2d_bytes_per_step": n * 6 * M * a * 16,
                    "d2h_bytes_per_step": int(2 * M * 16 * np.sum(ranks)),
                    "how": "host complex arrays through hcore_gpu_zgemm_batched: the native "
                           "complex kernels, complex factors in and out"},
            "single_call_ms": single_ms,
            "embedding_path": {"updates_per_s": n / (ms_embed / 1e3), "ms_per_step": ms_embed,
                               "how": "the same batch with HCORE_GPU_ZGEMM_EMBED=1: each update "
                                      "as a real update of order 2M through the real kernels"},
            "cpu_baseline": {"value": cpu1 * cores, "unit": "updates/s", "cores": cores,
                             "kind": "port", "sample": f"{nc} calls of the restated HCORE_zgemm "
                                                       "on one core, times the core count"}}
    if rank == 0:
        print(json.dumps(line))
        sys.stdout.flush()
    barrier(world)


FP64_PROBES = [("dfma", 0), ("dmma_m8n8k4", 1), ("dmma_m16n8k4", 2), ("dmma_m16n8k8", 3),
               ("dmma_m16n8k16", 4), ("dmma_m16n8k16_b_one_register", 5),
               ("dmma_m16n8k16_b_equal_values", 6)]


def run_fp64peak(args):
    """The FP64 ceiling, clock-stamped: every probe form of the library
    (hcore_gpu_fp64_probe: DFMA, DMMA shapes, and the m16n8k16 form with its
    B operands in one register or as equal values in distinct registers), at
    2, 4 and 8 accumulator chains, each timed for about `--probe-seconds`
    with nvidia-smi sampling SM clock, power and throttle reasons meanwhile."""
    import ctypes as C

    import torch

    import hcore_gb300 as hc
    from hcore_gb300 import build as hbuild

    rank, world, local = dist_init()
    if not os.path.exists(hbuild.LIB):
        hbuild.build()
    L = hc.lib()
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev).cuda_stream
    forms = [(nm, kd, ch) for nm, kd in FP64_PROBES for ch in (2, 4, 8)]
    if args.probe_forms:
        want = [f.split(":") for f in args.probe_forms.split(",")]
        kinds = dict(FP64_PROBES)
        forms = [(nm, kinds[nm], int(ch)) for nm, ch in want]
    rows = []
    for name, kind, chains in forms:
        tf, ms = C.c_double(), C.c_double()
        rc = L.hcore_gpu_fp64_probe(kind, chains, 8, 256, stream, C.byref(tf), C.byref(ms))
        if rc != 0:
            raise SystemExit(f"probe {name} failed: {rc}")
        iters = max(256, int(256 * args.probe_seconds * 1e3 / max(ms.value, 1e-3)))
        clocks = Clocks(local)
        clocks.start()
        time.sleep(0.3)
        rc = L.hcore_gpu_fp64_probe(kind, chains, 8, iters, stream, C.byref(tf), C.byref(ms))
        clk = clocks.stop()
        if rc != 0:
            raise SystemExit(f"probe {name} failed: {rc}")
        mhz = clk.get("sm_mhz")
        rows.append({"form": name, "chains": chains, "tflops": tf.value, "ms": ms.value,
                     "iters": iters, "sm_mhz": mhz, "power_w_max": clk.get("power_w_max"),
                     "reasons": clk.get("reasons"),
                     "flop_per_clk_per_sm": (tf.value * 1e12 / (mhz * 1e6) /
                                             torch.cuda.get_device_properties(dev).multi_processor_count)
                     if mhz else None})
    best = max(rows, key=lambda r: r["tflops"])
    line = {"metric": "FP64 issue rate (probe kernels, no memory traffic)", "value": best["tflops"],
            "unit": "TFLOP/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f64",
            "config": {"workload": "fp64 probes", "ctas_per_sm": 8, "threads_per_cta": 128},
            "best": best["form"], "probes": rows}
    print(json.dumps(line))
    sys.stdout.flush()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "precision":
        run_precision(args)
    elif args.workload == "dense":
        run_dense(args)
    elif args.workload == "predictor":
        run_predictor(args)
    elif args.workload == "tlr":
        run_tlr(args)
    elif args.workload == "compress":
        run_compress(args)
    elif args.workload == "zgemm":
        run_zgemm(args)
    elif args.workload == "fp64peak":
        run_fp64peak(args)
    elif args.workload == "panelstep":
        run_panelstep(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
