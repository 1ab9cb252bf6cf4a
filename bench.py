#!/usr/bin/env python
"""Throughput of the colored-ICP registration path on GB300.

Workload (default, "batch64"): 64 synthetic fragment pairs of uneven size (clouds
log-uniform in 20k-300k points, per-pair rotation 0-15 deg, translation 0-15 cm,
overlap 40-90 %), three-scale colored ICP (voxel 0.04/0.02/0.01 m, 50/30/14
iterations, max correspondence 1.5 x voxel, normal and gradient radius 2 x voxel).
A step registers the whole batch.  Metric: pairs/s (higher is better).

  value  chosen path: one CUDA graph per batch (all pairs in every launch,
         compensated FP32 accumulation, FP64 solve), inputs resident in HBM
  e2e    the same through the C ABI with host buffers: per step the 128 clouds are
         uploaded from pinned memory and the 64 results read back
  plain  the one-pair-per-launch FP32 path: 64 sequential single-pair calls, eager
         launches, convergence read back on the host after every iteration
  rows   the other workloads, each chosen vs plain where both exist: a 640x480
         frame pair end to end (ms/frame), one 250k-point pair through three
         scales, the adjoint of 5 unrolled Gauss-Newton steps on a 100k-point pair,
         and a tracked RGB-D stream at 640x480 and 1280x720 (frames/s, p50/p99
         latency, drift against the ground-truth trajectory)

--impl reference times the reference's algorithm on the host cores (the CPU port
in oracle/, FP32 in the reference's operation order, OpenMP) on the same workload.
Multi-GPU (torchrun): every rank registers its own batch (weak scaling); no data
moves between ranks, the barrier and the max-reduce of the step time are the only
collectives.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# the schedule of the precision and batching workloads
SCALES = [(0.04, 50, 0.06, 0.08, 0.08), (0.02, 30, 0.03, 0.04, 0.04), (0.01, 14, 0.015, 0.02, 0.02)]
ICP_BYTES_PER_POINT = 16 + 48  # source xyz+I; target record: xyz+cell, normal+I, gradient
ICP_BYTES_PER_BLOCK = 32 * 8   # one block partial (FP64)
ICP_CHUNK = 1024


def parse_args(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--pairs", type=int, default=64)
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--quick", action="store_true", help="value only (for profiler runs)")
    p.add_argument("--eager", action="store_true", help="with --quick: the chosen configuration launched "
                   "eagerly with host convergence checks (the same kernels and iteration counts as the graph; "
                   "for profilers that do not descend into conditional graph nodes)")
    p.add_argument("--no-extras", action="store_true", help="skip the per-row measurements (frame pair, "
                   "single pair, adjoint, stream)")
    p.add_argument("--no-tune", action="store_true", help="default launch shape instead of the autotuner's")
    p.add_argument("--stream-frames", type=int, default=1000, help="frames of each stream (640x480 and 1280x720)")
    p.add_argument("--single-pair", type=int, default=0, metavar="EXECUTES",
                   help="only the 250k-point pair through three scales: EXECUTES plan executes (graph mode, or "
                        "eager with --eager), one JSON line")
    p.add_argument("--frame-pair", type=int, default=0, metavar="PUSHES",
                   help="only the 640x480 frame pair: PUSHES alternating tracker pushes (graph mode, or eager "
                        "with --eager), one JSON line")
    return p.parse_args(argv)


# --------------------------------------------------------------------------- #
# ranks
# --------------------------------------------------------------------------- #
def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def dist_init(backend):
    import torch.distributed as dist

    rank, world, _ = dist_env()
    if world > 1 and not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        os.environ.setdefault("MASTER_PORT", "29511")
        dist.init_process_group(backend, rank=rank, world_size=world)
    return rank, world


def barrier():
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def reduce_max(x, device="cpu"):
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(x, device="cpu"):
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def rank_seed(base, rank):
    """each rank registers its own batch (weak scaling)"""
    return base + 1009 * rank


# --------------------------------------------------------------------------- #
# clocks during the timed region
# --------------------------------------------------------------------------- #
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, local=0):
        self.gpu_id = self.smi_id(local)
        self.proc = None
        self.path = None

    @staticmethod
    def smi_id(local):
        """the device's UUID as nvidia-smi names it: under CUDA_VISIBLE_DEVICES the CUDA
        ordinal is not the nvidia-smi index, the UUID is the same in both"""
        import torch

        u = str(torch.cuda.get_device_properties(local).uuid)
        return u if u.startswith("GPU-") else "GPU-" + u

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu_id}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        out = self.summarise(rows)
        if out is not None:
            out["gpu_id"] = self.gpu_id
        return out

    @staticmethod
    def summarise(rows):
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def committed_traffic():
    """DRAM bytes per ICP-iteration launch from the committed ncu capture, if any"""
    path = os.path.join(ROOT, "profiles", "icp_iter_traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


# --------------------------------------------------------------------------- #
# workload
# --------------------------------------------------------------------------- #
def make_workload(n_pairs, seed):
    from cuda_3d_gb300 import synth

    sampler = synth.RoomSampler()
    return synth.batch_pairs(n_pairs, seed=seed, sampler=sampler)


def icp_algorithmic_bytes(results):
    """compulsory HBM bytes of the ICP-iteration launches of one execute: per pair,
    scale and iteration every source point reads its 16-byte xyzI and gathers its
    48-byte target record (position, normal + intensity, gradient); each block
    writes one 256-byte partial"""
    total = 0
    for r in results:
        for s in range(len(SCALES)):
            n, it = r["scale_n_src"][s], r["scale_iterations"][s]
            total += it * (n * ICP_BYTES_PER_POINT + math.ceil(n / ICP_CHUNK) * ICP_BYTES_PER_BLOCK)
    return total


def workload_config(pairs, world):
    """the workload description both arms print (the reference arm times a sample of it)"""
    n_src = sum(len(p.src_xyz) for p in pairs)
    n_tgt = sum(len(p.tgt_xyz) for p in pairs)
    return {"workload": "batch64: 64 fragment pairs, clouds log-uniform 20k-300k points, rot 0-15 deg, "
                        "trans 0-15 cm, overlap 40-90 %, scales voxel 0.04/0.02/0.01 m x 50/30/14 iterations",
            "pairs_per_gpu": len(pairs), "src_points": n_src, "tgt_points": n_tgt,
            "scales": SCALES, "parallelism": f"replicas x{world} (pairs sharded per rank)",
            "l2": f"inputs larger than L2 ({(n_src + n_tgt) * 32 / 1e6:.0f} MB resident SoA)"}


def cpu_sample(pairs, k=4):
    """the fixed pair sample the CPU measurements time: pairs ranked by point count
    (source + target), one at the middle of each of k equal rank strata, so the sample
    spans the batch's size range"""
    k = min(k, len(pairs))
    order = sorted(range(len(pairs)), key=lambda i: len(pairs[i].src_xyz) + len(pairs[i].tgt_xyz))
    return sorted(order[(2 * j + 1) * len(pairs) // (2 * k)] for j in range(k))


def sample_text(pairs, idx):
    pts = sum(len(pairs[i].src_xyz) + len(pairs[i].tgt_xyz) for i in idx) / len(idx)
    mean = sum(len(p.src_xyz) + len(p.tgt_xyz) for p in pairs) / len(pairs)
    return (f"pairs {idx} of the batch (one per size stratum; {pts / 1e3:.0f}k points per pair against the "
            f"batch's mean {mean / 1e3:.0f}k), full three-scale schedule, FP32 in the reference's operation order "
            f"(oracle/gca_oracle.c), OpenMP")


def pose_spread(a, b):
    from cuda_3d_gb300 import synth

    errs = [synth.pose_error(x["T"], y["T"]) for x, y in zip(a, b)]
    return max(e[0] for e in errs), max(e[1] for e in errs)


# --------------------------------------------------------------------------- #
# our arm
# --------------------------------------------------------------------------- #
def run_ours(args):
    import torch

    from cuda_3d_gb300 import build, native as N
    from cuda_3d_gb300 import synth

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist_init("nccl")
    build.build()
    # a dedicated stream: the library and the timing events share it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = N.Context(local, stream=stream.cuda_stream)
    pairs = make_workload(args.pairs, rank_seed(args.seed, rank))
    P = len(pairs)
    srcs = [ctx.cloud_from(p.src_xyz, p.src_rgb) for p in pairs]
    tgts = [ctx.cloud_from(p.tgt_xyz, p.tgt_rgb) for p in pairs]
    scales = [N.scale(*s) for s in SCALES]
    chosen = N.icp_params(scales, update_map=N.UPDATE_SE3_EXP, compensated=True,
                          use_graph=not (args.quick and args.eager))
    # launch shape from the autotuner (outside every timed region; results do not depend on it)
    tuning, tune_ms = None, None
    if not args.no_tune and not args.quick:
        t0 = time.perf_counter()
        best, best_ms = N.icp_autotune(ctx, srcs, tgts, chosen, reps=2)
        chosen.tuning = best
        tuning = {"nn_item_points": best.nn_item_points, "nn_blocks_per_sm": best.nn_blocks_per_sm,
                  "accum_blocks_per_sm": best.accum_blocks_per_sm, "fused_finalize": best.fused_finalize,
                  "serial_prep": best.serial_prep,
                  "ms_per_execute": best_ms,
                  "search_s": time.perf_counter() - t0}
    plan = N.IcpPlan(ctx, srcs, tgts, chosen)
    res_chosen = None
    for _ in range(max(args.warmup, 3)):
        res_chosen = plan.execute(results=True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    # ---- value: resident inputs, graph replays -------------------------------
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0.record(stream)
    for _ in range(args.steps):
        plan.execute(results=False)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier()
    ms = reduce_max(ev0.elapsed_time(ev1) / args.steps, "cuda")
    value = world * P / (ms / 1000.0)

    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": "colored-ICP pairs/s (quick)", "value": value, "ms_per_step": ms,
                              "gpu_launches": plan.kernels() * args.steps}))
        return

    # ---- e2e: host buffers through the C ABI ----------------------------------
    host = []
    for p in pairs:
        bufs = []
        for a in (p.src_xyz, p.src_rgb, p.tgt_xyz, p.tgt_rgb):
            t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True)
            t.numpy()[:] = a
            bufs.append(t)
        host.append(bufs)
    h2d = sum(b.numel() * 4 for bufs in host for b in bufs)

    # Double-buffered through the public API: two cloud sets, a plan on each, and a
    # second context whose stream uploads the next step's 128 clouds (one call; the
    # copy engines move the pinned buffers, so the upload takes no SMs from the
    # registration) while the first context runs this step's plan; the plan's stream
    # waits on the upload's event.  Every step uploads its inputs and reads its 64
    # results back inside the timed region.
    up_stream = torch.cuda.Stream()
    ctx_up = N.Context(local, stream=up_stream.cuda_stream)
    ctx_up.check(ctx_up.L.gca3d_set_upload_mode(ctx_up.h, N.UPLOAD_COPY_ENGINE))
    sets = [(srcs, tgts), ([ctx.cloud(s.capacity) for s in srcs], [ctx.cloud(t.capacity) for t in tgts])]
    up_xyz = [b.data_ptr() for bufs in host for b in (bufs[0], bufs[2])]
    up_rgb = [b.data_ptr() for bufs in host for b in (bufs[1], bufs[3])]
    up_n = [b.shape[0] for bufs in host for b in (bufs[0], bufs[2])]
    up_events = [torch.cuda.Event(), torch.cuda.Event()]

    def upload(k):
        cl = [c for s, t in zip(*sets[k]) for c in (s, t)]
        N.upload_many(ctx_up, cl, up_xyz, up_rgb, up_n)
        up_events[k].record(up_stream)

    upload(1)
    up_stream.synchronize()
    plans = [plan, N.IcpPlan(ctx, sets[1][0], sets[1][1], chosen)]

    def run_e2e(steps):
        # step k+1 is queued behind step k before step k's results are read, so the
        # GPU never waits for the host; a set is refilled once its plan's results are in
        upload(0)
        stream.wait_event(up_events[0])
        plans[0].execute(results=False)
        out = None
        for k in range(steps):
            cur = k & 1
            if k + 1 < steps:
                upload(cur ^ 1)  # step k-1 used this set and has been read back
                stream.wait_event(up_events[cur ^ 1])
                plans[cur ^ 1].execute(results=False)
            out = plans[cur].results()
        return out

    run_e2e(4)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res_e2e = run_e2e(args.steps)
    torch.cuda.synchronize()
    ms_e2e = reduce_max((time.perf_counter() - t0) * 1e3 / args.steps, "cuda")
    barrier()
    d2h = plan.readback_bytes()  # the pair states and the error word read back per step
    same = all(np.array_equal(a["T"], b["T"]) for a, b in zip(res_e2e, res_chosen))
    e2e = {"value": world * P / (ms_e2e / 1000.0), "unit": "pairs/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": ms_e2e, "results_equal_resident_run": same,
           "pipeline": "two cloud sets and plans; step k+1's upload (second context's stream, copy-engine "
                       "mode) overlaps step k's registration and step k+1 is queued before step k's results are "
                       "read; host wall clock with a device synchronize on both "
                       "sides"}

    # ---- roofline of the ICP iteration kernel (eager run, CUDA events) ---------
    # the same launch shape with the preparation serialised, so that the timed kernels
    # run alone (in the timed schedule they share the SMs with the next scale's preparation)
    prof_tuning = N.Tuning.from_buffer_copy(chosen.tuning)
    prof_tuning.serial_prep = 1
    prof = N.icp_params(scales, update_map=N.UPDATE_SE3_EXP, compensated=True, use_graph=False,
                        tuning=prof_tuning)
    plan_prof = N.IcpPlan(ctx, srcs, tgts, prof)
    plan_prof.execute(results=True)
    ctx.profile_begin("icp_iter")
    res_prof = plan_prof.execute(results=True)
    icp_ms, _ = ctx.profile_read()
    # one launch of the iteration per scale and iteration that some pair ran (the
    # search and the update are timed as two intervals each)
    icp_launches = sum(max(r["scale_iterations"][s] for r in res_prof) for s in range(len(SCALES)))
    bytes_total = icp_algorithmic_bytes(res_prof)
    peak, peak_kind = measured_peaks()
    achieved = bytes_total / (icp_ms / 1e3) / 1e9
    traffic = committed_traffic()
    breakdown = {"icp_iter": {"ms": icp_ms, "launches": icp_launches}}
    for k in ("sort_pass", "normals", "voxel_reduce", "grid_scatter"):
        ctx.profile_begin(k)
        plan_prof.execute(results=True)
        t, n = ctx.profile_read()
        breakdown[k] = {"ms": t, "launches": n}
    roofline = {"kernel": "ICP iteration (k_icp_nn + k_icp_accum: transform, NN, residuals, Jacobians, "
                          "compensated JTJ/JTr, FP64 solve)", "bound": "hbm",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "traffic": traffic.get("dram_bytes_per_launch") if traffic else None,
                "algorithmic_bytes_per_launch": bytes_total / max(icp_launches, 1),
                "avg_launch_us": icp_ms * 1e3 / max(icp_launches, 1), "launches": icp_launches,
                "timing": "eager execute with the preparation serialised (tuning.serial_prep), CUDA events on "
                          "the launching stream around the ICP launches"}

    # ---- plain: one pair per call, FP32, host convergence checks ----------------
    # the 64 single-pair plans are built before the timed region (the timed calls
    # launch and read back only); the one-shot call that builds and frees its plan
    # every time is reported beside it
    plain, res_plain = None, None
    if not args.no_plain:
        pp = N.icp_params(scales, update_map=N.UPDATE_SE3_EXP, compensated=False, use_graph=False)
        plans = [N.IcpPlan(ctx, [s], [t], pp) for s, t in zip(srcs, tgts)]
        res_plain = [pl.execute(results=True)[0] for pl in plans]
        reps = 2
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            res_plain = [pl.execute(results=True)[0] for pl in plans]
        torch.cuda.synchronize()
        ms_plain = reduce_max((time.perf_counter() - t0) * 1e3 / reps, "cuda")
        del plans
        [N.color_icp(ctx, s, t, pp) for s, t in zip(srcs, tgts)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res_once = [N.color_icp(ctx, s, t, pp) for s, t in zip(srcs, tgts)]
        torch.cuda.synchronize()
        ms_once = reduce_max((time.perf_counter() - t0) * 1e3, "cuda")
        rot, tr = pose_spread(res_chosen, res_plain)
        assert all(np.array_equal(a["T"], b["T"]) for a, b in zip(res_plain, res_once))
        plain = {"value": world * P / (ms_plain / 1000.0), "unit": "pairs/s", "ms_per_step": ms_plain,
                 "chosen_over_plain": ms_plain / ms,
                 "max_pose_diff_vs_chosen": {"rad": rot, "m": tr},
                 "with_plan_setup": {"value": world * P / (ms_once / 1000.0), "unit": "pairs/s",
                                     "ms_per_step": ms_once, "chosen_over_plain": ms_once / ms,
                                     "note": "gca3d_color_icp per pair: plan built (device allocations, "
                                             "host-pinned buffers) and freed in every call"}}

    gt = [synth.pose_error(r["T"], p.T_gt) for r, p in zip(res_chosen, pairs)]
    rows = None
    if rank == 0 and not args.no_extras:
        rows = run_rows(ctx, N, synth, args)
    cpu, pose_check = None, None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu, pose_check = cpu_leg(pairs, res_chosen, res_plain)

    line = {
        "metric": "colored-ICP pairs/s (64-pair batch, three-scale)",
        "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (FP64 solve and cross-block sums)", "data": "synthetic",
        "config": workload_config(pairs, world),
        "tuning": tuning,
        "e2e": e2e,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "plain": plain,
        "pose_vs_fp64_oracle": pose_check,
        "kernel_breakdown_ms_per_execute": breakdown,
        "rows": rows,
        "gt_error_max": {"rad": max(g[0] for g in gt), "m": max(g[1] for g in gt)},
        "gt_error_median": {"rad": statistics.median(g[0] for g in gt), "m": statistics.median(g[1] for g in gt)},
        "clocks": clk,
        "gpu_launches": plan.kernels() * args.steps,
    }
    if rank == 0:
        print(json.dumps(line))


# --------------------------------------------------------------------------- #
# the other workloads
# --------------------------------------------------------------------------- #
C0_SCALE = (0.01, 30, 0.03, 0.02, 0.02, 30)  # voxel, iterations, max_corr, normal r, gradient r, max_nn


def _lat(ms):
    ms = np.asarray(ms)
    return {"p50_ms": float(np.median(ms)), "p99_ms": float(np.percentile(ms, 99)), "mean_ms": float(ms.mean())}


def _track(N, ctx, cam, frames, use_graph, compensated, constant_velocity=True):
    tr = N.Tracker(ctx, N.tracker_params(cam, [N.scale(*C0_SCALE)], use_graph=use_graph, compensated=compensated,
                                         constant_velocity=constant_velocity))
    lat, res, pose = [], [], None
    for d, c in frames:
        t0 = time.perf_counter()
        r, pose = tr.push(d, c)
        lat.append((time.perf_counter() - t0) * 1e3)
        res.append(r)
    return lat, res, pose, tr.kernels()


def run_rows(ctx, N, synth, args):
    """per-row measurements on rank 0 (host-timed around calls that return results)"""
    rows = {}
    # C0: a 640x480 frame pair end to end (upload, filter, cloud, voxel, normals,
    # ICP, pose read-back).  The two views alternate through one tracker, so every
    # push registers one frame pair; the first pushes build the two slot graphs and
    # are left out.
    fp = synth.frame_pair(seed=0)
    cam = fp.cam
    seq = [(fp.depth0, fp.bgr0), (fp.depth1, fp.bgr1)] * 10
    out = {}
    for name, g, comp in (("chosen", True, True), ("plain", False, False)):
        lat, res, pose, kern = _track(N, ctx, cam, seq, g, comp, constant_velocity=False)
        rot, tr = synth.pose_error(res[1]["T"], fp.T_gt)
        out[name] = dict(_lat(lat[4:]), iterations=res[1]["iterations"], n_src=res[1]["n_src"],
                         gt_error={"rad": rot, "m": tr}, kernels=kern, T=res[1]["T"])
    rot, tr = synth.pose_error(out["chosen"].pop("T"), out["plain"].pop("T"))
    rows["frame_pair_640x480"] = {"unit": "ms/frame pair (host buffers in, pose out; steady state)",
                                  **out, "chosen_vs_plain_pose_diff": {"rad": rot, "m": tr},
                                  "plain_over_chosen_ms": out["plain"]["p50_ms"] / out["chosen"]["p50_ms"]}

    # C1: one 250k-point pair, three scales
    pr = synth.room_pair(seed=1, n_points=250_000, rot_deg=10.0, trans=0.10)
    s = ctx.cloud_from(pr.src_xyz, pr.src_rgb)
    t = ctx.cloud_from(pr.tgt_xyz, pr.tgt_rgb)
    scales = [N.scale(*x) for x in SCALES]
    one = {}
    for name, g, comp in (("chosen", True, True), ("plain", False, False)):
        plan = N.IcpPlan(ctx, [s], [t], N.icp_params(scales, update_map=N.UPDATE_SE3_EXP, compensated=comp,
                                                      use_graph=g))
        ms = []
        for k in range(8):
            t0 = time.perf_counter()
            r = plan.execute(results=True)[0]
            ms.append((time.perf_counter() - t0) * 1e3)
        rot, tr = synth.pose_error(r["T"], pr.T_gt)
        one[name] = dict(_lat(ms[2:]), iterations=r["iterations"], gt_error={"rad": rot, "m": tr})
    rows["single_pair_250k_three_scale"] = {"unit": "ms/pair", **one,
                                            "plain_over_chosen_ms": one["plain"]["p50_ms"] / one["chosen"]["p50_ms"]}

    # C2: adjoint of 5 unrolled Gauss-Newton steps, 100k-point pair
    pr = synth.room_pair(seed=21, n_points=100_000, rot_deg=10.0, trans=0.10)
    s = ctx.cloud_from(pr.src_xyz, pr.src_rgb)
    t = ctx.cloud_from(pr.tgt_xyz, pr.tgt_rgb)
    ctx.check(ctx.L.gca3d_estimate_normals(ctx.h, t.h, 0.06, 0))
    ctx.check(ctx.L.gca3d_color_gradient(ctx.h, t.h, 0.06))
    G = np.random.default_rng(1).normal(size=(4, 4))
    G[3] = 0
    xi0 = np.zeros(6)
    bufs = {"dxyz": ctx.alloc(12 * 100_000), "drgb": ctx.alloc(12 * 100_000)}
    fwd, bwd = [], []
    for k in range(12):
        t0 = time.perf_counter()
        N.color_icp_vjp(ctx, s, t, xi0, K=5, max_corr=0.05, n_src=100_000)
        t1 = time.perf_counter()
        N.color_icp_vjp(ctx, s, t, xi0, K=5, max_corr=0.05, dT=G, dE=0.3, n_src=100_000, out=bufs)
        t2 = time.perf_counter()
        fwd.append((t1 - t0) * 1e3)
        bwd.append((t2 - t1) * 1e3)
    rows["adjoint_100k_K5"] = {"unit": "ms per call", "forward_only": _lat(fwd[2:]),
                               "forward_and_gradient": _lat(bwd[2:]),
                               "note": "gradient accuracy is tested against FP64 central differences and the "
                                       "FP64 adjoint (tests/test_gpu_vjp.py)"}

    # C4: tracked stream, 640x480 and 1280x720
    scene = synth.frame_scene(1234)
    for name, cam, nf in (("640x480", synth.Camera(), args.stream_frames),
                          ("1280x720", synth.Camera(1280, 720, 1050.0, 1050.0, 639.5, 359.5), args.stream_frames)):
        poses = synth.spline_poses(nf, seed=0)
        frames = [synth.render_rgbd_torch(scene, P, 1000 + k, cam) for k, P in enumerate(poses)]
        row = {"frames": nf}
        for arm, g, comp in (("chosen", True, True), ("plain", False, False)):
            lat, res, pose, kern = _track(N, ctx, cam, frames, g, comp)
            lat = lat[3:]
            rot, tr = synth.pose_error(pose, poses[-1])
            row[arm] = dict(_lat(lat), frames_per_s=1e3 / float(np.mean(lat)),
                            drift={"rad": rot, "m": tr, "per_frame_m": tr / (nf - 1)},
                            mean_iterations=float(np.mean([r["iterations"] for r in res[1:]])),
                            mean_src_points=float(np.mean([r["n_src"] for r in res[1:]])), kernels_per_frame=kern)
        rows[f"stream_{name}"] = row
    return rows


# --------------------------------------------------------------------------- #
# CPU: the reference's algorithm on the host cores
# --------------------------------------------------------------------------- #
def cpu_leg(pairs, res_chosen, res_plain):
    """the CPU baseline (the reference's FP32 algorithm timed on the sample pairs) and,
    untimed, the FP64 oracle as the checker of both GPU arms' poses on every pair"""
    from cuda_3d_gb300 import synth

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    threads = os.cpu_count() or 1
    O.set_threads(threads)
    scales = [O.Scale(*s) for s in SCALES]
    idx = cpu_sample(pairs)
    t0 = time.perf_counter()
    for i in idx:
        p = pairs[i]
        O.multiscale_ref32(p.src_xyz, p.src_rgb, p.tgt_xyz, p.tgt_rgb, scales)
    dt = time.perf_counter() - t0
    cpu = {"value": len(idx) / dt, "unit": "pairs/s", "cores": threads, "kind": "port",
           "sample": sample_text(pairs, idx)}

    runs = [O.multiscale_f64(p.src_xyz, p.src_rgb, p.tgt_xyz, p.tgt_rgb, scales, update_map=O.UPDATE_SE3_EXP)
            for p in pairs]
    runs32 = [O.multiscale_f64(p.src_xyz, p.src_rgb, p.tgt_xyz, p.tgt_rgb, scales, update_map=O.UPDATE_SE3_EXP,
                               search_f32=True) for p in pairs]
    check = {"pairs": len(pairs), "tolerance": {"rad": 1e-5, "m": 1e-5},
             "definition": "rotation angle of R_gpu R_fp64^T and |t_gpu - t_fp64| per pair, FP64 oracle "
                           "(oracle/gca_oracle.c) on the same clouds and schedule; fp32_search: the same oracle "
                           "with correspondences searched on the FP32 points the GPU searches"}
    split = [synth.pose_error(T, T32) for (T, _), (T32, _) in zip(runs, runs32)]
    check["oracle_modes_apart"] = {"max": {"rad": max(x[0] for x in split), "m": max(x[1] for x in split)},
                                   "pairs_beyond_tolerance": [i for i, x in enumerate(split)
                                                              if x[0] > 1e-5 or x[1] > 1e-5]}
    gt = [synth.pose_error(T, p.T_gt) for (T, _), p in zip(runs, pairs)]
    check["oracle_gt_error_max"] = {"rad": max(g[0] for g in gt), "m": max(g[1] for g in gt),
                                    "pair": int(np.argmax([g[0] for g in gt]))}
    for name, res in (("chosen", res_chosen), ("plain", res_plain)):
        if res is None:
            continue
        e = np.array([synth.pose_error(r["T"], T) for r, (T, _) in zip(res, runs)])
        e32 = np.array([synth.pose_error(r["T"], T) for r, (T, _) in zip(res, runs32)])
        same_it = all(list(r["scale_iterations"][:len(SCALES)]) == [x.iterations for x in rr]
                      for r, (_, rr) in zip(res, runs))
        either = [bool((a <= 1e-5).all() or (b <= 1e-5).all()) for a, b in zip(e, e32)]
        check[name] = {"max": {"rad": float(e[:, 0].max()), "m": float(e[:, 1].max())},
                       "median": {"rad": float(np.median(e[:, 0])), "m": float(np.median(e[:, 1]))},
                       "worst_pair": int(np.argmax(e.max(1))), "iterations_equal_oracle": same_it,
                       "within_tolerance": bool((e <= 1e-5).all()),
                       "fp32_search": {"max": {"rad": float(e32[:, 0].max()), "m": float(e32[:, 1].max())},
                                       "worst_pair": int(np.argmax(e32.max(1)))},
                       "within_tolerance_of_either_mode": all(either)}
    return cpu, check


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    pairs = make_workload(args.pairs, rank_seed(args.seed, 0))
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    scales = [O.Scale(*s) for s in SCALES]
    idx = cpu_sample(pairs)

    def step():
        for i in idx:
            p = pairs[i]
            O.multiscale_ref32(p.src_xyz, p.src_rgb, p.tgt_xyz, p.tgt_rgb, scales)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = (time.perf_counter() - t0) / args.steps
    value = len(idx) / dt
    print(json.dumps({
        "impl": "reference", "metric": "colored-ICP pairs/s (64-pair batch, three-scale)", "value": value,
        "unit": "pairs/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(pairs, world),
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                         "sample": "each step: " + sample_text(pairs, idx)},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def run_frame_pair(args):
    """the 640x480 frame pair alone (the per-row measurement of run_rows), e.g. under a
    profiler: the two views alternate through one tracker, every push registers one pair"""
    from cuda_3d_gb300 import build, native as N
    from cuda_3d_gb300 import synth

    build.build()
    ctx = N.Context(0)
    fp = synth.frame_pair(seed=0)
    seq = [(fp.depth0, fp.bgr0), (fp.depth1, fp.bgr1)] * ((args.frame_pair + 1) // 2)
    # --eager: launched eagerly with host convergence checks (what a profiler can follow)
    lat, res, _, kern = _track(N, ctx, fp.cam, seq[:args.frame_pair], not args.eager, True, constant_velocity=False)
    steady = lat[4:] if len(lat) > 6 else lat[1:]
    print(json.dumps({"metric": "640x480 frame pair (ms, host buffers in, pose out)", "pushes": len(lat),
                      **_lat(steady), "iterations": res[-1]["iterations"], "kernels_per_push": kern}))


def run_single_pair(args):
    """the 250k-point pair through three scales alone (the per-row measurement of
    run_rows), e.g. under a profiler"""
    from cuda_3d_gb300 import build, native as N
    from cuda_3d_gb300 import synth

    build.build()
    ctx = N.Context(0)
    pr = synth.room_pair(seed=1, n_points=250_000, rot_deg=10.0, trans=0.10)
    s = ctx.cloud_from(pr.src_xyz, pr.src_rgb)
    t = ctx.cloud_from(pr.tgt_xyz, pr.tgt_rgb)
    plan = N.IcpPlan(ctx, [s], [t], N.icp_params([N.scale(*x) for x in SCALES], update_map=N.UPDATE_SE3_EXP,
                                                 compensated=True, use_graph=not args.eager))
    ms = []
    for _ in range(args.single_pair):
        t0 = time.perf_counter()
        r = plan.execute(results=True)[0]
        ms.append((time.perf_counter() - t0) * 1e3)
    steady = ms[2:] if len(ms) > 4 else ms[1:] or ms
    print(json.dumps({"metric": "250k-point pair, three scales (ms per execute, resident clouds)",
                      "executes": len(ms), **_lat(steady), "iterations": r["iterations"]}))


def main(argv=None):
    args = parse_args(argv)
    if args.impl == "reference":
        run_reference(args)
    elif args.single_pair:
        run_single_pair(args)
    elif args.frame_pair:
        run_frame_pair(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
