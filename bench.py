"""Benchmark: band voxels/s of mesh -> narrow-band SDF + winding-number sign.

Workload (one step): both displaced tori of the boolean/offset workload —
R 1, r 0.3, 1024 x 512 parametric grid (1,048,576 triangles each), gradient
noise 0.02, the second rotated 90 degrees about x and shifted 0.5 in x —
converted to signed narrow-band volumes at voxel 0.002, band 3 voxels.
Synthetic, seeded (baby_shark_gb300.synthetic).

  value : band voxels / s with the meshes resident in HBM (bs_mesh_to_volume_device),
          L2 flushed (256 MiB write) between steps, per-step CUDA events on the
          library's stream.
  e2e   : the same through bs_mesh_to_volume with HOST buffers: vertex/index
          upload and the export of the resulting volumes (origins, values,
          masks) to host memory inside every timed step.
  roofline: the dominant kernel, timed live with CUDA events (stage timing),
          against the FP32 peak measured by bs_diag_fp32_peak when the kernel
          is FP32-bound, or the measured HBM copy bandwidth when it is
          memory-bound.
  cpu_baseline: the oracle (CPU restatement of the reference path, OpenMP,
          all host cores) on a bounded sample of the same workload.

The headline signs on the reference's own tree (the library's default, bit-exact
signs).  Beside it (default run): the boolean / offset / meshing tail on
those volumes (`pipeline`), the library's faster PLOC tree at the reference's
parameters (`fast_tree`) and with the order-3 far field at accuracy scale 1.5
(`order3_beta1.5`), each with its sign differences from the headline, the
256-mesh uneven batch (`batched`), the learned far field against the plain
traversal on 16 M points around the holed subdivision-9 icosphere, training
time included (`learned`), the launch shapes the autotuner picked during
warm-up (`autotuned_launch_shape`), and the other single-GPU workloads
(`other_configs`): the plain remesh of the subdivision-4 icosphere through
dual contouring to a CornerTable, and the holed subdivision-9 icosphere's
conversion on both trees.

Other workloads (`--workload`): `open-icosphere` (4.7 M triangles with
holes, voxel 0.001, signs of a sample checked against exact winding
numbers), `large-union` (16 tori, 12 M triangles, voxel 0.0005: batched
conversion, union, dual contouring, peak device memory), `learned` (the
learned far field against the traversal on points in the padded box).

`--impl reference` times the reference path's CPU implementation (the
oracle port; the Rust crate cannot be built here) on the same metric.
"""
import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

H = 0.002
BAND = 3
# Algorithmic work per unit, counted from the reference's operations.
FLOP_PER_PAIR = 84          # closest point + norm, triangle3.rs:317-382 (face-region path)
CULL_FLOP_PER_PAIR = 20     # voxel to bounding box distance and the cull comparison
WN_FLOP_FAR = 31            # far test + order-1/2 terms, aabb_tree.rs:662-671, 803-816
WN_FLOP_EXACT = 70          # Van Oosterom-Strackee solid angle, aabb_tree.rs:582-615 (atan2 as 20)
WN_FAR_PER_VOXEL = 141.46   # the oracle's traversal of the reference's SAH tree over the whole torus
WN_EXACT_PER_VOXEL = 14.96  # (1,048,576 triangles) from the 4.5 M band voxels of a 1/16 ring slice:
#                             counts per band voxel (oracle/traversal_counts.py)
WN_FLOP_PER_VOXEL = int(round(WN_FAR_PER_VOXEL * WN_FLOP_FAR + WN_EXACT_PER_VOXEL * WN_FLOP_EXACT))
# dram__bytes_read.sum + dram__bytes_write.sum per launch from one ncu capture of
# the half-ring case (k_wn_sign 322 MB for 17,900,503 band voxels,
# k_brick_distance 716 MB for 3,416,413,115 voxel pairs), scaled to a full
# torus by the units processed (35,669,277 voxels; 6,848,421,294 pairs);
# k_rt_sign captured on one full torus (582.8 MB read + 272.0 MB written)
TRAFFIC_PER_LAUNCH = {"k_wn_sign": 642e6, "k_brick_distance": 1436e6, "k_rt_sign": 854.8e6}
# smsp__inst_executed.sum per launch of the same capture of k_rt_sign (one
# full torus, 35,669,277 band voxels): warp instructions, the kernel's real
# bound (it issues on 86 % of the cycles); scaled by the voxels of a launch
RT_SIGN_WARP_INST_PER_VOXEL = 67.74e9 / 35669277
SM_COUNT_GB300 = 152
SCHEDULERS_PER_SM = 4
METRIC = "band voxels/s mesh→SDF+sign: learned/batched vs plain GPU, 0 sign flips"
UNIT = "band_voxels/s"
WORKLOAD = ("two displaced tori, 1,048,576 triangles each, voxel 0.002, band 3: mesh->SDF+sign (plain GPU path; "
            "signs on the reference's own SAH tree, bit-exact)")


def rank_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def meshes(fraction=1.0):
    """Both tori; with fraction < 1 only the triangles of the first part of
    each ring (a smaller case with the same triangle and voxel sizes)."""
    from baby_shark_gb300 import synthetic
    a, b = synthetic.config2()
    if fraction >= 1.0:
        return a, b
    out = []
    for v, f in (a, b):
        nv = 512
        keep = (f.max(axis=1) // nv) < int(1024 * fraction)
        out.append((v, np.ascontiguousarray(f[keep])))
    return out[0], out[1]


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cpu_baseline(seconds_target=15.0):
    """Oracle on a bounded sample: the first 1/16 of torus A's ring (65,536 triangles)."""
    from oracle import binding as ob
    (v, f), _ = meshes()
    nu, nv = 1024, 512
    take = nu // 16
    fs = f[np.isin(f[:, 0] // nv, np.arange(take)) & (f.max(axis=1) < (take + 1) * nv)]
    threads = os.cpu_count() or 1
    ob.set_threads(threads)
    t0 = time.perf_counter()
    vol, stats, _ = ob.mesh_to_volume(v, fs, H, BAND)
    dt = time.perf_counter() - t0
    del vol
    return {"value": stats["band_voxels"] / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "oracle mesh->SDF+sign on %d triangles (1/16 of torus A's ring), %d band voxels, %.2f s"
                      % (len(fs), stats["band_voxels"], dt)}


def combine_ranks(ms, band, world, device="cuda"):
    """Replicas: the job's step time is the slowest rank's, its band voxels
    the sum over ranks (every rank converts its own copy of the workload)."""
    if world == 1:
        return ms, band
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    b = torch.tensor([float(band)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(b, op=dist.ReduceOp.SUM)
    return float(t.item()), int(b.item())


def run_reference(args):
    rank, world, _ = rank_info()
    if rank != 0:
        return
    from oracle import binding as ob
    (v, f), _ = meshes()
    nu, nv = 1024, 512
    take = nu // 32
    fs = f[np.isin(f[:, 0] // nv, np.arange(take)) & (f.max(axis=1) < (take + 1) * nv)]
    threads = os.cpu_count() or 1
    ob.set_threads(threads)
    for _ in range(args.warmup):
        ob.mesh_to_volume(v, fs, H, BAND)
    times, band = [], 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        vol, stats, _ = ob.mesh_to_volume(v, fs, H, BAND)
        times.append(time.perf_counter() - t0)
        band = stats["band_voxels"]
        del vol
    tot = sum(times)
    value = band * args.steps / tot
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": WORKLOAD + "; reference CPU path on a bounded sample"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "oracle (CPU restatement of the reference path; the Rust crate cannot be "
                                       "built on this machine) on %d triangles (1/32 of torus A's ring), "
                                       "%d band voxels per step" % (len(fs), band)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args):
    import ctypes as C

    import torch

    import baby_shark_gb300 as bs
    from baby_shark_gb300 import _native as N
    from baby_shark_gb300 import build as bs_build

    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    bs_build.build()
    L = N.load()
    ctx = bs.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    (va, fa), (vb, fb) = meshes(args.tris_fraction)
    dev = [(torch.from_numpy(v).cuda(), torch.from_numpy(f.astype(np.int32)).cuda()) for v, f in ((va, fa), (vb, fb))]
    torch.cuda.synchronize()
    params = N.M2VParams()
    L.bs_m2v_params_default(C.byref(params))
    params.voxel_size = H
    params.band_width = BAND
    tune_choice = (C.c_int32 * 3)()
    tune_ms = (C.c_float * 11)()
    if args.pipeline_only:
        params.voxel_size = args.voxel_size
        # the boolean / offset / dual-contouring tail alone, once (a profiling case)
        print(json.dumps({"pipeline": pipeline_secondary(ctx, params, dev, L, N, bs, C),
                          "tris_fraction": args.tris_fraction, "voxel_size": args.voxel_size}))
        return
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step_device():
        outs = []
        band = 0
        for x, t in dev:
            out = C.c_void_p()
            N.check(L.bs_mesh_to_volume_device(ctx.h, x.data_ptr(), x.shape[0], t.data_ptr(), t.shape[0],
                                               C.byref(params), C.byref(out)), ctx.h)
            vol = bs.Volume(out, ctx)
            band += vol.counts()["active_voxels"]
            outs.append(vol)
        return band, outs

    # end to end: the meshes sit in pinned host memory; each step uploads them
    # through the host-pointer C ABI and exports every volume (origins, values,
    # masks) into pinned host buffers
    host_in = [(torch.from_numpy(v).pin_memory(), torch.from_numpy(f.astype(np.int32)).pin_memory())
               for v, f in ((va, fa), (vb, fb))]
    host_out = {}

    def export_pinned(vol, k):
        n = vol.counts()["leaves"]
        if k not in host_out or host_out[k][1].shape[0] < n:
            cap = int(n * 1.25) + 16
            host_out[k] = (torch.empty((cap, 3), dtype=torch.int32).pin_memory(),
                           torch.empty((cap, 512), dtype=torch.float32).pin_memory(),
                           torch.empty((cap, 16), dtype=torch.int32).pin_memory())
        o, val, m = host_out[k]
        N.check(L.bs_volume_export(ctx.h, vol.h, o.data_ptr(), val.data_ptr(), m.data_ptr()), ctx.h)
        return n * (12 + 2048 + 64)

    export_s = []  # host time of the exports of each step (the rest is upload + conversion)

    def step_e2e():
        band, h2d, d2h = 0, 0, 0
        te = 0.0
        for k, (x, t) in enumerate(host_in):
            out = C.c_void_p()
            N.check(L.bs_mesh_to_volume(ctx.h, x.data_ptr(), x.shape[0], t.data_ptr(), t.shape[0], C.byref(params),
                                        C.byref(out)), ctx.h)
            vol = bs.Volume(out, ctx)
            t0 = time.perf_counter()
            d2h += export_pinned(vol, k)
            te += time.perf_counter() - t0
            band += vol.counts()["active_voxels"]
            h2d += x.numel() * 4 + t.numel() * 4
            del vol
        export_s.append(te)
        return band, h2d, d2h

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # autotuned launch shapes (on torus A), part of the warm-up
    tuned = None
    if args.autotune:
        N.check(L.bs_autotune_mesh_to_volume(ctx.h, dev[0][0].data_ptr(), dev[0][0].shape[0], dev[0][1].data_ptr(),
                                             dev[0][1].shape[0], C.byref(params), tune_choice, tune_ms), ctx.h)
        shapes = ["64x8", "64x16", "64x32", "128x8", "128x16", "128x32", "256x8", "256x16"]
        tuned = {"dist_threads": int(tune_choice[0]), "wn_warps": int(tune_choice[1]),
                 "dist_tile": int(tune_choice[2]),
                 "distance_ms_threads_x_tile": {k: round(float(x), 2) for k, x in zip(shapes, tune_ms[:8])},
                 "sign_ms_2_4_8_warps": [round(float(x), 2) for x in tune_ms[8:]]}
    for _ in range(args.warmup):
        step_device()
    ctx.synchronize()
    # ---- timed region (device-resident inputs) ----
    ctx.set_stage_timing(True)
    ctx.stage_times(reset=True)
    launches0 = ctx.kernel_launches
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    ctx.synchronize()
    per_step, band = [], 0
    # the interpreter's collector stays off while steps are timed (a
    # collection pause would be host time between the library's launches)
    gc.collect()
    gc.disable()
    with torch.cuda.stream(stream):
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            band, outs = step_device()
            e1.record(stream)
            del outs
            flush.fill_(1.0)  # L2 flush between steps (outside the event pair)
            e1.synchronize()
            per_step.append(e0.elapsed_time(e1))
    ctx.synchronize()
    torch.cuda.synchronize()
    gc.enable()
    barrier()
    clk = clocks.stop()
    launches = ctx.kernel_launches - launches0
    stages = ctx.stage_times(reset=True)
    ctx.set_stage_timing(False)
    stats = ctx.last_stats()
    ms = sum(per_step) / len(per_step)
    ms, band_all = combine_ranks(ms, band, world, "cuda")
    value = band_all / (ms / 1000.0)

    # ---- e2e: host buffers through the C ABI, upload + export inside each step ----
    for _ in range(max(1, args.warmup)):
        step_e2e()
    t_e2e = []
    del export_s[:]
    gc.collect()
    gc.disable()
    clocks_e2e = ClockSampler(local)
    clocks_e2e.start()
    for _ in range(args.steps):
        ctx.synchronize()
        t0 = time.perf_counter()
        b_e2e, h2d, d2h = step_e2e()
        ctx.synchronize()
        t_e2e.append(time.perf_counter() - t0)
    gc.enable()
    clk_e2e = clocks_e2e.stop()
    e2e_ms, e2e_band = combine_ranks(1000.0 * sum(t_e2e) / len(t_e2e), b_e2e, world, "cuda")
    e2e_value = e2e_band / (e2e_ms / 1000.0)

    # ---- roofline of the dominant kernel ----
    top = max(stages.items(), key=lambda kv: kv[1][0])
    name, (tot_ms, nl) = top
    peaks, src = measured_peaks()
    fp32_peak = fp32_peak_tflops(ctx)
    per_launch_s = tot_ms / nl / 1000.0
    # stats are of the last conversion (torus B); both tori are the same size class
    extra = {}
    if name == "k_brick_distance":
        ev = stats["voxel_pairs_evaluated"]
        flops = FLOP_PER_PAIR * ev + CULL_FLOP_PER_PAIR * stats["voxel_pairs"]
        algo = ("%d FLOP x %d evaluated (voxel, sub-triangle) pairs + %d FLOP cull test x %d pairs per launch"
                % (FLOP_PER_PAIR, ev, CULL_FLOP_PER_PAIR, stats["voxel_pairs"]))
        extra["reference_equivalent_tflops"] = FLOP_PER_PAIR * stats["voxel_pairs"] / per_launch_s / 1e12
        extra["pairs_evaluated_fraction"] = ev / max(1, stats["voxel_pairs"])
    elif name == "k_rt_sign":
        flops = WN_FLOP_PER_VOXEL * stats["active_voxels"]
        # one traversal per voxel of the reference's own tree: the executed
        # far-field and exact counts are the reference's (per voxel)
        executed = WN_FLOP_FAR * stats["wn_far"] + WN_FLOP_EXACT * stats["wn_exact"]
        extra["executed_tflops"] = executed / per_launch_s / 1e12
        extra["executed_flop_per_launch"] = executed
        extra["far_per_voxel"] = stats["wn_far"] / max(1, stats["active_voxels"])
        extra["exact_per_voxel"] = stats["wn_exact"] / max(1, stats["active_voxels"])
        algo = ("%d FLOP per band voxel (the reference's own traversal: %.0f far-field nodes x %d FLOP + "
                "%.0f exact triangles x %d FLOP, counted by the oracle) x %d voxels per launch"
                % (WN_FLOP_PER_VOXEL, WN_FAR_PER_VOXEL, WN_FLOP_FAR, WN_EXACT_PER_VOXEL, WN_FLOP_EXACT,
                   stats["active_voxels"]))
        # the bound that holds it: warp-instruction issue (one per scheduler
        # per cycle) at the SM clock sampled during the timed region
        if clk.get("sm_mhz"):
            inst = RT_SIGN_WARP_INST_PER_VOXEL * stats["active_voxels"]
            issue_peak = SM_COUNT_GB300 * SCHEDULERS_PER_SM * clk["sm_mhz"] * 1e6
            extra["issue_bound"] = {
                "warp_instructions_per_launch": inst, "achieved_per_s": inst / per_launch_s,
                "peak_per_s": issue_peak, "frac": inst / per_launch_s / issue_peak,
                "source": "smsp__inst_executed.sum of one ncu capture (profiles/k_rt_sign_one_torus.md), per band "
                          "voxel; peak = 152 SMs x 4 schedulers x the sampled SM clock"}
    elif name == "k_wn_sign":
        flops = WN_FLOP_PER_VOXEL * stats["active_voxels"]
        # what the warp-coherent traversal executes: every lane of a warp evaluates
        # each node the warp takes as far, and each leaf the warp opens exactly
        executed = 32 * (WN_FLOP_FAR * stats["wn_warp_far"] + WN_FLOP_EXACT * stats["wn_warp_exact"])
        extra["executed_tflops"] = executed / per_launch_s / 1e12
        extra["executed_flop_per_launch"] = executed
        algo = ("%d FLOP per band voxel (the reference's own traversal: %.0f far-field nodes x %d FLOP + "
                "%.0f exact triangles x %d FLOP, counted by the oracle) x %d voxels per launch"
                % (WN_FLOP_PER_VOXEL, WN_FAR_PER_VOXEL, WN_FLOP_FAR, WN_EXACT_PER_VOXEL, WN_FLOP_EXACT,
                   stats["active_voxels"]))
    else:
        flops = None
        algo = None
    if flops is not None:
        achieved = flops / per_launch_s / 1e12
        roof = {"kernel": name, "bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": achieved / fp32_peak if fp32_peak else None, "traffic": TRAFFIC_PER_LAUNCH.get(name),
                "peak_source": "measured on this GPU by bs_diag_fp32_peak (FFMA loop); MEASURED_PEAKS.json "
                               "holds no FP32 figure",
                "algorithmic": algo, **extra}
    else:
        roof = {"kernel": name, "bound": "hbm", "achieved": None, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                "frac": None, "traffic": None, "peak_source": src}
    roof["share_of_step"] = tot_ms / sum(v[0] for v in stages.values())
    roof["launch_ms"] = tot_ms / nl

    pipe = pipeline_secondary(ctx, params, dev, L, N, bs, C) if args.pipeline else None
    fast_tree = variant_secondary(ctx, params, dev, L, N, bs, C, args) if args.order3 else None
    fast3 = variant_secondary(ctx, params, dev, L, N, bs, C, args, order=3, beta=1.5) if args.order3 else None
    batch = batch_secondary(ctx, L, N, bs, C, args.batch_meshes) if args.batch_meshes else None
    learned = None
    open_mesh = None
    if args.learned_queries or args.configs:
        from baby_shark_gb300 import synthetic as syn
        open_mesh = syn.open_icosphere()
    if args.learned_queries:
        vl, fl = open_mesh
        learned = learned_secondary(ctx, vl, fl, args.learned_queries, steps=2, warmup=1, validation=100000)
        learned["workload"] = ("subdivision-9 icosphere with holes (%d triangles), %d points uniform in the box "
                               "padded by 10 %%" % (len(fl), args.learned_queries))

    others = configs_secondary(ctx, L, N, bs, C, open_mesh) if args.configs else None

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD if args.tris_fraction >= 1.0 else
                       WORKLOAD + " (first %.3g of each ring)" % args.tris_fraction,
                       "triangles_per_step": int(len(fa) + len(fb)),
                       "band_voxels_per_step": int(band), "l2": "flushed between steps (256 MiB write)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "ms_per_step": e2e_ms, "steps_ms": [round(t * 1e3, 2) for t in t_e2e],
                    "export_ms": [round(t * 1e3, 2) for t in export_s], "clocks": clk_e2e},
            "gpu_launches": int(launches),
            "roofline": roof,
            "clocks": clk,
            "stages_ms_per_step": {k: v[0] / args.steps for k, v in sorted(stages.items(), key=lambda kv: -kv[1][0])},
            "last_stats": stats,
            "pipeline": pipe,
            "batched": batch,
            "autotuned_launch_shape": tuned,
            "fast_tree": fast_tree,
            "learned": learned,
            "order3_beta1.5": fast3,
            "other_configs": others}
    if rank == 0:
        if world == 1:
            line["cpu_baseline"] = cpu_baseline()
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_open(args):
    """The non-watertight workload: subdivision-9 icosphere (5,242,880
    triangles) with 4-octave radial noise of amplitude 0.1 and 10 % of faces
    removed, voxel 0.001, band 3.  Band voxels/s of mesh -> SDF + sign with the
    mesh resident in HBM, and the signs of a seeded sample of band voxels
    against exact winding numbers (direct sum, bs_winding_numbers_exact)."""
    import ctypes as C

    import torch

    import baby_shark_gb300 as bs
    from baby_shark_gb300 import _native as N
    from baby_shark_gb300 import build as bs_build
    from baby_shark_gb300 import synthetic

    bs_build.build()
    L = N.load()
    ctx = bs.Context(0)
    t_gen = time.perf_counter()
    v, f = synthetic.open_icosphere()
    t_gen = time.perf_counter() - t_gen
    h = 0.001
    x = torch.from_numpy(v).cuda()
    t = torch.from_numpy(f.astype(np.int32)).cuda()
    params = N.M2VParams()
    L.bs_m2v_params_default(C.byref(params))
    params.voxel_size = h
    params.band_width = BAND
    params.wn_order = args.wn_order
    params.wn_beta = args.wn_beta
    if args.wn_order == 3:
        params.wn_tree = 1  # the third-order term lives on the library's tree
    stream = torch.cuda.ExternalStream(ctx.stream)

    def step():
        out = C.c_void_p()
        N.check(L.bs_mesh_to_volume_device(ctx.h, x.data_ptr(), x.shape[0], t.data_ptr(), t.shape[0],
                                           C.byref(params), C.byref(out)), ctx.h)
        return bs.Volume(out, ctx)

    for _ in range(args.warmup):
        step()
    ctx.synchronize()
    ms = []
    vol = None
    for _ in range(args.steps):
        vol = None
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        vol = step()
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    band = vol.counts()["active_voxels"]
    stats = ctx.last_stats()
    # sign check on a seeded sample of band voxels
    o, val, m = vol.export()
    act = np.unpackbits(m.view(np.uint8), bitorder="little").reshape(len(o), 512).astype(bool)
    li, vi = np.nonzero(act)
    rng = np.random.default_rng(7)
    pick = rng.choice(len(li), size=min(args.validation, len(li)), replace=False)
    li, vi = li[pick], vi[pick]
    vox = o[li] + np.stack([vi >> 6, (vi >> 3) & 7, vi & 7], 1)
    pts = vox.astype(np.float32) * np.float32(h)
    t0 = time.perf_counter()
    wn = bs.winding_numbers_exact(x, t, pts, ctx=ctx).cpu().numpy()
    t_exact = time.perf_counter() - t0
    inside = np.signbit(val[li, vi])
    mism = inside != (wn >= 0.2)
    line = {"metric": METRIC, "value": band / (min(ms) / 1000.0), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": min(ms), "higher_is_better": True, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "open icosphere: subdivision 9, 4-octave radial noise 0.1, 10%% of faces "
                                   "removed (%d triangles), voxel 0.001, band 3, far field order %d, "
                                   "beta %g" % (len(f), args.wn_order, args.wn_beta),
                       "band_voxels_per_step": int(band), "generation_s": t_gen},
            "sign_vs_exact": {"sample": int(len(li)), "mismatches": int(mism.sum()),
                              "mismatches_within_0.01_of_threshold": int((mism & (np.abs(wn - 0.2) < 0.01)).sum()),
                              "exact_pass_s": t_exact},
            "last_stats": stats}
    print(json.dumps(line))


def variant_secondary(ctx, params, dev, L, N, bs, C, args, tree=1, order=2, beta=2.0):
    """The same conversion with another sign tree / far-field order /
    accuracy scale: band voxels/s, and how many band voxel signs differ from
    the headline (the reference's tree, order 2, scale 2).  tree 1 is the
    library's PLOC tree with its warp-coherent traversal."""
    import copy

    import torch
    p3 = copy.copy(params)
    p3.wn_tree = tree
    p3.wn_order = order
    p3.wn_beta = beta
    stream = torch.cuda.ExternalStream(ctx.stream)

    def conv(p):
        vols = []
        for x, t in dev:
            out = C.c_void_p()
            N.check(L.bs_mesh_to_volume_device(ctx.h, x.data_ptr(), x.shape[0], t.data_ptr(), t.shape[0],
                                               C.byref(p), C.byref(out)), ctx.h)
            vols.append(bs.Volume(out, ctx))
        return vols

    for _ in range(max(1, args.warmup // 2)):
        conv(p3)
    ms = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        v3 = conv(p3)
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    band = sum(v.counts()["active_voxels"] for v in v3)
    v2 = conv(params)
    diff = 0
    for a, b in zip(v2, v3):
        (_, va, ma), (_, vb, mb) = a.export(), b.export()
        act = np.unpackbits(ma.view(np.uint8), bitorder="little").reshape(len(ma), 512).astype(bool)
        diff += int(np.sum(np.signbit(va[act]) != np.signbit(vb[act])))
    return {"value": band / (min(ms) / 1000.0), "unit": UNIT, "ms_per_step": min(ms),
            "sign_differences_vs_headline": diff, "band_voxels": int(band),
            "tree": "PLOC (warp-coherent traversal)" if tree == 1 else "reference SAH", "order": order, "beta": beta}


def learned_secondary(ctx, v, f, n_q, steps=2, warmup=1, validation=200000, seed=12345):
    """The learned far field against the plain traversal on one mesh:
    winding numbers (signs at the 0.2 threshold) of n_q points uniform in the
    bounding box padded by 10 %.  Plain = the tree traversal (the reference's
    order-2 far field, accuracy scale 2, the library's PLOC tree with
    Morton-sorted queries) for every point; learned = train a network (band
    volume, sampling, traversal labels, training, calibration: all timed) and
    answer the points outside the band whose prediction is confident from the
    network, the rest from the same traversal.  Both include the tree build.
    Returns both times, their ratio, the share of points the network
    answered, the sign differences between the two, and signs of a seeded
    sample against exact winding numbers."""
    import torch

    import baby_shark_gb300 as bs

    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    lo = torch.from_numpy(v.min(axis=0)).cuda()
    hi = torch.from_numpy(v.max(axis=0)).cuda()
    ext = hi - lo
    q = (lo - 0.1 * ext + torch.rand(n_q, 3, generator=gen, device="cuda") * (1.2 * ext)).contiguous()
    torch.cuda.synchronize()

    def plain():
        ctx.synchronize()
        t0 = time.perf_counter()
        tree = bs.WindingNumbers.from_mesh((v, f), order=2, ctx=ctx)
        out = torch.empty(n_q, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        bs_native = bs._native
        bs_native.check(bs_native.load().bs_winding_numbers_approximate(ctx.h, tree.h, q.data_ptr(), n_q, 2.0,
                                                                        out.data_ptr()), ctx.h)
        ctx.synchronize()
        return time.perf_counter() - t0, out

    def learned():
        ctx.synchronize()
        t0 = time.perf_counter()
        lf = bs.LearnedFarField.train((v, f), ctx=ctx, seed=1)
        t1 = time.perf_counter()
        out, n_trav = lf.classify(q)
        ctx.synchronize()
        return time.perf_counter() - t0, time.perf_counter() - t1, out, n_trav, lf

    for _ in range(max(1, warmup)):
        plain()
        learned()
    tp, wp = min((plain() for _ in range(max(1, steps))), key=lambda r: r[0])
    runs = [learned() for _ in range(max(1, steps))]
    tl, tq, wl, n_trav, lf = min(runs, key=lambda r: r[0])
    diff = int((wp > 0.2).ne(wl > 0.2).sum().item())
    # exact check on a seeded sample
    idx = torch.randperm(n_q, generator=gen, device="cuda")[:validation]
    exact = bs.winding_numbers_exact(v, f, q[idx], ctx=ctx)
    ex = (exact > 0.2).cpu().numpy()
    mism_plain = int(np.sum(ex != (wp[idx] > 0.2).cpu().numpy()))
    mism_learned = int(np.sum(ex != (wl[idx] > 0.2).cpu().numpy()))
    answered = 1.0 - n_trav / n_q
    # tensor-core work of the network (forward 2 (64 x 64 + 64 x 64 + 64) FLOP a sample, training about 3x)
    fwd_flop = 2 * (64 * 64 + 64 * 64 + 64)
    train_samples = 2_000_000 * 16
    return {"points": n_q, "triangles": int(len(f)),
            "plain_s": tp, "plain_points_per_s": n_q / tp,
            "learned_s": tl, "learned_points_per_s": n_q / tl, "learned_over_plain": tp / tl,
            "learned_breakdown_s": dict(lf.timings, classify_s=tq),
            "network_answered_fraction": answered,
            "sign_differences_learned_vs_plain": diff,
            "validation": {"points": int(validation), "plain_vs_exact": mism_plain,
                           "learned_vs_exact": mism_learned},
            "calibration": lf.calibration, "margin": lf.margin,
            "epoch_loss": [float(x) for x in lf.epoch_loss],
            "network_tflops": {"training": 3 * fwd_flop * train_samples / lf.timings["training_s"] / 1e12,
                               "inference_in_classify": fwd_flop * n_q / tq / 1e12}}


def run_learned(args):
    """The learned far field on the non-watertight workload (subdivision-9
    icosphere, 4.7 M triangles, 4-octave noise 0.1, 10 % of faces removed):
    learned_secondary on --queries points."""
    import baby_shark_gb300 as bs
    from baby_shark_gb300 import build as bs_build
    from baby_shark_gb300 import synthetic

    bs_build.build()
    ctx = bs.Context(0)
    v, f = synthetic.open_icosphere()
    r = learned_secondary(ctx, v, f, args.queries, args.steps, args.warmup, args.validation)
    line = {"metric": "winding numbers / s of points in the padded box (learned far field vs traversal)",
            "value": r["learned_points_per_s"], "unit": "points/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "dtype": "bf16 network, f32 traversal",
            "data": "synthetic",
            "config": {"workload": "subdivision-9 icosphere, 4-octave noise 0.1, 10 %% of faces removed (%d "
                                   "triangles); %d query points uniform in the box padded by 10 %%"
                                   % (len(f), args.queries), "parallelism": "single GPU"},
            **r}
    print(json.dumps(line), flush=True)


def run_large_union(args):
    """The large combined workload: the union of 16 displaced tori
    (synthetic.large_union: major radius 0.5-1.5, minor 0.1-0.4, random
    rotation and centre in [-1, 1]^3, about 12 M triangles), voxel 0.0005,
    band 3.  All tori go to SDF + sign in one batched call with the meshes
    resident in HBM, the 16 volumes are united pairwise, and the union is
    dual-contoured (triangles counted on the device, not copied out).
    Reports band voxels/s of the conversion, the union and dual-contouring
    times, output triangles/s and the peak device memory of the library's
    pool (the whole run has to stay within 180 GB)."""
    import ctypes as C

    import torch

    import baby_shark_gb300 as bs
    from baby_shark_gb300 import _native as N
    from baby_shark_gb300 import build as bs_build
    from baby_shark_gb300 import synthetic

    bs_build.build()
    L = N.load()
    ctx = bs.Context(0)
    t_gen = time.perf_counter()
    meshes = synthetic.large_union()
    t_gen = time.perf_counter() - t_gen
    h = 0.0005
    K = len(meshes)
    xyz = torch.from_numpy(np.concatenate([v for v, _ in meshes])).cuda()
    tri = torch.from_numpy(np.concatenate([f for _, f in meshes]).astype(np.int32)).cuda()
    nv = np.array([len(v) for v, _ in meshes], np.uint64)
    nt = np.array([len(f) for _, f in meshes], np.uint64)
    P = (N.M2VParams * K)()
    for k in range(K):
        L.bs_m2v_params_default(C.byref(P[k]))
        P[k].voxel_size = h
        P[k].band_width = BAND
    torch.cuda.synchronize()

    def once():
        ctx.synchronize()
        t0 = time.perf_counter()
        outs = (C.c_void_p * K)()
        N.check(L.bs_mesh_to_volume_batch_device(ctx.h, K, xyz.data_ptr(), nv.ctypes.data, tri.data_ptr(),
                                                 nt.ctypes.data, P, outs), ctx.h)
        vols = [bs.Volume(C.c_void_p(outs[k]), ctx) for k in range(K)]
        ctx.synchronize()
        t1 = time.perf_counter()
        band = sum(v.counts()["active_voxels"] for v in vols)
        leaves_in = sum(v.counts()["leaves"] for v in vols)
        ctx.synchronize()
        t1b = time.perf_counter()
        while len(vols) > 1:
            nxt = [vols[i].union(vols[i + 1]) for i in range(0, len(vols) - 1, 2)]
            if len(vols) % 2:
                nxt.append(vols[-1])
            vols = nxt
        u = vols[0]
        ctx.synchronize()
        t2 = time.perf_counter()
        n_tris = C.c_uint64()
        N.check(L.bs_dual_contour(ctx.h, u.h, C.c_float(h), None, 0, C.byref(n_tris)), ctx.h)
        ctx.synchronize()
        t3 = time.perf_counter()
        cu = u.counts()
        return {"convert_s": t1 - t0, "union_s": t2 - t1b, "dc_s": t3 - t2, "band_voxels": int(band),
                "leaves_in": int(leaves_in), "union_leaves": int(cu["leaves"]), "union_tiles": int(cu["tiles"]),
                "union_active_voxels": int(cu["active_voxels"]), "dc_triangles": int(n_tris.value)}

    for _ in range(args.warmup):
        once()
    ctx.memory_reset(trim=True)
    runs = [once() for _ in range(max(1, args.steps))]
    mem = ctx.memory()
    best = min(runs, key=lambda r: r["convert_s"] + r["union_s"] + r["dc_s"])
    line = {"metric": "band voxels/s mesh->SDF+sign (batched, 16 tori) and output triangles/s",
            "value": best["band_voxels"] / best["convert_s"], "unit": UNIT, "n_gpus": 1,
            "steps": len(runs), "warmup": args.warmup, "higher_is_better": True, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "union of 16 displaced tori (synthetic.large_union, %d triangles), "
                                   "voxel 0.0005, band 3: batched mesh->SDF+sign, pairwise union, dual contouring"
                                   % int(nt.sum()),
                       "parallelism": "single GPU"},
            "convert_ms": best["convert_s"] * 1e3, "union_ms": best["union_s"] * 1e3,
            "dc_ms": best["dc_s"] * 1e3,
            "dc_triangles_per_s": best["dc_triangles"] / best["dc_s"] if best["dc_s"] else None,
            "pipeline_ms": (best["convert_s"] + best["union_s"] + best["dc_s"]) * 1e3,
            "counts": {k: best[k] for k in ("band_voxels", "leaves_in", "union_leaves", "union_tiles",
                                            "union_active_voxels", "dc_triangles")},
            "device_memory_gb": {"peak_in_use": mem["used_high"] / 1e9, "reserved": mem["reserved"] / 1e9,
                                 "workload_limit": 180.0},
            "generation_s": t_gen}
    print(json.dumps(line), flush=True)


def batch_secondary(ctx, L, N, bs, C, n_meshes, reps=3):
    """The uneven-batch workload (synthetic.uneven_batch: icospheres and
    displaced tori, 1k-500k triangles, grids 64^3-512^3, band 3), resident in
    HBM: the meshes one call each (bs_mesh_to_volume_device, volume freed
    after each) against one bs_mesh_to_volume_batch_device call.  Both are
    timed from the host around the whole set, best of `reps`, after one
    warm-up run each."""
    import torch
    from baby_shark_gb300 import synthetic
    t_gen = time.perf_counter()
    batch = synthetic.uneven_batch(n_meshes)
    t_gen = time.perf_counter() - t_gen
    K = len(batch)
    xyz = torch.from_numpy(np.concatenate([v for v, _, _ in batch])).cuda()
    tri = torch.from_numpy(np.concatenate([f for _, f, _ in batch]).astype(np.int32)).cuda()
    nv = np.array([len(v) for v, _, _ in batch], np.uint64)
    nt = np.array([len(f) for _, f, _ in batch], np.uint64)
    vb = np.concatenate([[0], np.cumsum(nv)]).astype(np.int64)
    tb = np.concatenate([[0], np.cumsum(nt)]).astype(np.int64)
    P = (N.M2VParams * K)()
    for k, (_, _, h) in enumerate(batch):
        L.bs_m2v_params_default(C.byref(P[k]))
        P[k].voxel_size = float(h)
        P[k].band_width = BAND
    torch.cuda.synchronize()

    def sequential():
        band = 0
        for k in range(K):
            out = C.c_void_p()
            N.check(L.bs_mesh_to_volume_device(ctx.h, xyz.data_ptr() + 12 * int(vb[k]), int(nv[k]),
                                               tri.data_ptr() + 12 * int(tb[k]), int(nt[k]), C.byref(P[k]),
                                               C.byref(out)), ctx.h)
            vol = bs.Volume(out, ctx)
            band += vol.counts()["active_voxels"]
            del vol
        return band

    def batched():
        outs = (C.c_void_p * K)()
        N.check(L.bs_mesh_to_volume_batch_device(ctx.h, K, xyz.data_ptr(), nv.ctypes.data, tri.data_ptr(),
                                                 nt.ctypes.data, P, outs), ctx.h)
        vols = [bs.Volume(C.c_void_p(outs[k]), ctx) for k in range(K)]
        band = sum(v.counts()["active_voxels"] for v in vols)
        del vols
        return band

    def best(fn):
        fn()
        ctx.synchronize()
        ts, band = [], 0
        for _ in range(reps):
            ctx.synchronize()
            t0 = time.perf_counter()
            band = fn()
            ctx.synchronize()
            ts.append(time.perf_counter() - t0)
        return min(ts), band

    l0 = ctx.kernel_launches
    t_seq, band_seq = best(sequential)
    l1 = ctx.kernel_launches
    t_bat, band_bat = best(batched)
    l2 = ctx.kernel_launches
    assert band_seq == band_bat
    return {"workload": "%d meshes (synthetic.uneven_batch): %d triangles, icospheres and displaced tori of "
                        "1k-500k triangles, grids 64^3-512^3, band 3" % (K, int(nt.sum())),
            "band_voxels": int(band_bat),
            "sequential_ms": t_seq * 1e3, "batched_ms": t_bat * 1e3,
            "sequential_band_voxels_per_s": band_seq / t_seq, "batched_band_voxels_per_s": band_bat / t_bat,
            "batched_over_sequential": t_seq / t_bat,
            "launches_sequential": int((l1 - l0) // (reps + 1)), "launches_batched": int((l2 - l1) // (reps + 1)),
            "generation_s": t_gen}


def configs_secondary(ctx, L, N, bs, C, open_mesh=None, reps=3):
    """The other single-GPU workloads, timed beside the headline:

    - the plain voxel remesh (icosphere subdivision 4, 5,120 triangles, noise
      0.05, voxel 0.02, band 3): mesh -> SDF + sign -> dual contouring ->
      CornerTable through the public API from host arrays, host clock around
      the whole remesh, best of `reps` after a warm-up;
    - the non-watertight conversion (subdivision-9 icosphere, 4-octave noise
      0.1, 10 % of faces removed, 5,242,880 -> about 4.7 M triangles, voxel
      0.001, band 3): mesh -> SDF + sign with the mesh resident in HBM, CUDA
      events on the library stream, best of `reps`, on the reference's tree
      (the bit-exact default) and on the library's fast tree."""
    import torch
    from baby_shark_gb300 import synthetic
    out = {}
    v1, f1 = synthetic.config1()

    def remesh():
        vol = bs.MeshToVolume(ctx).with_voxel_size(0.02).with_narrow_band_width(BAND).convert((v1, f1))
        ct = bs.CornerTable.from_dual_contouring(vol, 0.02)
        c = ct.counts()
        return vol.counts()["active_voxels"], c["faces"], c["vertices"]

    remesh()
    ts = []
    for _ in range(reps):
        ctx.synchronize()
        t0 = time.perf_counter()
        band, faces, verts = remesh()
        ts.append(time.perf_counter() - t0)
    t = min(ts)
    out["remesh_icosphere_sub4"] = {
        "workload": "icosphere subdivision 4 (%d triangles), radial noise 0.05, voxel 0.02, band 3: mesh -> SDF + "
                    "sign -> dual contouring -> CornerTable from host arrays" % len(f1),
        "ms": t * 1e3, "band_voxels": int(band), "band_voxels_per_s": band / t,
        "corner_table_faces": int(faces), "corner_table_vertices": int(verts), "faces_per_s": faces / t}
    if open_mesh is None:
        open_mesh = synthetic.open_icosphere()
    vo, fo = open_mesh
    x = torch.from_numpy(vo).cuda()
    tt = torch.from_numpy(fo.astype(np.int32)).cuda()
    stream = torch.cuda.ExternalStream(ctx.stream)
    res = {}
    for tree in (0, 1):
        P = N.M2VParams()
        L.bs_m2v_params_default(C.byref(P))
        P.voxel_size = 0.001
        P.band_width = BAND
        P.wn_tree = tree

        def step():
            o = C.c_void_p()
            N.check(L.bs_mesh_to_volume_device(ctx.h, x.data_ptr(), x.shape[0], tt.data_ptr(), tt.shape[0],
                                               C.byref(P), C.byref(o)), ctx.h)
            return bs.Volume(o, ctx)

        vol = step()
        del vol
        ms = []
        band = 0
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            vol = step()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            band = vol.counts()["active_voxels"]
            del vol
        res["reference_tree" if tree == 0 else "fast_tree"] = {"ms": min(ms), "band_voxels": int(band),
                                                               "band_voxels_per_s": band / (min(ms) / 1e3)}
    out["open_icosphere_sub9"] = {
        "workload": "subdivision-9 icosphere, 4-octave radial noise 0.1, 10 %% of faces removed (%d triangles), "
                    "voxel 0.001, band 3: mesh -> SDF + sign, mesh resident in HBM" % len(fo), **res}
    return out


def pipeline_secondary(ctx, params, dev, L, N, bs, C):
    """The boolean workload's tail, once per boolean: A op B, then offset +0.01
    and -0.01 (each on its own copy), then dual contouring of each (and, as the
    reference's other mesher, marching cubes); CUDA events on the library
    stream around every stage.  Returns ms per stage and the output triangles."""
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream)

    def m2v(k):
        out = C.c_void_p()
        x, t = dev[k]
        N.check(L.bs_mesh_to_volume_device(ctx.h, x.data_ptr(), x.shape[0], t.data_ptr(), t.shape[0],
                                           C.byref(params), C.byref(out)), ctx.h)
        return bs.Volume(out, ctx)

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = fn()
        e1.record(stream)
        e1.synchronize()
        return r, e0.elapsed_time(e1)

    res = {}
    tris_total, dc_ms_total, mc_total, mc_ms_total = 0, 0.0, 0, 0.0
    for op in ("subtract", "union", "intersect"):
        a, b = m2v(0), m2v(1)
        c, t_csg = timed(lambda: getattr(a, op)(b))
        d = {"csg_ms": t_csg, "leaves": c.counts()["leaves"], "tiles": c.counts()["tiles"]}
        for sign, dist in (("plus", 0.01), ("minus", -0.01)):
            cc = c.clone()
            _, t_off = timed(lambda: cc.offset(dist))
            st = ctx.last_stats()
            d["offset_%s_relax_passes" % sign] = st.get("offset_passes")
            d["offset_%s_leaf_sweeps" % sign] = st["offset_leaf_sweeps"]
            n = C.c_uint64()
            _, t_dc = timed(lambda: N.check(L.bs_dual_contour(ctx.h, cc.h, params.voxel_size, None, 0, C.byref(n)),
                                            ctx.h))
            d["offset_%s_ms" % sign] = t_off
            d["dc_%s_ms" % sign] = t_dc
            d["dc_%s_triangles" % sign] = int(n.value)
            tris_total += int(n.value)
            dc_ms_total += t_dc
            nm = C.c_uint64()
            _, t_mc = timed(lambda: N.check(L.bs_marching_cubes(ctx.h, cc.h, params.voxel_size, None, 0, C.byref(nm)),
                                            ctx.h))
            d["mc_%s_ms" % sign] = t_mc
            d["mc_%s_triangles" % sign] = int(nm.value)
            mc_total += int(nm.value)
            mc_ms_total += t_mc
            del cc
        res[op] = d
        del a, b, c
    res["output_triangles_per_s_dc"] = tris_total / (dc_ms_total / 1000.0) if dc_ms_total else None
    res["output_triangles_per_s_mc"] = mc_total / (mc_ms_total / 1000.0) if mc_ms_total else None
    return res


def fp32_peak_tflops(ctx):
    import ctypes as C
    from baby_shark_gb300 import _native as N
    L = N.load()
    if not hasattr(L, "bs_diag_fp32_peak"):
        return None
    out = C.c_double()
    N.check(L.bs_diag_fp32_peak(ctx.h, C.byref(out)), ctx.h)
    return out.value


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-pipeline", dest="pipeline", action="store_false",
                    help="skip the secondary boolean / offset / dual-contouring timings")
    ap.add_argument("--tris-fraction", type=float, default=1.0,
                    help="use only the first part of each torus ring (smaller case for profiling)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep the default launch shapes (128 threads per brick, 4 warps per sign block)")
    ap.add_argument("--no-order3", dest="order3", action="store_false",
                    help="skip the order-3 / accuracy-scale-1.5 sign-pass comparison")
    ap.add_argument("--batch-meshes", type=int, default=256,
                    help="meshes of the uneven-batch comparison (0 skips it)")
    ap.add_argument("--configs", type=int, default=1,
                    help="1: also time the plain remesh and the non-watertight conversion (other_configs)")
    ap.add_argument("--workload", default="tori", choices=["tori", "open-icosphere", "large-union", "learned"],
                    help="tori: the boolean workload's two tori (the headline line); open-icosphere: the "
                         "non-watertight subdivision-9 icosphere with an exact-sign check")
    ap.add_argument("--wn-order", type=int, default=2, choices=[2, 3],
                    help="far-field order of the sign pass for --workload open-icosphere (2 = the reference's)")
    ap.add_argument("--wn-beta", type=float, default=2.0,
                    help="accuracy scale of the sign pass for --workload open-icosphere (2 = the reference's)")
    ap.add_argument("--learned-queries", type=int, default=16_000_000,
                    help="points of the learned-vs-plain comparison beside the headline (0: skip it)")
    ap.add_argument("--queries", type=int, default=16_000_000,
                    help="query points of --workload learned")
    ap.add_argument("--validation", type=int, default=200000,
                    help="band voxels checked against exact winding numbers (open-icosphere)")
    ap.add_argument("--pipeline-only", action="store_true",
                    help="run only the boolean / offset / dual-contouring tail once and print its stage times")
    ap.add_argument("--voxel-size", type=float, default=H,
                    help="voxel size of the --pipeline-only case (the workload's is 0.002)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "open-icosphere":
        run_open(args)
    elif args.workload == "large-union":
        run_large_union(args)
    elif args.workload == "learned":
        run_learned(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
