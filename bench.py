"""Benchmark of the DE path on GB300: DE-traced Mrays/s of the Mandelbox
wavefront path trace (1280x720, 64 spp, 4 bounces, 512 steps, hit epsilon 1e-4).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one whole 64-spp frame rendered as one dispatch (58,982,400 paths,
15.3 GB of path state in HBM; --spp-per-step chooses a smaller progressive
pass). `value` is device-timed (CUDA events on the library stream, max over
ranks); `e2e` is the same metric through the public API with host buffers: one
full 64-spp frame via Renderer.render (scene and graph uploaded from the host,
dispatches of the step's size, film read back). With N > 1 (torchrun) every rank renders its
own replica (the path has no exchange step).

At N = 1 the same line also carries the other configurations, measured in the
same run: `c2_cone_rule` (the headline frame with the reference's cone-relative
hit test), `c1` (Mandelbulb primary rays), `c3` (the uneven 64-job batch against
plain launches), `c4` (the 3840x2160 deep zoom with its agreement against
binary128 and FP64) and `c5` (the 200 req/s serving stream against sequential
plain launches, and both capacities); --no-extras leaves them out. The other
workloads also run alone with --workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DE-traced Mrays/s"
UNIT = "Mrays/s"
WORKLOAD = "mandelbox_pathtrace_1280x720_64spp_4bounce"
SPP_PER_STEP = 8
# Algorithmic FP32 flops (FMA = 2) of the Mandelbox form: per Iterate iteration
# (box fold 6, |p| 5 + sqrt 1, trap |p| 5 + sqrt 1 + min, sphere fold 1 div + 4,
# scale 4, add origin 4 = 31) and per DE evaluation outside the loop (query point
# 6, NormFence 7 + sqrt 1, march update 15 = 29).
FLOPS_PER_ITER = 31
FLOPS_PER_EVAL = 29


def profiled_traffic():
    """DRAM bytes per trace launch at 1280x720 from the committed ncu summary (or None)."""
    path = os.path.join(ROOT, "profiles", "k_trace_mandelbox_ncu.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch_1280x720:"):
                return int(line.split(":")[1])
    except OSError:
        pass
    return None


def dist_env():
    n = int(os.environ.get("WORLD_SIZE", "1"))
    r = int(os.environ.get("RANK", "0"))
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    return n, r, lr


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def cpu_port_rate(seconds_target: float = 12.0):
    """The oracle (FP32 restatement of the reference, all host cores) on a bounded
    sample of the same frame: pixels on a stride, 8 spp. Returns (Mrays/s, sample)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle  # the CPU restatement; used only as the baseline here

    from syfrack_gb300 import workloads

    scene = workloads.mandelbox_scene()
    cfg = workloads.mandelbox_pathtrace_config()
    og = oracle.OracleGraph(scene.graph)
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(3)
    n = 64
    total_seg, total_t, used = 0, 0.0, 0
    while total_t < seconds_target and n <= 65536:
        pix = np.stack([rng.integers(0, cfg.width, n), rng.integers(0, cfg.height, n)], 1).astype(np.uint32)
        t0 = time.perf_counter()
        r = og.render(scene.desc(cfg.width, cfg.height), cfg.desc(), pix, 0, SPP_PER_STEP, precision=32,
                      threads=threads)
        dt = time.perf_counter() - t0
        total_seg += r["segments"]
        total_t += dt
        used += n
        n *= 2
    return total_seg / total_t / 1e6, threads, f"{used} random pixels x {SPP_PER_STEP} spp of the frame, FP32"


def workload_config(args, n_ranks):
    """The workload's description, the same in both arms."""
    from syfrack_gb300 import workloads

    cfg = workloads.mandelbox_pathtrace_config(width=args.width, height=args.height, spp=64,
                                               samples_per_dispatch=args.spp_per_step)
    paths = cfg.width * cfg.height * args.spp_per_step
    return {"workload": WORKLOAD if (cfg.width, cfg.height) == (1280, 720) else f"profiling case {cfg.width}x{cfg.height}",
            "width": cfg.width, "height": cfg.height, "spp_per_step": args.spp_per_step,
            "hit_rule": f"fixed epsilon {cfg.hit_epsilon:g} (radius <= epsilon)", "paths_per_step": paths,
            "max_bounces": cfg.max_bounces, "max_steps": cfg.max_steps, "parallelism": f"replicas{n_ranks}",
            "l2": f"inputs larger than L2 (path state {paths * 260 / 1e9:.1f} GB per step)"}


def run_reference(args):
    n, rank, _ = dist_env()
    if rank != 0:
        return
    rates = []
    # warm-up then K bounded samples of the workload, each a separate measurement
    cpu_port_rate(2.0)
    for _ in range(args.steps):
        rate, threads, sample = cpu_port_rate(max(3.0, 20.0 / max(args.steps, 1)))
        rates.append(rate)
    value = statistics.median(rates)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": n,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Mandelbox scene; no dataset)",
            "config": workload_config(args, n),
            "host_threads": threads,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample + " (the reference is Rust/WGSL and cannot be built here; "
                                                "timed: its C++ restatement in oracle/)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def reduce_ranks(dist, elapsed, work, device):
    """Replicas: the slowest rank's time (max) and every rank's work (sum); with no
    exchange on the data path these two numbers are all the ranks share."""
    import torch

    t = torch.tensor([float(elapsed), float(work)], dtype=torch.float64, device=device)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(mx[0]), float(t[1])


def run_ours(args):
    spp_step = args.spp_per_step
    import ctypes as C

    n_ranks, rank, local_rank = dist_env()
    dist = None
    if n_ranks > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")

    from syfrack_gb300 import GpuContext, Renderer, RenderSession, workloads
    from syfrack_gb300._lib import check

    ctx = GpuContext(device=local_rank if n_ranks > 1 else 0)
    renderer = Renderer(ctx)
    scene = workloads.mandelbox_scene()
    spp_total = spp_step * (args.warmup + args.steps)
    cfg = workloads.mandelbox_pathtrace_config(width=args.width, height=args.height, spp=spp_total,
                                               samples_per_dispatch=spp_step)
    sess = RenderSession(renderer, scene, cfg)
    sess.set_launch(args.min_blocks, args.quantum, args.regen)
    tile = (0, 0, cfg.width, cfg.height)
    peak = C.c_double()
    check(ctx.lib.sf_device_fp32_peak(ctx.h, C.byref(peak)))

    def step(k):
        sess.dispatch((*tile, k * spp_step), spp_step)

    for k in range(args.warmup):
        step(k)
    sess.sync(600000)
    ctx.set_profiling(True)
    ctx.reset_stats()
    if dist:
        dist.barrier()
    # timed region: events on the library stream bracket the K steps
    import torch

    stream = torch.cuda.ExternalStream(ctx.stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        torch.cuda.synchronize()
        ev0.record(stream)
        for k in range(args.warmup, args.warmup + args.steps):
            step(k)
        ev1.record(stream)
        ev1.synchronize()
    ms = ev0.elapsed_time(ev1)
    status = sess.sync(600000)
    st = ctx.stats()
    segs = st["segments"]
    if dist:
        ms_max, segs_all = reduce_ranks(dist, ms, segs, "cuda")
    else:
        ms_max, segs_all = ms, float(segs)
    value = segs_all / (ms_max * 1e-3) / 1e6
    # dominant kernel: the persistent trace kernel (CUDA events around each launch)
    trace_ms = st["trace_ms"]
    trace_launches = max(st["trace_launches"], 1)
    flops = FLOPS_PER_ITER * st["de_iterations"] + FLOPS_PER_EVAL * st["de_evals"]
    per_launch_flops = flops / trace_launches
    avg_launch_s = trace_ms * 1e-3 / trace_launches
    achieved = per_launch_flops / avg_launch_s / 1e12 if avg_launch_s > 0 else 0.0
    # after the timed region: one more step on the diagnostic trace kernel, which counts
    # warp-level DE calls and iteration slots (lane use), on a separate session
    ctx.set_profiling(True, lane_stats=True)
    ctx.reset_stats()
    lane_cfg = workloads.mandelbox_pathtrace_config(width=args.width, height=args.height, spp=spp_step,
                                                    samples_per_dispatch=spp_step)
    lane_sess = RenderSession(renderer, scene, lane_cfg)
    lane_sess.set_launch(args.min_blocks, args.quantum, args.regen)
    lane_sess.dispatch(tile + (0,), spp_step)
    lane_sess.sync(600000)
    lst = ctx.stats()
    lane_sess.close()
    ctx.set_profiling(False)
    sess.close()

    # end to end through the public API: one full 64-spp frame in dispatches of the
    # step's size, rendered from host descriptions, film read back
    e2e_cfg = workloads.mandelbox_pathtrace_config(width=args.width, height=args.height, spp=64,
                                                   samples_per_dispatch=spp_step)
    ctx.reset_stats()
    if dist:
        dist.barrier()
    e2e_s, e2e_segs = 1.0, 0
    if not args.no_e2e:
        t0 = time.perf_counter()
        renderer.render(scene, e2e_cfg)
        e2e_s = time.perf_counter() - t0
        e2e_segs = ctx.stats()["segments"]
    if dist:
        e2e_s, e2e_segs = reduce_ranks(dist, e2e_s, e2e_segs, "cuda")
    e2e = e2e_segs / e2e_s / 1e6
    px = e2e_cfg.width * e2e_cfg.height
    e2e_steps = max(1, e2e_cfg.samples_per_pixel // spp_step)
    d2h = px * (16 + 4 + 16)
    h2d = C.sizeof(__import__("syfrack_gb300").abi.sf_scene_desc) + 4096
    cone = None
    if n_ranks == 1 and not args.no_extras:
        cone = pathtrace_variant(renderer, ctx, scene, args, "cone")

    if rank == 0:
        cpu = None
        if n_ranks == 1 and not args.no_cpu_baseline:
            rate, threads, sample = cpu_port_rate(12.0)
            cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": n_ranks, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Mandelbox scene; no dataset)",
            "config": workload_config(args, n_ranks),
            "run": {"integrator": "wavefront",
                    "launch": {"min_blocks_per_sm": args.min_blocks, "quantum": args.quantum, "regen": args.regen},
                    "segments_per_step": segs_all / args.steps,
                    "pixel_samples_per_s": cfg.width * cfg.height * spp_step * args.steps * n_ranks
                    / (ms_max * 1e-3)},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d // e2e_steps,
                    "d2h_bytes_per_step": d2h // e2e_steps,
                    "call": f"Renderer.render: one full 64-spp frame ({e2e_steps} dispatch(es) of {spp_step} spp), "
                            f"film read back; bytes per {spp_step}-spp step"},
            "roofline": {"bound": "fp32", "kernel": "k_trace", "achieved": achieved, "peak": peak.value,
                         "unit": "TFLOP/s", "frac": achieved / peak.value if peak.value else None,
                         "traffic": profiled_traffic() if ((cfg.width, cfg.height) == (1280, 720)
                                                           and spp_step == 64) else None,
                         "traffic_source": "dram__bytes_read+write per k_trace launch, one-pass ncu capture of the "
                                           "1280x720 x 64-spp dispatch (profiles/k_trace_mandelbox_ncu.md)",
                         "peak_source": "measured FFMA probe (sf_device_fp32_peak)",
                         "flops_per_launch": per_launch_flops, "launch_ms": avg_launch_s * 1e3,
                         "de_evals_per_step": st["de_evals"] / args.steps,
                         "de_iterations_per_step": st["de_iterations"] / args.steps,
                         "simt_lane_efficiency": lst["de_evals"] / max(32 * lst["warp_de_calls"], 1),
                         "iterate_lane_efficiency": lst["de_iterations"] / max(lst["iteration_slots"], 1),
                         "launch_tail_fraction": lst["tail_cycles"] / max(lst["warp_cycles"], 1),
                         "lane_efficiency_source": f"one further {spp_step}-spp step on the diagnostic trace kernel"},
            "gpu_launches": st["launches"],
            "status_word": status,
            "clocks": clocks.summary(),
            "cpu_baseline": cpu,
        }
        if cone is not None:
            line["c2_cone_rule"] = cone
    if n_ranks == 1 and not args.no_extras:
        renderer = None
        ctx.close()
        ctx = None
        line.update(extras(args))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    renderer = None
    if ctx is not None:
        ctx.close()


def pathtrace_variant(renderer, ctx, scene, args, rule, steps=5, warmup=2):
    """The headline frame with another hit rule ("cone": the reference's
    cone-relative test at pixel tolerance 1), device-timed like the headline."""
    spp_step = args.spp_per_step
    from syfrack_gb300 import RenderSession, workloads

    cfg = workloads.mandelbox_pathtrace_config(width=args.width, height=args.height,
                                               spp=spp_step * (steps + warmup),
                                               samples_per_dispatch=spp_step, rule=rule)
    sess = RenderSession(renderer, scene, cfg)
    sess.set_launch(args.min_blocks, args.quantum, args.regen)
    for k in range(warmup):
        sess.dispatch((0, 0, cfg.width, cfg.height, k * spp_step), spp_step)
    sess.sync(600000)
    ctx.reset_stats()
    import torch

    stream = torch.cuda.ExternalStream(ctx.stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for k in range(warmup, warmup + steps):
        sess.dispatch((0, 0, cfg.width, cfg.height, k * spp_step), spp_step)
    ev1.record(stream)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1)
    st = ctx.stats()
    sess.close()
    return {"value": st["segments"] / (ms * 1e-3) / 1e6, "unit": UNIT, "ms_per_step": ms / steps, "steps": steps,
            "de_evals_per_segment": st["de_evals"] / max(st["segments"], 1),
            "hit_rule": "cone-relative radius / t < pixel_cone (the reference's rule, pixel tolerance 1)"}


def extras(args):
    """The other configurations, measured in the same run (one GPU): primary rays,
    the uneven batch, the deep zoom and the serving stream, each summarised."""
    base = dict(vars(args))

    def ns(**kw):
        d = dict(base)
        d.update(kw)
        return argparse.Namespace(**d)

    out = {}
    t0 = time.perf_counter()
    p = measure_primary(ns(steps=10, warmup=3))
    out["c1"] = {"workload": p["workload"], "value": p["value"], "unit": p["unit"],
                 "launch_ms": p["frames"]["256x256"]["launch_ms"], "e2e": p["e2e"],
                 "frame_2048x2048_mrays_per_s": p["frames"]["2048x2048"]["mrays_per_s"],
                 "cpu_baseline": p["cpu_baseline"]}
    b = measure_batch(ns(steps=3, jobs=64))
    out["c3"] = {"workload": b["workload"], "unit": UNIT, "batched": b["value"],
                 "batched_steady_replays": b["value_steady_replays"], "plain_megakernel": b["plain_megakernel"],
                 "plain_wavefront_sessions": b["plain_wavefront_sessions"],
                 "speedup_vs_plain_megakernel": b["value"] / b["plain_megakernel"],
                 "speedup_vs_plain_wavefront": b["value"] / b["plain_wavefront_sessions"],
                 "autotuned": b["autotuned"], "paths_per_pass": b["paths_per_pass"], "seconds": b["seconds"]}
    d = measure_deepzoom(ns(steps=3, warmup=3, frame=None))
    out["c4"] = {k: d[k] for k in ("workload", "value", "unit", "kernel_ms_per_frame", "orbit", "orbit_kernel_ms",
                                   "e2e", "host_orbit_variant", "agreement", "cpu_baseline") if k in d}
    sv = measure_serve(ns())
    summ = lambda r: {"p50_ms": r["latency"]["all"].get("p50_ms"), "p99_ms": r["latency"]["all"].get("p99_ms"),
                      "throughput_rps": r["throughput_rps"], "mrays_per_s": r["mrays_per_s"]}
    out["c5"] = {"workload": sv["workload"], "requests": sv["requests"],
                 "served": {**summ(sv["served"]), "mean_batch_requests": sv["served"]["mean_batch_requests"],
                            "per_kind_p99_ms": {k: sv["served"]["latency"][k].get("p99_ms")
                                                for k in ("tile", "preview", "refine")}},
                 "plain_sequential": summ(sv["plain_sequential"]), "capacity": sv["capacity"],
                 "throughput_ratio": sv["throughput_ratio"]}
    out["extras_seconds"] = time.perf_counter() - t0
    return out


def measure_batch(args):
    """Uneven mixed batch: 64 seeded jobs (Mandelbulb powers 2-12, Mandelbox scales
    -2.5..2.5, Menger levels 3-7; tiles 64-512 px; 1-16 spp; 2 bounces). Rendered
    (a) job after job by the per-pixel megakernel (the reference's plain path),
    (b) job after job by per-job wavefront sessions, (c) as one autotuned batch
    replayed from a CUDA graph. Wall time from host descriptions to finished films."""
    from syfrack_gb300 import Batch, GpuContext, Renderer, RenderSession, workloads

    ctx = GpuContext(0)
    r = Renderer(ctx)
    jobs = workloads.mixed_batch(seed=7, jobs=args.jobs)
    for sc, _ in jobs:
        r.compile(sc.graph)

    def sequential(integrator):
        ctx.reset_stats()
        t0 = time.perf_counter()
        for sc, cfg in jobs:
            c2 = type(cfg)(**{**cfg.__dict__, "integrator": integrator, "tile_size": 256 if integrator == "megakernel" else cfg.tile_size})
            s = RenderSession(r, sc, c2)
            while not s.step(0):
                pass
            s.close()
        dt = time.perf_counter() - t0
        return ctx.stats()["segments"] / dt / 1e6, dt

    # warm-up of every code path on a few jobs
    wb = Batch(r, jobs[:3])
    wb.run(1)
    wb.sync()
    wb.close()
    plain_mk, t_mk = sequential("megakernel")
    plain_wf, t_wf = sequential("wavefront")
    b = Batch(r, jobs)
    mb, q, rg, tune_ms = b.autotune()
    ctx.reset_stats()
    t0 = time.perf_counter()
    b.run(1, use_graph=True)
    b.sync(600000)
    t_b = time.perf_counter() - t0
    segs = ctx.stats()["segments"]
    batched = segs / t_b / 1e6
    # steady state: replays of the captured pass (accumulating further samples)
    ctx.reset_stats()
    t0 = time.perf_counter()
    b.run(args.steps, use_graph=True)
    b.sync(600000)
    t_r = time.perf_counter() - t0
    replay = ctx.stats()["segments"] / t_r / 1e6
    b.close()
    line = {"metric": METRIC, "workload": f"mixed_batch_{len(jobs)}_jobs", "unit": UNIT, "value": batched,
            "value_steady_replays": replay, "plain_megakernel": plain_mk, "plain_wavefront_sessions": plain_wf,
            "speedup_vs_plain_megakernel": batched / plain_mk, "seconds": {"megakernel": t_mk, "wavefront": t_wf,
            "batch_first_pass": t_b, "batch_replays": t_r, "autotune_ms_best_pass": tune_ms},
            "autotuned": {"min_blocks_per_sm": mb, "quantum": q, "regen": rg}, "segments_per_pass": segs,
            "paths_per_pass": int(sum(c.width * c.height * c.samples_per_pixel for _, c in jobs)),
            "dtype": "f32", "data": "synthetic (seeded jobs)"}
    ctx.close()
    return line


def _percentiles(xs):
    import numpy as np

    if not xs:
        return {"n": 0}
    a = np.asarray(xs, dtype=np.float64)
    return {"n": int(a.size), "p50_ms": float(np.percentile(a, 50)), "p99_ms": float(np.percentile(a, 99)),
            "mean_ms": float(a.mean()), "max_ms": float(a.max())}


def _latency_report(lat, kinds):
    out = {"all": _percentiles(list(lat.values()))}
    for k in ("tile", "preview", "refine"):
        out[k] = _percentiles([v for j, v in lat.items() if kinds[j] == k])
    return out


def serve_replay(renderer, ctx, events, args):
    """Replays the stream in real time against a Server; latency = completion on the
    server clock - scheduled arrival mapped onto that clock."""
    from syfrack_gb300 import Server
    from syfrack_gb300.serve import DONE, FAILED
    from syfrack_gb300.workloads import SERVE_REFINE_WINDOW

    srv = Server(renderer, hbm_budget=int(args.hbm_budget_gb * (1 << 30)), slots=args.slots,
                 host_result_bytes=int(args.host_result_gb * (1 << 30)))
    kinds = [e[1] for e in events]
    tickets = [0] * len(events)
    lat, failed, outstanding, window, lag = {}, 0, set(), [], 0.0
    ctx.reset_stats()
    t0 = time.perf_counter()
    off = min(srv.stats()["now_ms"] - (time.perf_counter() - t0) * 1e3 for _ in range(5))
    i = 0
    last_done = 0.0
    while i < len(events) or outstanding:
        now = time.perf_counter() - t0
        while i < len(events) and events[i][0] <= now:
            t_arr, kind, payload = events[i]
            if kind == "tile":
                tickets[i] = srv.tile(*payload)
            elif kind == "preview":
                tickets[i] = srv.preview(*payload)
                window.append(i)
            else:
                tickets[i] = srv.refine(tickets[payload], 8)
            lag = max(lag, time.perf_counter() - t0 - t_arr)
            outstanding.add(i)
            i += 1
        for j in list(outstanding):
            res = srv.poll(tickets[j], copy=False)
            if res.state == DONE or res.state == FAILED:
                outstanding.discard(j)
                if res.state == FAILED:
                    failed += 1
                lat[j] = res.done_ms - (events[j][0] * 1e3 + off)
                last_done = max(last_done, res.done_ms - off)
                if kinds[j] != "preview":
                    srv.release(tickets[j])
        # a preview's film is dropped once 16 newer previews exist (its queued refinements keep it)
        while len(window) > SERVE_REFINE_WINDOW and window[0] not in outstanding:
            srv.release(tickets[window.pop(0)])
        nxt = events[i][0] - (time.perf_counter() - t0) if i < len(events) else 0.0005
        time.sleep(min(max(nxt, 0.0), 0.0005))
    span_s = last_done / 1e3 - events[0][0]
    st = srv.stats()
    segs = ctx.stats()["segments"]
    srv.close()
    return {"latency": _latency_report(lat, kinds), "failed": failed, "throughput_rps": len(lat) / span_s,
            "span_s": span_s, "segments": segs, "mrays_per_s": segs / span_s / 1e6, "max_submit_lag_ms": lag * 1e3,
            "batches": st["batches"], "mean_batch_requests": st["batched_requests"] / max(st["batches"], 1),
            "admission_waits": st["admission_waits"], "hbm_peak_gb": st["hbm_peak"] / (1 << 30)}


def plain_replay(renderer, ctx, events, cap_s, integrator="wavefront"):
    """The same stream through the plain drop-in calls, one request at a time in
    arrival order: RenderSession + dispatch(1 spp) + readback per preview, a further
    dispatch(8) + readback on that session per refinement, sf_escape2d per tile.
    integrator: the sessions' ("megakernel" is the reference's per-pixel loop)."""
    from syfrack_gb300 import RenderSession, escape2d
    from syfrack_gb300.workloads import SERVE_REFINE_WINDOW

    kinds = [e[1] for e in events]
    sessions, window, lat = {}, [], {}
    ctx.reset_stats()
    t0 = time.perf_counter()
    unserved = 0
    last_done = 0.0
    for j, (t_arr, kind, payload) in enumerate(events):
        now = time.perf_counter() - t0
        if now < t_arr:
            time.sleep(t_arr - now)
        if time.perf_counter() - t0 > cap_s:
            unserved = len(events) - j
            break
        if kind == "tile":
            escape2d(ctx, *payload)
        elif kind == "preview":
            sc, cfg = payload
            # a session sized for its refinements: 8 samples per dispatch, open-ended target
            cfg = type(cfg)(**{**cfg.__dict__, "samples_per_pixel": 1 << 16, "samples_per_dispatch": 8,
                               "integrator": integrator})
            s = RenderSession(renderer, sc, cfg)
            n = payload[1].samples_per_pixel
            s.dispatch((0, 0, cfg.width, cfg.height, 0), n)
            s.sync()
            s.readback()
            sessions[j] = [s, n]
            window.append(j)
            while len(window) > SERVE_REFINE_WINDOW:
                sessions.pop(window.pop(0))[0].close()
        else:
            s, done = sessions[payload]
            s.dispatch((0, 0, s.cfg.width, s.cfg.height, done), 8)  # samples done..done+7
            s.sync()
            s.readback()
            sessions[payload][1] = done + 8
        last_done = time.perf_counter() - t0
        lat[j] = (last_done - t_arr) * 1e3
    span_s = last_done - events[0][0]
    segs = ctx.stats()["segments"]
    for s, _ in sessions.values():
        s.close()
    return {"latency": _latency_report(lat, kinds), "unserved_at_cap": unserved, "cap_s": cap_s,
            "throughput_rps": len(lat) / span_s, "span_s": span_s, "segments": segs,
            "mrays_per_s": segs / span_s / 1e6}


def measure_serve(args):
    """Serving stream: Poisson arrivals at --rate req/s for --duration s (seeded):
    40% 2D tiles (Julia c = 0.7885 e^{ia} or a Burning Ship view; side 256-2048;
    1k-20k iterations), 40% previews (480x270, 1 spp, 1 bounce, a random orbit of a
    Mandelbulb or Mandelbox), 20% refinements (+8 spp into one of the 16 latest
    previews' films). Replayed in real time against the Server (150 GB HBM budget)
    and as sequential plain launches; p50/p99 latency and throughput of both. Then
    the capacity of both: the stream's first --burst requests queued at once."""
    from syfrack_gb300 import GpuContext, Renderer, workloads

    ctx = GpuContext(0)
    r = Renderer(ctx)
    for g in workloads.serving_graphs():
        r.compile(g)
    events = workloads.serving_stream(seed=args.seed, rate=args.rate, duration=args.duration)
    warm = workloads.serving_stream(seed=args.seed + 1, rate=args.rate, duration=0.25)
    serve_replay(r, ctx, warm, args)
    plain_replay(r, ctx, warm, 60.0)
    served = serve_replay(r, ctx, events, args)
    plain = plain_replay(r, ctx, events, cap_s=args.duration * 3)
    # capacity: the first requests of the same stream all queued at once
    burst = [(0.0, k, pl) for _, k, pl in events[:args.burst]]
    cap_served = serve_replay(r, ctx, burst, args)
    cap_plain = plain_replay(r, ctx, burst, cap_s=600.0)
    # the plain drop-in proper: previews and refinements through the per-pixel megakernel
    cap_plain_mk = plain_replay(r, ctx, burst, cap_s=600.0, integrator="megakernel")
    capacity = {"requests": len(burst), "served_rps": cap_served["throughput_rps"],
                "plain_rps": cap_plain["throughput_rps"],
                "ratio": cap_served["throughput_rps"] / cap_plain["throughput_rps"],
                "served_mrays_per_s": cap_served["mrays_per_s"], "plain_mrays_per_s": cap_plain["mrays_per_s"],
                "plain_megakernel_rps": cap_plain_mk["throughput_rps"],
                "plain_megakernel_mrays_per_s": cap_plain_mk["mrays_per_s"],
                "ratio_vs_plain_megakernel": cap_served["throughput_rps"] / cap_plain_mk["throughput_rps"],
                "mrays_ratio_vs_plain_megakernel": cap_served["mrays_per_s"] / cap_plain_mk["mrays_per_s"],
                "served_batches": cap_served["batches"],
                "served_mean_batch_requests": cap_served["mean_batch_requests"]}
    line = {"metric": "served p99 latency", "unit": "ms", "value": served["latency"]["all"].get("p99_ms"),
            "higher_is_better": False, "workload": f"serving_stream_poisson{args.rate:g}_{args.duration:g}s",
            "requests": len(events), "served": served, "plain_sequential": plain, "capacity": capacity,
            "throughput_ratio": served["throughput_rps"] / plain["throughput_rps"],
            "config": {"slots": args.slots, "hbm_budget_gb": args.hbm_budget_gb,
                       "host_result_gb": args.host_result_gb, "seed": args.seed,
                       "preview": workloads.SERVE_PREVIEW, "refine_spp": workloads.SERVE_REFINE_SPP},
            "dtype": "f32", "data": "synthetic (seeded Poisson stream)"}
    ctx.close()
    return line


def measure_primary(args):
    """Plain Mandelbulb primary rays: 256x256, power 8, 12 iterations, bailout 2.0,
    pinhole at (0,0,-3) looking at the origin, 60 degree FOV, 256 steps, epsilon 1e-4,
    far 10; hit t, step count and central-difference normal per pixel. Device time
    per launch from CUDA events (profiling on); e2e through Renderer.primary with
    host outputs; the oracle in FP32 on all host cores over the same frame. A
    2048x2048 frame of the same view gives the kernel's sustained rate."""
    from syfrack_gb300 import GpuContext, Renderer, workloads

    ctx = GpuContext(0)
    r = Renderer(ctx)
    g, cam, W, H, steps, eps, far = workloads.mandelbulb_primary()
    for _ in range(max(args.warmup, 3)):
        r.primary(g, cam, W, H, steps, "absolute", eps, far)
        r.primary(g, cam, 2048, 2048, steps, "absolute", eps, far)
    ctx.set_profiling(True)
    frames = {}
    for (w, h) in ((W, H), (2048, 2048)):
        ctx.reset_stats()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            r.primary(g, cam, w, h, steps, "absolute", eps, far)
        wall = time.perf_counter() - t0
        st = ctx.stats()
        launch_ms = st["trace_ms"] / max(st["trace_launches"], 1)
        rays = w * h
        frames[f"{w}x{h}"] = {"mrays_per_s": rays / (launch_ms * 1e-3) / 1e6, "launch_ms": launch_ms,
                              "e2e_mrays_per_s": rays * args.steps / wall / 1e6,
                              "de_evals_per_frame": st["de_evals"] / args.steps,
                              "de_iterations_per_frame": st["de_iterations"] / args.steps}
    ctx.set_profiling(False)
    # oracle (FP32, all host cores) on the same 256x256 frame
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # the CPU restatement; used only as the baseline here

    from syfrack_gb300 import abi as sfabi

    og = oracle.OracleGraph(g)
    b = cam.basis()
    oc = sfabi.sf_camera()
    oc.origin[:] = [float(x) for x in b.origin]
    oc.forward[:] = [float(x) for x in b.forward]
    oc.right[:] = [float(x) for x in b.right]
    oc.up[:] = [float(x) for x in b.up]
    oc.tan_half_fov = b.tan_half_fov
    oc.aspect = 1.0
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    og.primary(oc, W, H, steps, 1, eps, far, precision=32, threads=threads)
    cpu_s = time.perf_counter() - t0
    main = frames[f"{W}x{H}"]
    line = {"metric": "primary Mrays/s", "unit": "Mrays/s", "value": main["mrays_per_s"], "higher_is_better": True,
            "workload": "mandelbulb_primary_256x256_256steps", "steps": args.steps, "frames": frames,
            "e2e": {"value": main["e2e_mrays_per_s"], "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": W * H * 20, "call": "Renderer.primary"},
            "cpu_baseline": {"value": W * H / cpu_s / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": f"the whole {W}x{H} frame, FP32"},
            "dtype": "f32", "data": "synthetic (the C1 view)"}
    ctx.close()
    return line


def frame_size(args, w, h):
    """The workload's frame, or --frame WxH (smaller frames are for profiler captures)."""
    if not args.frame:
        return w, h
    fw, fh = args.frame.lower().split("x")
    return int(fw), int(fh)


def measure_tile(args):
    """The largest 2D tile of the serving mix through the plain call sf_escape2d:
    Burning Ship, 2048x2048, 20,000 iterations, every trap (ring, stripe bands,
    final angle), the canvas around the ship (centre (-0.45, -0.5), zoom 1.8) at
    pixel centres. value = iterations per second of k_escape2d (CUDA events); e2e =
    the same through the call with host outputs (24 B per pixel read back); the
    oracle in FP32 on all host cores over a seeded pixel sample of the same tile."""
    import numpy as np

    from syfrack_gb300 import Canvas, GpuContext, PlanarFractal, escape2d

    ctx = GpuContext(0)
    W, H = frame_size(args, 2048, 2048)
    f = PlanarFractal(family="BurningShip", iterations=20000)
    canvas = Canvas(width=W, height=H, center=(-0.45, -0.5), zoom=1.8)
    for _ in range(max(args.warmup, 3)):
        escape2d(ctx, f, canvas)
    ctx.set_profiling(True)
    walls, kms, iters = [], [], []
    for _ in range(args.steps):
        ctx.reset_stats()
        t0 = time.perf_counter()
        out = escape2d(ctx, f, canvas)
        walls.append(time.perf_counter() - t0)
        st = ctx.stats()
        kms.append(st["trace_ms"])
        iters.append(st["de_iterations"])
    ctx.set_profiling(False)
    it_frame, kernel_ms, wall = float(np.median(iters)), float(np.median(kms)), float(np.median(walls))
    line = {"metric": "2D escape-time Giter/s", "unit": "Giter/s", "value": it_frame / (kernel_ms * 1e-3) / 1e9,
            "higher_is_better": True, "workload": f"burning_ship_{W}x{H}_20k_iter_traps", "steps": args.steps,
            "kernel_ms_per_tile": kernel_ms, "iterations_per_tile": it_frame,
            "mean_iterations_per_pixel": float(out["iterations"].mean()),
            "e2e": {"value": it_frame / wall / 1e9, "unit": "Giter/s", "tile_ms": wall * 1e3,
                    "h2d_bytes_per_step": 0, "d2h_bytes_per_step": W * H * 24, "call": "escape2d (sf_escape2d)"},
            "dtype": "f32", "data": "synthetic (the serving mix's largest tile)"}
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle  # the CPU restatement; used only as the baseline here

        from syfrack_gb300.render import FAMILIES

        rng = np.random.default_rng(4)
        idx = rng.choice(W * H, 4096, replace=False)
        f32 = np.float32
        u = (idx % W).astype(np.float32) + f32(0.5)
        v = (idx // W).astype(np.float32) + f32(0.5)
        scale = f32(6.0) / f32(canvas.zoom)
        qx = f32(canvas.center[0]) + (u / f32(W) - f32(0.5)) * scale
        qy = f32(canvas.center[1]) + ((f32(0.5) - v / f32(H)) / (f32(W) / f32(H))) * scale
        pp = oracle.PlanarParams()
        pp.family = FAMILIES.index(f.family)
        pp.power, pp.iterations = f.power, f.iterations
        for k in ("zoom", "angle", "inversion", "twist", "relaxation", "memory", "bailout", "trap_radius", "stripes"):
            setattr(pp, k, float(np.float32(getattr(f, k))))
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        ref = oracle.planar(pp, np.stack([qx, qy], 1), precision=32, threads=threads)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": float(ref["iterations"].sum()) / dt / 1e9, "unit": "Giter/s",
                                "cores": threads, "kind": "port", "sample": f"{len(idx)} seeded pixels of the tile, FP32"}
    ctx.close()
    return line


def measure_deepzoom(args):
    """Mandelbrot deep zoom: 3840x2160, max 50,000 iterations, width 1e-12 around a
    seeded boundary point (FP64 bisection of the escape label along a random ray from
    c = 0). FP64 reference orbit on the GPU, FP32 perturbation with rebasing. Reports
    the perturbation's Giter/s (kernel time from CUDA events), the frame time through
    the public call (host outputs) with the orbit on the GPU and, beside it, on a host
    core; agreement of iteration counts with full-FP64 direct iteration on the GPU over
    every pixel; smooth-colouring error against it; and on a seeded 4096-pixel sample,
    agreement with the oracle's binary128 iteration (the truth) for the perturbation
    with the FP64 orbit, with the oracle's binary128 orbit (the decomposition: orbit
    error against FP32-delta error) and for FP64 direct iteration, the sample timed as
    the CPU baseline."""
    import numpy as np

    from syfrack_gb300 import GpuContext, deep_zoom, workloads

    ctx = GpuContext(0)
    W, H = frame_size(args, 3840, 2160)
    MI, width = 50000, 1e-12
    c = workloads.deep_zoom_center(seed=2026, max_iter=MI)
    for _ in range(max(args.warmup, 3)):
        deep_zoom(ctx, c, (0.0, 0.0), width, min(W, 960), min(H, 540), MI, bailout=16.0)

    def frames(orbit):
        ctx.set_profiling(True)
        walls, kms, oms, iters, out = [], [], [], [], None
        for _ in range(args.steps):
            ctx.reset_stats()
            t0 = time.perf_counter()
            out = deep_zoom(ctx, c, (0.0, 0.0), width, W, H, MI, bailout=16.0, orbit=orbit)
            walls.append(time.perf_counter() - t0)
            st = ctx.stats()
            kms.append(st["trace_ms"])
            oms.append(st["kernel_ms"] - st["trace_ms"])
            iters.append(st["de_iterations"])
        ctx.set_profiling(False)
        return out, float(np.median(iters)), float(np.median(kms)), float(np.median(oms)), float(np.median(walls))

    out, iters_per_frame, kernel_ms, orbit_ms, wall = frames("device")
    out_h, _, kernel_ms_h, _, wall_h = frames("host")
    full = deep_zoom(ctx, c, (0.0, 0.0), width, W, H, MI, bailout=16.0, reference_f64=True)
    it, it64 = full["iterations"].ravel(), full["iterations_f64"].ravel()
    agree64 = float((it == it64).mean())
    near64 = float((np.abs(it.astype(np.int64) - it64.astype(np.int64)) <= 1).mean())
    both = (it == it64) & (it < MI)
    smooth_err = np.abs(full["smooth"].ravel()[both] - full["smooth_f64"].ravel()[both])
    line = {"metric": "deep-zoom perturbation Giter/s", "unit": "Giter/s",
            "value": iters_per_frame / (kernel_ms * 1e-3) / 1e9, "higher_is_better": True,
            "workload": f"mandelbrot_deep_zoom_{W}x{H}_50k_iter_width1e-12", "steps": args.steps,
            "center": list(c), "kernel_ms_per_frame": kernel_ms, "iterations_per_frame": iters_per_frame,
            "orbit": "FP64 on the GPU (k_ref_orbit, one thread)", "orbit_kernel_ms": orbit_ms,
            "e2e": {"value": iters_per_frame / wall / 1e9, "unit": "Giter/s", "frame_ms": wall * 1e3,
                    "h2d_bytes_per_step": 0, "d2h_bytes_per_step": W * H * 8, "call": "deep_zoom (sf_deep_zoom)"},
            "host_orbit_variant": {"e2e_giter_per_s": iters_per_frame / wall_h / 1e9, "frame_ms": wall_h * 1e3,
                                   "kernel_ms_per_frame": kernel_ms_h,
                                   "same_counts_as_device_orbit": bool(np.array_equal(out["iterations"],
                                                                                      out_h["iterations"]))},
            "rebases_per_frame": out["rebases"],
            "agreement": {"perturbation_vs_fp64_direct_all_pixels": agree64,
                          "perturbation_vs_fp64_direct_within_1": near64,
                          "smooth_abs_err_vs_fp64_where_counts_agree": {
                              "mean": float(smooth_err.mean()) if smooth_err.size else None,
                              "max": float(smooth_err.max()) if smooth_err.size else None}},
            "dtype": "f32 deltas, f64 reference orbit", "data": "synthetic (seeded boundary point)"}
    if args.no_cpu_baseline:
        ctx.close()
        return line
    # truth: binary128 on a seeded sample (oracle, all host cores), timed as the CPU baseline
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # the CPU restatement; the baseline here, and the truth for the counts

    rng = np.random.default_rng(11)
    idx = rng.choice(W * H, 4096, replace=False)
    f32 = np.float32
    pitch = f32(width / W)
    px, py = idx % W, idx // W
    off = np.stack([(px.astype(np.float32) - f32(W) * f32(0.5) + f32(0.5)) * pitch,
                    (f32(H) * f32(0.5) - py.astype(np.float32) - f32(0.5)) * pitch], 1).astype(np.float64)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    truth, _ = oracle.mandel_escape(np.array(c), np.zeros(2), off, MI, 16.0, precision=128, threads=threads)
    t128 = time.perf_counter() - t0
    t0 = time.perf_counter()
    cpu64, _ = oracle.mandel_escape(np.array(c), np.zeros(2), off, MI, 16.0, precision=64, threads=threads)
    t64 = time.perf_counter() - t0
    # the decomposition: the same frame on the oracle's binary128 orbit (as hi/lo float pairs)
    q = deep_zoom(ctx, c, (0.0, 0.0), width, W, H, MI, bailout=16.0, orbit="given",
                  given_orbit=oracle.mandel_orbit(c, MI, 16.0, precision=128))["iterations"].ravel()
    match = lambda a: float((a[idx] == truth).mean()) if len(a) == W * H else float((a == truth).mean())
    line["agreement"].update({
        "sample_pixels": len(idx),
        "perturbation_vs_binary128": match(it),
        "perturbation_vs_binary128_within_1": float(
            (np.abs(it[idx].astype(np.int64) - truth.astype(np.int64)) <= 1).mean()),
        "perturbation_binary128_orbit_vs_binary128": match(q),
        "fp64_direct_gpu_vs_binary128": match(it64),
        "fp64_direct_cpu_vs_binary128": match(cpu64),
        "sample_interior_fraction": float((truth == MI).mean())})
    line["cpu_baseline"] = {"value": float(np.sum(np.minimum(cpu64, MI))) / t64 / 1e9, "unit": "Giter/s",
                            "cores": threads, "kind": "port",
                            "sample": f"{len(idx)} seeded pixels, FP64 direct iteration "
                                      f"({t64:.2f} s; binary128 on the same pixels {t128:.2f} s)"}
    ctx.close()
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--min-blocks", type=int, default=7,
                    help="trace blocks per SM: 2-4 of 256 threads or 6-7 of 128 (batches take 2-4)")
    ap.add_argument("--quantum", type=int, default=0)
    ap.add_argument("--regen", type=int, default=4)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    # smaller frames are for profiler captures only; the measured workload is 1280x720
    ap.add_argument("--width", type=int, default=1280)
    ap.add_argument("--height", type=int, default=720)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--spp-per-step", type=int, default=64,
                    help="samples per pixel of the frame rendered by one step (one dispatch)")
    ap.add_argument("--no-extras", action="store_true",
                    help="the headline only (without the other configurations' summaries)")
    ap.add_argument("--workload", default="pathtrace",
                    choices=["pathtrace", "batch", "serve", "primary", "deepzoom", "tile"])
    ap.add_argument("--frame", default=None, help="WxH override of the deepzoom/tile frame (profiling only)")
    ap.add_argument("--jobs", type=int, default=64)
    # serving stream
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--duration", type=float, default=60.0)
    ap.add_argument("--slots", type=int, default=4)
    ap.add_argument("--hbm-budget-gb", type=float, default=150.0)
    ap.add_argument("--host-result-gb", type=float, default=8.0)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--burst", type=int, default=3000, help="requests queued at once for the capacity measure")
    args = ap.parse_args()
    measures = {"batch": measure_batch, "serve": measure_serve, "primary": measure_primary,
                "deepzoom": measure_deepzoom, "tile": measure_tile}
    if args.impl == "reference":
        run_reference(args)
    elif args.workload in measures:
        print(json.dumps(measures[args.workload](args)), flush=True)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
