#!/usr/bin/env python3
"""Benchmark of the GB300 MLS-MPM substep.

Workload (one GPU): the liquid throughput scene — 1,000,000 weakly compressible
liquid particles uniform in [0.1,0.5]x[0.1,0.7]x[0.1,0.9], N=32, dt=1e-4, cell
sort every 16 substeps.  A step is one substep of all particles.

Prints one JSON line (rank 0):
  value        particle-substeps/s over the timed steps (CUDA events on the
               launching stream, device time of the substeps; the L2 is flushed
               by a 512 MiB write between steps, outside the events)
  roofline     the fused substep kernel: algorithmic bytes (128 B per
               particle-substep + 32 B per grid node) / its mean launch time,
               against the measured HBM copy bandwidth
  e2e          the same metric through the C ABI with pinned host buffers:
               upload of the state, one substep, readback of the state
  cpu_baseline the CPU restatement of the reference substep (oracle, FP32,
               all host threads) on a bounded sample of the same scene

--impl reference: the reference's substep has no CPU implementation and cannot
be built here, so the arm times the oracle's CPU restatement of it (all host
threads) on the same scene.
Multi-GPU (torchrun): a single scene does not shard, so each rank runs an
independent replica ("replicas only"); value = all ranks' particle-substeps /
the slowest rank's time.
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

import numpy as np  # noqa: E402

B_ALG = {"liquid": 128.0, "snow": 200.0, "elastic": 200.0, "fixed_corotated": 200.0}
GRID_BYTES_PER_NODE = 32.0  # one float4 read + one float4 written per grid node and substep


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=8)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="liquid",
                    choices=["liquid", "snow", "elastic", "batched", "differentiable", "seeding", "mesh", "export",
                             "render"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--shape", default="auto",
                    help="launch shape of the fused kernel: 'auto' (the autotuner picks it) or "
                         "steps_per_warp,warps_per_cta,tile_box (e.g. 2,12,1) to fix it, as the profiles do")
    ap.add_argument("--diff-material", default="both", choices=["both", "fixed_corotated", "snow"],
                    help="materials timed by the differentiable workload")
    ap.add_argument("--no-extra", action="store_true",
                    help="headline workload only (no snow, batched and differentiable sections)")
    ap.add_argument("--e2e-steps", type=int, default=32,
                    help="e2e steps averaged (a multiple of the sort interval includes its sorts at their rate)")
    return ap.parse_args()


def make_cfg(name):
    from mpm_gb300 import scenes

    if name == "liquid":
        return scenes.config_liquid(), "liquid_1M_N32"
    if name == "snow":
        return scenes.config_snow(), "snow_500k_N64"
    return scenes.config_elastic(), "elastic_10k_N16"


def dist_setup(args):
    from mpm_gb300 import distributed as D

    return D.env()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self, t0=None, t1=None):
        """Median SM clock and active throttle reasons over the samples taken between
        wall-clock times t0 and t1 (all samples when not given)."""
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 10:
                continue
            try:
                ts = time.mktime(time.strptime(parts[0].split(".")[0], "%Y/%m/%d %H:%M:%S")) + \
                    float("0." + parts[0].split(".")[1]) if "." in parts[0] else 0.0
            except Exception:
                ts = None
            if t0 is not None and ts is not None and not (t0 - 0.05 <= ts <= t1 + 0.05):
                continue
            try:
                sm.append(float(parts[2]))
                smax.append(float(parts[3]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[6:10]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_summary(workload):
    """Figures of one substep (velocity pass + fused kernel) from the committed ncu summary
    of the workload: DRAM bytes and warp instructions per substep, the SM clock of the
    capture."""
    p = os.path.join(ROOT, "profiles", f"scene_step_{workload}.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def cpu_baseline(cfg, budget_s=12.0, max_particles=None):
    """The oracle's FP32 restatement on all host threads over a bounded sample."""
    import oracle

    mats = [m.derived() for m in cfg["materials"]]
    st = cfg["state"]
    n = st["x"].shape[0]
    if max_particles and n > max_particles:
        st = {k: v[:max_particles] for k, v in st.items()}
        n = max_particles
    threads = oracle.max_threads()
    t1 = oracle.time_f32(st, cfg["params"], mats, 1, threads)
    steps = int(max(1, min(500, budget_s / max(t1, 1e-6))))
    t = oracle.time_f32(st, cfg["params"], mats, steps, threads)
    return {"value": n * steps / t, "unit": "particle-substeps/s", "cores": threads, "kind": "port",
            "sample": f"{n} particles x {steps} substeps of the same scene (FP32 oracle, {threads} threads, "
                      f"{t:.1f} s)"}


def run_reference(args):
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return
    from oracle import build as ob

    ob.build_oracle()
    import oracle

    cfg, workload = make_cfg(args.config)
    mats = [m.derived() for m in cfg["materials"]]
    st = cfg["state"]
    n_full = st["x"].shape[0]
    threads = oracle.max_threads()
    # size the per-step sample so the whole run stays within a few minutes
    t1 = oracle.time_f32(st, cfg["params"], mats, 1, threads)
    total_steps = args.steps + args.warmup
    budget = 150.0
    n = n_full
    if t1 * total_steps > budget:
        n = max(10_000, int(n_full * budget / (t1 * total_steps)))
    sample = {k: v[:n] for k, v in st.items()}
    for _ in range(args.warmup):
        oracle.time_f32(sample, cfg["params"], mats, 1, threads)
    times = [oracle.time_f32(sample, cfg["params"], mats, 1, threads) for _ in range(args.steps)]
    tot = sum(times)
    value = n * args.steps / tot
    line = {
        "impl": "reference", "metric": "particle-substeps/s", "value": value, "unit": "particle-substeps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload, "particles": n_full, "N": cfg["params"]["N"], "sample_particles": n},
        "cpu_baseline": {"value": value, "unit": "particle-substeps/s", "cores": threads, "kind": "port",
                         "sample": f"{n} of {n_full} particles, one substep per step (the reference has no CPU "
                                   f"substep and does not build here; oracle FP32 restatement)"},
        "e2e": {"value": value, "unit": "particle-substeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def choose_shape(sim, shape):
    """The fused kernel's launch shape: the autotuner's pick, or a fixed one."""
    from mpm_gb300 import autotune

    if shape == "auto":
        return autotune.tune(sim, None, tune_sort_interval=False, budget_substeps=32)
    spw, warps, box = (int(t) for t in shape.split(","))
    sim.set_tuning(spw, warps, box)
    return dict(autotune.current(sim), fixed=True)


def time_substeps(sim, steps, warmup, stream, flush):
    """Device time of `steps` single substeps (CUDA events on the library's stream), the L2
    flushed by a 512 MiB write before each (outside the events).  Returns the per-step
    times (ms), whether each step ran only the two substep kernels (no sort), the kernel
    launches and the wall time of the timed loop."""
    import torch

    for _ in range(warmup):
        flush.fill_(1.0)
        sim.advance(1)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    pure = []
    launches0 = sim.launches
    wall0 = time.perf_counter()
    for k in range(steps):
        flush.fill_(float(k))
        l0 = sim.launches
        starts[k].record(stream)
        sim.advance(1)
        ends[k].record(stream)
        pure.append(sim.launches - l0 == 2)  # velocity pass + fused kernel, no sort
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    return ms, pure, sim.launches - launches0, wall


def substep_roofline(cfg, n, ms, pure, workload):
    """HBM roofline of one substep (velocity pass + fused kernel): algorithmic bytes
    (B_ALG per particle + 32 B per grid node) over the mean time of the steps that ran no
    sort, against the measured copy bandwidth."""
    N = cfg["params"]["N"]
    fused_ms = [m for m, p in zip(ms, pure) if p]
    kernel_ms = statistics.mean(fused_ms) if fused_ms else statistics.mean(ms)
    peak, peak_kind = measured_peaks()
    name = cfg["materials"][0].name
    bytes_per_launch = B_ALG[name if name in B_ALG else "liquid"] * n + GRID_BYTES_PER_NODE * N ** 3
    achieved = bytes_per_launch / (kernel_ms * 1e-3) / 1e9
    prof = profile_summary(workload)
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": prof.get("dram_bytes_per_substep"),
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "kernel": "mpm::grid_velocity_kernel + mpm::scene_step_kernel (one substep)", "kernel_ms": kernel_ms,
            "bytes_per_launch": bytes_per_launch}


def issue_fraction(roofline, workload, clocks, num_sms):
    """Share of the SMs' issue slots the substep kernels used: their warp instructions per
    substep (from the committed ncu summary of the same workload) over kernel time x SMs x
    4 schedulers x the median SM clock sampled during the timed region."""
    prof = profile_summary(workload)
    inst = prof.get("warp_instructions_per_substep")
    mhz = (clocks or {}).get("sm_mhz") or prof.get("sm_mhz")
    if not inst or not mhz:
        return None
    slots = roofline["kernel_ms"] * 1e-3 * num_sms * 4 * mhz * 1e6
    return inst / slots


def run_ours(args):
    import torch

    from mpm_gb300 import distributed as D

    world, rank, local = D.init("nccl")
    from mpm_gb300 import build

    if rank == 0 or world == 1:
        build.build()
    D.barrier()
    from mpm_gb300.simulation import Simulation

    cfg, workload = make_cfg(args.config)
    n = cfg["state"]["x"].shape[0]
    N = cfg["params"]["N"]
    # a dedicated (non-default) stream: the events and the L2 flush are ordered with the
    # library's kernels on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sim = Simulation.from_config(cfg)
    sim.set_stream(stream.cuda_stream)
    sim.upload(cfg["state"])
    # the launch shape comes from the autotuner (measured here, on a copy of the scene) unless
    # --shape fixes it; the workload fixes the sort interval
    tuning = choose_shape(sim, args.shape)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    num_sms = torch.cuda.get_device_properties(0).multi_processor_count

    torch.cuda.synchronize()
    D.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    for _ in range(args.warmup):
        flush.fill_(1.0)
        sim.advance(1)
    torch.cuda.synchronize()
    D.barrier()
    torch.cuda.synchronize()
    wall0_abs = time.time()
    ms, pure, launches, wall = time_substeps(sim, args.steps, 0, stream, flush)
    clocks = sampler.stop(wall0_abs, wall0_abs + wall)
    sim.sync()
    torch.cuda.synchronize()
    D.barrier()
    dev_ms = D.max_over_ranks(sum(ms))  # the slowest replica
    ms_per_step = dev_ms / args.steps
    value = D.job_rate(world * n * args.steps, dev_ms * 1e-3)
    roofline = substep_roofline(cfg, n, ms, pure, workload)
    roofline["issue_frac"] = issue_fraction(roofline, workload, clocks, num_sms)

    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(sim, cfg, args.e2e_steps, world)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(cfg, max_particles=None if args.config != "liquid" else 1_000_000)
    sim.close()
    extra = {}
    if world == 1 and args.config == "liquid" and not args.no_extra:
        del flush
        torch.cuda.empty_cache()
        extra["snow"] = snow_section(args, stream, num_sms)
        extra["batched"] = batched_section(args, stream)
        extra["differentiable"] = differentiable_section(args)
    if rank == 0:
        line = {
            "metric": "particle-substeps/s", "value": value, "unit": "particle-substeps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload, "particles": n, "N": N, "material": cfg["materials"][0].name,
                       "dt": cfg["params"]["dt"], "sort_interval": cfg["params"].get("sort_interval", 0),
                       "l2": "flushed between steps (512 MiB write, outside the timed events)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks, "gpu_launches": launches,
            "wall_s_timed_region": wall, "tuning": tuning,
        }
        if extra:
            line["snow"] = extra["snow"]
            line["batched"] = extra["batched"]
            line["differentiable"] = extra["differentiable"]
            line["snow_value"] = extra["snow"]["value"]
            line["snow_roofline_frac"] = extra["snow"]["roofline"]["frac"]
            line["batched_vs_looped"] = extra["batched"]["batched_vs_looped"]
            line["bwd_fwd_ratio"] = extra["differentiable"]["bwd_fwd_ratio"]
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def snow_section(args, stream, num_sms):
    """The snow workload (500,000 particles in two spheres, N = 64, SVD plasticity),
    timed like the headline: single substeps, L2 flushed between them."""
    import torch

    from mpm_gb300.simulation import Simulation

    cfg, workload = make_cfg("snow")
    n = cfg["state"]["x"].shape[0]
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    with Simulation.from_config(cfg) as sim:
        sim.set_stream(stream.cuda_stream)
        sim.upload(cfg["state"])
        tuning = choose_shape(sim, args.shape)
        ms, pure, launches, _ = time_substeps(sim, args.steps, max(args.warmup, 3), stream, flush)
        sim.sync()
    del flush
    roof = substep_roofline(cfg, n, ms, pure, workload)
    roof["issue_frac"] = issue_fraction(roof, workload, None, num_sms)
    return {"value": n * len(ms) / (sum(ms) * 1e-3), "unit": "particle-substeps/s", "ms_per_step": sum(ms) / len(ms),
            "steps": len(ms), "roofline": roof, "gpu_launches": launches, "tuning": tuning,
            "config": {"workload": workload, "particles": n, "N": cfg["params"]["N"], "material": "snow",
                       "sort_interval": cfg["params"]["sort_interval"], "l2": "flushed between steps"}}


def run_e2e(sim, cfg, steps, world):
    """Per step through the C ABI: pinned host state -> device, one substep,
    device -> pinned host state; wall clock around the blocking calls, averaged over the
    steps."""
    import ctypes

    import torch

    st = cfg["state"]
    n = st["x"].shape[0]
    liquid = cfg["materials"][0].kind == 3
    fields = {"x": 3, "v": 3, "C": 9, "Jp": 1} if liquid else {"x": 3, "v": 3, "C": 9, "F": 9, "Jp": 1}
    host = {k: torch.from_numpy(np.ascontiguousarray(np.asarray(st[k], np.float32).reshape(n, w))).pin_memory()
            for k, w in fields.items()}
    out = {k: torch.empty((n, w), dtype=torch.float32).pin_memory() for k, w in fields.items()}
    P = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
    L = sim.L
    times = []
    for k in range(steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc = L.mpm_upload_soa(sim.ctx, n, P(host["x"]), P(host["v"]), P(host["C"]), P(host.get("F")),
                              P(host["Jp"]), None)
        rc |= L.mpm_substep(sim.ctx, 1)
        rc |= L.mpm_download_soa(sim.ctx, P(out["x"]), P(out["v"]), P(out["C"]), P(out.get("F")), P(out["Jp"]),
                                 None)
        t1 = time.perf_counter()
        if rc != 0:
            raise RuntimeError("e2e C ABI call failed")
        if k > 0:
            times.append(t1 - t0)
    from mpm_gb300 import distributed as D

    # the mean, not the median: an upload of the same count keeps the device order and the
    # sort schedule, so every sort_interval-th step also sorts
    per = D.max_over_ranks(statistics.mean(times))  # the slowest replica
    nbytes = 4 * n * sum(fields.values())
    return {"value": D.job_rate(world * n, per), "unit": "particle-substeps/s", "h2d_bytes_per_step": nbytes,
            "d2h_bytes_per_step": nbytes, "ms_per_step": 1e3 * per,
            "path": "mpm_upload_soa + mpm_substep(1) + mpm_download_soa, pinned host buffers",
            "steps": len(times), "statistic": "mean over the steps (the periodic cell sort included)"}


def batched_section(args, stream, scs=None, rank=0, world=1):
    """The batched workload (256 scenes): one replayed CUDA graph of 50 substeps per step,
    against looping plain single-scene launches over the same scenes, measured two ways
    with no Python per-call dispatch: (a) a compiled host loop (mpm_substep_many) that
    enqueues substep by substep over one context per scene, and (b) that loop captured
    into one CUDA graph and replayed.  The ratio is taken against the faster looped arm."""
    import torch

    from mpm_gb300 import distributed as D
    from mpm_gb300 import scenes
    from mpm_gb300.batch import Batch
    from mpm_gb300.simulation import Simulation, advance_many

    all_scenes = scenes.config_batched(nscenes=256, seed=0)
    n_all = sum(s["state"]["x"].shape[0] for s in all_scenes)
    # scenes are independent: rank r takes scenes r, r + world, ... (no collective on the data path)
    scs = D.shard(all_scenes, rank, world)
    n = sum(s["state"]["x"].shape[0] for s in scs)
    sub = 50
    b = Batch(scs, sort_interval=16)
    b.set_stream(stream.cuda_stream)
    b.upload([s["state"] for s in scs])
    # the range size of the batched kernel, chosen by the batch autotuner on a copy of the batch
    from mpm_gb300 import autotune

    tuning = autotune.tune_batch(b, autotune.default_cache_path(), budget_substeps=24, tune_sort_interval=True)
    for _ in range(max(args.warmup, 3)):
        b.advance(sub, graph=True)
    torch.cuda.synchronize()
    D.barrier()
    torch.cuda.synchronize()
    steps = max(1, min(args.steps, 10))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    l0 = b.launches
    for a, e in ev:
        a.record(stream)
        b.advance(sub, graph=True)
        e.record(stream)
    torch.cuda.synchronize()
    batched_ms = sum(a.elapsed_time(e) for a, e in ev)
    local_rate = n * sub * steps / (batched_ms * 1e-3)
    batched_ms_max = D.max_over_ranks(batched_ms)  # the slowest rank's share
    launches = b.launches - l0
    b.sync()
    b.close()
    value = D.job_rate(n_all * sub * steps, batched_ms_max * 1e-3)

    # looped plain launches: one context per scene, all on one stream
    sims = []
    for sc in scs:
        sim = Simulation(materials=[sc["material"]], sort_interval=16, **sc["params"])
        sim.set_stream(stream.cuda_stream)
        sim.upload(sc["state"])
        sims.append(sim)
    advance_many(sims, 3)
    torch.cuda.synchronize()
    # (a) the compiled loop, 10 substeps of every scene: device time by events, wall time
    # of the enqueueing loop; the slower of the two is what the loop delivers
    loop_sub = 10
    a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    a.record(stream)
    advance_many(sims, loop_sub)
    e.record(stream)
    t_enq = time.perf_counter() - t0
    torch.cuda.synchronize()
    loop_wall = time.perf_counter() - t0
    loop_ms = a.elapsed_time(e)
    c_loop = n * loop_sub / max(loop_ms * 1e-3, loop_wall)
    # (b) the same loop over `sub` substeps captured once into a CUDA graph, replayed once
    # (a replay runs exactly the captured substeps, so the contexts stay consistent)
    graph_rate, graph_ms, nodes = None, None, None
    try:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream, capture_error_mode="thread_local"):
            advance_many(sims, sub)
        a.record(stream)
        g.replay()
        e.record(stream)
        torch.cuda.synchronize()
        graph_ms = a.elapsed_time(e)
        graph_rate = n * sub / (graph_ms * 1e-3)
        nodes = int(sum(s.launches for s in sims))
        del g
    except Exception as exc:  # report, do not hide: the compiled loop still stands
        graph_rate = None
        graph_ms = f"capture failed: {exc}"
    for sim in sims:
        sim.close()
    looped = max(c_loop, graph_rate or 0.0)
    return {"value": value, "unit": "particle-substeps/s", "ms_per_step": batched_ms_max / steps, "steps": steps,
            "substeps_per_step": sub, "gpu_launches": launches, "tuning": tuning,
            "config": {"workload": "batched_256_scenes", "particles": n_all, "scenes": 256, "graph": True,
                       "parallelism": f"scenes split over {world} ranks" if world > 1 else "single",
                       "l2": "inputs larger than L2 (state ~1 GB)"},
            "looped_c_loop": {"value": c_loop, "unit": "particle-substeps/s", "device_ms": loop_ms,
                              "wall_ms": 1e3 * loop_wall, "enqueue_ms": 1e3 * t_enq, "substeps": loop_sub,
                              "how": "mpm_substep_many: one compiled host loop, mpm_substep(ctx, 1) per scene per "
                                     "substep, one context per scene, one stream"},
            "looped_graph": {"value": graph_rate, "unit": "particle-substeps/s", "device_ms": graph_ms,
                             "substeps": sub,
                             "how": "the same compiled loop over 50 substeps captured into one CUDA graph, replayed "
                                    "once (device time by events)"},
            "batched_vs_looped": local_rate / looped,
            "looped_baseline": "the faster of looped_c_loop and looped_graph"}


def run_batched(args):
    import torch

    from mpm_gb300 import distributed as D

    world, rank, local = D.init("nccl")
    from mpm_gb300 import build

    if rank == 0 or world == 1:
        build.build()
    D.barrier()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sec = batched_section(args, stream, rank=rank, world=world)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    if rank != 0:
        return
    line = {"metric": "particle-substeps/s", "value": sec["value"], "unit": "particle-substeps/s", "n_gpus": world,
            "steps": sec["steps"], "warmup": args.warmup, "ms_per_step": sec["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic"}
    line.update({k: v for k, v in sec.items() if k not in line})
    print(json.dumps(line), flush=True)


def differentiable_section(args):
    """The differentiable workload (100,000 fixed-corotated particles, N = 64, 256
    substeps, a checkpoint every 16): the checkpointed forward and the backward
    (recompute of each segment + adjoint kernels), wall clock around the blocking
    mpm_diff_forward / mpm_diff_backward calls."""
    import torch

    from mpm_gb300 import scenes
    from mpm_gb300.autograd import DiffSim

    from mpm_gb300 import materials as M

    cfg = scenes.config_differentiable()
    st = cfg["state"]
    n = st["x"].shape[0]
    nsteps = 256
    target = np.array([0.6, 0.3, 0.5])

    def time_fwd_bwd(material):
        sim = DiffSim(cfg["params"], material, n, nsteps, 16)
        fw, bw = [], []
        for k in range(max(args.warmup, 1) + max(1, min(args.steps, 5))):
            t0 = time.perf_counter()
            xo, _ = sim.forward(st, nsteps)
            t1 = time.perf_counter()
            com = xo.astype(np.float64).mean(0)
            gx = np.tile(2.0 * (com - target) / n, (n, 1))
            t2 = time.perf_counter()
            sim.backward(gx)
            t3 = time.perf_counter()
            if k >= max(args.warmup, 1):
                fw.append(t1 - t0)
                bw.append(t3 - t2)
        sim.close()
        torch.cuda.synchronize()
        return statistics.median(fw), statistics.median(bw), len(fw)

    which = getattr(args, "diff_material", "both")
    f = b = k = None
    if which in ("both", "fixed_corotated"):
        f, b, k = time_fwd_bwd(cfg["materials"][0])
    snow = None
    if which in ("both", "snow"):
        # the same body as snow (plasticity and hardening in the adjoint)
        sf, sb, k2 = time_fwd_bwd(M.snow(cfg["materials"][0].particle_volume))
        snow = {"forward_s": sf, "backward_s": sb, "bwd_fwd_ratio": sb / sf,
                "material": "snow (E 1.4e5, nu 0.2, hardening 10, clamps [0.975, 1.0075])"}
        if f is None:
            f, b, k = sf, sb, k2
    return {"value": n * nsteps / f, "unit": "particle-substeps/s", "forward_s": f, "backward_s": b,
            "bwd_fwd_ratio": b / f, "steps": k, "snow": snow,
            "config": {"workload": "differentiable_100k_N64_256", "particles": n, "N": 64, "substeps": nsteps,
                       "checkpoint_every": 16},
            "timing": "wall clock around the blocking mpm_diff_forward / mpm_diff_backward calls (host copies of "
                      "the initial state and of the gradients included)"}


def run_differentiable(args):
    from mpm_gb300 import build

    build.build()
    sec = differentiable_section(args)
    line = {"metric": "particle-substeps/s", "value": sec["value"], "unit": "particle-substeps/s", "n_gpus": 1,
            "steps": sec["steps"], "warmup": args.warmup, "ms_per_step": 1e3 * sec["forward_s"] / 256,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic"}
    line.update({k: v for k, v in sec.items() if k not in line})
    print(json.dumps(line), flush=True)


def run_seeding(args):
    """Scene objects: GPU rejection sampling of a closed triangle mesh (an icosphere of
    20 x 4^4 triangles, size 0.5) at 2e7 candidates per unit volume, through
    mpm_add_object (seeding plus the append into the context); the oracle's restatement
    seeds a bounded sample of the same object on one host thread."""
    from mpm_gb300 import build

    build.build()
    import torch

    import oracle
    from mpm_gb300 import _lib
    from mpm_gb300 import materials as M
    from mpm_gb300.scene_file import SceneObject
    from mpm_gb300.simulation import Simulation

    V, F = _icosphere(4)
    dens = 20_000_000
    obj = SceneObject(shape=_lib.SHAPE_MESH, size=0.5, position=(0.25, 0.25, 0.25), vertices=V, triangles=F)
    def time_add(o):
        times, count = [], 0
        for k in range(max(args.warmup, 1) + max(1, min(args.steps, 10))):
            sim = Simulation(dt=1e-4, N=64, materials=[M.elastic(1.0 / dens)])
            o.seed = k
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            count = sim.add_object(o)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            sim.close()
            if k >= max(args.warmup, 1):
                times.append(t1 - t0)
        return statistics.median(times), count, len(times)

    dt_s, count, nsteps = time_add(obj)
    # the same object with the winding-number inside test (every triangle per candidate)
    wobj = SceneObject(shape=_lib.SHAPE_MESH, size=0.5, position=(0.25, 0.25, 0.25), vertices=V, triangles=F,
                       inside_test=_lib.INSIDE_WINDING)
    w_s, w_count, _ = time_add(wobj)
    cand = int(dens * 0.5 ** 3)
    # oracle: one host thread on a bounded sample (same object, smaller density)
    sdens = 400_000
    t0 = time.perf_counter()
    xs = oracle.seed_object(_lib.SHAPE_MESH, 0.5, (0.25, 0.25, 0.25), seed=0, density=sdens, vertices=V, triangles=F)
    cpu_s = time.perf_counter() - t0
    line = {"metric": "seeded particles/s", "value": count / dt_s, "unit": "particles/s", "n_gpus": 1,
            "steps": nsteps, "warmup": args.warmup, "ms_per_step": 1e3 * dt_s, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 tests, f32 positions", "data": "synthetic",
            "config": {"workload": "seed_icosphere_5120tri_2e7", "candidates": cand, "particles": count,
                       "triangles": int(F.shape[0])},
            "cpu_baseline": {"value": len(xs) / cpu_s, "unit": "particles/s", "cores": 1, "kind": "port",
                             "sample": f"{len(xs)} particles of the same object at density {sdens} (oracle, "
                                       f"all triangles per candidate, {cpu_s:.1f} s)"},
            "timing": "wall clock around mpm_add_object (GPU seeding, count readback, append)",
            "winding_number": {"value": w_count / w_s, "unit": "particles/s", "ms_per_step": 1e3 * w_s,
                               "particles": w_count,
                               "how": "the same object with inside_test = MPM_INSIDE_WINDING (FP32 solid angles over "
                                      "all 5,120 triangles per candidate, FP64 for points near the surface)"}}
    print(json.dumps(line), flush=True)


def run_mesh(args):
    """Surface reconstruction at the reference's mesh defaults (include/options.h:30-31:
    a 250^3 voxel grid, particle radius 5 voxels) of 500,000 particles (the reference's
    default particle count) filling a ball of radius 0.25 in an N=60 domain, after 10
    snow substeps.  A step is one surface extraction as MeshBuilder::computeMesh makes it
    (up to the OBJ text): distance field, marching-cubes count, scan, and the emit of
    libigl's vertex list and the faces.  value: device time (CUDA events on the context's
    stream) of mpm_surface_mesh_indexed_device, the mesh left in HBM; e2e: wall clock of
    mpm_surface_mesh_indexed, which also copies vertices and faces to pinned host memory.
    The oracle meshes the same particles on one host thread."""
    from mpm_gb300 import build

    build.build()
    import ctypes

    import torch

    import oracle
    from mpm_gb300 import _lib
    from mpm_gb300 import materials as M
    from mpm_gb300.simulation import Simulation

    G, radius, n, N = 250, 5, 500_000, 60
    rng = np.random.default_rng(0)
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    x = (0.5 + u * 0.25 * rng.random(n)[:, None] ** (1.0 / 3.0)).astype(np.float32)
    sim = Simulation(dt=1e-4, N=N, materials=[M.snow(1.0 / n)])
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    sim.upload({"x": x})
    sim.advance(10)
    sim.sync()
    cap = 4 * 1024 * 1024
    Vh = torch.empty((cap, 3), dtype=torch.float64, pin_memory=True)
    Fh = torch.empty((cap, 3), dtype=torch.int32, pin_memory=True)
    nv, cnt = ctypes.c_int64(), ctypes.c_int64()
    L = sim.L

    dptr, fptr = ctypes.c_void_p(), ctypes.c_void_p()

    def call_host():
        _lib.check(L.mpm_surface_mesh_indexed(sim.ctx, G, radius, ctypes.c_void_p(Vh.data_ptr()), cap,
                                              ctypes.c_void_p(Fh.data_ptr()), cap, ctypes.byref(nv),
                                              ctypes.byref(cnt)), sim.ctx)

    def call_device():
        _lib.check(L.mpm_surface_mesh_indexed_device(sim.ctx, G, radius, ctypes.byref(dptr), ctypes.byref(fptr),
                                                     ctypes.byref(nv), ctypes.byref(cnt)), sim.ctx)

    def call_field():
        _lib.check(L.mpm_surface_distance_device(sim.ctx, G, radius, ctypes.byref(dptr)), sim.ctx)

    for _ in range(max(args.warmup, 3)):
        call_host()
        call_device()
        call_field()
    steps = max(1, min(args.steps, 20))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(fn):
        """Device time (CUDA events on the context's stream) and wall time of fn, L2 flushed before."""
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        t1 = time.perf_counter()
        return e0.elapsed_time(e1) * 1e-3, t1 - t0

    clocks = ClockSampler(0)
    clocks.start()
    launches0 = sim.launches
    t_start = time.time()
    dev = [timed(call_device)[0] for _ in range(steps)]
    t_end = time.time()
    launches = (sim.launches - launches0) // steps
    wall = [timed(call_host)[1] for _ in range(steps)]
    field_s = statistics.median([timed(call_field)[0] for _ in range(steps)])
    clk = clocks.stop(t_start, t_end)
    ntri, nvert = int(cnt.value), int(nv.value)
    d_s, w_s = statistics.median(dev), statistics.median(wall)
    peak, peak_kind = measured_peaks()
    # oracle on one host thread: the same particles and grid
    xs = sim.download(("x",))["x"]
    vdx = oracle.voxel_dx(N, float(np.float32(1.0 / N)), G)
    c0 = time.perf_counter()
    f = oracle.distance_field(xs, G, radius, vdx)
    ref_V, ref_F = oracle.surface_indexed(f, radius, vdx)
    cpu_s = time.perf_counter() - c0
    # distance-field pass (fill, scatter, finish): minimal bytes = positions read once and
    # the field written once
    alg = 12.0 * n + 4.0 * G ** 3
    line = {"metric": "surface meshes/s", "value": 1.0 / d_s, "unit": "meshes/s", "n_gpus": 1, "steps": steps,
            "warmup": max(args.warmup, 3), "ms_per_step": 1e3 * d_s, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 field, f64 vertices", "data": "synthetic",
            "config": {"workload": "mesh_ball_500k_G250_r5", "particles": n, "grid_side": G, "radius": radius,
                       "N": N, "vertices": nvert, "faces": ntri,
                       "l2": "512 MiB flush between steps"},
            "e2e": {"value": 1.0 / w_s, "unit": "meshes/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 24 * nvert + 12 * ntri + 12},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": alg / field_s / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg / field_s / 1e9 / peak, "traffic": None,
                         "kernel": "distance field (fill + distance_kernel + finish)",
                         "note": f"positions read + field written once per pass; the scatter is bound by "
                                 f"shared-memory reductions (one per particle-node pair), not HBM; peak of "
                                 f"{peak_kind}"},
            "distance_field_ms": 1e3 * field_s,
            "clocks": clk,
            "oracle_faces": int(ref_F.shape[0]),
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "meshes/s", "cores": 1, "kind": "port",
                             "sample": f"the same {n} particles on the same grid (oracle distance field and "
                                       f"marching cubes, 1 thread, {cpu_s:.1f} s)"}}
    line["smooth"] = smooth_section(sim, Vh, Fh, nvert, ntri, timed, steps)
    print(json.dumps(line), flush=True)


def smooth_section(sim, Vh, Fh, nv, nf, timed, steps):
    """MeshBuilder::smoothMesh (include/mesh_builder.h:212-245, the reference's
    --laplacian_smooth) on the mesh just extracted: device time of mpm_surface_smooth_device
    on a copy of the vertices in HBM (CUDA events on the context's stream, L2 flushed
    before), the conjugate-gradient iteration count, the wall time of mpm_surface_smooth on
    host arrays, and the oracle's direct sparse solve of the same system on the host
    (scipy's SuperLU) with the largest difference between the two."""
    import ctypes

    import torch

    from mpm_gb300 import _lib
    from oracle import smooth_oracle

    V0 = Vh[:nv].clone().numpy()
    F0 = Fh[:nf].clone().numpy()
    V0d = torch.from_numpy(V0).cuda()
    Fd = torch.from_numpy(F0).cuda()
    Vd = torch.empty_like(V0d)
    it = ctypes.c_int32()

    def call_device():
        _lib.check(sim.L.mpm_surface_smooth_device(sim.ctx, ctypes.c_void_p(Vd.data_ptr()), nv,
                                                   ctypes.c_void_p(Fd.data_ptr()), nf, ctypes.byref(it)), sim.ctx)

    Vh2 = V0.copy()

    def call_host():
        Vh2[:] = V0
        _lib.check(sim.L.mpm_surface_smooth(sim.ctx, Vh2.ctypes.data_as(ctypes.c_void_p), nv,
                                            F0.ctypes.data_as(ctypes.c_void_p), nf, ctypes.byref(it)), sim.ctx)

    Vd.copy_(V0d)
    call_device()
    dev, launches = [], []
    for _ in range(steps):
        Vd.copy_(V0d)
        l0 = sim.launches
        dev.append(timed(call_device)[0])
        launches.append(sim.launches - l0)
    wall = [timed(call_host)[1] for _ in range(min(steps, 5))]
    c0 = time.perf_counter()
    ref = smooth_oracle.smooth_mesh(V0, F0)
    cpu_s = time.perf_counter() - c0
    U = Vd.cpu().numpy()
    d_s = statistics.median(dev)
    return {"ms": 1e3 * d_s, "iterations": int(it.value), "us_per_iteration": 1e6 * d_s / max(it.value, 1),
            "gpu_launches": int(statistics.median(launches)), "e2e_ms": 1e3 * statistics.median(wall),
            "max_rel_diff_vs_oracle": float(np.abs(U - ref).max() / np.abs(ref).max()),
            "cpu_baseline": {"ms": 1e3 * cpu_s, "cores": 1, "kind": "port",
                             "sample": f"scipy SuperLU direct solve of the same {nv}-vertex system"}}


def _liquid_sim(stream):
    """The liquid throughput scene (1M particles, N=32) advanced 16 substeps, on `stream`."""
    from mpm_gb300.simulation import Simulation

    cfg, _ = make_cfg("liquid")
    sim = Simulation.from_config(cfg)
    sim.set_stream(stream.cuda_stream)
    sim.upload(cfg["state"])
    sim.advance(16)
    sim.sync()
    return sim, cfg


def run_export(args):
    """Particle export of the liquid scene (1M particles): the reference's per-frame
    ParticleWriter::writeParticles (include/particle_writer.h:19-43) as .bgeo point records.
    A step is one frame: mpm_export_particles (records packed on the GPU in active-list
    order, copied to pinned memory on a copy stream) and mpm_export_wait.  value: exported
    particles/s of that pair (wall clock: the copy ends it); roofline: the packing kernel
    (24 B of x, v and 4 B of id read, 36 B written per particle) by CUDA events on the
    context's stream; e2e: the same frame with the uncompressed file written to /dev/shm
    (or the temp directory).  overlap: 16 substeps with and without a frame export between
    them.  The oracle writes the same file from host arrays with numpy (1 core)."""
    from mpm_gb300 import build

    build.build()
    import ctypes
    import tempfile

    import torch

    import oracle.export_oracle as E
    from mpm_gb300 import particle_writer as W

    stream = torch.cuda.Stream()
    sim, cfg = _liquid_sim(stream)
    n = sim.n
    for _ in range(max(args.warmup, 3)):
        W.export_records(sim, 0)
        W.wait_records(sim, 0)
    steps = max(1, min(args.steps, 50))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    clocks = ClockSampler(0)
    clocks.start()
    t_start = time.time()
    wall, pack = [], []
    launches0 = sim.launches
    for k in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(stream)
        W.export_records(sim, k & 1)
        e1.record(stream)
        W.wait_records(sim, k & 1)
        wall.append(time.perf_counter() - t0)
        torch.cuda.synchronize()
        pack.append(e0.elapsed_time(e1) * 1e-3)
    t_end = time.time()
    clk = clocks.stop(t_start, t_end)
    launches = (sim.launches - launches0) // steps
    outdir = "/dev/shm" if os.path.isdir("/dev/shm") else tempfile.gettempdir()
    path = os.path.join(outdir, f"mpm_export_{os.getpid()}.bgeo")
    e2e = []
    writer = W.ParticleWriter()
    for _ in range(min(steps, 10)):
        t0 = time.perf_counter()
        writer.writeParticles(path, sim)
        e2e.append(time.perf_counter() - t0)
    size = os.path.getsize(path)
    os.remove(path)
    # overlap: 16 substeps alone, then 16 substeps with a frame exported after the first
    def loop(export):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.advance(1)
        if export:
            W.export_records(sim, 0)
        sim.advance(15)
        if export:
            W.wait_records(sim, 0)
        sim.sync()
        return time.perf_counter() - t0
    loop(False), loop(True)
    plain = statistics.median([loop(False) for _ in range(5)])
    with_export = statistics.median([loop(True) for _ in range(5)])
    # oracle: the same file from host arrays
    st = sim.download(("x", "v"))
    c0 = time.perf_counter()
    ref = E.bgeo_file(st["x"], st["v"])
    cpu_s = time.perf_counter() - c0
    w_s, p_s = statistics.median(wall), statistics.median(pack)
    peak, peak_kind = measured_peaks()
    alg = 64.0 * n
    line = {"metric": "exported particles/s", "value": n / w_s, "unit": "particles/s", "n_gpus": 1, "steps": steps,
            "warmup": max(args.warmup, 3), "ms_per_step": 1e3 * w_s, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 records (big-endian)", "data": "synthetic",
            "config": {"workload": "export_liquid_1M", "particles": n, "record_bytes": 36, "file_bytes": size,
                       "l2": "512 MiB flush between steps"},
            "e2e": {"value": n / statistics.median(e2e), "unit": "particles/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 36 * n, "file": outdir},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": alg / p_s / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg / p_s / 1e9 / peak, "traffic": None, "kernel": "bgeo_pack_kernel",
                         "note": f"64 B per particle (x, v, id read; record written); peak of {peak_kind}"},
            "pack_ms": 1e3 * p_s, "copy_GBps": 36.0 * n / w_s / 1e9,
            "overlap": {"substeps_16_ms": 1e3 * plain, "substeps_16_with_export_ms": 1e3 * with_export},
            "clocks": clk, "oracle_bytes_equal": bool(len(ref) == size),
            "cpu_baseline": {"value": n / cpu_s, "unit": "particles/s", "cores": 1, "kind": "port",
                             "sample": f"the same {n} particles: numpy writer of the oracle from host arrays "
                                       f"({cpu_s:.3f} s)"}}
    print(json.dumps(line), flush=True)


def run_render(args):
    """Headless point rendering of the liquid scene (1M particles): the reference's
    Renderer::render (include/renderer.h:43-63) at 800 x 600 with 2-pixel points.  A step is
    one mpm_render_points call (clear, splat, colour, copy of the RGB8 image to host).
    value: frames/s by CUDA events on the context's stream (the copy included); e2e: wall
    clock of the call.  The oracle rasterises the same particles with numpy (1 core)."""
    from mpm_gb300 import build

    build.build()
    import torch

    import oracle.export_oracle as E
    from mpm_gb300.renderer import Renderer

    stream = torch.cuda.Stream()
    sim, cfg = _liquid_sim(stream)
    n = sim.n
    r = Renderer()
    for _ in range(max(args.warmup, 3)):
        r.render(sim)
    steps = max(1, min(args.steps, 50))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    clocks = ClockSampler(0)
    clocks.start()
    t_start = time.time()
    dev, wall = [], []
    launches0 = sim.launches
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(stream)
        img = r.render(sim)
        e1.record(stream)
        wall.append(time.perf_counter() - t0)
        torch.cuda.synchronize()
        dev.append(e0.elapsed_time(e1) * 1e-3)
    t_end = time.time()
    clk = clocks.stop(t_start, t_end)
    launches = (sim.launches - launches0) // steps
    x = sim.download(("x",))["x"]
    c0 = time.perf_counter()
    ref = E.render_points(x)
    cpu_s = time.perf_counter() - c0
    d_s, w_s = statistics.median(dev), statistics.median(wall)
    peak, peak_kind = measured_peaks()
    alg = 12.0 * n + 4.0 * 800 * 600
    line = {"metric": "rendered frames/s", "value": 1.0 / d_s, "unit": "frames/s", "n_gpus": 1, "steps": steps,
            "warmup": max(args.warmup, 3), "ms_per_step": 1e3 * d_s, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 positions, u8 image", "data": "synthetic",
            "config": {"workload": "render_liquid_1M_800x600", "particles": n, "width": 800, "height": 600,
                       "point_size": 2.0, "l2": "512 MiB flush between steps"},
            "e2e": {"value": 1.0 / w_s, "unit": "frames/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 3 * 800 * 600},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": alg / d_s / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg / d_s / 1e9 / peak, "traffic": None, "kernel": "whole call",
                         "note": f"positions read, mask and image written once; peak of {peak_kind}"},
            "clocks": clk, "oracle_image_equal": bool(np.array_equal(img, ref)),
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "frames/s", "cores": 1, "kind": "port",
                             "sample": f"the same {n} particles, numpy rasteriser of the oracle ({cpu_s:.3f} s)"}}
    print(json.dumps(line), flush=True)


def _icosphere(subdivisions):
    t = (1.0 + 5 ** 0.5) / 2.0
    V = [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]]
    F = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6],
         [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
         [8, 6, 7], [9, 8, 1]]
    V = [np.asarray(v, np.float64) / np.linalg.norm(v) for v in V]
    for _ in range(subdivisions):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                m = (V[a] + V[b]) / 2.0
                V.append(m / np.linalg.norm(m))
                mid[key] = len(V) - 1
            return mid[key]

        nf = []
        for a, b, c in F:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        F = nf
    return np.asarray(V, np.float32), np.asarray(F, np.int32)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "batched":
        run_batched(args)
    elif args.config == "differentiable":
        run_differentiable(args)
    elif args.config == "seeding":
        run_seeding(args)
    elif args.config == "mesh":
        run_mesh(args)
    elif args.config == "export":
        run_export(args)
    elif args.config == "render":
        run_render(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
