#!/usr/bin/env python
"""Benchmark of the particle-tracing hot path on GB300.

Workload (one "step"): the FTLE pipeline on a 256^3 FP32 ABC flow plus
N(0, 0.01) noise (seed 0): one seed per grid vertex (16,777,216 particles),
classical RK4 with four field samples per step, h = 0.01, at most 500 steps
(T = 5), flow map, then the fused gradient / Cauchy-Green / Jacobi eigenvalue /
log FTLE kernel (FP32).  Metric: RK4 particle-steps per second (steps actually
taken), with FTLE voxels per second beside it.

value : device-resident input, timed with CUDA events on the library's stream.
e2e   : the same through the C ABI from pinned HOST buffers: field upload
        (host -> device), flow map, FTLE, FTLE download (device -> host).
--impl reference : the reference's CPU algorithm (the oracle port of it,
        frozen-velocity RK4 as the reference computes it) on the host cores,
        on a bounded sample of the same workload.

Multi-GPU: independent replicas (one process per GPU under torchrun), weak
scaling; value = all ranks' steps / max-over-ranks time.
"""
import argparse
import json
import os
import platform
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RK4 particle-steps/s"
UNIT = "particle-steps/s"
BYTES_PER_RK4_STEP = 512          # 4 samples x 8 corners x 16 B (flow-map mode: no vertex store)
BYTES_PER_FTLE_VOXEL = 100        # 6 neighbour float4 reads + one FP32 write


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--size", type=int, default=256)
    p.add_argument("--iterations", type=int, default=501)
    p.add_argument("--cpu-stride", type=int, default=16,
                   help="CPU baseline's bounded sample: every cpu-stride-th seed of the C-order seed list")
    p.add_argument("--no-extra", action="store_true", help="headline workload only (skip the other workloads' lines)")
    p.add_argument("--dry-run", action="store_true",
                   help="check the multi-process launcher only: each rank reports on the CPU (gloo), no workload runs")
    p.add_argument("--requests", type=int, default=300, help="served workload: number of requests")
    p.add_argument("--serve-arms", default="plain,batched,cpu", help="served workload: arms to run (plain, batched, cpu)")
    p.add_argument("--serve-cpu-seconds", type=float, default=15.0, help="served workload: CPU reference arm's sample length")
    p.add_argument("--serve-loads", default="0.5,0.9", help="served workload: offered loads as fractions of saturation")
    p.add_argument("--serve-lanes", type=int, default=2, help="served workload: service lanes of the batched arm")
    p.add_argument("--serve-reply", choices=["curves", "image"], default="image",
                   help="served workload: what a streamline request returns to the client -- the pars_service reply, "
                        "an image of the curves ray traced on the GPU (pipeline.cpp:264-337), or every curve buffer")
    p.add_argument("--serve-image", default="960x540", help="served workload: image size of the image reply")
    p.add_argument("--domain-edge", type=int, default=512, help="domain workload: edge of the cube domain")
    p.add_argument("--domain-seeds", type=int, default=1_000_000, help="domain workload: seeds of the Gaussian mixture")
    p.add_argument("--workload", choices=["ftle", "streamlines", "domain", "pathlines", "serve", "render"], default="ftle",
                   help="ftle: the headline line; the others print one line for the other workloads")
    return p.parse_args()


def combine_ranks(dist, elapsed, steps, device):
    """Whole-job figures of N independent replicas: the slowest rank's time
    (max over ranks) and the steps all ranks took (sum).  dist is
    torch.distributed (or None for one process)."""
    if dist is None:
        return float(elapsed), float(steps)
    import torch
    t = torch.tensor([float(elapsed)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    s = torch.tensor([float(steps)], device=device, dtype=torch.float64)
    dist.all_reduce(s)
    return float(t.item()), float(s.item())


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic(steps_per_launch):
    """DRAM bytes per launch of the flow-map kernel from the committed ncu
    summary (bytes per particle-step measured there, scaled to this launch)."""
    path = os.path.join(ROOT, "profiles", "batch_advect_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("dram_bytes_per_particle_step:"):
            return float(line.split(":")[1]) * steps_per_launch
    return None


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        visible = os.environ.get("CUDA_VISIBLE_DEVICES")
        self.index = visible.split(",")[device] if visible else str(device)
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", self.index], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def wait_ready(self, timeout=10.0):
        """Blocks until the first sample arrives (at most `timeout` s): the
        first nvidia-smi start on a machine can take a second or more, and
        its NVML set-up stalls CUDA calls of this process meanwhile, so the
        timed region starts only after it."""
        deadline = time.time() + timeout
        while self.proc and not self.rows and self.proc.poll() is None and time.time() < deadline:
            time.sleep(0.02)
        time.sleep(0.2)

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def cpu_reference_run(field, iterations, stride, steps, warmup):
    """The reference's algorithm on the host cores: the oracle port's flow map
    (frozen-velocity RK4, FP32, the reference's operation order), all threads,
    on every stride-th seed of the C-order seed list (a uniform sample of the
    whole domain)."""
    import oracle
    port = oracle.port()
    threads = port.max_threads()
    for _ in range(warmup):
        port.flow_map(field, iterations, 1.0, 2, 0.01, 0, None, stride)
    total, t0 = 0, time.perf_counter()
    for _ in range(steps):
        _, s = port.flow_map(field, iterations, 1.0, 2, 0.01, 0, None, stride)
        total += s
    dt = time.perf_counter() - t0
    return total / dt, threads, dt


def host_cpu():
    """The host's CPU model and logical core count."""
    model = platform.processor() or platform.machine()
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                key = line.split(":")[0].strip().lower()
                if key in ("model name", "cpu model", "hardware"):
                    model = line.split(":", 1)[1].strip()
                    break
                if key == "cpu part" and model == platform.machine():
                    model = f"{platform.machine()} (CPU part {line.split(':', 1)[1].strip()})"
    except OSError:
        pass
    return {"cpu_model": model, "nproc": os.cpu_count()}


def cpu_single_thread(field, iterations, stride):
    """The same CPU leg on one thread, on every (16 stride)-th seed."""
    import oracle
    port = oracle.port()
    threads = port.max_threads()
    port.set_threads(1)
    try:
        value, _, _ = cpu_reference_run(field, iterations, stride * 16, 1, 0)
    finally:
        port.set_threads(threads)
    return {"value": value, "sample": f"every {stride * 16}th seed in C order, one thread"}


def cpu_sample_text(seeds, stride, n):
    count = (seeds + stride - 1) // stride
    return (f"every {stride}th of the {seeds} seeds in C order ({count} seeds spread over the whole {n}^3 domain) per step, "
            "frozen-velocity RK4 as the reference computes it (one field sample per step), FP32, all host threads")


def _events_time(torch, stream, fn):
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    out = fn()
    b.record(stream)
    torch.cuda.synchronize()
    return out, a.elapsed_time(b) * 1e-3


def run_streamlines(args):
    """The plain streamline workload: 64^3 ABC, 4096 seeds (stride 4), RK4
    h = 0.01, 1000 steps, rgb colours and indices; frozen (the reference's
    scheme) and re-sampled RK4."""
    import torch
    import oracle
    from pars_gb300 import native, workloads
    cfg = workloads.streamline_config()
    f = cfg["field"]
    ctx = native.Context(0)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    seeds = ctx.seed_generate(f.offset, f.size, cfg["stride"], cfg["iterations"])
    h = ctx.upload_field(f)
    out = {}
    for name, mode in (("frozen", native.STAGES_FROZEN), ("resampled", native.STAGES_RESAMPLED)):
        def once():
            s = ctx.trace(h, seeds, native.RUNGE_KUTTA_4, mode, cfg["step"])
            ctx.curves_index()
            ctx.curves_color("rgb")
            return s
        for _ in range(max(args.warmup, 3)):
            once()
        total, t = 0, 0.0
        for _ in range(args.steps):
            s, dt = _events_time(torch, stream, once)
            total += s["steps"]
            t += dt
        out[name] = total / t
        out[name + "_ms"] = 1e3 * t / args.steps
    port = oracle.port()
    t0 = time.perf_counter()
    ref = port.trace_single(f, seeds, 2, cfg["step"], "rgb", 0.5)
    cpu = ref.steps / (time.perf_counter() - t0)
    print(json.dumps({"workload": "streamlines_64: 64^3 ABC, 4096 seeds, RK4 h=0.01, <=1000 steps, index + rgb colour",
                      "metric": METRIC, "unit": UNIT, "value": out["resampled"], "ms_per_call_resampled": out["resampled_ms"],
                      "frozen_velocity_steps_per_s": out["frozen"], "ms_per_call_frozen": out["frozen_ms"],
                      "steps_per_call": ref.steps, "cpu_port_steps_per_s": cpu, "cpu_threads": port.max_threads()}))
    ctx.close()


def run_render(args):
    """The ray tracer (pars::ray_tracer's stage 6: set_integral_curves, trace,
    serialize) on the benchmark generator's settings
    (pars_benchmark_generator/source/main.cpp:7-28): image 1080 x 1920, one
    iteration, streamline radius 0.1 voxel, camera looking along +z, curves
    coloured hsv_constant_s 0.75.  Scenes: the 64^3 ABC streamlines (4096
    seeds, <= 1000 RK4 steps, h = 0.01), the same with a stride-2 lattice
    (32768 seeds), and the 64^3 scene with the field's normalised speed as the
    volume.  One image = set_integral_curves (BVH build) + trace(1) +
    serialize into host memory; the CPU restatement of the same shading on all
    host threads is timed on each scene beside it."""
    import oracle
    from pars_gb300 import native, workloads
    cfg = workloads.streamline_config()
    f = cfg["field"]
    ctx = native.Context(0)
    h = ctx.upload_field(f)
    port = oracle.port()
    width, height = 1080, 1920
    radius = float(np.float32(0.1) * f.spacing[0])
    camera = ((float(np.pi), float(np.pi), -9.0), (0.0, 0.0, 1.0), (0.0, 1.0, 0.0))
    speed = np.linalg.norm(f.xyz, axis=-1)
    volume = ((speed / speed.max()).astype(np.float32), f.offset, f.spacing)
    scenes = []
    for name, stride, vol in (("streamlines_64", 4, None), ("streamlines_64_stride2", 2, None), ("streamlines_64_volume", 4, volume)):
        seeds = ctx.seed_generate(f.offset, f.size, (f.spacing * np.float32(stride)).astype(np.float32), cfg["iterations"])
        s = ctx.trace(h, seeds, native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED, cfg["step"])
        ctx.curves_index()
        ctx.curves_color("hsv_constant_s", 0.75)
        if vol is None:
            ctx.ray_tracer_clear_volume()
        else:
            ctx.ray_tracer_set_volume(*vol)
        ctx.ray_tracer_set_image_size(width, height)
        ctx.ray_tracer_set_camera(*camera)

        phases = {"set_integral_curves": 0.0, "trace": 0.0, "serialize": 0.0}
        frame = np.zeros((height, width, 4), np.uint8)          # the client's image buffer, reused

        def image():
            t = [time.perf_counter()]
            ctx.ray_tracer_set_integral_curves(radius)
            t.append(time.perf_counter())
            ctx.ray_tracer_trace(1)
            t.append(time.perf_counter())
            out = ctx.ray_tracer_serialize(out=frame)
            t.append(time.perf_counter())
            for k, phase in enumerate(phases):
                phases[phase] += t[k + 1] - t[k]
            return out

        for _ in range(max(args.warmup, 3)):
            image()
        for phase in phases:
            phases[phase] = 0.0
        ctx.profile_enable(True)
        ctx.profile_reset()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            rgba = image()
        wall = (time.perf_counter() - t0) / args.steps
        build_ms, _ = ctx.profile_get("bvh_build")
        render_ms, _ = ctx.profile_get("render")
        ctx.profile_enable(False)
        batches = ctx.curves(s["batches"], vertices=True, colors=True, indices=True)
        host = [(b["vertices"], b["colors"], b["indices"]) for b in batches]
        segments = sum(len(b["indices"]) for b in batches)
        c0 = time.perf_counter()
        expected, _ = port.render(host, radius, camera, (width, height), frames=1, volume=vol)
        cpu = time.perf_counter() - c0
        scenes.append({"scene": name, "segments": segments, "volume": vol is not None,
                       "ms_per_image": 1e3 * wall, "images_per_s": 1.0 / wall,
                       "call_ms": {k: 1e3 * v / args.steps for k, v in phases.items()},
                       "bvh_build_ms": build_ms / args.steps, "render_ms": render_ms / args.steps,
                       "rays_per_s": width * height / (1e-3 * render_ms / args.steps),
                       "cpu_restatement_ms_per_image": 1e3 * cpu, "cpu_threads": port.max_threads(),
                       "pixels_equal_cpu": int(np.all(rgba == expected, axis=-1).sum()), "pixels": width * height})
    ctx.release_field(h)
    ctx.close()
    print(json.dumps({"workload": "render: the benchmark generator's ray-tracing settings (1080 x 1920, 1 iteration, radius "
                                  "0.1 voxel) on 64^3 ABC streamlines", "metric": "images/s", "unit": "images/s",
                      "value": scenes[0]["images_per_s"], "scenes": scenes}))


def run_domain(args):
    """The partitioned workload: 512^3 Arnold-Beltrami field + 8 Fourier modes
    (seed 1) split 4x4x4 into 64 blocks on one GPU; 1M seeds from a 4-centre
    Gaussian mixture (sigma = 0.05 of the domain, seed 2); RK4 h = 0.005,
    2000 steps; particles handed between blocks each round on the device."""
    import torch
    from pars_gb300 import native, workloads
    n = args.domain_edge
    ctx = native.Context(0)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    xyz, spacing = workloads.beltrami_fourier_device(torch, n, seed=1)
    ranks = 64
    d = ctx.domain_create_device(xyz.data_ptr(), (n, n, n), spacing, ranks)
    del xyz
    torch.cuda.empty_cache()
    info = native.partition(ranks, 0, (n, n, n))
    seeds, offsets = workloads.gaussian_mixture_seeds(args.domain_seeds, n, spacing, info, remaining=2002, seed=2)
    s, dt = None, 0.0
    for _ in range(max(args.warmup, 1)):
        ctx.trace_domain(d, seeds, offsets, native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED, 0.005)
    total, t = 0, 0.0
    for _ in range(args.steps):
        s, dt = _events_time(torch, stream, lambda: ctx.trace_domain(d, seeds, offsets, native.RUNGE_KUTTA_4,
                                                                     native.STAGES_RESAMPLED, 0.005))
        total += s["steps"]
        t += dt
    print(json.dumps({"workload": f"domain_{n}: {n}^3 Arnold-Beltrami + 8 Fourier modes, 64 blocks (4x4x4) on one GPU, "
                                  f"{args.domain_seeds} Gaussian-mixture seeds, RK4 h=0.005, <=2000 steps, device handoff queues",
                      "metric": METRIC, "unit": UNIT, "value": total / t, "ms_per_step": 1e3 * t / args.steps,
                      "steps_per_run": s["steps"], "rounds": s["rounds"], "batches": s["batches"],
                      "vertices": s["vertices"]}))
    ctx.domain_release(d)
    ctx.close()


def run_pathlines(args):
    """The batched-pathline workload: 32 unsteady double-gyre fields (edge
    log-uniform 32-256, 16-64 slices, seed counts log-uniform 1k-512k; seed 3),
    classical RK4 in space-time, h = 0.01 over one period (1000 steps), all
    fields in one persistent launch with the autotuned launch shape."""
    import torch
    from pars_gb300 import native, workloads
    ctx = native.Context(0)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    specs = workloads.pathline_batch_config(seed=3)
    jobs, keep = [], []
    gen = torch.Generator(device="cuda")
    gen.manual_seed(3)
    field_bytes = 0
    for spec in specs:
        xyz, offset, spacing, t0, dt = workloads.double_gyre_device(torch, spec["edge"], spec["slices"])
        n = spec["edge"]
        h = ctx.upload_unsteady_field_device(xyz.data_ptr(), (n, n, n), spec["slices"], offset,
                                              (np.array([n, n, n], np.float32) * spacing), spacing, t0, dt)
        field_bytes += n ** 3 * spec["slices"] * 16
        del xyz
        c = spec["seeds"]
        seeds = torch.zeros((c, 4), dtype=torch.float32, device="cuda")
        seeds[:, 0] = 0.05 + 1.9 * torch.rand(c, device="cuda", generator=gen)
        seeds[:, 1] = 0.05 + 0.9 * torch.rand(c, device="cuda", generator=gen)
        seeds[:, 2] = 0.05 + 0.9 * torch.rand(c, device="cuda", generator=gen)
        end = torch.empty((c, 4), dtype=torch.float32, device="cuda")
        j = native.BatchJob()
        j.field, j.integrator, j.stage_mode, j.max_steps, j.step_size = h, native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED, 1000, 0.01
        j.time_begin, j.seeds, j.seed_count, j.end_positions = 0.0, seeds.data_ptr(), c, end.data_ptr()
        jobs.append(j)
        keep.append((seeds, end))
    torch.cuda.empty_cache()
    ctx.batch_advect(jobs)   # tunes the launch shape on first use
    for _ in range(max(args.warmup - 1, 1)):
        ctx.batch_advect(jobs)
    total, t = 0, 0.0
    for _ in range(args.steps):
        steps, dt = _events_time(torch, stream, lambda: ctx.batch_advect(jobs))
        total += sum(steps)
        t += dt
    variant, threads = ctx.batch_tuned(1)
    print(json.dumps({"workload": "pathlines_32: 32 unsteady double-gyre fields (edge 32-256 log-uniform, 16-64 slices, "
                                  "1k-512k seeds log-uniform, seed 3), RK4 in space-time h=0.01, <=1000 steps, one persistent launch",
                      "metric": METRIC, "unit": UNIT, "value": total / t, "ms_per_step": 1e3 * t / args.steps,
                      "steps_per_run": total // args.steps, "seeds": sum(s["seeds"] for s in specs),
                      "field_bytes": field_bytes, "tuned_variant": variant, "threads_per_cta": threads}))
    ctx.close()


def run_cpu_reference(specs, host_fields, seconds):
    """The served stream through the reference's algorithm on the host cores:
    the oracle port (frozen-velocity RK4 in FP32 with the reference's operation
    order, OpenMP over particles on every host thread), request by request in
    stream order -- seeds, trace, indices and hsv_constant_s colours for a
    streamline request; flow map and FTLE for an FTLE request -- until
    `seconds` of work have been done.  Returns the sample's rates."""
    import oracle
    from pars_gb300 import workloads
    port = oracle.port()
    f32 = np.float32
    fields = {}
    done, steps, vertices, t0 = 0, 0, 0, time.perf_counter()
    for s in specs:
        if time.perf_counter() - t0 >= seconds:
            break
        if s["dataset"] not in fields:
            xyz, offset, size, spacing = host_fields[s["dataset"]]
            fields[s["dataset"]] = workloads.Field(xyz.numpy(), offset, spacing, size)
        f = fields[s["dataset"]]
        stride = (f.spacing * f32(s["stride"])).astype(f32)
        if s["kind"] == "streamlines":
            seeds = port.seed_generate(f.offset, f.size, stride, s["iterations"])
            curves = port.trace_single(f, seeds, 2, s["step"], "hsv_constant_s", 0.75)
            steps += curves.steps
            vertices += sum(len(b["vertices"]) for b in curves.batches)
        else:
            flow, n = port.flow_map(f, s["iterations"], float(f32(1.0) / f32(s["stride"])), 2, s["step"])
            port.ftle_fp64(flow, stride, float(f32(s["step"]) * f32(s["iterations"])))
            steps += n
        done += 1
    dt = time.perf_counter() - t0
    return {"requests_per_s": done / dt, "particle_steps_per_s": steps / dt, "cores": port.max_threads(),
            "kind": "port", "sample": f"the stream's first {done} requests ({steps} RK4 steps, {vertices} curve "
                                      f"vertices) in {dt:.1f} s"}


def run_serve(args):
    """The served mixed stream, end to end from host memory to host memory.

    plain   : one request at a time through the single-request C ABI, as a
              caller of the plain kernels serves it: upload the request's
              field from (pinned) host memory, seeds + trace + index + colour
              or flow map + FTLE, download every result buffer into pinned
              host buffers, release.
    batched : the service (two lanes by default, batches of up to 64, datasets
              resident, FTLE requests on the continuous engine; the other lane
              count is timed at saturation beside it, and the batched arm also
              runs at the plain path's 50 % offered load):
              requests are submitted as reference `settings` messages at their
              Poisson arrival times; a client thread collects each finished
              request's buffers into the same pinned host buffers.
    cpu     : the reference's algorithm on the host cores (run_cpu_reference),
              a bounded sample of the same stream from the same host fields.
    Latency runs from a request's arrival to its results being in host
    memory.  Both paths at saturation (every request present at t = 0) and at
    offered loads of 50 % and 90 % of their own saturation throughput."""
    import threading as th
    import torch
    from pars_gb300 import native, workloads
    from pars_gb300.requests import encode_settings
    ds, reqs = workloads.served_stream_config(seed=4, requests=args.requests)
    f32 = np.float32
    image_reply = args.serve_reply == "image"
    width, height = (int(x) for x in args.serve_image.split("x"))
    messages, specs = [], []
    for r in reqs:
        d = ds[r["dataset"]]
        step = 0.01 if d["kind"] == "abc" else 0.05
        iterations = r["steps"] + (2 if r["kind"] == "streamlines" else 1)
        # camera: the dataset's centre seen along +z from 1.6 extents away (fovy 68)
        extent = np.array([2 * np.pi] * 3 if d["kind"] == "abc" else [2.0, 1.0, 1.0])
        centre = extent / 2
        camera = (float(centre[0]), float(centre[1]), float(-1.6 * extent.max()))
        radius = float(f32(0.1) * f32(extent[0] / (d["edge"] - 1)))
        specs.append({"kind": r["kind"], "dataset": r["dataset"], "stride": r["stride"], "iterations": iterations, "step": step,
                      "camera": camera, "radius": radius})
        message = {
            "mode": r["kind"], "dataset_filepath": d["name"], "seed_generation_stride": [r["stride"]] * 3,
            "seed_generation_iterations": iterations,
            "particle_tracing_integrator": "runge_kutta_4", "particle_tracing_step_size": step,
            "color_generation_mode": "hsv_constant_s", "color_generation_free_parameter": 0.75}
        if image_reply and r["kind"] == "streamlines":
            message.update({"raytracing_camera_position": list(camera), "raytracing_camera_forward": [0.0, 0.0, 1.0],
                            "raytracing_camera_up": [0.0, 1.0, 0.0], "raytracing_image_size": [width, height],
                            "raytracing_streamline_radius": radius, "raytracing_iterations": 1})
        messages.append(encode_settings(message))

    # Datasets on the device (for the service) and in pinned host memory (for
    # the plain path, which uploads the request's field every time).
    device_fields, host_fields = [], []
    for d in ds:
        gen = workloads.abc_device if d["kind"] == "abc" else workloads.gyre_snapshot_device
        xyz, offset, size, spacing = gen(torch, d["edge"])
        pinned = torch.empty(xyz.shape, dtype=torch.float32, pin_memory=True)
        pinned.copy_(xyz)
        device_fields.append((xyz, offset, size, spacing))
        host_fields.append((pinned, offset, size, spacing))
    torch.cuda.synchronize()

    # Pinned collection buffers sized for the largest result.
    cap_vertices, cap_voxels = 1, 1
    for s in specs:
        _, offset, size, spacing = host_fields[s["dataset"]]
        if s["kind"] == "streamlines":
            st = (spacing * f32(s["stride"])).astype(f32)
            n = int(np.prod([int(f32(size[i]) / st[i]) for i in range(3)]))
            cap_vertices = max(cap_vertices, n * s["iterations"])
        else:
            scale = f32(1.0) / f32(s["stride"])
            edge = ds[s["dataset"]]["edge"]
            cap_voxels = max(cap_voxels, max(1, int(f32(edge) * scale)) ** 3)
    vbuf = torch.empty(cap_vertices * 4, dtype=torch.float32, pin_memory=True)
    cbuf = torch.empty(cap_vertices * 4, dtype=torch.float32, pin_memory=True)
    ibuf = torch.empty(cap_vertices, dtype=torch.int32, pin_memory=True)
    fbuf = torch.empty(cap_voxels, dtype=torch.float32, pin_memory=True)
    frame = torch.empty(width * height * 4, dtype=torch.uint8, pin_memory=True)
    collected = {"bytes": 0}

    def plain_request(ctx, k):
        s = specs[k]
        xyz, offset, size, spacing = host_fields[s["dataset"]]
        edge = ds[s["dataset"]]["edge"]
        h = ctx.upload_field_host(xyz.data_ptr(), (edge,) * 3, offset, size, spacing)
        if s["kind"] == "streamlines":
            seeds = ctx.seed_generate(offset, size, (spacing * f32(s["stride"])).astype(f32), s["iterations"])
            summary = ctx.trace(h, seeds, native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED, s["step"])
            ctx.curves_index()
            ctx.curves_color("hsv_constant_s", 0.75)
            if image_reply:
                # pipeline.cpp:264-337: the curves ray traced, the image to the client
                ctx.ray_tracer_set_image_size(width, height)
                ctx.ray_tracer_set_camera(s["camera"], (0.0, 0.0, 1.0), (0.0, 1.0, 0.0))
                ctx.ray_tracer_clear_volume()
                ctx.ray_tracer_set_integral_curves(s["radius"])
                ctx.ray_tracer_trace(1)
                size = np.zeros(2, np.int32)
                ctx._call("pars_gpu_ray_tracer_serialize", frame.data_ptr(), size.ctypes.data)
                collected["bytes"] += width * height * 4
            else:
                for b in range(summary["batches"]):
                    nv, ni, _, _ = ctx.batch_info(b)
                    ctx._call("pars_gpu_curves_download", b, vbuf.data_ptr(), cbuf.data_ptr(), ibuf.data_ptr())
                    collected["bytes"] += 32 * nv + 4 * ni
            steps = summary["steps"]
        else:
            fm, steps = ctx.flow_map_generate(h, s["iterations"], float(f32(1.0) / f32(s["stride"])), native.RUNGE_KUTTA_4,
                                              native.STAGES_RESAMPLED, s["step"])
            t = float(f32(s["step"]) * f32(s["iterations"]))
            shape = ctx.field_info(fm)["shape"]
            ctx._call("pars_gpu_ftle_generate", fm, t, native.FTLE_REGULAR, fbuf.data_ptr())
            collected["bytes"] += 4 * int(np.prod(shape))
            ctx.release_field(fm)
        ctx.release_field(h)
        return steps

    def run_plain(ctx, rate):
        t0 = time.perf_counter()
        at, lat, steps = 0.0, [], 0
        per_kind = {"streamlines": 0.0, "ftle": 0.0}
        for k in range(len(specs)):
            if rate:
                at += reqs[k]["gap"] / rate
                delay = t0 + at - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
            r0 = time.perf_counter()
            steps += plain_request(ctx, k)
            per_kind[specs[k]["kind"]] += time.perf_counter() - r0
            lat.append(1e3 * (time.perf_counter() - (t0 + at)))
        span = time.perf_counter() - t0
        breakdown.update({f"{kind}_fraction": v / span for kind, v in per_kind.items()})
        return span, np.array(lat), steps

    def collect(svc, ticket):
        info = svc.info(ticket)
        if info.kind == 0 and image_reply:
            w, hgt = svc.image_into(ticket, frame.data_ptr())
            collected["bytes"] += w * hgt * 4
        elif info.kind == 0:
            for b in range(info.batches):
                nv, ni = svc.batch_into(ticket, b, vbuf.data_ptr(), cbuf.data_ptr(), ibuf.data_ptr())
                collected["bytes"] += 32 * nv + 4 * ni
        else:
            svc.ftle_into(ticket, fbuf.data_ptr())
            collected["bytes"] += 4 * int(np.prod(list(info.ftle_shape)))
        steps = info.steps
        svc.release(ticket)
        return steps

    def run_service(svc, rate):
        n = len(messages)
        tickets, arrival = [None] * n, [0.0] * n
        t0 = time.perf_counter()

        def submitter():
            at = 0.0
            for k, m in enumerate(messages):
                if rate:
                    at += reqs[k]["gap"] / rate
                    delay = t0 + at - time.perf_counter()
                    if delay > 0:
                        time.sleep(delay)
                arrival[k] = t0 + at
                tickets[k] = svc.submit(m)

        thread = th.Thread(target=submitter)
        thread.start()
        lat, steps, pending, nxt = [], 0, [], 0
        running, collecting = [], 0.0
        while len(lat) < n:
            while nxt < n and tickets[nxt] is not None:
                pending.append(nxt)
                nxt += 1
            progress = False
            for k in list(pending):
                if svc.wait(tickets[k], 0) == 2:
                    info = svc.info(tickets[k])
                    start = arrival[k] + info.queue_ms / 1e3
                    running.append((start, start + info.run_ms / 1e3))
                    c0 = time.perf_counter()
                    steps += collect(svc, tickets[k])
                    collecting += time.perf_counter() - c0
                    lat.append(1e3 * (time.perf_counter() - arrival[k]))
                    pending.remove(k)
                    progress = True
            if not progress:
                time.sleep(0.0002)
        thread.join()
        span = time.perf_counter() - t0
        # wall time during which at least one batch ran, and the collector's share
        busy, end = 0.0, -1e30
        for a, b in sorted(running):
            if b > end:
                busy += b - max(a, end)
                end = b
        breakdown["batch_running_fraction"] = busy / span
        breakdown["collecting_fraction"] = collecting / span
        return span, np.array(lat), steps

    breakdown = {}

    def summarise(run, target):
        collected["bytes"] = 0
        breakdown.clear()
        span, lat, steps = run(target, None)
        saturation = len(messages) / span
        out = {"saturation_requests_per_s": saturation, "saturation_particle_steps_per_s": steps / span,
               "saturation_p50_ms": float(np.percentile(lat, 50)), "saturation_p99_ms": float(np.percentile(lat, 99)),
               "result_bytes_to_host": collected["bytes"], "saturation_breakdown": dict(breakdown)}
        for load in loads:
            span, lat, _ = run(target, load * saturation)
            out[f"load{int(load * 100)}"] = {"offered_requests_per_s": load * saturation,
                                             "achieved_requests_per_s": len(messages) / span,
                                             "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))}
        return out

    arms = args.serve_arms.split(",")
    loads = [float(x) for x in args.serve_loads.split(",") if x]
    results = {}
    if "plain" in arms:
        ctx = native.Context(0)
        for k in range(8):                           # warm-up (autotuning, allocations)
            plain_request(ctx, k)
        results["plain"] = summarise(run_plain, ctx)
        ctx.close()

    if "batched" in arms:
        def service(lanes):
            svc = native.Service(0, budget_bytes=160 << 30, lanes=lanes, max_batch=64)
            for d, (xyz, offset, size, spacing) in zip(ds, device_fields):
                svc.add_dataset_device(d["name"], xyz.data_ptr(), (d["edge"],) * 3, offset, size, spacing)
            torch.cuda.synchronize()
            for m in messages[:8]:                   # warm-up
                t = svc.submit(m)
                svc.wait(t)
                collect(svc, t)
            return svc

        svc = service(args.serve_lanes)
        results["batched"] = summarise(run_service, svc)
        results["batched"]["lanes"] = args.serve_lanes
        if "plain" in results and "load50" in results["plain"]:
            # latency at the plain path's own 50 % load: both arms at one offered rate
            rate = results["plain"]["load50"]["offered_requests_per_s"]
            span, lat, _ = run_service(svc, rate)
            results["batched"]["at_plain_load50"] = {"offered_requests_per_s": rate,
                                                     "achieved_requests_per_s": len(messages) / span,
                                                     "p50_ms": float(np.percentile(lat, 50)),
                                                     "p99_ms": float(np.percentile(lat, 99))}
        svc.close()
        # the other lane count, at saturation only
        other = 2 if args.serve_lanes == 1 else 1
        svc = service(other)
        span, _, _ = run_service(svc, None)
        results["batched"][f"saturation_requests_per_s_lanes{other}"] = len(messages) / span
        svc.close()

    if "cpu" in arms:
        results["cpu_reference"] = run_cpu_reference(specs, host_fields, args.serve_cpu_seconds)
    reply = (f"streamline requests reply with a {width}x{height} image of their curves ray traced on the GPU (the "
             "pars_service reply)" if image_reply else "streamline requests return every curve buffer")
    line = {"workload": f"served_{len(messages)}: {len(messages)} requests (seed 4), 70% streamlines / 30% FTLE on "
                        f"{len(ds)} ABC / double-gyre fields (edge 64-512), seeds 1k-2M (streamlines <= 16384), "
                        f"200-2000 RK4 steps, Poisson arrivals; {reply}, FTLE requests their FTLE field; results "
                        "collected into pinned host buffers",
            "reply": args.serve_reply, "datasets": ds}
    line.update(results)
    if "plain" in results and "batched" in results:
        line["throughput_ratio_at_saturation"] = (results["batched"]["saturation_requests_per_s"] /
                                                  results["plain"]["saturation_requests_per_s"])
    if "batched" in results and "cpu_reference" in results:
        line["particle_steps_ratio_batched_to_cpu"] = (results["batched"]["saturation_particle_steps_per_s"] /
                                                       results["cpu_reference"]["particle_steps_per_s"])
    print(json.dumps(line))


def _free_port():
    import socket
    with socket.socket() as sock:
        sock.bind(("127.0.0.1", 0))
        return sock.getsockname()[1]


def launch_replicas(args):
    """--gpus N > 1 started as a plain process: runs N ranks, one process per
    GPU, through torch.distributed.run on this node (rendezvous on
    127.0.0.1), with the same arguments; rank 0 prints the line."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def launcher_check(args):
    """--dry-run: every rank joins a gloo group on the CPU and reports its rank
    through combine_ranks (rank r: r + 1 seconds, 1000 (r + 1) units), so the
    launcher and the reduction are checked without a GPU or a workload."""
    import torch.distributed as dist
    rank, world, _ = dist_env()
    dist.init_process_group("gloo")
    elapsed, units = combine_ranks(dist, float(rank + 1), 1000 * (rank + 1), "cpu")
    if rank == 0:
        print(json.dumps({"launcher_check": True, "n_gpus": world, "requested_gpus": args.gpus,
                          "max_rank_seconds": elapsed, "sum_units": units}))
    dist.destroy_process_group()


def gather_peaks(ctx):
    """Measured gather ceilings of this GPU (GB/s of 16-byte loads delivered
    to registers; best of two per case): L1-resident (32 KiB) and
    L2-resident (64 MiB) buffers, coalesced 512-byte warp requests, one random
    sector per lane, and eight-corner cell gathers."""
    out = {}
    for size, level in ((32 << 10, "l1"), (64 << 20, "l2")):
        for pattern in ("coalesced", "random", "cells"):
            out[f"{level}_{pattern}"] = max(ctx.gather_peak(size, pattern) for _ in range(2)) / 1e9
    return out


def extra_workloads(args):
    """The other workloads, each in its own process (one JSON line each), for
    the default single-GPU run: streamlines, the partitioned domain, batched
    pathlines, the ray tracer and a reduced served stream."""
    runs = {"streamlines": ["--workload", "streamlines", "--steps", "20", "--warmup", "3"],
            "domain": ["--workload", "domain", "--steps", "3", "--warmup", "1"],
            "pathlines": ["--workload", "pathlines", "--steps", "2", "--warmup", "1"],
            "render": ["--workload", "render", "--steps", "5", "--warmup", "3"],
            "serve": ["--workload", "serve", "--requests", "100", "--serve-loads", "0.5", "--serve-cpu-seconds", "5"]}
    out = {}
    for name, extra in runs.items():
        t0 = time.perf_counter()
        r = subprocess.run([sys.executable, os.path.abspath(__file__)] + extra, capture_output=True, text=True)
        line = None
        for text in reversed(r.stdout.strip().splitlines()):
            if text.startswith("{"):
                line = json.loads(text)
                break
        out[name] = line if (r.returncode == 0 and line) else {"error": (r.stderr or r.stdout)[-400:],
                                                              "returncode": r.returncode}
        out[name]["wall_s"] = time.perf_counter() - t0
    return out


def served_summary(serve):
    """The served stream's headline figures (batched service against the plain
    single-request path), from the served workload's own line."""
    if not serve or "batched" not in serve or "plain" not in serve:
        return None
    b, p = serve["batched"], serve["plain"]
    return {"workload": serve.get("workload", "").split(":")[0], "reply": serve.get("reply"), "lanes": b.get("lanes"),
            "req_per_s": b["saturation_requests_per_s"], "plain_req_per_s": p["saturation_requests_per_s"],
            "ratio": b["saturation_requests_per_s"] / p["saturation_requests_per_s"],
            "p50_ms": b.get("load50", {}).get("p50_ms"), "p99_ms": b.get("load50", {}).get("p99_ms"),
            "plain_p50_ms": p.get("load50", {}).get("p50_ms"), "plain_p99_ms": p.get("load50", {}).get("p99_ms"),
            "load": "50 % of each arm's own saturation throughput",
            "at_plain_load50": b.get("at_plain_load50")}


def main():
    args = parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_replicas(args))
    if args.dry_run:
        launcher_check(args)
        return
    if args.workload != "ftle":
        {"streamlines": run_streamlines, "domain": run_domain, "pathlines": run_pathlines, "serve": run_serve,
         "render": run_render}[args.workload](args)
        return
    rank, world, local = dist_env()
    from pars_gb300 import workloads

    n = args.size
    seeds = n ** 3
    max_steps = args.iterations - 1
    config = {"workload": f"ftle_{n}: ABC + N(0,0.01) noise (seed 0) on {n}^3 FP32 vertices of [0,2pi]^3, one seed per vertex "
                          f"({seeds} particles), classical RK4 (4 samples/step) h=0.01, <= {max_steps} steps (T=5), "
                          "flow map + fused central-difference / Cauchy-Green / FP32 Jacobi eigenvalue / log FTLE",
              "grid": n, "seeds": seeds, "max_steps": max_steps, "step_size": 0.01, "stage_mode": "resampled",
              "field_samples_per_step": 4, "reference_field_samples_per_step": 1,
              "ranks": world, "l2": f"inputs larger than L2 ({16 * n ** 3 / 1e6:.0f} MB float4 field) and a 256 MB L2 flush "
                                    "before every step",
              "tested_at_this_size": "tests/test_gpu_fullsize.py: flow map of 100k strided seeds within 1e-3 cells of FP64, "
                                     "FTLE of an interior 48^3 window within 1e-4 of FP64"}

    if args.impl == "reference":
        if rank != 0:
            return
        field = workloads.abc_field(n, noise_sigma=0.01, seed=0)
        value, threads, dt = cpu_reference_run(field, args.iterations, args.cpu_stride, args.steps, args.warmup)
        sample = cpu_sample_text(seeds, args.cpu_stride, n)
        print(json.dumps({"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                          "data": "synthetic", "config": config,
                          "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                                           **host_cpu()},
                          "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return

    import torch
    from pars_gb300 import native

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    field = workloads.abc_field(n, noise_sigma=0.01, seed=0)
    ctx = native.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    handle = ctx.upload_field(field)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    T = 0.01 * max_steps

    def device_step(stage_mode=native.STAGES_RESAMPLED):
        fm, steps = ctx.flow_map_generate(handle, args.iterations, 1.0, native.RUNGE_KUTTA_4, stage_mode, 0.01)
        ctx.ftle_generate(fm, T, native.FTLE_REGULAR, download=False)
        ctx.release_field(fm)
        return steps

    # the warm-up also runs the L2 flush: its first launch in a process loads
    # the fill kernel's module, which on a cold machine pages in from disk
    for _ in range(max(args.warmup, 3)):
        flush.zero_()
        device_step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    ctx.profile_reset()
    ctx.profile_enable(True)
    launches0 = ctx.launch_count()
    sampler.start()
    sampler.wait_ready()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    total_steps = 0
    start.record(stream)
    for _ in range(args.steps):
        flush.zero_()
        total_steps += device_step()
    stop.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    launches = ctx.launch_count() - launches0
    ctx.profile_enable(False)
    elapsed_ms = start.elapsed_time(stop)
    advect_ms, advect_n = ctx.profile_get("batch_advect")
    ftle_ms, ftle_n = ctx.profile_get("ftle_fused")

    elapsed_ms, total_steps_all = combine_ranks(dist, elapsed_ms, total_steps, "cuda")
    value = total_steps_all / (elapsed_ms * 1e-3)
    ftle_voxels_per_s = world * seeds * args.steps / (elapsed_ms * 1e-3)
    steps_per_launch = total_steps / args.steps
    hbm_peak, hbm_kind = measured_peaks()
    advect_avg_s = advect_ms / max(advect_n, 1) * 1e-3
    achieved = steps_per_launch * BYTES_PER_RK4_STEP / advect_avg_s / 1e9
    ftle_avg_s = ftle_ms / max(ftle_n, 1) * 1e-3
    traffic = committed_traffic(steps_per_launch)
    peaks = gather_peaks(ctx)

    # The reference's scheme (frozen velocity, one sample per step) on the GPU.
    device_step(native.STAGES_FROZEN)
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    frozen_steps = 0
    f0.record(stream)
    for _ in range(2):
        flush.zero_()
        frozen_steps += device_step(native.STAGES_FROZEN)
    f1.record(stream)
    torch.cuda.synchronize()
    frozen_value = frozen_steps / (f0.elapsed_time(f1) * 1e-3)

    # End to end through the C ABI from pinned host buffers.
    pinned = torch.empty((n, n, n, 3), dtype=torch.float32, pin_memory=True).numpy()
    pinned[...] = field.xyz
    host_field = workloads.Field(pinned, field.offset, field.spacing, field.size)
    ftle_out = torch.empty((n, n, n), dtype=torch.float32, pin_memory=True).numpy()

    def e2e_step():
        h = ctx.upload_field(host_field)
        fm, steps = ctx.flow_map_generate(h, args.iterations, 1.0, native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED, 0.01)
        ctx.ftle_generate(fm, T, native.FTLE_REGULAR, out=ftle_out)
        ctx.release_field(fm)
        ctx.release_field(h)
        return steps

    e2e_step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    e2e_steps, t0 = 0, time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        e2e_steps += e2e_step()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_s, e2e_steps_all = combine_ranks(dist, e2e_s, e2e_steps, "cuda")
    e2e_value = e2e_steps_all / e2e_s

    cpu = None
    if rank == 0 and world == 1:
        cpu_value, threads, _ = cpu_reference_run(field, args.iterations, args.cpu_stride, 1, 0)
        cpu = {"value": cpu_value, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": cpu_sample_text(seeds, args.cpu_stride, n),
               "single_thread": cpu_single_thread(field, args.iterations, args.cpu_stride), **host_cpu()}

    if rank == 0:
        l1 = peaks["l1_coalesced"]
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config,
                "ftle_voxels_per_s": ftle_voxels_per_s,
                "frozen_velocity_steps_per_s": frozen_value,
                "roofline": {"bound": "l1_gather", "achieved": achieved, "peak": l1, "unit": "GB/s", "frac": achieved / l1,
                             "traffic": traffic, "kernel": "batch_advect",
                             "bytes_per_unit": BYTES_PER_RK4_STEP, "units_per_launch": steps_per_launch,
                             "avg_launch_ms": advect_avg_s * 1e3,
                             "peak_source": "measured in this run on this GPU (pars_gpu_gather_peak): 16-byte "
                                            "ld.global.nc loads, warp requests of 512 contiguous bytes in a 32 KiB "
                                            "L1-resident buffer; the kernel's corner gathers are served by L1 "
                                            "(ncu: L1 data-pipe wavefronts are its top unit)",
                             "gather_peaks_gbs": peaks,
                             "frac_of_l2_coalesced": achieved / peaks["l2_coalesced"],
                             "hbm": {"peak_gbs": hbm_peak, "peak_source": hbm_kind,
                                     "traffic_gbs": (traffic / advect_avg_s / 1e9) if traffic else None},
                             "ftle_kernel": {"avg_launch_ms": ftle_avg_s * 1e3,
                                             "achieved_gbs": seeds * BYTES_PER_FTLE_VOXEL / ftle_avg_s / 1e9}},
                "cpu_baseline": cpu,
                "same_scheme_ratio": (frozen_value / cpu["value"]) if cpu else None,
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(field.xyz.nbytes),
                        "d2h_bytes_per_step": int(ftle_out.nbytes)},
                "clocks": clocks, "gpu_launches": launches}
    ctx.close()
    del flush
    torch.cuda.empty_cache()
    if dist:
        dist.destroy_process_group()
    if rank == 0:
        if world == 1 and not args.no_extra:
            line["workloads"] = extra_workloads(args)
            line["served"] = served_summary(line["workloads"].get("serve"))
        print(json.dumps(line))


if __name__ == "__main__":
    main()
