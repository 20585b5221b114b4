#!/usr/bin/env python3
"""Benchmark: batched atmosphere LUT precompute on GB300.

Headline workload (one "step"): a batch of 256 seeded synthetic atmospheres
(fuzzyblue_gb300.workloads.uniform_batch, seed 0) at the crate's default table
sizes (transmittance 256x64, irradiance 64x16, scattering r32 mu128 mu_s32 nu8),
4 scattering orders, MIXED precision (max relative error <= 1e-3 against the
FP64 oracle), built with one persistent launch per pass group.

  value   atmospheres/s with the work resident on the device (CUDA events on the
          build stream; per-launch events give the kernel times)
  e2e     atmospheres/s through the public API: parameters from the host, every
          table of every atmosphere copied back into pinned host memory
  plain   the plain path, one default atmosphere per call, FP32 (for the
          batched/plain ratio)
  cpu_baseline  the reference's own shader code compiled as C++ (oracle/_ref), or
          the oracle port where that is unavailable, on a bounded sample, all
          host threads
  uneven  one step of the uneven batch (96 atmospheres, three table classes,
          orders 2-8), batched against the plain path per class
  serve   a 12 s Poisson sample at 50 req/s through the request loop: p50/p99
          latency overall and per class beside the plain FIFO replay

--impl reference times the reference's CPU implementation on the same metric.
Multi-GPU: replicas only (each rank builds its own batch; no collective on the
data path); value is the whole-job rate.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

BATCH = 256
ORDERS = 4
WORKLOAD = ("uniform batch: 256 seeded atmospheres (seed 0), default table sizes "
            "(TR 256x64, IR 64x16, SC r32 mu128 mu_s32 nu8), 4 orders, mixed precision")
E2E_PARTS = 8                 # batches per step in the end-to-end measurement
SERVE_SAMPLE_RATE = 50.0      # req/s of the serving sample in the headline line
SERVE_SAMPLE_SECONDS = 12.0   # seconds of arrivals of that sample
METRIC = "atmospheres/s, uniform batch of 256 at default table sizes, 4 orders, mixed precision (<=1e-3 rel err vs FP64)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=BATCH)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline only: leave out the short uneven-batch and serving measurements")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "plain"],
                    help="arithmetic of the batch (the headline is mixed)")
    ap.add_argument("--workload", default="uniform", choices=["uniform", "uneven", "serve", "render"],
                    help="uniform: the headline batch; uneven: 96 atmospheres over three table classes, "
                         "orders 2-8; serve: open-loop Poisson requests through the request loop; "
                         "render: the headless sky pass over the tables, 1920x1080 frames")
    ap.add_argument("--rates", default="50,200,1000", help="serve: offered request rates (req/s)")
    ap.add_argument("--duration", type=float, default=60.0, help="serve: seconds of arrivals per rate")
    ap.add_argument("--max-queue", type=int, default=512,
                    help="serve: queued requests beyond which new ones are refused (load shedding)")
    return ap.parse_args()


# ------------------------------------------------------------------ clocks --
class Clocks:
    """Samples nvidia-smi every 200 ms while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return None

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ------------------------------------------------------------ distributed --
def dist():
    from fuzzyblue_gb300.ranks import layout
    return layout()


def barrier(world):
    from fuzzyblue_gb300.ranks import barrier as rank_barrier
    rank_barrier(world)


def max_over_ranks(world, v):
    from fuzzyblue_gb300.ranks import max_over_ranks as rank_max
    return rank_max(world, v)


# ------------------------------------------------------------- roofline ---
# The roofline of the dominant launch (scattering density of order n >= 3 plus
# the indirect irradiance of order n - 1) is reported on the FP32 pipe: the
# FLOPs the kernel executes per direction evaluation (measured with ncu on the
# same launch, a committed profile summary) times the directions of the
# launch, over its CUDA-event time. Beside it: the reference's quadrature
# arithmetic per output texel, op-counted on the oracle's restatement over the
# first 16 atmospheres of this workload (`python oracle/count_flops.py`; adds,
# muls, divs, sqrts and transcendentals one FLOP each, sampler filtering and
# literal-only expressions not counted; 162.6 FLOPs per direction at n >= 3).
FLOP_PER_TEXEL = {
    "transmittance": 28311.7,
    "direct_irradiance": 34.0,
    "single_scattering": 8033.8,
    "density_order2": 133663.8,
    "density_order3": 83260.2,
    "indirect_order1": 163843.0,
    "indirect_order2": 74755.0,
    "multiple_scattering": 8332.2,
}
FLOP_PER_ATMOSPHERE = 350185724984.0  # default sizes, 4 orders (same count)
# Counts of the dominant launch measured with ncu on the kernel sources whose
# SHA-256 (first 16 hex digits, over KERNEL_SOURCES) is `sources`: the
# executed FP32 FLOPs and thread instructions per direction evaluation (a
# --set full capture of 16 atmospheres) and the DRAM bytes per launch (the same
# capture, scaled to the launch's atmospheres). The commands are in the profile
# summaries named by `profile`. When the sources on disk differ, the roofline
# is reported with "stale": true.
KERNEL_SOURCES = ("fuzzyblue_gb300/csrc/fb_passes.cuh", "fuzzyblue_gb300/csrc/fb_device.cuh")
DENSITY_NCU = {
    "sources": "3c8e1ac1b66b0be0",
    "profile": "profiles/passes_uniform16_mixed_ncu.md",
    "atmospheres": 16,
    "fp32_flop_per_direction_order3": 24.49,
    "thread_instr_per_direction_order3": 20.54,
    "dram_bytes_per_atmosphere_order3": 13.16e6,
}


def kernel_sources_sha():
    """SHA-256 prefix of the kernel sources' code: comments, trailing blanks and
    empty lines removed, so that an edit of a comment keeps the counts current."""
    import hashlib
    import re
    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        with open(os.path.join(ROOT, f), encoding="utf-8") as fh:
            text = re.sub(r"/\*.*?\*/", "", fh.read(), flags=re.S)
        lines = (re.sub(r"//.*", "", line).rstrip() for line in text.splitlines())
        h.update("\n".join(line for line in lines if line).encode())
    return h.hexdigest()[:16]


def fp32_peak_tflops(sms, mhz):
    return sms * 128 * 2 * mhz * 1e6 / 1e12


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


# ------------------------------------------------------------------ ours ---
def run_ours(a):
    world, rank, local = dist()
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as td
        td.init_process_group("nccl")
    from fuzzyblue_gb300 import workloads
    from fuzzyblue_gb300.api import Atmosphere, Builder, build_batch, device_bytes
    from fuzzyblue_gb300.params import PRECISION_MIXED, PRECISION_PLAIN, Parameters

    builder = Builder(local)
    stream = torch.cuda.Stream()
    prec = PRECISION_MIXED if a.precision == "mixed" else PRECISION_PLAIN
    params = workloads.uniform_batch(a.batch, seed=0, order=ORDERS, precision=prec)

    def step(profile=False):
        builder.set_profiling(profile)
        pend = build_batch(builder, params, stream=stream)
        return pend

    # tile shapes of the workload's table class from the autotuner (untimed)
    tuned = None
    if not a.no_autotune:
        builder.autotune([params[0]], batch=8)
        tuned = builder.tuned_shape(params[0])

    # warm-up (graph path)
    for _ in range(a.warmup):
        p = step()
        p.wait()
        p.release()
    torch.cuda.synchronize()

    # timed region: device-resident work, per-launch timing events
    clocks = Clocks(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    step_ms, prof = [], []
    ev0.record(stream)
    torch.cuda.nvtx.range_push("timed")  # lets a profiler select the timed launches
    for _ in range(a.steps):
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        p = step(profile=True)
        s1.record(stream)
        p.wait()
        prof.append(p.profile())
        p.release()
        step_ms.append(s0.elapsed_time(s1))
    torch.cuda.nvtx.range_pop()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    total_ms = max_over_ranks(world, ev0.elapsed_time(ev1))
    ms_per_step = total_ms / a.steps
    from fuzzyblue_gb300.ranks import whole_job_rate
    value = whole_job_rate(world, a.batch, ms_per_step / 1e3)

    # the same steps replayed from the CUDA graph (no per-launch events)
    builder.set_profiling(False)
    torch.cuda.synchronize()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    for _ in range(a.steps):
        p = step()
        p.wait()
        p.release()
    g1.record(stream)
    torch.cuda.synchronize()
    graph_ms = max_over_ranks(world, g0.elapsed_time(g1)) / a.steps

    # end to end through the public API with host buffers: every step's
    # parameters go in with its builds and all three tables of every
    # atmosphere come back into page-locked host memory
    # (fb_atmosphere_copy_to_host_async). A step's atmospheres are built as
    # E2E_PARTS batches (one default atmosphere already fills the GPU, so a
    # batch of 32 runs at the rate of the whole 256), alternating between two
    # streams, each with its own host buffer: a batch's build waits on the
    # device for the previous batch (fb_pending_acquire), so builds run back to
    # back while each batch's copies overlap the next batch's kernels; the
    # timed region ends when the last copy is done.
    sizes = params[0].texel_counts()
    per_atm = 16 * sum(sizes)
    parts = E2E_PARTS if a.batch % E2E_PARTS == 0 else 1
    sub = a.batch // parts
    hosts = [torch.empty((a.batch, per_atm // 4), dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
    streams = [stream, torch.cuda.Stream()]
    tw, th = params[0].transmittance_extent()
    iw, ih = params[0].irradiance_extent()
    n_tr, n_ir = 4 * tw * th, 4 * iw * ih
    from fuzzyblue_gb300 import _native as N
    h2d = a.batch * 384
    inflight = [None, None]
    # untimed: one build on each stream, so that the memory pool holds two
    # batches' tables and temporaries before the timed steps
    warm = [build_batch(builder, params[:sub], stream=streams[k]) for k in (0, 1)]
    for w in warm:
        w.wait()
        w.release()
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    prev = None
    for u in range(a.steps * parts):
        k = u & 1
        b = u % parts
        if inflight[k] is not None:  # that stream's previous batch: copies done, then release
            streams[k].synchronize()
            inflight[k].release()
        if prev is not None:
            prev.acquire(streams[k])
        p = build_batch(builder, params[b * sub:(b + 1) * sub], stream=streams[k])
        prev = p
        for i in range(sub):
            base = hosts[k][b * sub + i].ctypes.data
            N.check(N.lib().fb_atmosphere_copy_to_host_async(p.atmosphere(i)._h, streams[k].cuda_stream, base,
                                                             base + 4 * n_tr, base + 4 * (n_tr + n_ir)),
                    "fb_atmosphere_copy_to_host_async")
        inflight[k] = p
    for k in (0, 1):
        streams[k].synchronize()
        if inflight[k] is not None:
            inflight[k].release()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(world, time.perf_counter() - t0) / a.steps
    e2e = whole_job_rate(world, a.batch, e2e_s)

    # plain path: one default-size atmosphere per call, FP32
    plain_p = Parameters()
    for _ in range(2):
        q = Atmosphere.build(builder, plain_p, stream=stream)
        q.wait()
        q.release()
    pe0, pe1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n_plain = 20
    pe0.record(stream)
    for _ in range(n_plain):
        q = Atmosphere.build(builder, plain_p, stream=stream)
        q.release()
    pe1.record(stream)
    torch.cuda.synchronize()
    plain_ms = pe0.elapsed_time(pe1) / n_plain

    # kernel times from the timed region
    kernels = {}
    for launches in prof:
        for r in launches:
            key = r["kernel"] + ("" if r["order"] == 0 else "_order%d" % min(r["order"], 3))
            kernels.setdefault(key, []).append(r)
    dens = [r for launches in prof for r in launches if r["kernel"] == "density+indirect" and r["order"] >= 3]
    dens_ms = sum(r["ms"] for r in dens) / max(len(dens), 1)
    sms = builder.sm_count
    # executed FP32 FLOPs per direction evaluation of this launch (ncu) and
    # the reference's quadrature FLOPs per texel (oracle op count)
    directions = a.batch * sizes[2] * 2 * params[0].density_samples ** 2
    exec_per_dir = DENSITY_NCU["fp32_flop_per_direction_order3"]
    stale = kernel_sources_sha() != DENSITY_NCU["sources"]
    ref_flops = a.batch * (sizes[2] * FLOP_PER_TEXEL["density_order3"] + sizes[1] * FLOP_PER_TEXEL["indirect_order2"])
    mhz = (clk or {}).get("sm_mhz") or 2070.0
    peak = fp32_peak_tflops(sms, mhz)
    exec_flops = directions * exec_per_dir if exec_per_dir else None
    achieved = exec_flops / (dens_ms / 1e3) / 1e12 if exec_flops else None
    ref_achieved = ref_flops / (dens_ms / 1e3) / 1e12
    traffic = DENSITY_NCU["dram_bytes_per_atmosphere_order3"] * a.batch
    peaks = measured_peaks()
    # the launch's binding limit is instruction issue: warp instructions per
    # launch (ncu's thread instructions per direction / 32) against one per
    # cycle per scheduler, 4 schedulers per SM
    instr_per_dir = DENSITY_NCU["thread_instr_per_direction_order3"]
    issue = None
    if instr_per_dir:
        issue_achieved = directions * instr_per_dir / 32.0 / (dens_ms / 1e3) / 1e9
        issue_peak = sms * 4 * mhz * 1e6 / 1e9
        issue = {"achieved": issue_achieved, "peak": issue_peak, "unit": "G warp instructions/s",
                 "frac": issue_achieved / issue_peak, "thread_instr_per_unit": instr_per_dir,
                 "source": "thread instructions per direction, ncu, " + DENSITY_NCU["profile"]}

    out = {
        "metric": METRIC if a.precision == "mixed" else METRIC.replace(
            "mixed precision (<=1e-3 rel err vs FP64)", "plain FP32"),
        "value": value,
        "unit": "atmospheres/s",
        "n_gpus": world,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 with f64 ray geometry and order accumulation" if a.precision == "mixed" else "f32",
        "data": "synthetic: seeded atmospheres (fuzzyblue_gb300.workloads, seed 0)",
        "config": {"workload": WORKLOAD if a.precision == "mixed" else WORKLOAD.replace("mixed", "plain FP32"),
                   "batch_per_gpu": a.batch, "orders": ORDERS, "precision": a.precision,
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "inputs larger than L2: ~%d GB of tables and temporaries per step" % round(
                       sum(sum(device_bytes(p)) for p in params) / 1e9)},
        "clocks": clk,
        "e2e": {"value": e2e, "unit": "atmospheres/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": a.batch * per_atm,
                "overlap": "each step built as %d batches of %d on two streams: a batch's copies overlap the next "
                           "batch's kernels" % (parts, sub)},
        "gpu_launches": sum(len(x) for x in prof),
        "roofline": {"bound": "fp32", "kernel": "k_density (scattering density + indirect irradiance), order >= 3",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if achieved else None,
                     "peak_source": "152 SMs x 128 FP32 lanes x 2 FLOP x median SM clock under load (%d MHz); "
                                    "no tensor-core work, HBM far from its limit" % mhz,
                     "launch_ms": dens_ms, "flop_per_unit": exec_per_dir, "units_per_launch": directions,
                     "unit_name": "direction evaluations (texels x 512 sphere directions)",
                     "flop_source": "executed FP32 FLOPs (FADD + FMUL + 2 FFMA) per direction, ncu, "
                                    + DENSITY_NCU["profile"],
                     "traffic": traffic,
                     "traffic_source": "ncu DRAM bytes of the same launch on %d atmospheres (%s), scaled to %d"
                                       % (DENSITY_NCU["atmospheres"], DENSITY_NCU["profile"], a.batch),
                     "stale": stale, "kernel_sources_sha256_16": kernel_sources_sha(),
                     "counts_measured_on_sha256_16": DENSITY_NCU["sources"],
                     "hbm": {"achieved_gbs": traffic / (dens_ms / 1e3) / 1e9 if traffic else None,
                             "peak_gbs": peaks.get("hbm_gbs"), "peak_source": "MEASURED_PEAKS.json"},
                     "issue": issue,
                     "reference_algorithm": {
                         "achieved": ref_achieved, "frac": ref_achieved / peak,
                         "flop_per_texel": FLOP_PER_TEXEL["density_order3"],
                         "note": "the reference's quadrature arithmetic (oracle op count, oracle/count_flops.py) "
                                 "delivered per second: the kernel executes fewer FLOPs per direction than the "
                                 "reference's shader code (per-tile reduced tables replace the 4D lookups)"}},
        "kernels_ms": {k: sum(r["ms"] for r in v) / len(v) for k, v in sorted(kernels.items())},
        "latency_ms": {"p50": statistics.median(step_ms), "p99": float(np.quantile(step_ms, 0.99))},
        "graph": {"ms_per_step": graph_ms, "value": world * a.batch / (graph_ms / 1e3)},
        "plain": {"ms_per_atmosphere": plain_ms, "atmospheres_per_s": 1e3 / plain_ms, "precision": "plain"},
        "batched_over_plain": value / (world * 1e3 / plain_ms),
        "algorithmic_tflops": value * FLOP_PER_ATMOSPHERE / 1e12,
        "tile_shape": tuned,
    }
    if rank == 0 and world == 1 and not a.no_extras:
        # the other configurations in short form: one step of the uneven batch
        # and a Poisson sample at 50 req/s through the request loop
        u = measure_uneven(a, builder, stream, steps=1, warmup=1)
        out["uneven"] = {k: u[k] for k in ("metric", "value", "unit", "ms_per_step", "e2e", "plain",
                                           "batched_over_plain", "per_class", "clocks")}
        out["uneven"]["steps"], out["uneven"]["warmup"] = 1, 1
        sv = measure_serve(a, builder, [SERVE_SAMPLE_RATE], SERVE_SAMPLE_SECONDS)
        line = sv["rates"][0]
        out["serve"] = {"metric": sv["metric"], "offered_rate": line["offered_rate"],
                        "duration_s": SERVE_SAMPLE_SECONDS, "requests": line["requests"],
                        "served": line["served"], "plain_fifo": line["plain"],
                        "served_over_plain_throughput": line["served_over_plain_throughput"],
                        "config": sv["config"]}
    if rank == 0 and not a.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(params[0])
    if rank == 0:
        print(json.dumps(out))
    builder.close()
    if world > 1:
        import torch.distributed as td
        td.destroy_process_group()


def cpu_baseline(p, fraction=1.0):
    from oracle import cpu_baseline as C
    kind = "reference" if C.reference_available() else "port"
    r = C.estimate(p, "reference" if kind == "reference" else "port", fraction=fraction)
    return {"value": 1.0 / r["seconds_per_atmosphere"], "unit": "atmospheres/s", "cores": r["threads"],
            "kind": kind, "sample": r["sample"], "sample_seconds": r["sample_seconds"]}


# ------------------------------------------------------------- reference ---
def run_reference(a):
    world, rank, local = dist()
    if rank != 0:
        return
    from fuzzyblue_gb300 import workloads
    from oracle import cpu_baseline as C
    kind = "reference" if C.reference_available() else "port"
    p = workloads.uniform_batch(1, seed=0, order=ORDERS)[0]
    frac = 1.0 / 32
    for _ in range(a.warmup):
        C.estimate(p, kind, fraction=frac)
    t0 = time.perf_counter()
    est = []
    for _ in range(a.steps):
        est.append(C.estimate(p, kind, fraction=frac))
    wall = time.perf_counter() - t0
    sec = statistics.mean(r["seconds_per_atmosphere"] for r in est)
    value = 1.0 / sec
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "atmospheres/s", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": wall / a.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded atmospheres (fuzzyblue_gb300.workloads, seed 0)",
        "config": {"workload": WORKLOAD, "batch_per_gpu": a.batch, "orders": ORDERS, "precision": "reference FP32",
                   "implementation": "the reference's shaders compiled as C++ (oracle/_ref), host threads"
                   if kind == "reference" else "the oracle's C++ restatement (oracle/fb_oracle.cpp), host threads"},
        "cpu_baseline": {"value": value, "unit": "atmospheres/s", "cores": est[0]["threads"], "kind": kind,
                         "sample": est[0]["sample"]},
        "e2e": {"value": value, "unit": "atmospheres/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


# ---------------------------------------------------------------- render ---
RENDER_W, RENDER_H = 1920, 1080


def render_scene(p):
    """Camera 1 km above the ground looking just above the horizon, the sun
    45 degrees up; depth: a seeded half of the pixels at finite depth (aerial
    perspective, 20 m to 5 km), the rest sky."""
    import numpy as np
    from fuzzyblue_gb300.render import DrawParameters
    d = DrawParameters.look_at((0.0, p.bottom_radius + 1.0, 0.0), forward=(1.0, 0.15, 0.3), up=(0, 1, 0),
                               fov_y_deg=70.0, aspect=RENDER_W / RENDER_H, sun_direction=(0.4, 0.7071, 0.58))
    rng = np.random.default_rng(3)
    depth = np.where(rng.random((RENDER_H, RENDER_W)) < 0.5,
                     rng.uniform(2e-5, 5e-3, (RENDER_H, RENDER_W)), 0.0).astype(np.float32)
    return d, depth


def run_render(a):
    """The headless sky pass of the crate's renderer (render_sky.frag over
    render_sky.h; fb_atmosphere_render_sky) over the tables of one default
    atmosphere (uniform batch seed 0, mixed precision): one 1920x1080 frame per
    step, radiance and transmittance written as float4. value: device-resident
    frames; e2e: the depth buffer copied in from pinned host memory and the
    radiance copied out every frame. CPU baseline: the reference's own shading
    code compiled as C++ (oracle/_ref), all host cores, on a 240x135 frame of
    the same view, scaled by the pixel count."""
    world, rank, local = dist()
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    from fuzzyblue_gb300 import workloads
    from fuzzyblue_gb300.api import Atmosphere, Builder
    from fuzzyblue_gb300.params import PRECISION_MIXED
    from fuzzyblue_gb300.render import render_sky
    builder = Builder(local)
    p = workloads.uniform_batch(1, seed=0, order=ORDERS, precision=PRECISION_MIXED)[0]
    pend = Atmosphere.build(builder, p)
    pend.wait()
    atm = pend.take(0)
    pend.release()
    draw, depth_h = render_scene(p)
    stream = torch.cuda.Stream()
    depth = torch.as_tensor(depth_h).to("cuda")
    for _ in range(max(a.warmup, 3)):
        render_sky(atm, draw, RENDER_W, RENDER_H, depth=depth, stream=stream)
    stream.synchronize()
    # Frames are short (well under a millisecond) and the tables fit in L2, so
    # each timed frame has its own events and a 256 MB write between frames,
    # outside them, evicts the tables and buffers from L2 (cold tables every
    # frame); enough frames for the clock sampler to see the timed region.
    frames = max(a.steps, 1000)
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(frames)]
    clocks = Clocks(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    with torch.cuda.stream(stream):
        for f0, f1 in evs:
            flush.fill_(1.0)
            f0.record(stream)
            render_sky(atm, draw, RENDER_W, RENDER_H, depth=depth, stream=stream)
            f1.record(stream)
    stream.synchronize()
    clk = clocks.stop()
    ms = max_over_ranks(world, sum(f0.elapsed_time(f1) for f0, f1 in evs)) / frames
    pixels = RENDER_W * RENDER_H
    from fuzzyblue_gb300.ranks import whole_job_rate
    value = whole_job_rate(world, 1, ms / 1e3)
    # end to end: depth in from pinned host memory, radiance out to it, every frame
    depth_pin = torch.empty((RENDER_H, RENDER_W), dtype=torch.float32, pin_memory=True)
    depth_pin.copy_(torch.from_numpy(depth_h))
    out_pin = torch.empty((RENDER_H, RENDER_W, 4), dtype=torch.float32, pin_memory=True)
    dev_depth = torch.empty((RENDER_H, RENDER_W), dtype=torch.float32, device="cuda")
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(frames):
        with torch.cuda.stream(stream):
            dev_depth.copy_(depth_pin, non_blocking=True)
            color, _ = render_sky(atm, draw, RENDER_W, RENDER_H, depth=dev_depth, stream=stream)
            out_pin.copy_(color, non_blocking=True)
        stream.synchronize()
    e2e_s = max_over_ranks(world, time.perf_counter() - t0) / frames
    out = {
        "metric": "frames/s, headless sky pass (radiance + transmittance) over the tables of one atmosphere",
        "value": value, "unit": "frames/s", "n_gpus": world, "steps": frames, "warmup": max(a.warmup, 3),
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic: the default-size tables of atmosphere 0 of the uniform batch (seed 0), "
                                "seeded depth buffer",
        "config": {"workload": "sky pass, 1920x1080, half the pixels at finite depth (aerial perspective)",
                   "width": RENDER_W, "height": RENDER_H, "pixels_per_s": value * pixels,
                   "l2": "flushed between frames (256 MB written outside the timed events): cold tables "
                         "(16.3 MB) and buffers every frame"},
        "clocks": clk,
        "e2e": {"value": whole_job_rate(world, 1, e2e_s), "unit": "frames/s",
                "h2d_bytes_per_step": 4 * pixels, "d2h_bytes_per_step": 16 * pixels},
        "gpu_launches": frames,
        "roofline": {"bound": "hbm", "achieved": 36 * pixels / (ms / 1e3) / 1e9,
                     "peak": measured_peaks().get("hbm_gbs"), "unit": "GB/s",
                     "frac": (36 * pixels / (ms / 1e3) / 1e9) / measured_peaks()["hbm_gbs"]
                     if measured_peaks().get("hbm_gbs") else None,
                     "traffic": None,
                     "note": "algorithmic bytes: the depth read and the radiance and transmittance written, "
                             "36 B per pixel; the pass is bound by its table gathers (two 4D lookups of the "
                             "scattering table and up to four transmittance lookups per pixel, L2-resident), "
                             "not by HBM"},
    }
    if rank == 0 and not a.no_cpu_baseline:
        from oracle import cpu_baseline as C
        from oracle import py_oracle
        t = atm.to_host()
        w, h = RENDER_W // 8, RENDER_H // 8  # the same view at 1/64 of the pixels
        dep = np.ascontiguousarray(depth_h[::8, ::8])
        ref = C.reference_available()
        t0 = time.perf_counter()
        reps = 0
        while reps < 3 or time.perf_counter() - t0 < 2.0:
            py_oracle.render_sky(p, t["transmittance"], t["scattering"], draw, w, h, depth=dep, reference=ref)
            reps += 1
        sec = (time.perf_counter() - t0) / reps * (pixels / (w * h))
        out["cpu_baseline"] = {"value": 1.0 / sec, "unit": "frames/s", "cores": os.cpu_count(),
                               "kind": "reference" if ref else "port",
                               "sample": "%dx%d frames of the same view, %d repetitions, scaled by the pixel count"
                               % (w, h, reps)}
    if rank == 0:
        print(json.dumps(out))
    atm.close()
    builder.close()


# ----------------------------------------------------------- uneven batch ---
def run_uneven(a):
    """96 atmospheres (seed 1) split evenly over the default, half and double
    table classes, orders uniform in 2-8, one batch build per step (one
    persistent launch per pass group, replayed from a CUDA graph)."""
    world, rank, local = dist()
    import torch
    torch.cuda.set_device(local)
    from fuzzyblue_gb300.api import Builder
    builder = Builder(local)
    stream = torch.cuda.Stream()
    print(json.dumps(measure_uneven(a, builder, stream, a.steps, a.warmup)))
    builder.close()


def measure_uneven(a, builder, stream, steps, warmup):
    """The uneven batch's line: device-resident rate, end to end, and batched
    against the plain path overall and per table class."""
    import torch
    from fuzzyblue_gb300 import workloads
    from fuzzyblue_gb300.api import build_batch
    from fuzzyblue_gb300.params import PRECISION_MIXED, PRECISION_PLAIN
    from fuzzyblue_gb300 import _native as N
    prec = PRECISION_MIXED if a.precision == "mixed" else PRECISION_PLAIN
    params = workloads.uneven_batch(96, seed=1, precision=prec)
    classes, seen = [], set()
    for p in params:
        key = p.scattering_extent()
        if key not in seen:
            seen.add(key)
            classes.append(p)
    if not a.no_autotune:
        builder.autotune(classes, batch=4)
    tuned = [builder.tuned_shape(c) for c in classes]
    for _ in range(warmup):
        q = build_batch(builder, params, stream=stream)
        q.wait()
        q.release()
    torch.cuda.synchronize()
    clocks = Clocks(torch.cuda.current_device())
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        q = build_batch(builder, params, stream=stream)
        q.wait()
        q.release()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / steps
    # end to end: every table of every atmosphere into pinned host memory
    bufs = {}
    for p in params:
        n = 4 * sum(p.texel_counts())
        key = p.scattering_extent()
        if key not in bufs:
            bufs[key] = torch.empty(n, dtype=torch.float32, pin_memory=True).numpy()
    d2h = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        q = build_batch(builder, params, stream=stream)
        q.wait()
        for i, p in enumerate(params):
            ntr, nir, nsc = p.texel_counts()
            base = bufs[p.scattering_extent()].ctypes.data
            N.check(N.lib().fb_atmosphere_copy_to_host(q.atmosphere(i)._h, stream.cuda_stream, base,
                                                       base + 16 * ntr, base + 16 * (ntr + nir)), "copy_to_host")
            d2h += 16 * (ntr + nir + nsc)
        q.release()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / steps
    per_class = {}
    for p in params:
        c = "x".join(str(v) for v in p.scattering_extent())
        per_class[c] = per_class.get(c, 0) + 1
    # batched vs plain per table class: each class's atmospheres as one batch,
    # and the plain path, each atmosphere alone in FP32 (one call each)
    from fuzzyblue_gb300.api import Atmosphere
    compare = {}
    plain_total = 0.0
    for c in per_class:
        members = [p for p in params if "x".join(str(v) for v in p.scattering_extent()) == c]
        best = None
        for _ in range(2):
            t0 = time.perf_counter()
            q = build_batch(builder, members, stream=stream)
            q.wait()
            q.release()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        plain = [p.replace(precision=PRECISION_PLAIN) for p in members]
        w = Atmosphere.build(builder, plain[0], stream=stream)
        w.wait()
        w.release()
        t0 = time.perf_counter()
        for p in plain:
            q = Atmosphere.build(builder, p, stream=stream)
            q.wait()
            q.release()
        pt = time.perf_counter() - t0
        plain_total += pt
        compare[c] = {"atmospheres": len(members), "batched_atmospheres_per_s": len(members) / best,
                      "plain_atmospheres_per_s": len(members) / pt, "batched_over_plain": pt / best}
    out = {
        "metric": "atmospheres/s, uneven batch of 96 over three table classes, orders 2-8, %s precision"
                  % a.precision,
        "value": 96 / (ms / 1e3), "unit": "atmospheres/s", "n_gpus": 1, "steps": steps, "warmup": warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 with f64 ray geometry and order accumulation" if a.precision == "mixed" else "f32",
        "data": "synthetic: seeded atmospheres (fuzzyblue_gb300.workloads.uneven_batch, seed 1)",
        "config": {"workload": "uneven batch: 96 seeded atmospheres (seed 1), default / half / double table "
                               "classes 32 each, orders uniform in 2-8", "classes": per_class,
                   "orders": sorted(set(p.order for p in params)), "precision": a.precision,
                   "l2": "inputs larger than L2"},
        "clocks": clk,
        "e2e": {"value": 96 / e2e_s, "unit": "atmospheres/s", "h2d_bytes_per_step": 96 * 384,
                "d2h_bytes_per_step": d2h // steps},
        "tile_shapes": tuned,
        "plain": {"atmospheres_per_s": 96 / plain_total, "precision": "plain",
                  "path": "each atmosphere alone, one call each, FP32"},
        "batched_over_plain": (96 / (ms / 1e3)) / (96 / plain_total),
        "per_class": compare,
    }
    return out


# ---------------------------------------------------------------- serving ---
def _class_percentiles(lat):
    """{class: {"n", "p50_ms", "p99_ms"}} of per-class latency arrays (ms)."""
    import numpy as np
    return {c: {"n": int(len(v)), "p50_ms": float(np.percentile(v, 50)) if len(v) else None,
                "p99_ms": float(np.percentile(v, 99)) if len(v) else None} for c, v in lat.items()}


def run_serve(a):
    """Open-loop Poisson request stream (seed 2) through the request loop
    (fb_server_*): each request one atmosphere drawn from the uniform-batch
    distributions, table class 60/30/10 default / half / double, orders 2-8,
    admitted under a 120 GB HBM budget, finished tables resident (LRU). The
    plain one-at-a-time path is measured as per-request build times of plain
    FP32 single builds per (class, order), replayed in arrival order through
    one FIFO server with the same queue limit."""
    import torch
    torch.cuda.set_device(0)
    from fuzzyblue_gb300.api import Builder
    builder = Builder(0)
    print(json.dumps(measure_serve(a, builder, [float(x) for x in a.rates.split(",")], a.duration)))
    builder.close()


def measure_serve(a, builder, rates, duration):
    """The serving line: per offered rate, served throughput and latency
    percentiles (overall and per class) beside the plain FIFO replay."""
    import threading
    import numpy as np
    from fuzzyblue_gb300 import workloads
    from fuzzyblue_gb300 import _native as N
    from fuzzyblue_gb300.api import Atmosphere, Server
    from fuzzyblue_gb300.params import PRECISION_MIXED, PRECISION_PLAIN
    names = ("default", "half", "double")
    prec = PRECISION_MIXED if a.precision == "mixed" else PRECISION_PLAIN
    probe = workloads.draw_atmosphere(np.random.default_rng(99), precision=prec)
    if not a.no_autotune:
        builder.autotune([probe.replace(**workloads.CLASSES[c]) for c in names], batch=4)

    def cls_of(p):
        for c in ("double", "half"):  # the default class has no overrides: test it last
            if all(getattr(p, k) == v for k, v in workloads.CLASSES[c].items()):
                return c
        return "default"

    # plain one-at-a-time service times per (class, order), FP32
    service = {}
    for c in names:
        for order in range(2, 9):
            q0 = probe.replace(precision=PRECISION_PLAIN, order=order, **workloads.CLASSES[c])
            ts = []
            for rep in range(3):
                t0 = time.perf_counter()
                q = Atmosphere.build(builder, q0)
                q.wait()
                ts.append(time.perf_counter() - t0)
                q.release()
            service[(c, order)] = min(ts[1:])
    lines = []
    for rate in rates:
        rng = np.random.default_rng(2)
        arrivals, t = [], 0.0
        while True:
            t += float(rng.exponential(1.0 / rate))
            if t > duration:
                break
            arrivals.append(t)
        reqs = [workloads.serving_request(rng, precision=prec) for _ in arrivals]
        srv = Server(builder, hbm_budget_bytes=120 * 10 ** 9, max_queue=a.max_queue)
        submit_at, done_at, rejected, cls_at = {}, {}, [0], {}
        lock = threading.Lock()
        start = time.perf_counter() + 0.05

        def submitter():
            for at, p in zip(arrivals, reqs):
                delay = start + at - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                try:
                    tk = srv.submit(p)
                except N.FuzzyblueError:
                    with lock:
                        rejected[0] += 1
                    continue
                with lock:
                    submit_at[tk] = start + at
                    cls_at[tk] = cls_of(p)
        th = threading.Thread(target=submitter)
        th.start()
        # finished tickets come from the server's completion queue
        # (fb_server_completed): one call per wake-up, not a poll per ticket
        failed = [0]
        deadline = start + duration + 120.0
        while time.perf_counter() < deadline:
            for tk in srv.completed(timeout_ms=1):
                now = time.perf_counter()
                try:
                    ok = srv.poll(tk) is not None
                except N.FuzzyblueError:
                    ok = False
                if ok:
                    done_at[tk] = now
                else:
                    failed[0] += 1
                srv.release(tk)
            if not th.is_alive():
                with lock:
                    if len(done_at) + failed[0] >= len(submit_at):
                        break
        th.join()
        st = srv.stats()
        srv.close()
        lat = np.array([done_at[k] - submit_at[k] for k in done_at]) * 1e3
        lat_cls = {c: np.array([done_at[k] - submit_at[k] for k in done_at if cls_at[k] == c]) * 1e3 for c in names}
        end = max(done_at.values()) if done_at else start
        served = {"completed": len(done_at), "rejected": rejected[0], "failed": failed[0],
                  "throughput": len(done_at) / max(end - start, 1e-9),
                  "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
                  "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
                  "server_p50_ms": st["p50_ms"], "server_p99_ms": st["p99_ms"], "batches": st["batches"],
                  "mean_batch": st["mean_batch"], "evictions": st["evictions"],
                  "by_class": _class_percentiles(lat_cls)}
        # the plain path on the same arrivals: one FIFO server, same queue limit
        free_at, lat_p, comp, rej_p, queue = 0.0, [], 0, 0, []
        lat_pc = {c: [] for c in names}
        for at, p in zip(arrivals, reqs):
            queue = [x for x in queue if x > at]  # completion times still ahead
            if len(queue) > a.max_queue:
                rej_p += 1
                continue
            s_t = service[(cls_of(p), p.order)]
            begin = max(at, free_at)
            free_at = begin + s_t
            queue.append(free_at)
            lat_p.append((free_at - at) * 1e3)
            lat_pc[cls_of(p)].append(lat_p[-1])
            comp += 1
        plain = {"completed": comp, "rejected": rej_p, "throughput": comp / max(free_at, 1e-9),
                 "p50_ms": float(np.percentile(lat_p, 50)), "p99_ms": float(np.percentile(lat_p, 99)),
                 "by_class": _class_percentiles({c: np.array(v) for c, v in lat_pc.items()})}
        lines.append({"offered_rate": rate, "requests": len(arrivals), "served": served, "plain": plain,
                      "served_over_plain_throughput": served["throughput"] / plain["throughput"]})
    out = {
        "metric": "served atmospheres/s and p50/p99 request latency, Poisson open loop",
        "value": max(l["served"]["throughput"] for l in lines), "unit": "atmospheres/s", "n_gpus": 1,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 with f64 ray geometry and order accumulation" if a.precision == "mixed" else "f32",
        "data": "synthetic: seeded requests (fuzzyblue_gb300.workloads.serving_request, seed 2)",
        "config": {"workload": "serving: open-loop Poisson requests, class 60/30/10 default / half / double, "
                               "orders 2-8, 120 GB HBM budget, LRU-resident tables",
                   "duration_s": duration, "max_queue": a.max_queue, "precision": a.precision,
                   "plain_path": "plain FP32 single builds per (class, order), measured, replayed FIFO"},
        "rates": lines,
    }
    return out


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "uneven":
        run_uneven(a)
    elif a.workload == "serve":
        run_serve(a)
    elif a.workload == "render":
        run_render(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
