"""Benchmark of the point-cloud hologram path on GB300.

Workload (default): the full-HD three-colour sphere — 1920x1080 SLM at
8.0 um pitch, 638/532/473 nm channels, 100,000 points on a randomly
perturbed sphere of radius 3 mm at z = 0.5 m (seeded synthetic data; the
reference ships no dataset). One step = generateHologram(PC_DIFF_RS) for all
three channels + phase encoding + 8-bit normalisation over all channels.

The headline `value` is RS point x pixel interactions per second over the
device-timed steps (inputs resident in HBM, L2 flushed between steps), with
RS on the tensor cores (OPHPC_MODE_TENSOR_BF16X3: split-BF16 contraction of
per-tile row and column factors, relL2 ~1e-5 against FP64, stated in
`relL2_vs_fp64`); `e2e` is the same metric through the host-facing C ABI
with host buffers, host->device copy of the vertices and device->host copy
of the complex field and the 8-bit codes inside every timed step. The plain
FP32-core RS kernel (`rs_plain`) and Fresnel (plain FP32 kernel and tensor
cores) are timed the same way and reported beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

For N > 1 (torchrun) every rank generates its own hologram of the workload
(independent jobs, no data-path collective: weak scaling); `value` is the
sum over ranks divided by the slowest rank's time.

`--impl reference` times the reference's CPU point-cloud path on the host
cores instead: the reference's own sources (oracle/_ref) where they were
compiled, else the C restatement of that path (oracle/), each step a
bounded sample (a subset of the points at full resolution) of the same
workload.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "pt*px/s RS & Fresnel at relL2<=1e-4 vs FP64; serving p50/p99 ms vs plain"
UNIT = "interactions/s"
WORKLOAD = "sphere_fhd"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--cpu-points", type=int, default=0, help="points in the CPU sample (0 = auto)")
    ap.add_argument("--serving-jobs", type=int, default=512, help="jobs in the serving stream")
    ap.add_argument("--profile-case", default=None,
                    help="run one fixed case for a profiler and exit: rs_1k, fresnel_1k, rs_fhd (sphere_fhd "
                         "RS generate), tc_fp16_4k, tc_bf16x3_4k (box_4k distribution, 131,072 points), "
                         "tcrs_fhd (tensor-core RS, sphere_fhd, 20,000 points), tcrs_fhd_full (all 100,000), "
                         "step_fhd (the headline step: tensor-core RS + phase codes), "
                         "tcf_fhd_full (tensor-core Fresnel, sphere_fhd), tcf_4k (tensor-core Fresnel, box_4k "
                         "geometry, 131,072 points), codes_fhd (the headline step's generate, then the phase "
                         "codes twice)")
    ap.add_argument("--serving-max-points", type=int, default=500_000,
                    help="largest point count of a serving job")
    return ap.parse_args()


def env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(x: float, dist, device: str) -> float:
    """The largest x over the ranks (the slowest rank's step time): an
    all-reduce of one value, on `device` ("cuda" under NCCL, "cpu" under
    gloo). With no process group, x itself."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_rank: float, world: int, t_slowest: float) -> float:
    """Whole-job throughput: every rank processes its own units (weak
    scaling), the job ends with the slowest rank."""
    return units_per_rank * world / t_slowest


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_model() -> str:
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part", "hardware")):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"ophpc_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        except Exception:
            return out
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for nm, val in zip(names, r[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if sm:
            out.update(sm_mhz=statistics.median(sm), sm_max_mhz=max(mx), reasons=sorted(reasons), samples=len(sm))
        return out


# ------------------------------------------------------------------ CPU arm

def cpu_sample_run(w, n_points: int, diff_flag: int):
    """Times the CPU point-cloud path on `n_points` of the workload at full
    resolution with all host threads. Returns (interactions/s, seconds,
    kind, field)."""
    import oracle
    sub = w.subset(n_points)
    g = oracle.Geometry(pnx=sub.pnx, pny=sub.pny, ppx=sub.pp, ppy=sub.pp, wavelengths=list(sub.wavelengths))
    if oracle.ref_available():
        import tempfile
        with tempfile.TemporaryDirectory() as d:
            xml = os.path.join(d, "cfg.xml")
            with open(xml, "w") as f:
                f.write(g.xml())
            # generateHologram's own elapsed time (ophgen/src/ophPointCloud.cpp:187-190)
            field, _, _, secs = oracle.ref_run(xml, vertices=sub.vertices, diff_flag=diff_flag, encode_flag=3)
        kind = "reference"
    else:
        t0 = time.perf_counter()
        field = oracle.generate(g, sub.vertices, diff_flag)
        secs = time.perf_counter() - t0
        kind = "port"
    return sub.interactions / secs, secs, kind, field


def reference_arm(args, w):
    rank, world, _ = env_rank()
    if rank != 0:
        return
    # 300 points: enough for the OpenMP point loop to keep 16+ threads busy
    # (60 points left it starved and under-reported the CPU by 2.5x)
    n = args.cpu_points or 300
    for _ in range(max(0, args.warmup)):
        cpu_sample_run(w, n, 0)
    times = []
    kind = "port"
    for _ in range(args.steps):
        _, secs, kind, _ = cpu_sample_run(w, n, 0)
        times.append(secs)
    t = sum(times) / len(times)
    inter = w.subset(n).interactions
    value = inter / t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": w.name, "pnx": w.pnx, "pny": w.pny, "channels": w.n_channels,
                   "n_points": w.n_points, "diff": "RS", "sample_points": n},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": host_cores(), "kind": kind,
                         "sample": f"{n} of {w.n_points} points, full {w.pnx}x{w.pny}, {w.n_channels} channels, "
                                   f"RS; OpenMP over {host_cores()} threads ({cpu_model()})"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ serving

def single_server_p99(iso: np.ndarray, arrivals: np.ndarray, key) -> float:
    """p99 latency (s) of an ideal preemptive single server that runs one job
    at a time at its isolated speed, highest priority first (key(j, arrival)
    -> sort key, smaller first). A queueing bound for the serving stream:
    whatever the GPU overlaps beyond this is gained by running jobs side by
    side."""
    n = len(iso)
    rem = iso.astype(np.float64).copy()
    done = np.zeros(n)
    active = []
    t, i = 0.0, 0
    while i < n or active:
        if not active:
            t = max(t, arrivals[i])
        while i < n and arrivals[i] <= t + 1e-12:
            active.append(i)
            i += 1
        j = min(active, key=lambda q: key(q, arrivals[q]))
        nxt = arrivals[i] if i < n else np.inf
        dt = min(rem[j], nxt - t)
        rem[j] -= dt
        t += dt
        if rem[j] <= 1e-12:
            done[j] = t
            active.remove(j)
    return float(np.percentile(done - arrivals, 99))


def serving_leg(n_jobs: int, max_points: int, loads=(0.5, 0.8, 0.95), seed: int = 4):
    """Mixed hologram jobs with Poisson arrivals through the serving engine.

    Every job is first run alone (isolated latency = its service time); the
    mean isolated service time sets the arrival rate of each offered load.
    Latency = completion - arrival (server clock). Jobs return their 8-bit
    phase holograms (the field stays on the device). The default policy
    (every job by earliest deadline) runs every load; shortest remaining
    work and short-jobs-first run the 80% load beside it."""
    import threading

    import torch

    from openholo_gb300 import make_config, workloads
    from openholo_gb300.serving import POLICY_DEADLINE, POLICY_EARLIEST_DEADLINE, POLICY_SHORTEST_REMAINING, Server

    jobs = workloads.serving_stream(n_jobs, rate_per_s=1.0, seed=seed, max_points=max_points)
    prepared = []
    for jb in jobs:
        w = jb.workload
        hv = torch.from_numpy(w.vertices).pin_memory()
        hc = torch.empty((w.n_channels, w.pny, w.pnx), dtype=torch.uint8).pin_memory()
        prepared.append((make_config(**w.geometry_kwargs()), hv, hc, w.n_points, jb.diff_flag, w.interactions))
    # every job on the tensor cores, split-BF16 (RS: tensor-core RS; Fresnel:
    # factor tables + tcgen05 GEMM), relL2 ~1e-5 against FP64
    mode_of = lambda d: 0x200   # noqa: E731
    out = {"jobs": n_jobs, "max_points": max_points, "loads": {}}
    rng = np.random.default_rng(seed + 1)
    gaps = rng.exponential(1.0, n_jobs)
    iso = None

    def run_load(srv, load, mean_s):
        arrivals = np.cumsum(gaps) * mean_s / load
        tickets = [None] * n_jobs

        def feeder():
            t0 = time.perf_counter()
            for i, (cfg, hv, hc, n, d, _) in enumerate(prepared):
                dt = arrivals[i] - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
                tickets[i] = srv.submit_raw(cfg, hv.data_ptr(), n, d, None, hc.data_ptr(), 0, mode_of(d))

        th = threading.Thread(target=feeder)
        th.start()
        th.join()
        res = [srv.wait_stats(t) for t in tickets]
        lat = np.array([r.t_done - r.t_submit for r in res])
        span = max(r.t_done for r in res) - min(r.t_submit for r in res)
        slow = lat / iso
        arr_rel = arrivals - arrivals[0]
        p99_iso = float(np.percentile(iso, 99))
        # the same, and with the jobs above the isolated p99 deferred behind
        # all others (the top 1 % may be late without moving the p99)
        model = {"fcfs_p99_over_isolated_p99": single_server_p99(iso, arr_rel, lambda q, a: a) / p99_iso,
                 "edf_p99_over_isolated_p99": single_server_p99(iso, arr_rel, lambda q, a: a + 2 * iso[q] + 0.02)
                 / p99_iso,
                 "edf_largest_last_p99_over_isolated_p99": single_server_p99(
                     iso, arr_rel, lambda q, a: (1e9 if iso[q] > p99_iso else 0.0) + a + 2 * iso[q] + 0.02)
                 / p99_iso}
        return {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "single_server_model": model,
                "p99_over_isolated_p99": float(np.percentile(lat, 99) / np.percentile(iso, 99)),
                "slowdown_p50": float(np.percentile(slow, 50)), "slowdown_p99": float(np.percentile(slow, 99)),
                "throughput_interactions_per_s": float(sum(p[5] for p in prepared) / span),
                "jobs_per_s": n_jobs / span}

    with Server(0, max_in_flight=16, step_ms=2.0, policy=POLICY_EARLIEST_DEADLINE) as srv:
        iso = []
        for cfg, hv, hc, n, d, _ in prepared:
            r = srv.wait_stats(srv.submit_raw(cfg, hv.data_ptr(), n, d, None, hc.data_ptr(), 0, mode_of(d)))
            iso.append(r.t_done - r.t_submit)
        iso = np.array(iso)
        mean_s = float(iso.mean())
        out["isolated_ms"] = {"p50": float(np.percentile(iso, 50) * 1e3), "p99": float(np.percentile(iso, 99) * 1e3),
                              "mean": mean_s * 1e3}
        out["policy"] = "earliest deadline (submission + 2 x estimated isolated time + 20 ms)"
        out["kernels"] = "every job on the tensor cores, split-BF16 (RS and Fresnel)"
        for load in loads:
            out["loads"][f"{load:.2f}"] = run_load(srv, load, mean_s)
    with Server(0, max_in_flight=16, step_ms=2.0, policy=POLICY_SHORTEST_REMAINING) as srv:
        out["shortest_remaining_0.80"] = run_load(srv, 0.8, mean_s)
    with Server(0, max_in_flight=16, step_ms=2.0, policy=POLICY_DEADLINE) as srv:
        out["short_first_deadline_0.80"] = run_load(srv, 0.8, mean_s)
    return out


def plan_leg(ctx, sp, reps: int = 50):
    """Small repeated jobs: host wall time of one synchronised generate +
    phase encode through the direct calls and through a plan (the same calls
    captured once into a CUDA graph and replayed; ophpc_plan_*), 512x512,
    2,000 points, per tensor-core path."""
    import torch

    import openholo_gb300 as oph
    n, pnx, pny = 2000, 512, 512
    rng = np.random.default_rng(11)
    v = np.zeros((n, 7))
    v[:, 0:2] = rng.uniform(-1e-3, 1e-3, (n, 2))
    v[:, 2] = rng.uniform(0.45, 0.55, n)
    v[:, 3:6] = 1.0 - rng.uniform(0.0, 1.0, (n, 3))
    cfg = oph.make_config(pnx=pnx, pny=pny, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9])
    dv = torch.from_numpy(v).cuda()
    f = torch.empty((1, pny, pnx, 2), dtype=torch.float64, device="cuda")
    codes = torch.empty((1, pnx * pny), dtype=torch.uint8, device="cuda")
    out = {"workload": "512x512, 2,000 points, 532 nm, generate + phase encode, synchronised"}
    for name, diff in (("rs_tc_bf16x3", oph.DIFF_RS), ("fresnel_tc_bf16x3", oph.DIFF_FRESNEL)):
        def direct():
            ctx.generate(cfg, dv.data_ptr(), n, diff, oph.MODE_TENSOR_BF16X3, f.data_ptr(), sp)
            ctx.encode(f.data_ptr(), 1, pnx * pny, oph.ENCODE_PHASE, None, codes.data_ptr(), sp)
            torch.cuda.synchronize()
        with ctx.plan(cfg, dv.data_ptr(), n, diff, oph.MODE_TENSOR_BF16X3, f.data_ptr(), oph.ENCODE_PHASE, None,
                      codes.data_ptr()) as plan:
            def replay():
                plan.launch(sp)
                plan.wait(sp)
            ms = {}
            for key, fn in (("direct_ms", direct), ("plan_ms", replay)):
                for _ in range(5):
                    fn()
                t0 = time.perf_counter()
                for _ in range(reps):
                    fn()
                ms[key] = (time.perf_counter() - t0) / reps * 1e3
        out[name] = ms
    return out


def facade_e2e(w, mode: int, steps: int) -> dict:
    """The reference caller's sequence through the ophPointCloud façade's C
    ABI with host buffers: setPointCloudModel, generateHologram(RS),
    encoding(PHASE), normalize. Wall clock around the synchronous calls
    (after 3 untimed repetitions); bytes are those the façade copies."""
    from openholo_gb300.pointcloud import PointCloud
    with tempfile.TemporaryDirectory() as d:
        xml = os.path.join(d, "cfg.xml")
        with open(xml, "w") as f:
            f.write(w.config_xml())
        h = PointCloud()
        try:
            if not h.readConfig(xml):
                raise RuntimeError(f"readConfig: {h.lastError()}")
            h.SetMode(mode)
            v = np.ascontiguousarray(w.vertices)
            gen_s = []
            calls = {"setPointCloudModel": [], "generateHologram": [], "encoding": [], "normalize": []}

            def step():
                t0 = time.perf_counter()
                h.setPointCloudModel(v)
                t1 = time.perf_counter()
                secs = h.generateHologram(0)
                if secs <= 0.0:
                    raise RuntimeError(f"generateHologram: {h.lastError()}")
                t2 = time.perf_counter()
                h.encoding(0)
                t3 = time.perf_counter()
                h.normalize()
                t4 = time.perf_counter()
                gen_s.append(secs)
                for k, a, b in (("setPointCloudModel", t0, t1), ("generateHologram", t1, t2), ("encoding", t2, t3),
                                ("normalize", t3, t4)):
                    calls[k].append((b - a) * 1e3)

            for _ in range(3):
                step()
            gen_s.clear()
            for c in calls.values():
                c.clear()
            t0 = time.perf_counter()
            for _ in range(steps):
                step()
            t = (time.perf_counter() - t0) / steps
        finally:
            h.release()
    npx = w.pnx * w.pny * w.n_channels
    return {"s_per_step": t, "generate_s": sum(gen_s) / len(gen_s),
            "calls_ms_median": {k: float(np.median(c)) for k, c in calls.items()},
            "h2d": w.n_points * 56 + npx * 16 + npx * 8, "d2h": npx * 16 + npx * 8 + npx}


def generate_host_e2e(ctx, w, cfg, mode: int, steps: int) -> dict:
    """ophpc_generate_host: host vertices in, one host complex_H buffer per
    channel out (page-locked here), synchronous; wall clock per call."""
    import torch
    hv = torch.from_numpy(np.ascontiguousarray(w.vertices)).pin_memory()
    hf = [torch.empty((w.pny, w.pnx, 2), dtype=torch.float64).pin_memory() for _ in range(w.n_channels)]
    ptrs = [t.data_ptr() for t in hf]
    for _ in range(3):
        ctx.generate_host(cfg, hv.data_ptr(), w.n_points, 0, mode, ptrs)
    t0 = time.perf_counter()
    for _ in range(steps):
        ctx.generate_host(cfg, hv.data_ptr(), w.n_points, 0, mode, ptrs)
    t = (time.perf_counter() - t0) / steps
    return {"value": w.interactions / t, "unit": UNIT, "ms_per_call": t * 1e3,
            "h2d_bytes_per_step": w.n_points * 56, "d2h_bytes_per_step": w.pnx * w.pny * w.n_channels * 16,
            "call": "ophpc_generate_host (RS, tensor cores): host Vertex[] in, host complex_H per channel out"}


def relL2_at_pixels(ctx, w, diff: int, mode: int, n_pix: int = 256, seed: int = 17):
    """relL2 of one generate against the FP64 oracle at seeded pixels of
    every channel, all points (accuracy leg; outside any timed region)."""
    import torch

    import openholo_gb300 as oph
    import oracle
    cfg = oph.make_config(**w.geometry_kwargs())
    npx = w.pnx * w.pny
    dv = torch.from_numpy(w.vertices).cuda()
    f = torch.empty((w.n_channels, npx, 2), dtype=torch.float64, device="cuda")
    ctx.generate(cfg, dv.data_ptr(), w.n_points, diff, mode, f.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    pix = np.sort(np.random.default_rng(seed).choice(npx, n_pix, replace=False))
    g = f[:, torch.from_numpy(pix).cuda()].cpu().numpy()
    got = g[..., 0] + 1j * g[..., 1]
    gw = oracle.Geometry(pnx=w.pnx, pny=w.pny, ppx=w.pp, ppy=w.pp, wavelengths=list(w.wavelengths),
                         scale=w.scale, distance=w.distance)
    want = np.stack([oracle.field_at(gw, w.vertices, diff, c, pix) for c in range(w.n_channels)])
    del dv, f
    return float(np.linalg.norm(got - want) / np.linalg.norm(want))


def extra_workload_leg(ctx, w, variants, steps: int) -> dict:
    """Device-timed generate calls of one more benchmark workload (L2 is
    flushed by the inputs: every field here is larger than the 129 MB L2,
    except rs_1k's, whose steps flush it with a 256 MB write), each with its
    relL2 against the FP64 oracle at 256 seeded pixels per channel."""
    import torch

    import openholo_gb300 as oph
    cfg = oph.make_config(**w.geometry_kwargs())
    s = torch.cuda.current_stream()
    dv = torch.from_numpy(w.vertices).cuda()
    f = torch.empty((w.n_channels, w.pny, w.pnx, 2), dtype=torch.float64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    out = {"pnx": w.pnx, "pny": w.pny, "channels": w.n_channels, "n_points": w.n_points,
           "interactions_per_call": w.interactions}
    for name, diff, mode in variants:
        ctx.generate(cfg, dv.data_ptr(), w.n_points, diff, mode, f.data_ptr(), s.cuda_stream)
        torch.cuda.synchronize()
        ts = []
        for _ in range(steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(s)
            ctx.generate(cfg, dv.data_ptr(), w.n_points, diff, mode, f.data_ptr(), s.cuda_stream)
            b.record(s)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b) / 1e3)
        t = sum(ts) / len(ts)
        out[name] = {"value": w.interactions / t, "unit": UNIT, "ms_per_generate": t * 1e3}
    del dv, f, flush
    torch.cuda.empty_cache()
    for name, diff, mode in variants:
        out[name]["relL2_vs_fp64"] = relL2_at_pixels(ctx, w, diff, mode)
    out["relL2_samples"] = f"all {w.n_points} points at 256 seeded pixels per channel (FP64 oracle)"
    return out


def wrp_leg(ctx, steps: int) -> dict:
    """WRP generator (ophWRP::generateHologram): the reference's own example
    (Example/dataset/Dice/WRP/Dice_WRP.xml geometry: 1920x1080, 4.3 um, 532
    nm, scale 0.0015/0.0015/0.0003, WRP at 300 um, propagation 0.1 m, the
    Dice point cloud's shape as seeded points: 7,493 points on a cube's
    faces) and the sphere_fhd point cloud (100,000 points, three colours)
    with its WRP 1 mm in front of the sphere and 0.5 m of propagation.
    Device-timed per hologram (L2 flushed), relL2 against the FP64 oracle
    (splat restated, propagation by numpy FFT)."""
    import torch

    import openholo_gb300 as oph
    import oracle
    from openholo_gb300 import workloads as W
    s = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    rng = np.random.default_rng(7)
    n = 7493
    face = rng.integers(0, 6, n)
    uv = rng.uniform(-1, 1, (n, 2))
    cube = np.zeros((n, 3))
    for f in range(6):
        m = face == f
        ax, sg = f // 2, 1.0 if f % 2 else -1.0
        others = [a for a in range(3) if a != ax]
        cube[m, ax] = sg * 0.37
        cube[m, others[0]] = 0.37 * uv[m, 0]
        cube[m, others[1]] = 0.37 * uv[m, 1]
    dice = np.zeros((n, 7))
    dice[:, 0:3] = cube * np.array([1.0, 1.45, 1.2])
    dice[:, 3:6] = 1.0 - rng.uniform(0.0, 1.0, (n, 3))
    sph = W.sphere_fhd()
    cases = {
        "dice_example": (dict(pnx=1920, pny=1080, ppx=4.3e-6, ppy=4.3e-6, wavelengths=[532e-9],
                              scale=(0.0015, 0.0015, 0.0003), wrp_location=300e-6, distance=0.1), dice),
        "sphere_fhd": (dict(pnx=1920, pny=1080, ppx=8e-6, ppy=8e-6, wavelengths=list(sph.wavelengths),
                            scale=(1.0, 1.0, 1.0), wrp_location=float(sph.vertices[:, 2].max()) + 1e-3,
                            distance=0.5), sph.vertices),
    }
    out = {}
    for name, (kw, v) in cases.items():
        cfg = oph.make_wrp_config(**kw)
        dv = torch.from_numpy(np.ascontiguousarray(v)).cuda()
        f = torch.empty((cfg.n_channels, kw["pny"], kw["pnx"], 2), dtype=torch.float64, device="cuda")
        run = lambda: ctx.wrp_generate(cfg, dv.data_ptr(), v.shape[0], f.data_ptr(), s.cuda_stream)  # noqa: E731
        run()
        torch.cuda.synchronize()
        ts = []
        for _ in range(steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(s)
            run()
            b.record(s)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b) / 1e3)
        t = sum(ts) / len(ts)
        g = oracle.WrpGeometry(**kw)
        zmax = oracle.wrp_zmax(g, v)
        wsq = [int(abs(lam * (kw["wrp_location"] - zmax) / (kw["ppx"] ** 2 * 2)) * 2) for lam in kw["wavelengths"]]
        res = {"pnx": kw["pnx"], "pny": kw["pny"], "channels": cfg.n_channels, "n_points": int(v.shape[0]),
               "splat_half_width_px": wsq, "ms_per_hologram": t * 1e3, "holograms_per_s": 1.0 / t,
               "note": "synchronises once per call to read the depth range"}
        t0 = time.perf_counter()
        want = oracle.wrp_generate(g, v)
        res["oracle_cpu_s"] = time.perf_counter() - t0
        h = f.cpu().numpy()
        got = h[..., 0] + 1j * h[..., 1]
        res["relL2_vs_fp64"] = float(np.linalg.norm(got - want) / np.linalg.norm(want))
        out[name] = res
        del dv, f
    return out


def full_field_codes(ctx, w, mode: int) -> dict:
    """8-bit codes of the headline step (generate + encode + normalise over
    all channels) against the codes of the reference's own FP64 GPU kernel's
    field over every pixel (accuracy leg, outside any timed region; the
    reference kernel takes ~3 minutes at sphere_fhd)."""
    import torch

    import oracle
    from oracle import ref_gpu
    if not ref_gpu.available():
        return {"unavailable": "reference GPU kernels not built"}
    import openholo_gb300 as oph
    k = ref_gpu.RefGpuKernels()
    try:
        ref = k.generate(w.geometry_kwargs(), w.vertices, 0, chunk_points=5000)
    finally:
        k.close()
    cfg = oph.make_config(**w.geometry_kwargs())
    npx = w.pnx * w.pny
    dv = torch.from_numpy(w.vertices).cuda()
    f = torch.empty((w.n_channels, npx, 2), dtype=torch.float64, device="cuda")
    codes = torch.empty((w.n_channels, npx), dtype=torch.uint8, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    ctx.generate(cfg, dv.data_ptr(), w.n_points, 0, mode, f.data_ptr(), sp)
    torch.cuda.synchronize()
    h = f.cpu().numpy()
    got_field = (h[..., 0] + 1j * h[..., 1]).reshape(ref.shape)
    out = {"checker": "reference FP64 GPU kernel (ophgen/src/ophPCKernel.cu, compiled for sm_103a), every pixel",
           "field_relL2": float(np.linalg.norm(got_field - ref) / np.linalg.norm(ref))}
    for flag, name in ((0, "phase"), (1, "amplitude")):
        ctx.encode(f.data_ptr(), w.n_channels, npx, flag, None, codes.data_ptr(), sp)
        torch.cuda.synchronize()
        got = codes.cpu().numpy().astype(np.int32)
        want, _, _ = oracle.normalize(oracle.encode(ref, flag))
        dlt = got - want.reshape(got.shape).astype(np.int32)
        if flag == 0:
            dlt = (dlt + 128) % 256 - 128
        out[name] = {"codes_exact_frac": float(np.mean(dlt == 0)), "codes_max_lsb": int(np.abs(dlt).max())}
    del dv, f, codes
    return out


# ------------------------------------------------------------------ GPU arm

def gpu_arm(args, w):
    import torch

    import openholo_gb300 as oph

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    ctx = oph.Context(local)
    lib = oph.lib()
    cfg = oph.make_config(**w.geometry_kwargs())
    nch, pnx, pny = w.n_channels, w.pnx, w.pny
    npx = pnx * pny
    s = torch.cuda.current_stream()
    sp = s.cuda_stream
    dv = torch.from_numpy(w.vertices).cuda()
    field = torch.empty((nch, pny, pnx, 2), dtype=torch.float64, device="cuda")
    codes = torch.empty((nch, npx), dtype=torch.uint8, device="cuda")
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")   # > 129 MB L2

    # headline RS path: the tensor-core RS (split-BF16, relL2 ~1e-5 vs FP64)
    rs_mode = oph.MODE_TENSOR_BF16X3

    def step(diff):
        ctx.generate(cfg, dv.data_ptr(), w.n_points, diff, rs_mode, field.data_ptr(), sp)
        ctx.encode(field.data_ptr(), nch, npx, oph.ENCODE_PHASE, None, codes.data_ptr(), sp)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(fn, steps):
        """Per-step CUDA events on the launching stream, L2 flushed between steps."""
        evs = []
        for _ in range(steps):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(s)
            fn()
            b.record(s)
            evs.append((a, b))
        torch.cuda.synchronize()
        return [a.elapsed_time(b) / 1e3 for a, b in evs]

    # warm-up
    for _ in range(max(3, args.warmup)):
        step(oph.DIFF_RS)
    torch.cuda.synchronize()

    # --- headline: device-resident RS step ---------------------------------
    barrier()
    l0 = lib.ophpc_kernel_launches()
    wall0 = time.perf_counter()
    with ClockSampler(local) as clk:
        step_times = timed(lambda: step(oph.DIFF_RS), args.steps)
    barrier()
    wall = time.perf_counter() - wall0
    launches = lib.ophpc_kernel_launches() - l0
    t_step = max_over_ranks(sum(step_times) / len(step_times), dist, "cuda")
    inter = w.interactions
    value = job_value(inter, world, t_step)

    # --- dominant kernel alone for the roofline: the tensor-core RS generate
    # (prep + amax + tc_rs_kernel + CUDA-core complement, which exits at once
    # when every pair went to the tensor cores)
    gen_tc = timed(lambda: ctx.generate(cfg, dv.data_ptr(), w.n_points, oph.DIFF_RS, rs_mode, field.data_ptr(), sp), 3)
    t_tc = sum(gen_tc) / len(gen_tc)
    # the plain FP32-core RS kernel (prep + rs_kernel), reported beside it
    gen_rs = timed(lambda: ctx.generate(cfg, dv.data_ptr(), w.n_points, oph.DIFF_RS, 0, field.data_ptr(), sp), 3)
    t_rs = max_over_ranks(sum(gen_rs) / len(gen_rs), dist, "cuda")
    gen_fr = timed(lambda: ctx.generate(cfg, dv.data_ptr(), w.n_points, oph.DIFF_FRESNEL, 0, field.data_ptr(), sp),
                   max(3, args.steps // 2))
    t_fr = max_over_ranks(sum(gen_fr) / len(gen_fr), dist, "cuda")

    # --- tensor-core Fresnel (tcgen05): FP16 and split-BF16, relL2 against the
    # plain FP32 Fresnel field (itself within ~1e-6 of FP64)
    def tensor_leg(wl, d_vert, cfg_l, out, steps):
        res = {}
        plain = torch.empty_like(out)
        t_plain = None
        gen_p = timed(lambda: ctx.generate(cfg_l, d_vert.data_ptr(), wl.n_points, oph.DIFF_FRESNEL, 0,
                                           plain.data_ptr(), sp), 1)
        t_plain = gen_p[0]
        for name, mode in (("fp16", oph.MODE_TENSOR_FP16), ("bf16x3", oph.MODE_TENSOR_BF16X3)):
            ctx.generate(cfg_l, d_vert.data_ptr(), wl.n_points, oph.DIFF_FRESNEL, mode, out.data_ptr(), sp)
            torch.cuda.synchronize()
            ts = timed(lambda: ctx.generate(cfg_l, d_vert.data_ptr(), wl.n_points, oph.DIFF_FRESNEL, mode,
                                            out.data_ptr(), sp), steps)
            t = sum(ts) / len(ts)
            rel = float(torch.linalg.vector_norm(out - plain) / torch.linalg.vector_norm(plain))
            res[name] = {"value": wl.interactions / t, "unit": UNIT, "ms_per_generate": t * 1e3,
                         "relL2_vs_plain_fp32": rel, "speedup_vs_plain_fresnel": t_plain / t}
        res["plain_fresnel_ms"] = t_plain * 1e3
        return res

    tensor = {"sphere_fhd": tensor_leg(w, dv, cfg, field, max(3, args.steps // 2))}
    from openholo_gb300 import workloads as W
    w4 = W.box_4k()
    cfg4 = oph.make_config(**w4.geometry_kwargs())
    dv4 = torch.from_numpy(w4.vertices).cuda()
    f4 = torch.empty((1, w4.pny, w4.pnx, 2), dtype=torch.float64, device="cuda")
    tensor["box_4k"] = tensor_leg(w4, dv4, cfg4, f4, 2)
    del dv4, f4
    for name, mode in (("fp16", oph.MODE_TENSOR_FP16), ("bf16x3", oph.MODE_TENSOR_BF16X3)):
        tensor["box_4k"][name]["relL2_vs_fp64"] = relL2_at_pixels(ctx, w4, 1, mode)
    tensor["box_4k"]["relL2_vs_fp64_samples"] = "all 1,000,000 points at 256 seeded pixels (FP64 oracle)"

    # the other benchmark workloads: rs_1k (1024x1024, 5,000 points) and
    # box_8k (7680x4320, 2,000,000 points; tensor-core RS only: the FP32-core
    # kernel would take ~30 s a call)
    from openholo_gb300 import workloads as W
    more = {}
    more["rs_1k"] = extra_workload_leg(ctx, W.rs_1k(), [("rs_plain", 0, 0), ("rs_tc_bf16x3", 0, rs_mode),
                                                         ("fresnel_plain", 1, 0),
                                                         ("fresnel_tc_bf16x3", 1, oph.MODE_TENSOR_BF16X3)],
                                       max(3, args.steps // 2))
    more["box_8k"] = extra_workload_leg(ctx, W.box_8k(), [("rs_tc_bf16x3", 0, rs_mode)], 2)
    wrp = None
    if rank == 0:
        wrp = wrp_leg(ctx, max(3, args.steps // 2))
    codes_full = None
    if rank == 0:
        codes_full = full_field_codes(ctx, w, rs_mode)

    serving = None
    if world == 1:
        serving = serving_leg(args.serving_jobs, args.serving_max_points)
    plan_replay = plan_leg(ctx, sp)

    # --- end to end through the reference-facing API, host buffers ---------
    # What a reference caller runs (Example/examPointCloud/examPointCloud.cpp:
    # setPointCloudModel, generateHologram, encoding, normalize): the
    # ophPointCloud façade's C ABI, every buffer on the host. Each step copies
    # the vertices into the object and uploads them, downloads complex_H,
    # uploads it again for encoding (the caller may have edited it), downloads
    # m_lpEncoded, uploads it for normalize and downloads m_lpNormalized.
    e2e = facade_e2e(w, rs_mode | oph.MODE_GPU, max(3, args.steps // 2))
    e2e_value = job_value(inter, world, max_over_ranks(e2e["s_per_step"], dist, "cuda"))
    # ophpc_generate_host alone (host vertices in, host complex_H out): the
    # genCghPointCloudGPU equivalent, without encoding
    gh = generate_host_e2e(ctx, w, cfg, rs_mode, max(3, args.steps // 2))

    # --- the encoders on the device-resident sphere_fhd field (the last RS
    # generate above): FP64 phase values (m_lpEncoded), normalize of those
    # values into codes, and the codes-only phase path; L2 flushed between
    # calls
    import ctypes
    lib.ophpc_normalize.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64,
                                    ctypes.c_void_p, ctypes.c_void_p]
    lib.ophpc_normalize.restype = ctypes.c_int
    enc_vals = torch.empty((nch, npx), dtype=torch.float64, device="cuda")

    def normalize_call():
        if lib.ophpc_normalize(ctx._h, enc_vals.data_ptr(), nch, npx, codes.data_ptr(), sp) != 0:
            raise RuntimeError("ophpc_normalize failed")

    encoders = {}
    for name, fn in (
            ("phase_values", lambda: ctx.encode(field.data_ptr(), nch, npx, oph.ENCODE_PHASE, enc_vals.data_ptr(),
                                                None, sp)),
            ("normalize", normalize_call),
            ("phase_codes_only", lambda: ctx.encode(field.data_ptr(), nch, npx, oph.ENCODE_PHASE, None,
                                                    codes.data_ptr(), sp)),
            ("amplitude_values", lambda: ctx.encode(field.data_ptr(), nch, npx, oph.ENCODE_AMPLITUDE,
                                                    enc_vals.data_ptr(), None, sp)),
            ("ssb", lambda: ctx.encode_ssb(field.data_ptr(), nch, pnx, pny, w.pp, w.pp, oph.ENCODE_SSB, 0,
                                           (0.0, 0.5), enc_vals.data_ptr(), codes.data_ptr(), sp)),
            ("off_axis_ssb", lambda: ctx.encode_ssb(field.data_ptr(), nch, pnx, pny, w.pp, w.pp, oph.ENCODE_OFFSSB,
                                                    oph.SSB_LEFT, (0.0, 0.5), enc_vals.data_ptr(), codes.data_ptr(),
                                                    sp)),
            ("sideband", lambda: ctx.encode_sideband(field.data_ptr(), nch, pnx, pny, w.pp, w.pp, oph.SSB_TOP,
                                                     enc_vals.data_ptr(), codes.data_ptr(), sp))):
        fn()
        ts = timed(fn, 10)
        encoders[name] = {"ms": 1e3 * sum(ts) / len(ts)}
    encoders["pixels"] = nch * npx
    encoders["note"] = ("phase_values: FP64 (atan2(im, re) + pi) / (2 pi) per pixel, 16 B read and 8 B written; "
                        "normalize: min/max and codes of 8 B values; phase_codes_only: the single-pass FP32-estimate "
                        "codes kernel; ssb (encodeHologram, two shifted FP64 transforms per channel), off_axis_ssb "
                        "(SSB_LEFT: four transforms of channel 0) and sideband (SSB_TOP: one transform per channel), "
                        "each with its 8-bit codes")

    clocks = clk.summary()
    sm_mhz = clocks["sm_mhz"] or 1995.0
    props = torch.cuda.get_device_properties(local)
    sms = props.multi_processor_count
    # plain RS, SFU roofline: every interaction needs one sin and one cos
    # (2 MUFU ops); 16 MUFU results per clock per SM.
    peak_rs = sms * 16 / 2 * sm_mhz * 1e6
    achieved_rs = inter / t_rs
    # tensor-core RS, tensor roofline: per interaction four complex MACs
    # (split-BF16 hi*hi, hi*lo, lo*hi and the FP16 cross pair) = 32 real
    # flops executed, of which one complex MAC (8 flops) is the useful work
    peaks = measured_peaks()
    peak_tensor = peaks.get("bf16_tflops", 1900.0) * 1e12
    achieved_tc = inter * 32 / t_tc

    line = None
    if rank == 0:
        cpu = None
        rel = None
        rel_fp64 = {}
        # cpu_baseline leg: the CPU point-cloud path on a bounded sample of
        # the same workload, and the GPU result on that sample checked
        # against it (relative L2 error, FP64 CPU result as reference).
        n_cpu = args.cpu_points or 300
        rate, secs, kind, ref_field = cpu_sample_run(w, n_cpu, 0)
        sub = w.subset(n_cpu)
        dsub = torch.from_numpy(sub.vertices).cuda()
        fsub = torch.empty_like(field)
        ctx.generate(cfg, dsub.data_ptr(), sub.n_points, oph.DIFF_RS, rs_mode, fsub.data_ptr(), sp)
        torch.cuda.synchronize()
        g = fsub.cpu().numpy()
        got = g[..., 0] + 1j * g[..., 1]
        rel = float(np.linalg.norm(got - ref_field) / np.linalg.norm(ref_field))
        # every Fresnel variant against the FP64 CPU field on a smaller sample
        n_fr = max(50, n_cpu // 3)
        _, _, _, ref_fr = cpu_sample_run(w, n_fr, 1)
        subf = w.subset(n_fr)
        dsubf = torch.from_numpy(subf.vertices).cuda()
        for name, mode in (("fresnel_plain", 0), ("fresnel_tc_fp16", oph.MODE_TENSOR_FP16),
                           ("fresnel_tc_bf16x3", oph.MODE_TENSOR_BF16X3)):
            ctx.generate(cfg, dsubf.data_ptr(), subf.n_points, oph.DIFF_FRESNEL, mode, fsub.data_ptr(), sp)
            torch.cuda.synchronize()
            g = fsub.cpu().numpy()
            got = g[..., 0] + 1j * g[..., 1]
            rel_fp64[name] = float(np.linalg.norm(got - ref_fr) / np.linalg.norm(ref_fr))
        rel_fp64["rs_tc_bf16x3"] = rel
        ctx.generate(cfg, dsub.data_ptr(), sub.n_points, oph.DIFF_RS, 0, fsub.data_ptr(), sp)
        torch.cuda.synchronize()
        g = fsub.cpu().numpy()
        rel_fp64["rs_plain"] = float(np.linalg.norm(g[..., 0] + 1j * g[..., 1] - ref_field) /
                                     np.linalg.norm(ref_field))
        rel_fp64["samples"] = f"RS {n_cpu} points, Fresnel {n_fr} points, full {w.pnx}x{w.pny}x{w.n_channels}"
        # all points at seeded pixels: the error at the workload's full
        # size (it grows with the point count: part of it is common to
        # every point's phase)
        import oracle
        gw = oracle.Geometry(pnx=w.pnx, pny=w.pny, ppx=w.pp, ppy=w.pp, wavelengths=list(w.wavelengths),
                             scale=w.scale, distance=w.distance)
        pix = np.sort(np.random.default_rng(17).choice(npx, 256, replace=False))
        full, wants = {}, {}
        for name, diff, mode in (("rs_tc_bf16x3", 0, rs_mode), ("rs_plain", 0, 0), ("fresnel_plain", 1, 0),
                                 ("fresnel_tc_bf16x3", 1, oph.MODE_TENSOR_BF16X3),
                                 ("fresnel_tc_fp16", 1, oph.MODE_TENSOR_FP16)):
            ctx.generate(cfg, dv.data_ptr(), w.n_points, diff, mode, fsub.data_ptr(), sp)
            torch.cuda.synchronize()
            g = fsub.reshape(nch, npx, 2)[:, torch.from_numpy(pix).cuda()].cpu().numpy()
            got = g[..., 0] + 1j * g[..., 1]
            if diff not in wants:
                wants[diff] = np.stack([oracle.field_at(gw, w.vertices, diff, c, pix) for c in range(nch)])
            want = wants[diff]
            full[name] = float(np.linalg.norm(got - want) / np.linalg.norm(want))
        full["samples"] = f"all {w.n_points} points at 256 seeded pixels per channel"
        rel_fp64["full_size"] = full
        cpu = {"value": rate, "unit": UNIT, "cores": host_cores(), "kind": kind,
               "sample": f"{n_cpu} of {w.n_points} points at full {w.pnx}x{w.pny}, {w.n_channels} channels, RS "
                         f"({secs:.1f} s, OpenMP, {cpu_model()})",
               "relL2_gpu_vs_cpu_on_sample": rel}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "bf16x3+fp16 (tcgen05 split-BF16 hi*hi+hi*lo+lo*hi and an FP16 cross pair, FP32 "
                     "accumulation; FP64 phase reduction and FP64 field)", "data": "synthetic",
            "config": {"workload": w.name, "pnx": pnx, "pny": pny, "pixel_pitch_m": w.pp,
                       "wavelengths_m": list(w.wavelengths), "n_points": w.n_points, "diff": "RS",
                       "step": "generateHologram(RS, 3 channels; tensor-core RS, split-BF16) + phase encode + "
                               "normalise",
                       "l2": "flushed (256 MB write) between timed steps", "parallelism": f"replicas x{world}"},
            "relL2": rel,
            "relL2_vs_fp64": rel_fp64 or None,
            "roofline": {"bound": "tensor", "kernel": "tc_rs_kernel", "achieved": achieved_tc / 1e12,
                         "peak": peak_tensor / 1e12, "unit": "TFLOP/s", "frac": achieved_tc / peak_tensor,
                         "traffic": TCRS_TRAFFIC_BYTES.get(w.name), "traffic_unit": "bytes per launch (DRAM)",
                         "algorithmic_flops": inter * 32, "useful_flops": inter * 8,
                         "useful_frac": achieved_tc / 4 / peak_tensor,
                         "peak_basis": "MEASURED_PEAKS.json bf16_tflops (cuBLAS bf16 GEMM, burst): of measured",
                         "flops_basis": "32 executed flops per point x pixel interaction (four complex MACs: "
                                        "split-BF16 hi*hi, hi*lo, lo*hi, FP16 cross pair); 8 useful"},
            "rs_plain": {"value": job_value(inter, world, t_rs), "unit": UNIT, "ms_per_generate": t_rs * 1e3,
                         "kernel": "rs_kernel (FP32 cores + MUFU)",
                         "speedup_of_tensor_core_rs": t_rs / t_tc,
                         "roofline": {"bound": "sfu", "achieved": achieved_rs, "peak": peak_rs,
                                      "unit": "interactions/s", "frac": achieved_rs / peak_rs,
                                      "traffic": RS_TRAFFIC_BYTES.get(w.name),
                                      "traffic_unit": "bytes per launch (DRAM)",
                                      "algorithmic_bytes": w.n_points * nch * 64 + npx * nch * 16,
                                      "peak_basis": f"{sms} SMs x 16 MUFU/clk / 2 MUFU (sin, cos) per "
                                                    f"interaction x {sm_mhz:.0f} MHz median SM clock under load"}},
            "fresnel": {"value": job_value(inter, world, t_fr), "unit": UNIT, "ms_per_generate": t_fr * 1e3,
                        "kernel": "fresnel_kernel (FP32 cores, separable)"},
            "tensor_fresnel": tensor,
            "rs_1k": more.get("rs_1k"),
            "box_8k": more.get("box_8k"),
            "wrp": wrp,
            "codes_vs_reference": codes_full,
            "codes_exact_frac": (codes_full or {}).get("phase", {}).get("codes_exact_frac"),
            "codes_max_lsb": (codes_full or {}).get("phase", {}).get("codes_max_lsb"),
            "serving": serving,
            "plan_replay": plan_replay,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": e2e["h2d"],
                    "d2h_bytes_per_step": e2e["d2h"], "ms_per_step": e2e["s_per_step"] * 1e3,
                    "call": "ophPointCloud facade C ABI (ophpc_pc_set_point_cloud, ophpc_pc_generate_hologram, "
                            "ophpc_pc_encoding(PHASE), ophpc_pc_normalize): host Vertex[] in, host complex_H, "
                            "m_lpEncoded and m_lpNormalized out; wall clock around the synchronous calls",
                    "generate_s_reported": e2e["generate_s"], "calls_ms_median": e2e["calls_ms_median"]},
            "e2e_generate_host": gh,
            "encoders": encoders,
            "gpu_launches": int(launches),
            "clocks": {"sm_mhz": clocks["sm_mhz"], "sm_max_mhz": clocks["sm_max_mhz"],
                       "reasons": clocks["reasons"], "samples": clocks["samples"]},
            "wall_s_timed_region": wall,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    ctx.close()
    return line


def measured_peaks() -> dict:
    """MEASURED_PEAKS.json (HBM copy and cuBLAS bf16 throughput measured on
    this GPU pool), or {} when absent."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


# dram__bytes_read.sum + dram__bytes_write.sum of one tc_rs_kernel launch of
# the workload's tensor-core RS generate, from a 1-pass ncu capture of
# `bench.py --profile-case tcrs_fhd_full` (profiles/tc_tile_kernels_sphere_fhd_dram.md).
TCRS_TRAFFIC_BYTES = {"sphere_fhd": 21014784 + 83691008}


# dram__bytes_read.sum + dram__bytes_write.sum of one rs_kernel launch of the
# workload's RS generate, from a 1-pass ncu capture of
# `bench.py --profile-case rs_fhd` (profiles/rs_kernel_sphere_fhd_dram.md).
RS_TRAFFIC_BYTES = {"sphere_fhd": 27.46e6 + 151.67e6}


def profile_case(name: str) -> None:
    """One call of one path on a small fixed case (for ncu captures): no
    timing, no CPU work, a few GB of device memory at most."""
    import torch

    import openholo_gb300 as oph
    from openholo_gb300 import workloads
    if name in ("rs_1k", "fresnel_1k"):
        w, diff, mode = workloads.rs_1k(), (0 if name == "rs_1k" else 1), 0
    elif name == "rs_fhd":   # the headline step's generate: ~110 MB on the device
        w, diff, mode = workloads.sphere_fhd(), 0, 0
    elif name in ("tc_fp16_4k", "tc_bf16x3_4k"):
        w = workloads.box_4k(n_points=131_072)
        diff = 1
        mode = oph.MODE_TENSOR_FP16 if name == "tc_fp16_4k" else oph.MODE_TENSOR_BF16X3
    elif name == "tcrs_fhd":   # tensor-core RS, sphere_fhd geometry, 20,000 of its points
        w, diff, mode = workloads.sphere_fhd().subset(20_000), 0, oph.MODE_TENSOR_BF16X3
    elif name == "tcrs_fhd_full":   # the headline step's tensor-core RS generate (~110 MB on the device)
        w, diff, mode = workloads.sphere_fhd(), 0, oph.MODE_TENSOR_BF16X3
    elif name in ("step_fhd", "codes_fhd"):   # tensor-core RS generate + phase codes, sphere_fhd
        w, diff, mode = workloads.sphere_fhd(), 0, oph.MODE_TENSOR_BF16X3
    elif name == "tcf_fhd_full":    # tensor-core Fresnel (on-chip factors), sphere_fhd, all points
        w, diff, mode = workloads.sphere_fhd(), 1, oph.MODE_TENSOR_BF16X3
    elif name == "tcf_4k":          # tensor-core Fresnel (on-chip factors), box_4k geometry, 131,072 points
        w, diff, mode = workloads.box_4k(n_points=131_072), 1, oph.MODE_TENSOR_BF16X3
    elif name == "values_fhd":      # FP64 phase values of the sphere_fhd field, then normalize of them
        w, diff, mode = workloads.sphere_fhd(), 0, oph.MODE_TENSOR_BF16X3
    elif name == "wrp_fhd":         # WRP generator, sphere_fhd points, WRP 1 mm in front, 0.5 m propagation
        w = workloads.sphere_fhd()
        ctx = oph.Context(0)
        wcfg = oph.make_wrp_config(pnx=w.pnx, pny=w.pny, ppx=w.pp, ppy=w.pp, wavelengths=list(w.wavelengths),
                                   wrp_location=float(w.vertices[:, 2].max()) + 1e-3, distance=0.5)
        dv = torch.from_numpy(w.vertices).cuda()
        f = torch.empty((w.n_channels, w.pny, w.pnx, 2), dtype=torch.float64, device="cuda")
        for _ in range(2):
            ctx.wrp_generate(wcfg, dv.data_ptr(), w.n_points, f.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        print(f"profile case {name}: done")
        return
    else:
        raise SystemExit(f"unknown profile case {name}")
    ctx = oph.Context(0)
    cfg = oph.make_config(**w.geometry_kwargs())
    dv = torch.from_numpy(w.vertices).cuda()
    f = torch.empty((w.n_channels, w.pny, w.pnx, 2), dtype=torch.float64, device="cuda")
    codes = torch.empty((w.n_channels, w.pny * w.pnx), dtype=torch.uint8, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    npx = w.pny * w.pnx
    for it in range(2):
        if name not in ("codes_fhd", "values_fhd") or it == 0:
            ctx.generate(cfg, dv.data_ptr(), w.n_points, diff, mode, f.data_ptr(), sp)
        if name in ("step_fhd", "codes_fhd"):
            ctx.encode(f.data_ptr(), w.n_channels, npx, oph.ENCODE_PHASE, None, codes.data_ptr(), sp)
        if name == "values_fhd":
            import ctypes
            lib = oph.lib()
            lib.ophpc_normalize.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64,
                                            ctypes.c_void_p, ctypes.c_void_p]
            lib.ophpc_normalize.restype = ctypes.c_int
            vals = torch.empty((w.n_channels, npx), dtype=torch.float64, device="cuda")
            ctx.encode(f.data_ptr(), w.n_channels, npx, oph.ENCODE_PHASE, vals.data_ptr(), None, sp)
            if lib.ophpc_normalize(ctx._h, vals.data_ptr(), w.n_channels, npx, codes.data_ptr(), sp) != 0:
                raise RuntimeError("ophpc_normalize failed")
    torch.cuda.synchronize()
    print(f"profile case {name}: done")


def main():
    args = parse()
    if args.profile_case:
        profile_case(args.profile_case)
        return
    from openholo_gb300 import workloads
    w = workloads.BY_NAME[args.workload]()
    if args.impl == "reference":
        reference_arm(args, w)
    else:
        gpu_arm(args, w)


if __name__ == "__main__":
    main()
