"""Benchmark: pixel-iterations/s of the perturbation method at 2^-1000 zoom.

Workload (one step = one full frame): 1920x1080 pixels, real-axis width
2^-1000 around a 1088-bit centre found by seeded ray bisection
(tests/golden/views.json "c4"), maxiter 200000, Mandelbrot.  A step renders
the reference orbit on the GPU and every pixel of the frame.

Lines printed (rank 0, one JSON line):
  value     whole-job pixel-iterations/s with inputs resident on the device
            (device output buffer), summed over ranks / max step time;
  e2e       the same metric through the public C ABI call with host output
            buffers (host->device inputs and device->host counts in the
            timed region);
  plain_mp  the plain multi-limb kernel on a band of the same frame (the
            "perturbation vs plain MP on GPU" half of the metric);
  roofline  the perturbation kernel against the measured FP32 pipe peak;
  cpu_baseline  the oracle's MPFR loop (the reference's deep-zoom path at
            1088 bits) on a bounded pixel sample, all host threads;
  plain_configs  config 2 (FP64) and config 3 (multi-limb) frames, each
            beside the reference CPU loop on a band of rows;
  serving   the seeded mixed request stream (mdz_gb300.stream) through the
            serving engine: capacity (closed loop) and p50/p99 latency under
            Poisson arrivals at 80% of that capacity (rank 0).
--impl reference times that CPU path alone on the same metric.

Multi-GPU: pixels are independent; every rank renders its own frame (weak
scaling, no collective on the data path), rank 0 reports the sum.
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
from fractions import Fraction
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

VIEWS = json.loads((ROOT / "tests" / "golden" / "views.json").read_text())
# FP32 operations (flops) of one perturbation step: complex 2 Z dz (4 mul +
# 2 add), dz^2 (3 mul + 2 add), two adds of dc, |z|^2 (2) and its compare.
# At 2^-1000 the dz^2 terms vanish exactly and the step executes as 4 FFMA
# (8 flops); the roofline counts the algorithmic 16 against the FP32 flop
# peak (2 flops per FFMA lane).
ALGO_OPS_PER_PIXEL_ITER = 16
# DRAM bytes (read + written) of one perturb_step_kernel launch of the
# 1920x1080 2^-1000 frame: ncu dram__bytes_read.sum + dram__bytes_write.sum
# (one pass, --clock-control none) over launches 61-63 of one frame, 74.7 MB
# read and 11.6-14.6 MB written each (profiles/perturb_step_kernel_c4_traffic.md).
# The pixel state (32 B per unfinished pixel) goes in and out once a launch;
# the reference orbit (3.2 MB of float4 entries) is read from L2.
STEP_LAUNCH_DRAM_BYTES = 87.6e6
# rows of the frame rendered by the plain multi-limb kernel: 1920 x 64 pixels
# = 3840 warps of 8x4-pixel tiles, about three full waves of the resident
# warps at 34 words (240 registers: 8 warps per SM x 152 SMs)
PLAIN_BAND_ROWS = 64


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="c4")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=200,
                    help="requests of the seeded mixed stream for the serving latency run "
                         "(0 = skip)")
    ap.add_argument("--serve-capacity-requests", type=int, default=32,
                    help="first requests of the stream run closed loop to measure capacity")
    ap.add_argument("--serve-seed", type=int, default=5005)
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the config 2 (FP64) and config 3 (multi-limb) frames")
    ap.add_argument("--serve-load", type=float, default=0.8)
    ap.add_argument("--frame", default=None,
                    help="WxH override of the frame size (same centre, pixel spacing scaled) "
                         "for small profiling cases")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = max(smax, float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def c4_values(view):
    from mdz_gb300 import MpVal, parse_number
    prec = int(view["precision"])
    cx = MpVal.from_fraction(parse_number(view["cx"]), prec)
    cy = MpVal.from_fraction(parse_number(view["cy"]), prec)
    width = MpVal.from_fraction(parse_number(view["size"]), prec)
    return cx, cy, width, prec


def workload_config(view, world: int) -> dict:
    """The `config` object both arms print (identical, so the two lines
    describe the same workload)."""
    return {"workload": f"c4: {view['width']}x{view['height']}, width 2^-1000, "
                        f"{view['precision']}-bit centre (seeded ray bisection), "
                        f"maxiter {view['depth']}, Mandelbrot",
            "l2": "flushed between steps (256 MB write)",
            "parallelism": f"replicas x{world}"}


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x: float, op="max") -> float:
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def cpu_baseline(view, seconds: float) -> dict:
    """The reference's deep-zoom path (per-pixel MPFR loop at the view's
    precision, src/frac_mandel.c:25-52) on a bounded sample of the frame's
    pixels, all host threads.  Returns pixel-iterations/s."""
    from mdz_gb300 import perturb_pixel_c
    from mdz_gb300.mpval import hexfloat
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    if not O.has_mpfr():
        return {"value": None, "unit": "pixel-iters/s", "cores": threads, "kind": "port",
                "sample": "unavailable: libmpfr.so.6 not found on this host"}
    cx, cy, width, prec = c4_values(view)
    W, H, depth = view["width"], view["height"], view["depth"]
    rng = np.random.default_rng(44)
    done_its, elapsed, n_done = 0, 0.0, 0
    batch = max(threads, 8)
    while elapsed < seconds and n_done < 4096:
        ix = rng.integers(0, W, batch)
        ln = rng.integers(0, H, batch)
        cs = [perturb_pixel_c(cx, cy, width, W, H, int(a), int(b)) for a, b in zip(ix, ln)]
        t0 = time.perf_counter()
        counts, _ = O.points_mpfr([hexfloat(c[0]) for c in cs], [hexfloat(c[1]) for c in cs],
                                  depth, prec, threads=threads)
        elapsed += time.perf_counter() - t0
        done_its += int(np.where(counts == 0, depth, counts).sum())
        n_done += batch
    return {"value": done_its / elapsed, "unit": "pixel-iters/s", "cores": threads,
            "kind": "port",
            "sample": f"{n_done} random pixels of the frame, MPFR {prec}-bit loop to depth "
                      f"{depth}, {elapsed:.1f}s"}


def run_reference(args, view, world, rank, dist):
    if rank != 0:
        return
    base = cpu_baseline(view, args.cpu_seconds)
    vals = []
    for _ in range(args.steps):
        b = cpu_baseline(view, max(2.0, args.cpu_seconds / max(1, args.steps)))
        vals.append(b["value"])
    value = statistics.median(vals) if vals and vals[0] else None
    line = {"metric": "pixel-iters/s at 2^-1000 zoom", "impl": "reference", "value": value,
            "unit": "pixel-iters/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": f"mpfr-{view['precision']}", "data": "synthetic",
            "config": workload_config(view, world),
            "path": "the reference's per-pixel MPFR loop (frac_mandel_mpfr) restated in "
                    "oracle/mdz_oracle.c, on host cores; each step a bounded random-pixel "
                    "sample of the frame",
            "cpu_baseline": dict(base, value=value),
            "e2e": {"value": value, "unit": "pixel-iters/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_plain_configs(args, local) -> dict:
    """The plain methods on their own configurations, each beside the
    reference's CPU loop (the oracle restatement, all host threads) on a band
    of rows of the same frame: config 2 (FP64, 1920x1080 with 3x3
    supersampling = 5760x3240 counts, maxiter 20000) and config 3 (multi-limb,
    640x480 at 256 bits, maxiter 50000).  GPU numbers are the whole frame
    through the public call with a host output buffer (counts copied back)."""
    from mdz_gb300 import Renderer
    from mdz_gb300.cases import view as case_view
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    out = {}
    with Renderer(local) as r:
        v = case_view("c2", None, aa=True)
        xmin, xmax, ymax = v.rect().doubles()
        W, H = v.real_width, v.real_height
        r.render_fp64(W, 64, v.depth, xmin, xmax, ymax)              # warm-up
        t0 = time.perf_counter()
        _, st = r.render_fp64(W, H, v.depth, xmin, xmax, ymax)
        wall = time.perf_counter() - t0
        gpu = st["pixel_iters"] / wall
        # CPU: rows from the middle of the frame, doubling until ~seconds
        rows, cpu_its, cpu_s = 8, 0, 0.0
        while cpu_s < args.cpu_seconds / 2 and rows <= H:
            row0 = H // 2 - rows // 2
            t0 = time.perf_counter()
            band = O.render_fp64_rows(W, H, row0, rows, v.depth, xmin, xmax, ymax,
                                      threads=threads)
            cpu_s = time.perf_counter() - t0
            cpu_its = int(np.where(band == 0, v.depth, band).sum())
            rows *= 2
        cpu = cpu_its / cpu_s
        out["c2_fp64"] = {"value": gpu, "unit": "pixel-iters/s", "frame": f"{W}x{H}",
                          "kernel_ms": st["kernel_ms"], "wall_ms": wall * 1e3,
                          "cpu_baseline": {"value": cpu, "cores": threads, "kind": "port",
                                           "sample": f"{rows // 2} middle rows, {cpu_s:.1f}s"},
                          "gpu_vs_cpu": gpu / cpu}
        v = case_view("c3", None, aa=False)
        rc = v.rect()
        W, H = v.real_width, v.real_height
        r.render_mp(W, 8, v.depth, rc.xmin, rc.ymax, rc.width, v.precision)   # warm-up
        t0 = time.perf_counter()
        _, st = r.render_mp(W, H, v.depth, rc.xmin, rc.ymax, rc.width, v.precision)
        wall = time.perf_counter() - t0
        gpu = st["pixel_iters"] / wall
        rows, cpu_its, cpu_s = 2, 0, 0.0
        if O.has_mpfr():
            while cpu_s < args.cpu_seconds / 2 and rows <= H:
                row0 = H // 2 - rows // 2
                t0 = time.perf_counter()
                _, cpu_its = O.render_mpfr(W, H, v.depth, v.precision, rc.xmin, rc.ymax,
                                           rc.width, row0=row0, nrows=rows, threads=threads)
                cpu_s = time.perf_counter() - t0
                rows *= 2
        cpu = cpu_its / cpu_s if cpu_s else None
        out["c3_multi_limb"] = {"value": gpu, "unit": "pixel-iters/s", "frame": f"{W}x{H}",
                                "words": st["words"], "kernel_ms": st["kernel_ms"],
                                "wall_ms": wall * 1e3,
                                "cpu_baseline": {"value": cpu, "cores": threads, "kind": "port",
                                                 "sample": f"{rows // 2} middle rows, MPFR "
                                                           f"{v.precision}-bit, {cpu_s:.1f}s"},
                                "gpu_vs_cpu": (gpu / cpu) if cpu else None}
    return out


def latency_summary(lat: np.ndarray) -> dict:
    def pct(q):
        return float(np.percentile(lat, q, method="inverted_cdf"))
    return {"n": int(lat.size), "p50": pct(50), "p90": pct(90), "p99": pct(99),
            "max": float(lat.max()), "mean": float(lat.mean())}


def tail_phases(sts: list, lat: np.ndarray) -> dict:
    """Where the slowest tenth of the requests spent their time: submission
    to the end of the main pass, waiting for the escalation passes, and in
    them (means, ms), with their flagged pixel counts."""
    cut = float(np.percentile(lat, 90, method="inverted_cdf"))
    sel = [s for s, x in zip(sts, lat) if x >= cut]
    def mean(k):
        return float(np.mean([s[k] for s in sel])) if sel else None
    return {"from_ms": cut, "n": len(sel), "main_ms": mean("main_ms"),
            "esc_wait_ms": mean("esc_wait_ms"), "esc_ms": mean("esc_ms"),
            "escalated_fp64": mean("escalated_fp64"), "escalated_mp": mean("escalated_mp"),
            "with_escalation": sum(1 for s in sel if s["escalated_fp64"] > 0)}


def run_serving(args, local) -> dict:
    """The mixed request stream through the serving engine: the first
    `serve_capacity_requests` requests closed loop (all submitted at once)
    measure the capacity; then `serve_requests` requests arrive as a Poisson
    process at `serve_load` of that capacity, for p50/p90/p99 latency (also
    per image size and per method).  Every request of the closed-loop run
    must equal its result in the Poisson run (each request the same alone or
    in any mix).  The engine's own log gives the device time of the steps
    against their host wall time (the share the step loop and its graph
    launches add)."""
    import tempfile
    from mdz_gb300.serve import Server
    from mdz_gb300.stream import load_pool, make_stream
    pool = load_pool()
    items = make_stream(max(args.serve_requests, args.serve_capacity_requests), pool,
                        seed=args.serve_seed)

    def run(sel, arrivals):
        reqs = [items[i].request(pool) for i in sel]
        with tempfile.NamedTemporaryFile(suffix=".json", delete=False) as tf:
            log_path = tf.name
        with Server(local, arena_bytes=48 << 30, staging_bytes=2 << 30,
                    queue_pixels=1 << 25, log_path=log_path) as srv:
            t0 = time.perf_counter()
            ids = []
            for a, rq in zip(arrivals, reqs):
                dt = t0 + a - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                ids.append(srv.submit(rq))
            sts = [srv.wait(i, 1_800_000) for i in ids]
            wall = time.perf_counter() - t0
            stats = srv.stats()
        try:
            engine = json.loads(Path(log_path).read_text().strip().splitlines()[-1])
        except (OSError, ValueError, IndexError):
            engine = {}
        Path(log_path).unlink(missing_ok=True)
        return reqs, sts, wall, stats, engine

    ncap = min(args.serve_capacity_requests, len(items))
    reqs1, sts1, wall1, stats1, _ = run(range(ncap), [0.0] * ncap)
    its = sum(s["pixel_iters"] for s in sts1)
    rate = args.serve_load * ncap / wall1
    n = args.serve_requests
    gaps = np.array([it.gap for it in items[:n]]) / rate
    arrivals = np.cumsum(gaps) - gaps[0]
    reqs2, sts2, wall2, stats2, engine = run(range(n), list(arrivals))
    same = all(np.array_equal(a.counts, b.counts) for a, b in zip(reqs1, reqs2[:ncap]))
    lat = np.array([s["latency_ms"] for s in sts2])
    ok = all(s["state"] == "done" for s in sts1 + sts2)
    sizes = np.array([f"{it.width}x{it.height}" for it in items[:n]])
    meth = np.array(["perturbation" if s["method"] == 1 else "multi_limb" for s in sts2])
    busy = stats2["busy_ms"]
    dev = engine.get("device_step_ms")
    return {
        "requests": n, "seed": args.serve_seed, "all_done": ok,
        "stream": "sizes {240x180..1920x1080}, log2 span U[-1000,-10], prec ceil(-log2 span)+64, "
                  "mandelbrot/burning ship/celtic 0.7/0.2/0.1, maxiter log-U[1e3,1e5]",
        "capacity": {"requests": ncap, "run_s": wall1,
                     "throughput": {"value": its / wall1, "unit": "pixel-iters/s"},
                     "note": "closed loop, all requests submitted at once, through the public "
                             "submit/wait API with host result buffers"},
        "poisson_rate_per_s": rate, "load": args.serve_load, "poisson_run_s": wall2,
        "latency_ms": latency_summary(lat),
        "latency_ms_by_size": {k: latency_summary(lat[sizes == k]) for k in sorted(set(sizes))},
        "latency_ms_by_method": {k: latency_summary(lat[meth == k]) for k in sorted(set(meth))},
        "latency_tail": tail_phases(sts2, lat),
        "results_equal_across_runs": same,
        "steps": stats2["steps"], "gpu_launches": stats2["launches"],
        "step_loop": {"host_ms": busy, "device_ms": dev,
                      "host_share_above_device": (1.0 - dev / busy) if dev and busy else None,
                      "graph_launch_ms": engine.get("loop_ms", {}).get("graph_launch"),
                      "step_gap_ms": engine.get("step_gap_ms"),
                      "fixed_overhead_share": (engine["step_gap_ms"]["p10"] * stats2["steps"] / dev)
                      if dev and engine.get("step_gap_ms") else None,
                      "note": "per step, host wall (graph launch to sync) minus the step's device "
                              "span; its 10th percentile (steps not held up behind other "
                              "kernels) times the step count, over the device time, is the fixed "
                              "launch-and-sync overhead"},
        "device_bytes_peak": stats2["device_bytes_peak"],
    }


def run_ours(args, view, world, rank, local, dist):
    import torch
    from mdz_gb300 import Renderer, native
    lib = native.load()
    import ctypes as C
    cx, cy, width, prec = c4_values(view)
    W, H, depth = view["width"], view["height"], view["depth"]
    r = Renderer(local)
    torch.cuda.set_device(local)
    d_counts = torch.empty((H, W), dtype=torch.int32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")   # > 129 MB L2

    def step_device():
        return r.render_perturb_device(W, H, depth, cx, cy, width, prec, d_counts.data_ptr())

    for _ in range(args.warmup):
        step_device()
    # measured FP32 pipe peak (roofline denominator)
    peak = C.c_double()
    lib.mdzgpu_measure_peak(local, 0, C.byref(peak))
    torch.cuda.synchronize()
    barrier(dist)
    kernel_ms, orbit_ms, pixel_ms, its, rebases, wall = [], [], [], 0, 0, []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st = step_device()
            wall.append((time.perf_counter() - t0) * 1e3)
            kernel_ms.append(st["kernel_ms"])
            orbit_ms.append(st["orbit_ms"])
            pixel_ms.append(st["pixel_ms"])
            pixel_launches = st["pixel_launches"]
            its += st["pixel_iters"]
            rebases += st["rebases"]
            launches = st["launches"]
            orbit_len = st["orbit_len"]
    torch.cuda.synchronize()
    barrier(dist)
    total_ms = sum(kernel_ms)
    total_ms_max = max_over_ranks(dist, total_ms)
    its_all = max_over_ranks(dist, float(its), op="sum")
    value = its_all / (total_ms_max * 1e-3)

    # e2e: the public C ABI with host buffers
    host = np.empty((H, W), np.int32)
    e2e_ms, e2e_its, h2d, d2h = [], 0, 0, 0
    barrier(dist)
    for _ in range(args.steps):
        flush.fill_(2)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, _, st = r.render_perturb(W, H, depth, cx, cy, width, prec, out=host)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        e2e_its += st["pixel_iters"]
        h2d, d2h = st["h2d_bytes"], st["d2h_bytes"]
    e2e_max = max_over_ranks(dist, sum(e2e_ms))
    e2e_its_all = max_over_ranks(dist, float(e2e_its), op="sum")

    # plain multi-limb kernel on a band of the same frame (same precision)
    plain = None
    if not args.no_plain:
        from mdz_gb300 import MpVal
        hs = Fraction(width.to_fraction()) / W
        band = PLAIN_BAND_ROWS
        y0 = H // 2 - band // 2
        xmin = MpVal.from_fraction(cx.to_fraction() - W * hs / 2, prec + 64)
        ymax = MpVal.from_fraction(cy.to_fraction() + (H / 2 - y0) * hs, prec + 64)
        wv = MpVal.from_fraction(width.to_fraction(), prec + 64)
        _, pst = r.render_mp(W, band, depth, xmin, ymax, wv, prec, words=34)
        plain = {"value": pst["pixel_iters"] / (pst["kernel_ms"] * 1e-3),
                 "unit": "pixel-iters/s", "words": pst["words"],
                 "sample": f"{W}x{band} band at the frame centre, 34x32-bit words"}

    if rank != 0:
        r.close()
        return
    ms_per_step = total_ms_max / args.steps
    # the dominant kernel is the FP32 pixel pass (perturb_step_kernel, one
    # launch per step of the frame): its device time is the sum of CUDA-event
    # intervals around each launch, on the stream it runs on
    avg_pixel_ms = sum(pixel_ms) / len(pixel_ms)
    achieved = (its / args.steps) * ALGO_OPS_PER_PIXEL_ITER / (avg_pixel_ms * 1e-3) / 1e9
    peak_gflops = 2.0 * peak.value / 1e9     # FFMA lane-instructions/s x 2 flops
    traffic_gbs = STEP_LAUNCH_DRAM_BYTES / (avg_pixel_ms / max(pixel_launches, 1) * 1e-3) / 1e9
    try:
        hbm_gbs = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("hbm_gbs")
    except (OSError, ValueError):
        hbm_gbs = None
    line = {
        "metric": "pixel-iters/s at 2^-1000 zoom", "value": value, "unit": "pixel-iters/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32+int32 floatexp (fp64 rebase)", "data": "synthetic",
        "config": workload_config(view, world),
        "method": {"name": "perturbation", "orbit_limbs": int(lib.mdzgpu_perturb_limbs(prec)),
                   "orbit_len": orbit_len},
        "gpu_launches": launches * args.steps,
        "orbit_ms": (sum(orbit_ms) / len(orbit_ms)) if min(orbit_ms) >= 0 else "fused",
        "rebases_per_step": rebases / args.steps,
        "e2e": {"value": e2e_its_all / (e2e_max * 1e-3), "unit": "pixel-iters/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "fp32-pipe", "kernel": "perturb_step_kernel",
                     "achieved": achieved, "peak": peak_gflops,
                     "unit": "GFLOP/s", "frac": achieved / peak_gflops,
                     "algorithmic_flops_per_pixel_iter": ALGO_OPS_PER_PIXEL_ITER,
                     "executed_frac": achieved * 8 / ALGO_OPS_PER_PIXEL_ITER / peak_gflops,
                     "peak_source": "mdzgpu_measure_peak FFMA microbenchmark (this run), "
                                    "2 flops per FFMA",
                     "pixel_pass_ms_per_step": avg_pixel_ms,
                     "pixel_pass_launches_per_step": pixel_launches,
                     "traffic": STEP_LAUNCH_DRAM_BYTES,
                     "traffic_unit": "bytes per launch (ncu dram__bytes_read+write)",
                     "traffic_gbs": traffic_gbs,
                     "traffic_frac_of_measured_hbm": (traffic_gbs / hbm_gbs) if hbm_gbs else None},
        "clocks": clocks.summary(),
        "plain_mp": plain,
        "perturb_vs_plain": (value / world / plain["value"]) if plain else None,
    }
    r.close()
    if not args.no_configs:
        line["plain_configs"] = run_plain_configs(args, local)
    if args.serve_requests > 0:
        line["serving"] = run_serving(args, local)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(view, args.cpu_seconds)
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    view = dict(VIEWS[args.workload])
    if args.frame:
        from fractions import Fraction
        from mdz_gb300 import parse_number
        from mdz_gb300.mpval import hexfloat
        w, h = (int(x) for x in args.frame.lower().split("x"))
        # keep the pixel spacing: a crop around the centre
        view["size"] = hexfloat(parse_number(view["size"]) * Fraction(w, view["width"]))
        view["width"], view["height"] = w, h
    world, rank, local, dist = dist_init(args)
    try:
        if args.impl == "reference":
            run_reference(args, view, world, rank, dist)
        else:
            run_ours(args, view, world, rank, local, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
