"""Benchmark of the GB300 BIRP render path.

Workload (default): 512 renders of a 256^3 stretched-axis FP32 cube (x in
[-40, 30], y, z in [-40, 40] Re, trilinear, PREFIX march), poses on the
SMILE-like orbit aimed at (9, 0, 0), image sizes from {144x84, 288x168,
576x336, 1024x600} and steps from {0.025, 0.05, 0.1} Re, seeded. One step =
one pass over all 512 requests.

  value      images/s of the batched path (one persistent-kernel launch from a
             CUDA graph), device time, inputs resident, L2 flushed between steps
  e2e        the same through the C ABI birp_batch_render with HOST output
             buffers (descriptor H2D + image D2H + copies to the caller inside)
  plain      images/s of the one-render-per-call path (birp_render, host output)
  serving    p50/p99 latency of the continuous-batching server at 70% of the
             saturated rate (Poisson arrivals)
  roofline   the batched kernel against the slower of its FP32 work and its
             gathered bytes at the L2 read rate, both peaks measured in-run;
             roofline_issue: its warp instructions (per cell segment, from the
             committed ncu capture) against the SM issue rate at the sampled
             clock, the bound it actually runs into
  cpu_baseline  the reference's FP32 render arithmetic (oracle port) on all
             host cores over a bounded random pixel sample of the same
             workload, and on one core

`--impl reference` times only that CPU implementation (bounded samples).
Multi-GPU (torchrun): replicas, one per rank, barrier + max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "images/s & p99 latency: batched/served vs plain GPU render at ≤1e-5 rel err"
UNIT = "images/s"
# Per trilinear ray-sample (the reference's formulation): 8 FP32 corners
# gathered, 6 position + 6 index + 3 fraction + 21 lerp + 4 Kahan flops.
FLOP_PER_SAMPLE = 40.0
BYTES_PER_SAMPLE = 32.0
# Per cell segment (what the kernel does: the samples inside one cell summed
# in closed form): one 32-byte coefficient record + one 8-byte walk-table
# entry for the face crossed into the cell; 65 FP32 operations for the run
# end, the closed-form sum and the Kahan update (FMA = 2) plus 3 for the new
# base offset and exit index of the crossed axis.
FLOP_PER_CELL = 68.0
BYTES_PER_CELL = 40.0


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(world, x: float) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- workload

def make_workload(B, n_req: int, seed_cube: int = 1, seed_req: int = 2):
    from birp_cpp_gb300 import synth
    xs, ys, zs, v64 = synth.cube_config1(seed=seed_cube)
    v32 = v64.astype(np.float32)
    cube = B.Cube(xs, ys, zs, v32)
    reqs = synth.config2_requests(n_req, seed=seed_req)
    cams = [B.camera(pos, aim, synth.FOV_W, synth.FOV_H, nx, ny, n_samples=synth.n_samples(step),
                     ray_length=synth.RAY_LENGTH, trilinear=True) for pos, aim, nx, ny, step in reqs]
    return dict(cube=cube, cams=cams, reqs=reqs, host=(xs, ys, zs, v32))


def _gen_cube(spec):
    from birp_cpp_gb300 import synth
    nx, ny, nz, r0, seed = spec
    xs, ys, zs, v = synth.cube_stretched(nx, ny, nz, r0, seed)
    return xs, ys, zs, v.astype(np.float32)


def make_workload_c3(B, host_cubes, specs):
    """Config 3: 48 uneven stretched cubes (16 cameras each) + 8 CMEM requests."""
    from birp_cpp_gb300 import synth
    cubes = [B.Cube(*hc) for hc in host_cubes]
    cmem = B.Cmem()
    items = []
    for src, pos, aim, nx, ny, step in specs:
        cam = B.camera(pos, aim, synth.FOV_W, synth.FOV_H, nx, ny, n_samples=synth.n_samples(step),
                       ray_length=synth.RAY_LENGTH, trilinear=True)
        items.append((cubes[src] if src >= 0 else cmem, cam))
    return cubes, cmem, items


def run_c3(args, B):
    """One-launch multi-cube batch (config 3) vs plain renders of the same requests."""
    import concurrent.futures as cf
    import multiprocessing as mp
    from birp_cpp_gb300 import synth
    cube_specs, specs = synth.config3_specs()
    with cf.ProcessPoolExecutor(max_workers=os.cpu_count() or 4, mp_context=mp.get_context("spawn")) as ex:
        host = list(ex.map(_gen_cube, cube_specs))
    from birp_cpp_gb300 import build
    build.build()
    B.init(0)
    cubes, cmem, items = make_workload_c3(B, host, specs)
    total_px = sum(c.nx * c.ny for _, c in items)
    batch = B.Batch(len(items), total_px)
    for _ in range(max(args.warmup, 2)):
        batch.render(items)
    km = []
    for _ in range(args.steps):
        B.flush_l2()
        batch.submit(items)
        batch.wait()
        km.append(batch.last_ms()[0])
    ms = float(np.mean(km))
    outs = [np.empty((c.ny, c.nx), np.float32) for _, c in items]
    t0 = time.perf_counter()
    for (sp, c), o in zip(items, outs):
        B.render(sp, c, out=o)
    plain_s = time.perf_counter() - t0
    dev_bytes = sum(c.info().device_bytes for c in cubes)
    print(json.dumps({"workload": "config 3: 48 uneven stretched cubes x 16 cameras + 8 CMEM, one launch",
                      "requests": len(items), "images_s": len(items) / (ms / 1000), "ms_per_launch": ms,
                      "plain_images_s": len(items) / plain_s, "batched_vs_plain": (len(items) / (ms / 1000)) /
                      (len(items) / plain_s), "cube_device_bytes": dev_bytes}))


def run_c4(args, B):
    """Serving sweep (config 4): Poisson arrivals at each rate for a fixed time;
    requests pick a cube by Zipf(1.1) popularity over a pool of cubes held in
    host (pinned) memory, rendered through the server under a GPU byte budget
    with LRU eviction; poses, sizes and steps from the orbit sampler.
    Reports images/s and p50/p99 latency per rate beside the plain per-call
    render's latency."""
    from birp_cpp_gb300 import build, synth
    nx, ny, nz = (int(v) for v in args.c4_dims.split("x"))
    rng = np.random.default_rng(4)
    # a few base fields (standoff r0 groups) and per-cube sheath noise
    xs, ys, zs = synth.stretched_axis(-40, 30, nx), synth.stretched_axis(-40, 40, ny), synth.stretched_axis(-40, 40, nz)
    r0_groups = [7.5, 9.0, 10.5, 12.0]
    bases = [synth.sheath_field(xs, ys, zs, np.random.default_rng(40 + g), r0=r0, noise=0.0).astype(np.float32)
             for g, r0 in enumerate(r0_groups)]
    build.build()
    B.init(0)
    layout = B.CUBE_COMPACT if args.c4_layout == "compact" else B.CUBE_RECORDS
    srv = B.Server(B.server_config(cube_budget_bytes=int(args.c4_budget_gb * (1 << 30)), slots=3,
                                   max_batch_requests=64, max_batch_pixels=16 << 20, max_wait_ms=1.0,
                                   max_queue=1 << 16, cube_layout=layout))
    ids = []
    for i in range(args.c4_cubes):
        # base * (1 + 0.3 U(-1, 1)), in FP32 and in place (256 cubes of 75 M
        # nodes are generated in minutes)
        v = rng.random(bases[0].shape, dtype=np.float32)
        v *= np.float32(0.6)
        v += np.float32(0.7)
        v *= bases[i % len(bases)]
        ids.append(srv.add_cube(xs, ys, zs, v))
        del v
    zipf_w = 1.0 / np.arange(1, args.c4_cubes + 1) ** 1.1
    zipf_w /= zipf_w.sum()
    reqs = synth.config2_requests(8192, seed=44)
    cams = [B.camera(p, a, synth.FOV_W, synth.FOV_H, w, h, n_samples=synth.n_samples(st)) for p, a, w, h, st in reqs]
    max_px = max(c.nx * c.ny for c in cams)
    # written once here: a client reuses its result buffers, and the first
    # touch of fresh pages (OS zero-fill, ~100 ms process-wide stalls at
    # 2.5 GB) is allocation cost, not serving latency
    bufs = [np.full(max_px, 0.0, np.float32) for _ in range(1024)]
    results = []
    for rate in (float(r) for r in args.c4_rates.split(",")):
        t0 = time.perf_counter()
        nxt, k, tickets = t0, 0, []
        st0 = srv.stats()
        while nxt - t0 < args.c4_seconds:
            now = time.perf_counter()
            if now < nxt:
                time.sleep(min(nxt - now, 0.002))
                continue
            cid = ids[int(rng.choice(args.c4_cubes, p=zipf_w))]
            try:
                tickets.append(srv.submit(cid, cams[k % len(cams)], bufs[k % len(bufs)]))
            except B.BirpError:
                pass
            k += 1
            nxt += rng.exponential(1.0 / rate)
        done = [r for r in (srv.wait(t, 120000) for t in tickets) if r.status == 0]
        t1 = time.perf_counter()
        st1 = srv.stats()
        lat = np.array([r.latency_ms for r in done]) if done else np.zeros(1)
        qms = np.array([r.queue_ms for r in done]) if done else np.zeros(1)
        results.append({"offered_req_s": rate, "completed": len(done), "images_s": len(done) / (t1 - t0),
                        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                        "queue_p99_ms": float(np.percentile(qms, 99)),
                        "uploads": st1.cube_uploads - st0.cube_uploads, "evictions": st1.cube_evictions - st0.cube_evictions,
                        "hits": st1.cube_hits - st0.cube_hits, "rejected": st1.rejected - st0.rejected})
        print(json.dumps(results[-1]), flush=True)
    srv.close()
    # plain per-call latency on one resident cube of the same layout
    cube = B.Cube(xs, ys, zs, bases[0], layout=layout)
    for c in cams[:5]:  # untimed: the server's released pool memory is returned meanwhile
        B.render(cube, c, out=bufs[0][: c.nx * c.ny].reshape(c.ny, c.nx))
    pl = []
    for c in cams[:200]:
        t = time.perf_counter()
        B.render(cube, c, out=bufs[0][: c.nx * c.ny].reshape(c.ny, c.nx))
        pl.append(1000 * (time.perf_counter() - t))
    print(json.dumps({"workload": f"config 4 serving sweep: {args.c4_cubes} cubes of {nx}x{ny}x{nz}, Zipf(1.1), "
                                  f"{args.c4_budget_gb} GB budget, {args.c4_seconds} s per rate, "
                                  f"{args.c4_layout} layout",
                      "sweep": results, "plain_p50_ms": float(np.percentile(pl, 50)),
                      "plain_p99_ms": float(np.percentile(pl, 99)), "plain_images_s": len(pl) / (sum(pl) / 1000)}))


def cpu_sample(reqs, host, seconds: float, threads: int, seed: int = 7):
    """The reference's FP32 render arithmetic (oracle port, per-cell lookup on
    the stretched axes) over random pixels drawn uniformly from all pixels of
    all requests, until `seconds` of wall time; returns (images/s, pixels,
    wall s). images/s = n_requests / (time per pixel * total pixels). The
    requests of a round are spread over `threads` host threads, one oracle
    call (one thread inside) per request: the library call releases the GIL,
    and a round holds ~1000 pixels per thread, so every thread has work."""
    import concurrent.futures as cf
    from birp_cpp_gb300 import synth
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    O.build()
    xs, ys, zs, v32 = host
    cube = O.Cube32(xs.astype(np.float32), ys.astype(np.float32), zs.astype(np.float32), v32, 1, 1)
    cams = [O.camera32(pos, aim, synth.FOV_W, synth.FOV_H, nx, ny, n_samples=synth.n_samples(step), ray_max=44)
            for pos, aim, nx, ny, step in reqs]
    npx = np.array([nx * ny for _, _, nx, ny, _ in reqs], np.int64)
    total_px = int(npx.sum())
    cum = np.cumsum(npx)
    rng = np.random.default_rng(seed)
    done_px, t_used = 0, 0.0
    chunk = 1024 * max(1, threads)

    def job(args):
        r, loc = args
        nx = reqs[r][2]
        O.render32_pixels(cube, cams[r], loc % nx, loc // nx, threads=1)

    t_start = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=max(1, threads)) as ex:
        while t_used < seconds or done_px == 0:
            flat = rng.integers(0, total_px, chunk)
            which = np.searchsorted(cum, flat, side="right")
            local = flat - np.concatenate([[0], cum[:-1]])[which]
            jobs = [(int(r), local[which == r]) for r in np.unique(which)]
            t0 = time.perf_counter()
            list(ex.map(job, jobs))
            t_used += time.perf_counter() - t0
            done_px += chunk
            if time.perf_counter() - t_start > 4 * seconds + 30:
                break
    per_px = t_used / done_px
    return len(reqs) / (per_px * total_px), done_px, t_used


def run_reference(args, world, rank):
    """--impl reference: the reference's CPU render arithmetic (oracle port)."""
    if rank != 0:
        return
    from birp_cpp_gb300 import synth
    reqs = synth.config2_requests(args.requests, seed=2)
    xs, ys, zs, v64 = synth.cube_config1(seed=1)
    host = (xs, ys, zs, v64.astype(np.float32))
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample(reqs, host, 0.5, threads, seed=100)
    vals, pxs, t_tot = [], 0, 0.0
    for k in range(args.steps):
        v, px, t = cpu_sample(reqs, host, args.ref_seconds, threads, seed=200 + k)
        vals.append(v)
        pxs += px
        t_tot += t
    value = float(np.mean(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * args.requests / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_dict(args),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{pxs} random pixels of the workload ({t_tot:.1f} s); images/s extrapolated "
                                   f"by total pixels"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def config_dict(args):
    return {"workload": f"{args.requests} orbit renders of a 256^3 stretched FP32 cube (config 2 on config 1's "
                        "cube): 144x84..1024x600 px, step 0.025-0.1 Re, trilinear, PREFIX",
            "cube": "256x256x256 stretched axes, FP32 (FP64 oracle copy)", "requests": args.requests,
            "fov_deg": [27.0, 16.0], "ray_length_re": 44.0,
            "l2": "flushed between timed steps (512 MB write); images (~445 MB) exceed L2",
            "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "1 GPU"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="birp", choices=["birp", "reference"])
    ap.add_argument("--requests", type=int, default=512)
    ap.add_argument("--ref-seconds", type=float, default=3.0)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--serve-seconds", type=float, default=3.0)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c4"],
                    help="c2: the 512-request single-cube batch (default); c3: 48-cube + CMEM batch; "
                         "c4: serving sweep")
    ap.add_argument("--c4-cubes", type=int, default=64)
    ap.add_argument("--c4-dims", default="512x384x384")
    ap.add_argument("--c4-budget-gb", type=float, default=60.0)
    ap.add_argument("--c4-rates", default="50,200,500,1000,2000")
    ap.add_argument("--c4-seconds", type=float, default=10.0)
    ap.add_argument("--c4-layout", default="compact", choices=["compact", "records"],
                    help="device layout of the served cubes")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload in ("c3", "c4"):
        import birp_cpp_gb300 as B
        (run_c3 if args.workload == "c3" else run_c4)(args, B)
        return

    import birp_cpp_gb300 as B
    from birp_cpp_gb300 import build
    build.build()
    B.init(local)
    W = make_workload(B, args.requests)
    cube, cams = W["cube"], W["cams"]
    npx = [c.nx * c.ny for c in cams]
    total_px = int(sum(npx))
    batch = B.Batch(len(cams), total_px)
    items = [(cube, c) for c in cams]

    for _ in range(max(args.warmup, 3)):
        batch.render(items)

    # ---- device-timed batched steps (inputs resident, L2 flushed before each)
    B.kernel_stats(reset=True)
    barrier(world)
    kern_ms, dev_ms = [], []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            B.flush_l2()
            batch.submit(items)
            batch.wait()
            k, t = batch.last_ms()
            kern_ms.append(k)
            dev_ms.append(t)
    barrier(world)
    ks = B.kernel_stats(reset=True)
    step_ms = allreduce_max(world, float(np.mean(kern_ms)))
    value = world * args.requests / (step_ms / 1000.0)
    samples_per_step = ks["samples"] / args.steps

    # ---- end to end through the C ABI with host buffers
    outs = [np.empty((c.ny, c.nx), np.float32) for c in cams]
    e2e_t = []
    import ctypes as C
    arr = B.Batch._reqs(items)
    ptrs = (C.c_void_p * len(items))(*[o.ctypes.data for o in outs])
    # untimed calls with the same output buffers (their pages are then mapped,
    # as in a serving loop that reuses its buffers)
    for _ in range(max(args.warmup, 1)):
        B.check(B.lib().birp_batch_render(batch.h, arr, len(items), ptrs))
    e2e_dev = []
    for _ in range(args.steps):
        B.flush_l2()
        barrier(world)
        t0 = time.perf_counter()
        B.check(B.lib().birp_batch_render(batch.h, arr, len(items), ptrs))
        e2e_t.append(time.perf_counter() - t0)
        e2e_dev.append(batch.last_ms())
    e2e_s = allreduce_max(world, float(np.mean(e2e_t)))
    e2e = world * args.requests / e2e_s
    # where the end-to-end time goes: kernel, device->host copy, host side
    k_mean = float(np.mean([k for k, _ in e2e_dev]))
    t_mean = float(np.mean([t for _, t in e2e_dev]))
    e2e_breakdown = {"kernel_ms": k_mean, "d2h_ms": t_mean - k_mean,
                     "host_ms": float(np.mean(e2e_t)) * 1e3 - t_mean}

    # ---- parity spot check of the timed images against the FP64 oracle
    parity = spot_check(W, outs) if rank == 0 else None

    # ---- plain per-call path on the same requests
    plain = None
    if not args.no_plain:
        pt = []
        for rep in range(2):
            B.flush_l2()
            t0 = time.perf_counter()
            for c, o in zip(cams, outs):
                B.render(cube, c, out=o)
            pt.append(time.perf_counter() - t0)
        plain_s = allreduce_max(world, min(pt))
        plain = world * args.requests / plain_s

    # ---- batched vs plain per image size (each class alone)
    by_size = None
    if not args.no_plain and rank == 0:
        by_size = {}
        img_buf = np.empty(max(c.nx * c.ny for c in cams), np.float32)
        for sz in sorted({(c.nx, c.ny) for c in cams}):
            sel = [c for c in cams if (c.nx, c.ny) == sz]
            its = [(cube, c) for c in sel]
            tb, tp = [], []
            for rep in range(2):
                B.flush_l2()
                batch.submit(its)
                batch.wait()
                tb.append(batch.last_ms()[0])
                B.flush_l2()
                t0 = time.perf_counter()
                for c in sel:
                    B.render(cube, c, out=img_buf[: c.nx * c.ny].reshape(c.ny, c.nx))
                tp.append(1000 * (time.perf_counter() - t0))
            bi, pi = len(sel) / (min(tb) / 1000), len(sel) / (min(tp) / 1000)
            by_size[f"{sz[0]}x{sz[1]}"] = {"requests": len(sel), "batched_images_s": bi, "plain_images_s": pi,
                                          "batched_vs_plain": bi / pi}

    # ---- roofline of the batched kernel (measured peaks)
    fp32_tflops, l2_gbs = B.measure_peaks()
    t_k = step_ms / 1000.0
    cells_per_step = ks["cells"] / args.steps

    def roof(units, flop_per, bytes_per, label):
        af = units * flop_per / t_k / 1e12
        ab = units * bytes_per / t_k / 1e9
        if units * flop_per / (fp32_tflops * 1e12) >= units * bytes_per / (l2_gbs * 1e9):
            r = {"bound": "fp32", "achieved": af, "peak": fp32_tflops, "unit": "TFLOP/s", "frac": af / fp32_tflops}
        else:
            r = {"bound": "l2", "achieved": ab, "peak": l2_gbs, "unit": "GB/s", "frac": ab / l2_gbs}
        r["units"] = label
        return r

    roofline = roof(cells_per_step, FLOP_PER_CELL, BYTES_PER_CELL,
                    f"{cells_per_step:.4g} cell segments/launch x {FLOP_PER_CELL:.0f} flop, {BYTES_PER_CELL:.0f} B")
    roofline.update({"traffic": traffic_from_profile(), "kernel": "render_batch_kernel",
                     "peak_source": "measured in-run: FP32 FMA loop and L2-resident read (birp_measure_peaks)",
                     "fp32_frac": cells_per_step * FLOP_PER_CELL / t_k / 1e12 / fp32_tflops,
                     "l2_frac": cells_per_step * BYTES_PER_CELL / t_k / 1e9 / l2_gbs})
    # the kernel is bound by instruction issue: warp instructions per cell
    # segment (ncu, profiles/) against one warp instruction per scheduler and
    # cycle (4 per SM) at the SM clock sampled during the timed steps
    wipc = profile_value("warp_instructions_per_cell")

    def issue_roofline(sm_mhz):
        if not wipc or not sm_mhz:
            return None
        try:
            import torch
            sms = torch.cuda.get_device_properties(local).multi_processor_count
        except Exception as e:  # a reporting extra: never fails the run
            return {"bound": "issue", "achieved": None, "error": str(e)[:120]}
        ai, peak = wipc * cells_per_step / t_k, 4.0 * sms * sm_mhz * 1e6
        return {"bound": "issue", "achieved": ai, "peak": peak, "unit": "warp-inst/s", "frac": ai / peak,
                "note": f"{wipc:.3f} warp instructions per cell segment (ncu, 64-request launch); peak = 4 x "
                        f"{sms} SMs x {sm_mhz:.0f} MHz (median SM clock of the timed steps)"}
    roofline_per_sample = roof(samples_per_step, FLOP_PER_SAMPLE, BYTES_PER_SAMPLE,
                               f"{samples_per_step:.4g} ray-samples/launch x {FLOP_PER_SAMPLE:.0f} flop, "
                               f"{BYTES_PER_SAMPLE:.0f} B (per-sample formulation; the kernel sums "
                               f"{samples_per_step / max(cells_per_step, 1):.2f} samples per cell in closed form)")
    peaks_file = os.path.join(ROOT, "MEASURED_PEAKS.json")
    hbm = None
    if os.path.exists(peaks_file):
        hbm = json.load(open(peaks_file)).get("hbm_gbs")
    unique_bytes = cube.info().device_bytes + 4 * total_px
    roofline_hbm = {"bound": "hbm", "achieved": unique_bytes / t_k / 1e9, "peak": hbm, "unit": "GB/s",
                    "frac": (unique_bytes / t_k / 1e9 / hbm) if hbm else None,
                    "note": "unique bytes: cube read once + images written; peak of measured (MEASURED_PEAKS.json)"}

    # ---- serving at 70% of the saturated batched rate
    serving = serve_latency(B, W, rate=0.7 * value / world, seconds=args.serve_seconds) if args.serve_seconds > 0 \
        else None

    # ---- CPU baseline (rank 0, N = 1)
    cpu = None
    if rank == 0 and world == 1 and args.cpu_seconds > 0:
        threads = os.cpu_count() or 1
        v, px, t = cpu_sample(W["reqs"], W["host"], args.cpu_seconds, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{px} random pixels of the {args.requests}-request workload, {t:.1f} s on {threads} "
                         f"threads; images/s extrapolated by total pixels"}
        v1, px1, t1 = cpu_sample(W["reqs"], W["host"], max(2.0, args.cpu_seconds / 3), 1, seed=11)
        cpu["single_core"] = {"value": v1, "unit": UNIT, "cores": 1,
                              "sample": f"{px1} random pixels, {t1:.1f} s on 1 thread"}

    if rank == 0:
        h2d = batch.upload_bytes()  # request descriptors and work tables, copied each step
        clock_summary = clocks.summary()
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config_dict(args),
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 4 * total_px},
            "plain": {"value": plain, "unit": UNIT} if plain else None,
            "batched_vs_plain": (value / plain) if plain else None,
            "by_size": by_size,
            "e2e_vs_plain": (e2e / plain) if plain else None,
            "e2e_breakdown": e2e_breakdown,
            "serving": serving,
            "ray_samples_per_s": samples_per_step * world / (step_ms / 1000.0),
            "roofline": roofline, "roofline_issue": issue_roofline(clock_summary.get("sm_mhz")),
            "roofline_per_sample": roofline_per_sample,
            "roofline_hbm": roofline_hbm,
            "cpu_baseline": cpu, "parity": parity,
            # each step replays one graph with four kernels: the CMEM, nearest
            # and compact-layout ones (no work here) and the records-layout
            # trilinear one
            "gpu_launches": 4 * args.steps, "clocks": clock_summary,
            "exact_fp64_rays_per_step": ks["exact_range_rays"] / args.steps,
            "samples_per_cell": (ks["samples"] / ks["cells"]) if ks.get("cells") else None,
        }
        print(json.dumps(line))


def spot_check(W, outs, n_pix: int = 3000):
    """Max/RMS relative error of random pixels of the timed images against the
    FP64 oracle."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    from birp_cpp_gb300 import synth
    O.build()
    xs, ys, zs, v32 = W["host"]
    oc = O.Cube64(xs, ys, zs, v32.astype(np.float64), 1)
    rng = np.random.default_rng(5)
    errs = []
    for r in rng.choice(len(W["reqs"]), 8, replace=False):
        pos, aim, nx, ny, step = W["reqs"][r]
        cam = O.camera64(pos, aim, synth.FOV_W, synth.FOV_H, nx, ny, synth.n_samples(step), synth.RAY_LENGTH, 0)
        pi = rng.integers(0, nx, n_pix // 8)
        pj = rng.integers(0, ny, n_pix // 8)
        ref = O.render64_pixels(oc, cam, pi, pj, threads=os.cpu_count() or 4)
        got = outs[r][pj, pi].astype(np.float64)
        m = ref > 1e-3 * max(ref.max(), 1e-300)
        if m.any():
            errs.append(np.abs(got[m] - ref[m]) / ref[m])
    e = np.concatenate(errs) if errs else np.zeros(1)
    return {"max_rel_err": float(e.max()), "rms_rel_err": float(np.sqrt(np.mean(e * e))), "pixels": int(e.size),
            "tolerance": 1e-5}


def serve_latency(B, W, rate: float, seconds: float, seed: int = 13):
    """Poisson arrivals at `rate` req/s for `seconds` into the server; returns
    p50/p99 latency and achieved throughput."""
    from birp_cpp_gb300 import synth
    srv = B.Server(B.server_config(slots=3, max_batch_requests=64, max_batch_pixels=16 << 20, max_wait_ms=1.0))
    sid = srv.add_cube(*W["host"])
    reqs = synth.config2_requests(4096, seed=seed)
    rng = np.random.default_rng(seed)
    cams = [B.camera(p, a, synth.FOV_W, synth.FOV_H, nx, ny, n_samples=synth.n_samples(s)) for p, a, nx, ny, s in reqs]
    # one buffer per in-flight request slot, each large enough for any image
    max_px = max(c.nx * c.ny for c in cams)
    bufs = [np.full(max_px, 0.0, np.float32) for _ in range(256)]  # pages resident before the timed arrivals
    # warm the cube into GPU memory
    t = srv.submit(sid, cams[0], bufs[0])
    srv.wait(t)
    tickets = []
    t0 = time.perf_counter()
    next_t = t0
    k = 0
    while next_t - t0 < seconds:
        now = time.perf_counter()
        if now < next_t:
            time.sleep(min(next_t - now, 0.002))
            continue
        c = cams[k % len(cams)]
        try:
            tickets.append(srv.submit(sid, c, bufs[k % len(bufs)]))
        except B.BirpError:
            pass
        k += 1
        next_t += rng.exponential(1.0 / rate)
    lat = []
    for t in tickets:
        r = srv.wait(t, 60000)
        if r.status == 0:
            lat.append(r.latency_ms)
    t_end = time.perf_counter()
    st = srv.stats()
    srv.close()
    lat = np.array(lat)
    return {"offered_rate": rate, "requests": len(tickets), "completed": int(len(lat)),
            "achieved_images_s": len(lat) / (t_end - t0), "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None, "batches": int(st.batches),
            "load": "70% of the saturated batched rate, Poisson"}


def profile_value(key):
    """One figure of the batched kernel from the committed ncu summary
    (profiles/render_batch_kernel_traffic.json), or None."""
    p = os.path.join(ROOT, "profiles", "render_batch_kernel_traffic.json")
    if os.path.exists(p):
        try:
            return json.load(open(p)).get(key)
        except (OSError, ValueError):
            return None
    return None


def traffic_from_profile():
    """DRAM bytes per launch of the batched kernel (ncu), if recorded."""
    return profile_value("dram_bytes_per_launch")


if __name__ == "__main__":
    main()
