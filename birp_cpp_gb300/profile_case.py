"""A small fixed workload for profiling one render kernel class: the first N
requests of the benchmark's orbit sampler (sizes 144x84..1024x600, steps
0.025-0.1 Re) on the 256^3 stretched cube (trilinear or nearest, either
layout) or on the default CMEM model, batched, launched a fixed number of
times. Run it under a profiler, e.g.

    python -m birp_cpp_gb300.profile_case --mode nearest --requests 64 --launches 4
"""
from __future__ import annotations

import argparse

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--mode", choices=["trilinear", "nearest", "compact", "cmem"], default="trilinear")
    ap.add_argument("--requests", type=int, default=64)
    ap.add_argument("--launches", type=int, default=4)
    args = ap.parse_args()

    import birp_cpp_gb300 as B
    from birp_cpp_gb300 import build, synth
    build.build()
    B.init(0)
    reqs = synth.config2_requests(args.requests, seed=2)
    if args.mode == "cmem":
        space = B.Cmem()
    else:
        xs, ys, zs, v = synth.cube_config1(seed=1)
        layout = B.CUBE_COMPACT if args.mode == "compact" else B.CUBE_RECORDS
        space = B.Cube(xs, ys, zs, v.astype(np.float32), layout=layout)
    cams = [B.camera(p, a, synth.FOV_W, synth.FOV_H, nx, ny, n_samples=synth.n_samples(s),
                     ray_length=synth.RAY_LENGTH, trilinear=args.mode != "nearest") for p, a, nx, ny, s in reqs]
    items = [(space, c) for c in cams]
    batch = B.Batch(len(items), sum(c.nx * c.ny for c in cams))
    for _ in range(args.launches):
        batch.submit(items)
        batch.wait()
    print(f"{args.mode}: {len(items)} requests, last launch {batch.last_ms()[0]:.3f} ms")
    batch.close()


if __name__ == "__main__":
    main()
