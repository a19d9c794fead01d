"""Autotuner for the lanes-per-ray choice (S = 1, 2, 4, 8) of the render
kernels. For each image-size class and sample-count class of the benchmark
workloads it times, with every S, (a) plain renders of the 256^3 stretched
cube from several orbit poses and (b) batches of 32 such requests (CUDA
events around the kernels, L2 flushed before each), and writes the fastest
choice per class for a request rendered alone and for one inside a batch to
csrc/tune_table.inc (or the path given), which the library compiles in. Run
on the GPU:

    python -m birp_cpp_gb300.autotune --out birp_cpp_gb300/csrc/tune_table.inc
"""
from __future__ import annotations

import argparse
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

SIZES = [(144, 84), (288, 168), (576, 336), (1024, 600)]
SAMPLES = [440, 880, 1760]
SEGMENTS = [1, 2, 4, 8]


def tune(n_poses: int = 4, repeats: int = 3, kind: str = "cube"):
    import ctypes as C

    import birp_cpp_gb300 as B
    from birp_cpp_gb300 import build, synth
    build.build()
    B.init(0)
    if kind == "cube":
        xs, ys, zs, v = synth.cube_config1(seed=1)
        space = B.Cube(xs, ys, zs, v.astype(np.float32))
        src = (space.h, None)
    else:
        space = B.Cmem()
        src = (None, space.h)
    poses = [(p, a) for p, a, *_ in synth.config2_requests(n_poses, seed=77)]
    results = {}
    L = B.lib()
    import torch  # device memory for the timed renders' output
    out = torch.empty(1024 * 600, dtype=torch.float32, device="cuda:0")
    for nx, ny in SIZES:
        for n in SAMPLES:
            best = None
            times = {}
            for s in SEGMENTS:
                tot = 0.0
                for pos, aim in poses:
                    cam = B.camera(pos, aim, synth.FOV_W, synth.FOV_H, nx, ny, n_samples=n, segments=s)
                    ms = C.c_float()
                    B.check(L.birp_time_render_device(src[0], src[1], C.byref(cam), C.c_void_p(out.data_ptr()),
                                                      repeats, 1, C.byref(ms)))
                    tot += ms.value
                times[s] = tot / len(poses)
                if best is None or times[s] < times[best]:
                    best = s
            results[(nx * ny, n)] = (best, times)
            print(json.dumps({"context": "plain", "pixels": nx * ny, "n_samples": n, "best": best,
                              "ms": {str(k): round(v, 4) for k, v in times.items()}}), flush=True)
    return results


def tune_batch(batch_size: int = 32, repeats: int = 3):
    """Kernel time of a batch of `batch_size` requests of one class (orbit
    poses) for every S; returns {(pixels, samples): (best S, times)}."""
    import birp_cpp_gb300 as B
    from birp_cpp_gb300 import build, synth
    build.build()
    B.init(0)
    xs, ys, zs, v = synth.cube_config1(seed=1)
    cube = B.Cube(xs, ys, zs, v.astype(np.float32))
    poses = [(p, a) for p, a, *_ in synth.config2_requests(batch_size, seed=78)]
    batch = B.Batch(batch_size, batch_size * 1024 * 600)
    results = {}
    for nx, ny in SIZES:
        for n in SAMPLES:
            times = {}
            for s in SEGMENTS:
                items = [(cube, B.camera(p, a, synth.FOV_W, synth.FOV_H, nx, ny, n_samples=n, segments=s))
                         for p, a in poses]
                ms = []
                for _ in range(repeats):
                    B.flush_l2()
                    batch.submit(items)
                    batch.wait()
                    ms.append(batch.last_ms()[0])
                times[s] = float(np.median(ms))
            best = min(times, key=times.get)
            results[(nx * ny, n)] = (best, times)
            print(json.dumps({"context": "batch", "pixels": nx * ny, "n_samples": n, "best": best,
                              "ms": {str(k): round(v, 4) for k, v in times.items()}}), flush=True)
    return results


def _rows(results, kind_code=-1):
    """Rows ordered by pixels then samples; each row covers pixels up to its
    class (and the geometric midpoint to the next class)."""
    pix = sorted({p for p, _ in results})
    smp = sorted({n for _, n in results})
    out = []
    for i, p in enumerate(pix):
        pmax = int(np.sqrt(p * pix[i + 1])) if i + 1 < len(pix) else (1 << 40)
        for j, n in enumerate(smp):
            nmax = int(np.sqrt(n * smp[j + 1])) if j + 1 < len(smp) else (1 << 30)
            best = results[(p, n)][0]
            out.append(f"    {{(int64_t){pmax}, {nmax}, {kind_code}, -1, {int(np.log2(best))}}},")
    return out


def write_table(plain, batch, path):
    lines = ["// Lanes-per-ray tables: the first row whose bounds hold gives log2(lanes).",
             "// Columns: max pixels, max samples, kind (0 cube, 1 CMEM, -1 any), trilinear",
             "// (-1 any), log2(lanes). Written by birp_cpp_gb300/autotune.py from timings on",
             "// a GB300 (256^3 stretched cube, orbit poses, L2 flushed before each launch):",
             "// plain renders for a request alone, 32-request batches for one in a batch.",
             "static const TuneRow kTuneRowsPlain[] = {"] + _rows(plain) + ["};",
             "static const TuneRow kTuneRowsBatch[] = {"] + _rows(batch) + ["};"]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "csrc", "tune_table.inc"))
    ap.add_argument("--poses", type=int, default=4)
    ap.add_argument("--repeats", type=int, default=3)
    args = ap.parse_args()
    plain = tune(args.poses, args.repeats)
    batch = tune_batch(repeats=args.repeats)
    write_table(plain, batch, args.out)
    print("wrote", args.out)


if __name__ == "__main__":
    main()
