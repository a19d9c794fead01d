"""Autotuner for the lanes-per-ray choice (S = 1, 2, 4, 8) of the render
kernels. For each image-size class and sample-count class of the benchmark
workloads it times plain renders of the 256^3 stretched cube from several
orbit poses with every S (CUDA events around the kernel, L2 flushed before
each) and writes the fastest choice per class to csrc/tune_table.inc (or the
path given), which the library compiles in. Run on the GPU:

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
            print(json.dumps({"pixels": nx * ny, "n_samples": n, "best": best,
                              "ms": {str(k): round(v, 4) for k, v in times.items()}}), flush=True)
    return results


def write_table(results, path, kind_code=-1):
    """Rows ordered by pixels then samples; each row covers pixels up to its
    class (and the geometric midpoint to the next class)."""
    pix = sorted({p for p, _ in results})
    smp = sorted({n for _, n in results})
    lines = ["// Lanes-per-ray table: the first row whose bounds hold gives log2(lanes).",
             "// kind: 0 cube, 1 CMEM, -1 any; trilinear: -1 any.",
             "// Written by birp_cpp_gb300/autotune.py from plain-render timings on a GB300",
             "// (256^3 stretched cube, orbit poses, L2 flushed before each render).",
             "static const TuneRow kTuneRows[] = {"]
    for i, p in enumerate(pix):
        pmax = int(np.sqrt(p * pix[i + 1])) if i + 1 < len(pix) else (1 << 40)
        for j, n in enumerate(smp):
            nmax = int(np.sqrt(n * smp[j + 1])) if j + 1 < len(smp) else (1 << 30)
            best = results[(p, n)][0]
            lines.append(f"    {{(int64_t){pmax}, {nmax}, {kind_code}, -1, {int(np.log2(best))}}},")
    lines.append("};")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "csrc", "tune_table.inc"))
    ap.add_argument("--poses", type=int, default=4)
    ap.add_argument("--repeats", type=int, default=3)
    args = ap.parse_args()
    res = tune(args.poses, args.repeats)
    write_table(res, args.out)
    print("wrote", args.out)


if __name__ == "__main__":
    main()
