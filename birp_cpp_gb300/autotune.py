"""Autotuner of the render kernels' launch shape, run on the GPU.

It searches, by timing the kernels (CUDA events, L2 flushed before each
launch), over
  * the tile shape of a request: lanes per ray S (1, 2, 4, 8), the width of
    the block of rays one warp marches (its 32 / S rays as 2^k across), and
    the arrangement of the CTA's 4 warps over the pixel tile (4x1, 2x2, 1x4),
    tiles up to 32 pixels a side;
      - for a request rendered alone (plain renders of the 256^3 stretched
        cube and of the default CMEM model from orbit poses), per
        image-size and sample-count class, cube and CMEM requests apart;
      - for a request inside a batch: 32-request batches of one class for
        trilinear and nearest cube requests, a 16-request batch of mixed
        sizes for CMEM requests;
  * the resident CTAs per SM each persistent batch kernel class is compiled
    for (records, pairs and compact-layout trilinear, nearest, CMEM):
    the library is rebuilt with each candidate and the class's batch kernel
    timed on a fixed workload (64 orbit requests; 16 for CMEM) in a child
    process.
It writes the tile-shape tables to csrc/tune_table.inc and the CTAs per SM to
csrc/tune_launch.inc (or the paths given); the library compiles both in.

    python -m birp_cpp_gb300.autotune               # everything
    python -m birp_cpp_gb300.autotune --skip-occupancy
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

SIZES = [(144, 84), (288, 168), (576, 336), (1024, 600)]
SAMPLES = [440, 880, 1760]
SEGMENTS = [1, 2, 4, 8]
MAX_TILE = 32


def shapes(seg: int):
    """(warp_rays_x, tile_warps_x) pairs the kernels take for S = seg."""
    rays = 32 // seg
    out = []
    for wx in (1, 2, 4, 8, 16, 32):
        if wx > rays:
            continue
        wy = rays // wx
        for gx in (1, 2, 4):
            gy = 4 // gx
            if wx * gx <= MAX_TILE and wy * gy <= MAX_TILE:
                out.append((wx, gx))
    return out


def _timer(B, kind):
    import ctypes as C
    import torch  # device memory for the timed renders' output
    from birp_cpp_gb300 import synth
    if kind == "cube":
        xs, ys, zs, v = synth.cube_config1(seed=1)
        space = B.Cube(xs, ys, zs, v.astype(np.float32))
        src = (space.h, None)
    else:
        space = B.Cmem()
        src = (None, space.h)
    out = torch.empty(1024 * 600, dtype=torch.float32, device="cuda:0")
    L = B.lib()

    def time_plain(cam, repeats):
        ms = C.c_float()
        B.check(L.birp_time_render_device(src[0], src[1], C.byref(cam), C.c_void_p(out.data_ptr()), repeats, 1,
                                          C.byref(ms)))
        return ms.value

    return space, time_plain


def tune_plain(n_poses: int = 4, repeats: int = 3, kind: str = "cube"):
    """{(pixels, samples): (best (S, wx, gx), times)} for plain renders of
    the 256^3 cube (kind "cube") or the default CMEM model ("cmem")."""
    import birp_cpp_gb300 as B
    from birp_cpp_gb300 import synth
    _space, time_plain = _timer(B, kind)
    poses = [(p, a) for p, a, *_ in synth.config2_requests(n_poses, seed=77)]
    results = {}
    for nx, ny in SIZES:
        for n in SAMPLES:
            times = {}
            for s in SEGMENTS:
                for wx, gx in shapes(s):
                    tot = 0.0
                    for pos, aim in poses:
                        cam = B.camera(pos, aim, synth.FOV_W, synth.FOV_H, nx, ny, n_samples=n, segments=s,
                                       warp_rays_x=wx, tile_warps_x=gx)
                        tot += time_plain(cam, repeats)
                    times[(s, wx, gx)] = tot / len(poses)
            best = min(times, key=times.get)
            results[(nx * ny, n)] = (best, times)
            default = (best[0], 1 << [3, 2, 2, 1][SEGMENTS.index(best[0])], 2)  # the untuned shape of that S
            print(json.dumps({"context": f"plain {kind}", "pixels": nx * ny, "n_samples": n, "best": best,
                              "ms_best": round(times[best], 4), "ms_default_shape": round(times[default], 4)}),
                  flush=True)
    return results


def tune_batch(kind: str, batch_size: int = 32, repeats: int = 3, sizes=SIZES, samples=SAMPLES, segs=(1, 2)):
    """{(pixels, samples): (best (S, wx, gx), times)} for batches of one
    request class: kind "tri" (trilinear cube), "nearest" or "cmem"."""
    import birp_cpp_gb300 as B
    from birp_cpp_gb300 import synth
    if kind == "cmem":
        space = B.Cmem()
    else:
        xs, ys, zs, v = synth.cube_config1(seed=1)
        space = B.Cube(xs, ys, zs, v.astype(np.float32))
    poses = [(p, a) for p, a, *_ in synth.config2_requests(batch_size, seed=78)]
    batch = B.Batch(batch_size, batch_size * 1024 * 600)
    results = {}
    for nx, ny in sizes:
        for n in samples:
            times = {}
            for s in segs:
                for wx, gx in shapes(s):
                    items = [(space, B.camera(p, a, synth.FOV_W, synth.FOV_H, nx, ny, n_samples=n, segments=s,
                                              warp_rays_x=wx, tile_warps_x=gx, trilinear=kind != "nearest"))
                             for p, a in poses]
                    ms = []
                    for _ in range(repeats):
                        B.flush_l2()
                        batch.submit(items)
                        batch.wait()
                        ms.append(batch.last_ms()[0])
                    times[(s, wx, gx)] = float(np.median(ms))
            best = min(times, key=times.get)
            results[(nx * ny, n)] = (best, times)
            print(json.dumps({"context": f"batch {kind}", "pixels": nx * ny, "n_samples": n, "best": best,
                              "ms_best": round(times[best], 4), "ms_2x2_S1": round(times.get((1, 8, 2), -1), 4)}),
                  flush=True)
    batch.close()
    return results


def tune_batch_cmem(repeats: int = 3):
    """{(pixels, samples): (best (S, wx, gx), times)}, one entry standing for
    every size: 16 orbit requests of mixed sizes on the default CMEM model
    in one batch, every tile shape of 1, 2, 4 and 8 lanes per ray."""
    import birp_cpp_gb300 as B
    from birp_cpp_gb300 import synth
    space = B.Cmem()
    reqs = synth.config2_requests(16, seed=2)
    batch = B.Batch(len(reqs), len(reqs) * 1024 * 600)
    times = {}
    for s in SEGMENTS:
        for wx, gx in shapes(s):
            items = [(space, B.camera(p, a, synth.FOV_W, synth.FOV_H, nx, ny, n_samples=synth.n_samples(st),
                                      ray_length=synth.RAY_LENGTH, segments=s, warp_rays_x=wx, tile_warps_x=gx))
                     for p, a, nx, ny, st in reqs]
            ms = []
            for _ in range(repeats + 1):
                B.flush_l2()
                batch.submit(items)
                batch.wait()
                ms.append(batch.last_ms()[0])
            times[(s, wx, gx)] = float(np.median(ms[1:]))
    batch.close()
    best = min(times, key=times.get)
    print(json.dumps({"context": "batch cmem (16 orbit requests)", "best": best, "ms_best": round(times[best], 4)}),
          flush=True)
    return {(1024 * 600, 880): (best, times)}


def _rows(results, kind_code=-1, trilinear=-1, all_sizes=False):
    """Rows ordered by pixels then samples; each row covers pixels up to its
    class (and the geometric midpoint to the next class). all_sizes: one
    result stands for every class."""
    pix = sorted({p for p, _ in results})
    smp = sorted({n for _, n in results})
    out = []
    for i, p in enumerate(pix):
        pmax = int(np.sqrt(p * pix[i + 1])) if i + 1 < len(pix) else (1 << 40)
        if all_sizes:
            pmax = 1 << 40
        for j, n in enumerate(smp):
            nmax = int(np.sqrt(n * smp[j + 1])) if j + 1 < len(smp) else (1 << 30)
            if all_sizes:
                nmax = 1 << 30
            s, wx, gx = results[(p, n)][0]
            out.append(f"    {{(int64_t){pmax}, {nmax}, {kind_code}, {trilinear}, {int(np.log2(s))}, "
                       f"{int(np.log2(wx))}, {int(np.log2(gx))}}},")
    return out


def write_table(plain, plain_cmem, batch_tri, batch_near, batch_cmem, path):
    lines = ["// Tile-shape tables: the first row whose bounds hold gives the shape.",
             "// Columns: max pixels, max samples, kind (0 cube, 1 CMEM, -1 any), trilinear",
             "// (-1 any), log2(lanes per ray), log2(rays across a warp block), log2(warps",
             "// across a tile) (-1: the default for the lanes per ray). Written by",
             "// birp_cpp_gb300/autotune.py from timings on a GB300 (256^3 stretched cube or",
             "// the default CMEM model, orbit poses, L2 flushed before each launch): plain",
             "// renders for a request alone (CMEM and cube requests), 32-request batches of",
             "// one cube class and a 16-request mixed-size CMEM batch for a request inside",
             "// a batch.",
             "static const TuneRow kTuneRowsPlain[] = {"] + _rows(plain_cmem, 1, -1) + _rows(plain) + ["};",
             "static const TuneRow kTuneRowsBatch[] = {"] + _rows(batch_cmem, 1, -1, all_sizes=True) + \
            _rows(batch_near, 0, 0) + _rows(batch_tri, -1, -1) + ["};"]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


# ------------------------------------------------------------------ occupancy

CLASSES = {  # class: (macro, candidates of resident CTAs per SM, profile case)
    "records": ("BIRP_WALK_MINB", [6, 7, 8], "trilinear"),
    "compact": ("BIRP_COMPACT_MINB", [5, 6, 7, 8], "compact"),
    "pairs": ("BIRP_PAIRS_MINB", [6, 7, 8], "pairs"),
    "nearest": ("BIRP_NEAREST_MINB", [6, 7, 8], "nearest"),
    "cmem": ("BIRP_CMEM_MINB", [5, 6, 7, 8, 9, 10, 12], "cmem"),
}


def _variant_defines(k):
    return {macro: cands[min(k, len(cands) - 1)] for macro, cands, _ in CLASSES.values()}


def time_case(lib_path: str, case: str, launches: int = 5) -> float:
    """Median batch-kernel time (ms) of one profile case with the library at
    lib_path, in a child process."""
    n = 16 if case == "cmem" else 64
    code = f"""
import json, numpy as np, sys
sys.path.insert(0, {ROOT!r})
import birp_cpp_gb300 as B
from birp_cpp_gb300 import synth
B.init(0)
reqs = synth.config2_requests({n}, seed=2)
mode = {case!r}
if mode == "cmem":
    space = B.Cmem()
else:
    xs, ys, zs, v = synth.cube_config1(seed=1)
    layout = {{"compact": B.CUBE_COMPACT, "pairs": B.CUBE_PAIRS}}.get(mode, B.CUBE_RECORDS)
    space = B.Cube(xs, ys, zs, v.astype(np.float32), layout=layout)
cams = [B.camera(p, a, synth.FOV_W, synth.FOV_H, nx, ny, n_samples=synth.n_samples(s), trilinear=mode != "nearest")
        for p, a, nx, ny, s in reqs]
items = [(space, c) for c in cams]
b = B.Batch(len(items), sum(c.nx * c.ny for c in cams))
ms = []
for i in range({launches} + 2):
    B.flush_l2(); b.submit(items); b.wait()
    if i >= 2: ms.append(b.last_ms()[0])
print(json.dumps(float(np.median(ms))))
"""
    env = dict(os.environ, BIRP_LIB=lib_path)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        raise RuntimeError(r.stderr[-2000:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def tune_occupancy():
    """{class: (best CTAs per SM, {candidate: ms})}."""
    from birp_cpp_gb300 import build
    build.build()
    n_var = max(len(c) for _, c, _ in CLASSES.values())
    with cf.ThreadPoolExecutor(max_workers=n_var) as ex:
        libs = list(ex.map(lambda k: build.build_variant(_variant_defines(k), f"minb{k}"), range(n_var)))
    out = {}
    for cls, (macro, cands, case) in CLASSES.items():
        times = {}
        for k, lib in enumerate(libs):
            v = _variant_defines(k)[macro]
            if v in times:
                continue
            times[v] = time_case(lib, case)
        best = min(times, key=times.get)
        out[cls] = (best, times)
        print(json.dumps({"context": "occupancy", "class": cls, "best": best,
                          "ms": {str(k): round(t, 4) for k, t in times.items()}}), flush=True)
    return out


def write_launch(occ, path):
    lines = ["// Resident CTAs per SM each persistent batch kernel class is compiled for",
             "// (__launch_bounds__ minimum; fewer allow more registers per thread). Written",
             "// by birp_cpp_gb300/autotune.py from the batch kernel's time on a fixed",
             "// workload per class (64 orbit requests on the 256^3 stretched cube, 16 on the",
             "// default CMEM model) with each candidate, on a GB300."]
    for cls, (macro, _c, _case) in CLASSES.items():
        times = ", ".join(f"{k}: {t:.3f} ms" for k, t in sorted(occ[cls][1].items()))
        lines.append(f"#define {macro}_TUNED {occ[cls][0]}  // {times}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "csrc", "tune_table.inc"))
    ap.add_argument("--launch-out", default=os.path.join(HERE, "csrc", "tune_launch.inc"))
    ap.add_argument("--poses", type=int, default=4)
    ap.add_argument("--repeats", type=int, default=3)
    ap.add_argument("--skip-occupancy", action="store_true")
    ap.add_argument("--skip-shapes", action="store_true")
    args = ap.parse_args()
    if not args.skip_occupancy:
        occ = tune_occupancy()
        write_launch(occ, args.launch_out)
        print("wrote", args.launch_out, flush=True)
    if not args.skip_shapes:
        import birp_cpp_gb300 as B
        from birp_cpp_gb300 import build
        build.build()
        B.init(0)
        plain = tune_plain(args.poses, args.repeats)
        plain_cmem = tune_plain(args.poses, args.repeats, kind="cmem")
        tri = tune_batch("tri", repeats=args.repeats)
        near = tune_batch("nearest", repeats=args.repeats)
        cm = tune_batch_cmem(repeats=args.repeats)
        write_table(plain, plain_cmem, tri, near, cm, args.out)
        print("wrote", args.out)


if __name__ == "__main__":
    main()
