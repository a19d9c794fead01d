"""Generates the golden fixtures in tests/golden/ by running the UNMODIFIED
reference renderer, built from its own sources by oracle/build_ref.sh.

Run with the reference project's directory (or BIRP_REFERENCE_DIR set):
    python tests/golden/make_golden.py <reference project directory>
The fixtures pin the oracle restatement (oracle/birp_oracle.cpp) bit for bit;
the tests never need the reference itself. Inputs are seeded, so rerunning
reproduces the files exactly.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle as O  # noqa: E402

# CMEM::Init argument sets (in the reference's positional order):
# v, b, dipole, p0, p1, p2, p3, B, alpha, beta, bs, A1, A2, ay_bs, az_bs, density.
# "default" is CMEM::Init(); "test_shifted" is the call in the reference's own
# tests/CMEM_test.cpp:63, whose arguments land one slot to the left.
CMEM_SETS = {
    "default": None,
    "test_shifted": [[400, 0, 0], [0, 0, 4], 0.0, 1.0, 4, 6, 3, 3.6, -1.0, -1.6, 12.6400003,
                     7.2e-06, 3.5000000000000004e-06, 0.0, 0.0, 0.0],
    "custom": [[380, 20, -10], [2, -3, 7], 0.3, 0.9, 2, 5, 3, 1.0, 2.2, -1.2, 13.0, 6e-6, 4e-6,
               0.6, 0.7, 7.0],
}

# Known answers from the reference's own tests (tests/CMEM_test.cpp:21-44, 63-89).
CMEM_KATS = {
    "default": [[[8, 4, 4], 0.0], [[4, 12, 10], 4.46853346e-06], [[3, 1.5, 1.2], 0.0],
                [[8, 10, 10], 8.15947317e-07], [[8, -10, -10], 8.15947317e-07],
                [[8, 10, -10], 8.15947317e-07]],
    "test_shifted": [[[8, 4, 4], 0.0], [[12, 12, 10], 4.57952495e-07], [[3, 1.5, 1.2], 0.0],
                     [[12, 10, 10], 5.48567925e-07], [[12, -10, -10], 5.48567925e-07],
                     [[12, 10, -10], 5.48567925e-07]],
}

POSES = [
    ((5.91813, 6.74116, 17.7067), (7.81768, 0.0, 0.0)),   # CLI default pose (src/main.cpp:37-40)
    ((1.0, 1.0, 1.0), (1.0, 0.0, 0.0)),                    # reference Camera test pose
    ((-5.0, -8.0, 3.0), (9.0, 0.0, 0.0)),
    ((2.0, 3.0, -4.0), (4.0, 2.0, 1.0)),                   # aim.y/aim.z are ignored by the pose
    ((-2.0, -12.0, 16.0), (10.0, 0.0, 0.0)),
]


def small_cube(rng):
    xs = np.linspace(-10, 20, 12).astype(np.float32)
    ys = np.linspace(-15, 15, 10).astype(np.float32)
    zs = np.linspace(-12, 14, 9).astype(np.float32)
    vals = rng.uniform(0, 5, size=(9, 10, 12)).astype(np.float32)
    return xs, ys, zs, vals


def main():
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BIRP_REFERENCE_DIR", "")
    r = subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh"), ref_dir], capture_output=True, text=True)
    if r.returncode != 0 or not os.path.exists(O.REF_PATH):
        sys.exit("reference build unavailable: " + r.stdout + r.stderr)
    R = O.Reference()
    rng = np.random.default_rng(20241203)

    # --- CMEM samples
    pts = rng.uniform(-30, 30, size=(3000, 3)).astype(np.float32)
    pts[:50, 1] = 0.0       # y == 0 branch of ShueCoords
    pts[50:100, 0] = 0.0    # x == 0 branch
    cm = {"points": pts}
    for name, args in CMEM_SETS.items():
        h = R.cmem_default() if args is None else R.cmem(*args)
        cm[name] = R.sample(h, pts)
        R.free(h)
    np.savez_compressed(os.path.join(HERE, "cmem_samples.npz"), **cm)

    # --- DataCube samples (nearest + trilinear)
    xs, ys, zs, vals = small_cube(rng)
    pts = np.stack([rng.uniform(-12, 22, 3000), rng.uniform(-17, 17, 3000), rng.uniform(-14, 16, 3000)],
                   1).astype(np.float32)
    cs = dict(xs=xs, ys=ys, zs=zs, values=vals, points=pts)
    for tri in (0, 1):
        h = R.cube(xs, ys, zs, vals, tri)
        cs[f"tri{tri}"] = R.sample(h, pts)
        R.free(h)
    np.savez_compressed(os.path.join(HERE, "cube_samples.npz"), **cs)

    # --- Renders through Camera::Render
    rd = dict(xs=xs, ys=ys, zs=zs, values=vals)
    meta = []
    k = 0
    for pos, aim in POSES:
        for tri in (0, 1):
            h = R.cube(xs, ys, zs, vals, tri)
            img = R.render(h, 2.0, 36.0, 30.0, pos, aim)
            R.free(h)
            rd[f"img{k}"] = img
            meta.append(dict(key=f"img{k}", space="cube", trilinear=tri, pixel=2.0, fov_h=36.0,
                             fov_w=30.0, pos=pos, aim=aim, renders=1))
            k += 1
        h = R.cmem_default()
        img = R.render(h, 1.0, 20.0, 24.0, pos, aim)
        R.free(h)
        rd[f"img{k}"] = img
        meta.append(dict(key=f"img{k}", space="cmem_default", trilinear=0, pixel=1.0, fov_h=20.0,
                         fov_w=24.0, pos=pos, aim=aim, renders=1))
        k += 1
    for renders in (1, 2):
        h = R.const()
        img = R.render(h, 3.0, 36.0, 36.0, (1.0, 1.0, 1.0), (1.0, 0.0, 0.0), renders=renders)
        R.free(h)
        rd[f"img{k}"] = img
        meta.append(dict(key=f"img{k}", space="const", trilinear=0, pixel=3.0, fov_h=36.0, fov_w=36.0,
                         pos=(1.0, 1.0, 1.0), aim=(1.0, 0.0, 0.0), renders=renders))
        k += 1
    # a signed field: the reference stops a ray at its first negative sample,
    # not only at the box edge (own seed: the fixtures above are unchanged)
    srng = np.random.default_rng(20261204)
    vals_s = srng.uniform(-1.5, 5.0, size=vals.shape).astype(np.float32)
    rd["values_signed"] = vals_s
    for pos, aim in POSES[:3]:
        for tri in (0, 1):
            h = R.cube(xs, ys, zs, vals_s, tri)
            img = R.render(h, 2.0, 36.0, 30.0, pos, aim)
            R.free(h)
            rd[f"img{k}"] = img
            meta.append(dict(key=f"img{k}", space="cube_signed", trilinear=tri, pixel=2.0, fov_h=36.0,
                             fov_w=30.0, pos=pos, aim=aim, renders=1))
            k += 1
    np.savez_compressed(os.path.join(HERE, "renders.npz"), **rd)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(dict(cmem_sets=CMEM_SETS, cmem_kats=CMEM_KATS, renders=meta,
                       generator="tests/golden/make_golden.py",
                       source="reference src/{Camera,DataCube,Cmem,Helper}.cpp via oracle/build_ref.sh"),
                  f, indent=1)
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main()
