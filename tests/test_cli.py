"""The command-line front-end (birp_cpp_gb300/lib/birp, the reference's
`birp` program): argument handling on the CPU; directory (batch) mode and
CMEM mode on a GPU, checked against the Python batch path on the same data
and against the reference's output naming."""
import os
import subprocess

import numpy as np
import pytest

from test_cpp_classes import read_fits

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "birp_cpp_gb300", "lib", "birp")


def _build():
    from birp_cpp_gb300 import build
    build.build()


def write_dat(path, xs, ys, zs, vals):
    """A cube in the reference's .dat layout: 9 header lines, the dims on line
    10, then the x, y, z node coordinates and the values x fastest."""
    with open(path, "w") as f:
        for i in range(9):
            f.write(f"header line {i + 1}\n")
        f.write(f"{len(xs)} {len(ys)} {len(zs)}\n")
        for ax in (xs, ys, zs):
            f.write(" ".join(f"{v:.9g}" for v in ax) + "\n")
        flat = np.asarray(vals, np.float32).reshape(-1)
        for k in range(0, len(flat), 16):
            f.write(" ".join(f"{v:.9g}" for v in flat[k:k + 16]) + "\n")


def test_cli_arguments_cpu(tmp_path):
    _build()
    r = subprocess.run([CLI], capture_output=True, text=True)
    assert r.returncode == 3 and "Please provide valid .dat" in r.stdout
    r = subprocess.run([CLI, "-i", str(tmp_path / "cube")], capture_output=True, text=True)
    assert r.returncode == 3
    r = subprocess.run([CLI, "-c", "-m", "bogus"], capture_output=True, text=True)
    assert r.returncode == 1 and "records, pairs or compact" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("layout", ["records", "pairs", "compact"])
def test_cli_batch_directory_matches_batch_api(tmp_path, birp, layout):
    from birp_cpp_gb300 import synth
    _build()
    indir, outdir = tmp_path / "cubes", tmp_path / "out"
    indir.mkdir()
    outdir.mkdir()
    cubes = []
    for k in range(5):
        xs, ys, zs = np.linspace(-20, 25, 30 + k), synth.stretched_axis(-30, 30, 34), np.linspace(-22, 22, 28)
        rng = np.random.default_rng(k)
        v = synth.sheath_field(xs, ys, zs, rng, r0=8.0 + k).astype(np.float32)
        write_dat(indir / f"cube{k}.dat", xs.astype(np.float32), ys.astype(np.float32), zs.astype(np.float32), v)
        cubes.append((xs.astype(np.float32).astype(np.float64), ys.astype(np.float32).astype(np.float64),
                      zs.astype(np.float32).astype(np.float64), v))
    args = [CLI, "-i", str(indir) + "/", "-o", str(outdir) + "/", "-t", "-s", "0.5", "-x", "4", "-y", "-9", "-z", "6",
            "-a", "9", "-m", layout, "-M", "2"]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Using batch mode" in r.stdout and r.stdout.count("Exported to") == 5
    # the same renders through the batch API (same batch lanes-per-ray table)
    lay = {"records": birp.CUBE_RECORDS, "pairs": birp.CUBE_PAIRS, "compact": birp.CUBE_COMPACT}[layout]
    gcubes = [birp.Cube(*c, layout=lay) for c in cubes]
    cams = [birp.camera((4.0, -9.0, 6.0), (9.0, 0.0, 0.0), 36.0, 36.0, 72, 72, n_samples=200, trilinear=True)
            for _ in cubes]
    b = birp.Batch(8, 8 * 72 * 72)
    want = b.render(list(zip(gcubes, cams)))
    for k in range(5):
        _, img = read_fits(outdir / f"cube{k}.dat.fits")
        assert img.shape == (72, 72)
        assert np.array_equal(img.astype(np.float32), want[k]), k
    b.close()


@pytest.mark.gpu
def test_cli_cmem_single(tmp_path, birp):
    _build()
    r = subprocess.run([CLI, "-c", "-o", str(tmp_path) + "/", "-s", "1.0"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    _, img = read_fits(tmp_path / "cmembirp.fits")
    assert img.shape == (36, 36) and np.isfinite(img).all() and img.max() > 0
