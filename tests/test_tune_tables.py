"""The committed tuning tables (birp_cpp_gb300/csrc/tune_table.inc,
tune_launch.inc), checked on the host: every tile-shape row is a shape the
kernels take (the rule of tile_shape_ok in csrc/render.cu: 1 to 32 lanes per
ray, a warp block no wider than its rays, 1, 2 or 4 warps across, tiles up
to 32 pixels a side), each table ends with rows that cover every
image size and sample count for every request kind, and every batch kernel
class has a CTAs-per-SM value the register file allows at 128 threads."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "birp_cpp_gb300", "csrc")
MAX_TILE = 32


def tables():
    text = open(os.path.join(CSRC, "tune_table.inc")).read()
    out = {}
    for name in ("kTuneRowsPlain", "kTuneRowsBatch"):
        body = re.search(name + r"\[\] = \{(.*?)\};", text, re.S).group(1)
        rows = [tuple(int(v) for v in re.findall(r"-?\d+", r.replace("(int64_t)", "")))
                for r in re.findall(r"\{([^{}]*)\}", body)]
        out[name] = rows
    return out


def shape_ok(segl2, wbx, wgx):
    if wbx < 0:  # the default width for the lanes per ray
        wbx = 3 if segl2 == 0 else 2 if segl2 <= 2 else 1 if segl2 <= 4 else 0
    if wgx < 0:
        wgx = 1
    tile_w = (1 << wgx) << wbx
    tile_h = ((32 >> segl2) >> wbx) * (4 >> wgx)
    return (0 <= segl2 <= 5 and wbx >= 0 and (1 << wbx) <= (32 >> segl2) and 0 <= wgx <= 2
            and tile_w <= MAX_TILE and tile_h <= MAX_TILE)


def test_every_row_is_a_shape_the_kernels_take():
    for name, rows in tables().items():
        assert rows, name
        for r in rows:
            assert len(r) == 7, (name, r)
            assert shape_ok(r[4], r[5], r[6]), (name, r)


def test_tables_cover_every_request():
    for name, rows in tables().items():
        for kind in (0, 1):
            for tri in (0, 1):
                for pixels in (1, 12096, 1 << 22, 1 << 39):
                    for samples in (1, 880, 1 << 29):
                        hit = [r for r in rows if pixels <= r[0] and samples <= r[1] and r[2] in (-1, kind)
                               and r[3] in (-1, tri)]
                        assert hit, (name, kind, tri, pixels, samples)


def test_launch_bounds_fit_the_register_file():
    text = open(os.path.join(CSRC, "tune_launch.inc")).read()
    vals = dict(re.findall(r"#define (BIRP_\w+_MINB_TUNED) (\d+)", text))
    for macro in ("BIRP_WALK_MINB_TUNED", "BIRP_COMPACT_MINB_TUNED", "BIRP_PAIRS_MINB_TUNED",
                  "BIRP_NEAREST_MINB_TUNED", "BIRP_CMEM_MINB_TUNED"):
        n = int(vals[macro])
        # 65536 registers per SM, 128 threads per CTA: at least 32 registers a thread
        assert 1 <= n <= 16, (macro, n)
