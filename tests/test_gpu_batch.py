"""The batched path (one persistent-kernel launch from a CUDA graph) and the
continuous-batching server give the same images as the plain per-call render,
bit for bit, alone and in a mix."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def spaces(birp):
    from birp_cpp_gb300 import synth
    xs, ys, zs, v = synth.cube_config1(seed=1, n=96)
    c1 = birp.Cube(xs, ys, zs, v.astype(np.float32))
    xs0, ys0, zs0, v0 = synth.cube_config0(seed=0)
    c0 = birp.Cube(xs0, ys0, zs0, v0.astype(np.float32))
    return dict(c1=c1, c0=c0, cmem=birp.Cmem(), host=dict(c1=(xs, ys, zs, v.astype(np.float32)),
                                                          c0=(xs0, ys0, zs0, v0.astype(np.float32))))


def mixed_items(birp, spaces, n=24, seed=9):
    from birp_cpp_gb300 import synth
    rng = np.random.default_rng(seed)
    reqs = synth.config2_requests(n, seed=seed)
    items = []
    for k, (pos, aim, nx, ny, step) in enumerate(reqs):
        nx, ny = max(8, nx // 8), max(6, ny // 8)
        kind = rng.integers(0, 4)
        space = [spaces["c1"], spaces["c1"], spaces["c0"], spaces["cmem"]][kind]
        # explicit lanes per ray: a batch and a plain render then sum each
        # ray in the same order (automatic choices differ between the two)
        cam = birp.camera(pos, aim, 27.0, 16.0, nx, ny, n_samples=synth.n_samples(step), segments=2 ** (k % 4),
                          trilinear=bool(rng.integers(0, 2)), march=int(rng.integers(0, 2)))
        items.append((space, cam))
    return items


def test_batch_equals_plain_bitwise(birp, spaces):
    items = mixed_items(birp, spaces)
    b = birp.Batch(64, 1 << 22)
    outs = b.render(items)
    for (space, cam), img in zip(items, outs):
        ref = birp.render(space, cam)
        assert np.array_equal(img, ref)
    kms, tms = b.last_ms()
    assert 0 < kms <= tms
    # a second launch of the same graph with other requests
    items2 = mixed_items(birp, spaces, n=7, seed=3)
    outs2 = b.render(items2)
    for (space, cam), img in zip(items2, outs2):
        assert np.array_equal(img, birp.render(space, cam))
    b.close()


def test_batch_auto_lanes_close_to_plain(birp, spaces):
    """With automatic lanes per ray a batch may split rays differently from a
    plain render (its own tuned table); the images then differ only by FP32
    summation order."""
    from conftest import rel_err
    items = [(sp, birp.camera(tuple(c.pos), tuple(c.aim), c.fov_w_deg, c.fov_h_deg, c.nx, c.ny,
                              n_samples=c.n_samples, trilinear=bool(c.trilinear), march=c.march))
             for sp, c in mixed_items(birp, spaces, n=16, seed=17)]
    b = birp.Batch(32, 1 << 22)
    for (sp, cam), img in zip(items, b.render(items)):
        ref = birp.render(sp, cam)
        if ref.max() > 0:
            mx, _, _ = rel_err(img, ref.astype(np.float64))
            assert mx <= 1e-5, mx  # the parity tolerance; both paths sit within it of the oracle
        assert np.array_equal(img == 0, ref == 0)
    b.close()


def test_batch_single_and_empty(birp, spaces):
    b = birp.Batch(4, 1 << 16)
    cam = birp.camera((3, 1, 2), (9, 0, 0), 27.0, 16.0, 40, 24, n_samples=440, segments=2)
    [img] = b.render([(spaces["c1"], cam)])
    assert np.array_equal(img, birp.render(spaces["c1"], cam))
    assert b.render([]) == []
    with pytest.raises(birp.BirpError):
        b.render([(spaces["c1"], birp.camera((3, 1, 2), (9, 0, 0), 27.0, 16.0, 400, 240))])  # > max_pixels
    b.close()


def test_host_outputs_direct_and_copied(birp, spaces, monkeypatch):
    """birp_batch_render and birp_render give the same bits whether the kernel
    writes the caller's host buffers itself (devices with coherent pageable
    host access) or the images are copied back (BIRP_HOST_DIRECT=0), and the
    same as the pinned-buffer path of submit / wait."""
    import ctypes as C
    items = mixed_items(birp, spaces, n=20, seed=21)
    b = birp.Batch(64, 1 << 22)
    direct = b.render(items)
    monkeypatch.setenv("BIRP_HOST_DIRECT", "0")
    copied = b.render(items)
    plain_copied = [birp.render(sp, cam) for sp, cam in items]
    monkeypatch.delenv("BIRP_HOST_DIRECT")
    plain_direct = [birp.render(sp, cam) for sp, cam in items]
    b.submit(items)
    b.wait()
    lib = birp.lib()
    lib.birp_batch_image.restype = C.POINTER(C.c_float)
    for i, (sp, cam) in enumerate(items):
        p = lib.birp_batch_image(b.h, i)
        pinned = np.ctypeslib.as_array(p, shape=(cam.ny, cam.nx)).copy()
        for other in (copied[i], plain_copied[i], plain_direct[i], pinned):
            assert np.array_equal(direct[i], other)
    b.close()


def test_server_same_alone_and_in_mix(birp, spaces):
    """Each request's image from the server equals its plain render, whether
    it ran alone or mixed with others arriving concurrently."""
    srv = birp.Server(birp.server_config(slots=3, max_batch_requests=16, max_batch_pixels=1 << 20,
                                         max_wait_ms=0.5))
    ids = {"c1": srv.add_cube(*spaces["host"]["c1"]), "c0": srv.add_cube(*spaces["host"]["c0"]),
           "cmem": srv.add_cmem()}
    name_of = {id(spaces["c1"]): "c1", id(spaces["c0"]): "c0", id(spaces["cmem"]): "cmem"}
    items = mixed_items(birp, spaces, n=40, seed=21)
    # alone
    space, cam = items[0]
    out = np.empty((cam.ny, cam.nx), np.float32)
    t = srv.submit(ids[name_of[id(space)]], cam, out)
    r = srv.wait(t)
    assert r.status == 0 and r.latency_ms > 0
    assert np.array_equal(out, birp.render(space, cam))
    # in a mix: all submitted at once and in bursts
    outs, tickets = [], []
    for k, (space, cam) in enumerate(items):
        o = np.empty((cam.ny, cam.nx), np.float32)
        outs.append(o)
        tickets.append(srv.submit(ids[name_of[id(space)]], cam, o))
        if k % 10 == 9:
            time.sleep(0.002)
    for t in tickets:
        assert srv.wait(t, 30000).status == 0
    for (space, cam), o in zip(items, outs):
        assert np.array_equal(o, birp.render(space, cam))
    st = srv.stats()
    assert st.completed == len(items) + 1 and st.batches >= 2
    srv.close()


@pytest.mark.parametrize("base,promoted", [("compact", "records"), ("compact", "pairs"), ("pairs", "records")])
def test_server_promotes_popular_cube(birp, base, promoted):
    """A server with a promotion share: the cube that gets most requests is
    rebuilt in the promoted layout while requests keep arriving; every image,
    before, during and after the swap, equals the plain render of the same
    cube in the layout it was rendered from (the promoted one after the
    swap), and the promoted copy stays within the share."""
    from birp_cpp_gb300 import synth
    code = {"records": birp.CUBE_RECORDS, "compact": birp.CUBE_COMPACT, "pairs": birp.CUBE_PAIRS}
    cubes = []
    for s in range(3):
        xs, ys, zs, v = synth.cube_config1(seed=60 + s, n=64)
        cubes.append((xs, ys, zs, v.astype(np.float32)))
    fast = [birp.Cube(*c, layout=code[promoted]) for c in cubes]
    slow = [birp.Cube(*c, layout=code[base]) for c in cubes]
    share = int(1.5 * fast[0].info().device_bytes)  # room for one promoted cube
    srv = birp.Server(birp.server_config(cube_budget_bytes=1 << 32, slots=2, max_batch_requests=8,
                                         max_batch_pixels=1 << 20, max_wait_ms=0.2, cube_layout=code[base],
                                         promoted_layout=code[promoted], promoted_budget_bytes=share))
    ids = [srv.add_cube(*c) for c in cubes]
    cams = [birp.camera(p, a, 27.0, 16.0, 48, 28, n_samples=440, segments=1)
            for p, a, *_ in synth.config2_requests(8, seed=61)]
    work = []
    for rnd in range(40):
        k = 0 if rnd % 4 else 1 + (rnd // 4) % 2  # cube 0 most requested
        cam = cams[rnd % len(cams)]
        o = np.empty((cam.ny, cam.nx), np.float32)
        work.append((k, cam, o, srv.submit(ids[k], cam, o)))
        time.sleep(0.003)
    deadline = time.time() + 10
    while srv.stats().cube_promotions == 0 and time.time() < deadline:
        time.sleep(0.02)
    for rnd in range(24):
        cam = cams[rnd % len(cams)]
        o = np.empty((cam.ny, cam.nx), np.float32)
        work.append((0, cam, o, srv.submit(ids[0], cam, o)))
    for k, cam, o, t in work:
        assert srv.wait(t, 30000).status == 0
        assert np.array_equal(o, birp.render(fast[k], cam)) or np.array_equal(o, birp.render(slow[k], cam)), k
    st = srv.stats()
    assert st.cube_promotions == 1, st.cube_promotions
    assert 0 < st.promoted_bytes <= share
    # after the swap, cube 0 renders from its promoted copy
    for cam in cams[:4]:
        o = np.empty((cam.ny, cam.nx), np.float32)
        assert srv.wait(srv.submit(ids[0], cam, o), 30000).status == 0
        assert np.array_equal(o, birp.render(fast[0], cam))
    srv.close()
    for c in fast + slow:
        c.close()


def test_server_rejects_bad_promotion(birp):
    """A promoted layout must be faster than the server's own: records over
    compact or pairs, pairs over compact."""
    for base, promoted in [(birp.CUBE_RECORDS, birp.CUBE_RECORDS), (birp.CUBE_RECORDS, birp.CUBE_PAIRS),
                           (birp.CUBE_PAIRS, birp.CUBE_PAIRS), (birp.CUBE_COMPACT, birp.CUBE_COMPACT),
                           (birp.CUBE_COMPACT, 7)]:
        with pytest.raises(birp.BirpError):
            birp.Server(birp.server_config(cube_layout=base, promoted_layout=promoted, promoted_budget_bytes=1 << 30))


def test_server_lru_eviction_and_errors(birp, spaces):
    from birp_cpp_gb300 import synth
    cubes = []
    for s in range(3):
        xs, ys, zs, v = synth.cube_config1(seed=40 + s, n=64)
        cubes.append((xs, ys, zs, v.astype(np.float32)))
    one = birp.Cube(*cubes[0]).info().device_bytes
    # budget for two cubes: cycling through three forces evictions + re-uploads
    srv = birp.Server(birp.server_config(cube_budget_bytes=int(2.5 * one), slots=2, max_batch_requests=4,
                                         max_batch_pixels=1 << 18, max_wait_ms=0.0))
    ids = [srv.add_cube(*c) for c in cubes]
    gpu_cubes = [birp.Cube(*c) for c in cubes]
    cam = birp.camera((2, -3, 4), (9, 0, 0), 27.0, 16.0, 48, 28, n_samples=440, segments=1)
    for rnd in range(3):
        for k in (0, 1, 2):
            o = np.empty((28, 48), np.float32)
            t = srv.submit(ids[k], cam, o)
            assert srv.wait(t, 30000).status == 0
            assert np.array_equal(o, birp.render(gpu_cubes[k], cam))
    st = srv.stats()
    assert st.cube_evictions >= 3 and st.cube_uploads >= 4
    assert st.resident_bytes <= int(2.5 * one)
    srv.close()
    # a cube larger than the budget fails cleanly with NOMEM
    srv = birp.Server(birp.server_config(cube_budget_bytes=1000, slots=1))
    cid = srv.add_cube(*cubes[0])
    o = np.empty((28, 48), np.float32)
    t = srv.submit(cid, cam, o)
    r = srv.wait(t, 30000)
    assert r.status == birp.ERR_NOMEM
    srv.close()
    # a full queue rejects with BUSY; a short wait times out without harm
    srv = birp.Server(birp.server_config(max_queue=1, slots=1, max_wait_ms=0.0))
    cid = srv.add_cmem()
    big = birp.camera((2, -3, 4), (9, 0, 0), 27.0, 16.0, 512, 300, n_samples=1760)
    outs = [np.empty((300, 512), np.float32) for _ in range(6)]
    tickets, busy = [], 0
    for o in outs:
        try:
            tickets.append(srv.submit(cid, big, o))
        except birp.BirpError as e:
            assert e.status == birp.ERR_BUSY
            busy += 1
    assert busy >= 1
    with pytest.raises(birp.BirpError) as e:
        srv.wait(tickets[-1], 0.0)
    assert e.value.status == birp.ERR_TIMEOUT
    for t in tickets:
        assert srv.wait(t, 60000).status == 0
    srv.close()


def test_tile_shapes_give_the_same_images(birp, spaces):
    """Every tile shape the kernels take (rays across a warp block, warps
    across a tile) renders the same image, bit for bit, for a given number of
    lanes per ray: the shape only maps rays to lanes. Plain and batched, cube
    (both interpolations) and CMEM; shapes the kernels do not take are
    rejected."""
    from birp_cpp_gb300 import autotune
    pos, aim = (-2.0, -12.0, 16.0), (9.0, 0.0, 0.0)
    b = birp.Batch(64, 1 << 22)
    for space, tri in ((spaces["c1"], True), (spaces["c1"], False), (spaces["cmem"], True)):
        for seg in (1, 2, 8):
            ref = None
            items = []
            for wx, gx in autotune.shapes(seg):
                cam = birp.camera(pos, aim, 27.0, 16.0, 37, 23, n_samples=300, segments=seg, warp_rays_x=wx,
                                  tile_warps_x=gx, trilinear=tri)
                img = birp.render(space, cam)
                if ref is None:
                    ref = img
                assert np.array_equal(img, ref), (seg, wx, gx)
                items.append((space, cam))
            for img in b.render(items):
                assert np.array_equal(img, ref)
    b.close()
    for wx, gx, seg in ((3, 2, 1), (64, 1, 1), (32, 2, 1), (8, 8, 1), (16, 1, 8)):
        cam = birp.camera(pos, aim, 27.0, 16.0, 37, 23, n_samples=300, segments=seg, warp_rays_x=wx, tile_warps_x=gx)
        with pytest.raises(birp.BirpError):
            birp.render(spaces["c1"], cam)
