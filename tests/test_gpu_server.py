"""The request server: each result is the same served alone and in a mix with other
requests, edits keep their order within a world, and the memory budget refuses what
cannot fit."""
import ctypes as C

import numpy as np
import pytest

import scenes
import vrt
from helpers import gpu_render, make_world

pytestmark = pytest.mark.gpu


def make_server(budget=1 << 30, slots=3, max_batch=4, max_wait_us=0, image_memory=0, max_batch_pixels=0):
    cfg = vrt.ServerConfig(budget, slots, max_batch, max_wait_us, image_memory, max_batch_pixels)
    h = C.c_void_p()
    vrt.check(vrt.lib().vrt_server_create(C.byref(cfg), C.byref(h)))
    return h


def add_world(srv, w):
    wid = C.c_int32()
    vrt.check(vrt.lib().vrt_server_add_world(srv, w.handle, C.byref(wid)))
    return wid.value


def submit_render(srv, wid, u, width, height, out, tag):
    q = vrt.Request()
    q.kind = vrt.REQ_RENDER
    q.world_id = wid
    q.uniforms = u
    q.width, q.height = width, height
    q.host_rgba = (out.ctypes.data if isinstance(out, np.ndarray) else out.data_ptr()) if out is not None else None
    q.user_tag = tag
    vrt.check(vrt.lib().vrt_server_submit(srv, C.byref(q)))


def submit_edit(srv, wid, c, r, tag):
    q = vrt.Request()
    q.kind = vrt.REQ_EDIT
    q.world_id = wid
    q.cx, q.cy, q.cz = c
    q.radius = r
    q.user_tag = tag
    vrt.check(vrt.lib().vrt_server_submit(srv, C.byref(q)))


def collect(srv, n):
    buf = (vrt.Completion * 256)()
    out = []
    vrt.check(vrt.lib().vrt_server_drain(srv))
    while True:
        k = vrt.check(vrt.lib().vrt_server_poll(srv, buf, 256))
        out += [buf[i] for i in range(k)]
        if k == 0:
            break
    assert len(out) == n
    return {c.user_tag: c for c in out}


@pytest.fixture(scope="module")
def worlds():
    a = scenes.full(2, W=128, H=64, width=64, height=64, max_steps=256)
    b = scenes.small(4)
    return a, b


def host_image(n, pinned):
    """A result buffer: page-locked (the kernel stores into it) or pageable (copied)."""
    if not pinned:
        return np.zeros(n, np.uint8)
    import torch
    return torch.zeros(n, dtype=torch.uint8, pin_memory=True)


def as_array(img):
    return img if isinstance(img, np.ndarray) else img.numpy()


@pytest.mark.parametrize("image_memory, pinned", [(0, False), (0, True), (1, False), (1, True)])
def test_served_in_mix_equals_alone(cuda, worlds, image_memory, pinned):
    """Images stored by the kernel into page-locked memory (the request's own buffer, or the
    slot's and then copied to a pageable one), or rendered on the device and copied."""
    a, b = worlds
    wa, wb = make_world(a.words, a.W, a.H), make_world(b.words, b.W, b.H)
    views = scenes.batch_views(a, 10, seed=9, max_steps=256)
    views = [(u, w // 8 + 8, h // 8 + 6) for (u, w, h) in views]
    srv = make_server(image_memory=image_memory)
    ia, ib = add_world(srv, wa), add_world(srv, wb)
    outs = {}
    for i, (u, w, h) in enumerate(views):
        u.aspectRatio = w / h
        outs[i] = (host_image(w * h * 4, pinned), wa, u, w, h)
        submit_render(srv, ia, u, w, h, outs[i][0], i)
        ub2 = vrt.Uniforms.from_buffer_copy(b.uniforms)
        ub2.aspectRatio = 96 / 64
        outs[100 + i] = (host_image(96 * 64 * 4, pinned), wb, ub2, 96, 64)
        submit_render(srv, ib, ub2, 96, 64, outs[100 + i][0], 100 + i)
    done = collect(srv, len(outs))
    for tag, (img, world, u, w, h) in outs.items():
        assert done[tag].status == 0
        alone = gpu_render(world, u, w, h)
        assert np.array_equal(as_array(img).reshape(h, w, 4), alone["rgba"]), f"request {tag}"
        assert done[tag].rays == int(alone["stats"][vrt.STAT_RAYS])
        assert done[tag].done_ms >= done[tag].submit_ms
    vrt.lib().vrt_server_destroy(srv)


def test_edits_are_ordered_within_a_world(cuda, worlds):
    a, _ = worlds
    w = make_world(a.words, a.W, a.H)
    u = vrt.Uniforms.from_buffer_copy(a.uniforms)
    u.aspectRatio = 1.0
    cam = [int(v) for v in u.camPos]
    edit = ((cam[0], cam[1] - 3, cam[2]), 6)
    before = gpu_render(w, u, 48, 48)["rgba"]
    w2 = make_world(a.words, a.W, a.H)
    w2.remove_sphere(*edit[0], edit[1], 0)
    after = gpu_render(w2, u, 48, 48)["rgba"]
    assert not np.array_equal(before, after)
    srv = make_server(slots=4, max_batch=2)
    wid = add_world(srv, w)
    imgs = [np.zeros(48 * 48 * 4, np.uint8) for _ in range(6)]
    for i in range(3):
        submit_render(srv, wid, u, 48, 48, imgs[i], i)
    submit_edit(srv, wid, edit[0], edit[1], 50)
    for i in range(3, 6):
        submit_render(srv, wid, u, 48, 48, imgs[i], i)
    done = collect(srv, 7)
    assert done[50].status == 0
    for i in range(3):
        assert np.array_equal(imgs[i].reshape(48, 48, 4), before), f"render {i} saw the edit"
    for i in range(3, 6):
        assert np.array_equal(imgs[i].reshape(48, 48, 4), after), f"render {i} missed the edit"
    vrt.lib().vrt_server_destroy(srv)


def test_bad_configs_are_refused(cuda):
    for cfg in [(1 << 30, 0, 4, 0, 0), (1 << 30, 3, 0, 0, 0), (0, 3, 4, 0, 0), (1 << 30, 3, 4, -1, 0),
                (1 << 30, 3, 4, 0, 2), (1 << 30, 3, 4, 0, 0, -1)]:
        h = C.c_void_p()
        assert vrt.lib().vrt_server_create(C.byref(vrt.ServerConfig(*cfg)), C.byref(h)) == vrt.EINVAL, cfg
        assert not h.value


def test_budget_refuses_oversized_requests(cuda, worlds):
    _, b = worlds
    w = make_world(b.words, b.W, b.H)
    srv = make_server(budget=w.info().device_bytes + 64 * 64 * 4 * 2)
    wid = add_world(srv, w)
    small = np.zeros(64 * 64 * 4, np.uint8)
    submit_render(srv, wid, b.uniforms, 64, 64, small, 1)
    submit_render(srv, wid, b.uniforms, 640, 480, None, 2)  # larger than the whole budget
    done = collect(srv, 2)
    assert done[1].status == 0 and done[2].status == vrt.EBUDGET
    with pytest.raises(vrt.VrtError):
        big = make_world(np.full(128 * 64 * 128, -1, np.int32), 128, 64)
        add_world(srv, big)
    vrt.lib().vrt_server_destroy(srv)


def test_depth_field_world_served(cuda, oracle, vrt_lib):
    """A world in the reference's own format (with depth-field words) served with edits:
    renders before and after each edit equal the oracle on the words of that moment."""
    W, H = 64, 32
    w = make_world(vrt_lib.terrain_generate(W, H, 8, 2), W, H)
    w.fix_depth_field()
    srv = make_server(slots=2, max_batch=2)
    wid = add_world(srv, w)
    u = vrt.default_uniforms()
    u.camPos[:] = [20.5, 29.25, 14.5]
    u.rotateMatrix[:] = vrt.rotate_matrix(0.6, 0.5)
    u.lightPos[:] = [32.0, 300.0, 10.0]
    u.maxSteps = 120
    u.aspectRatio = 48 / 32
    edits = [(30, 14, 34, 5), (38, 12, 30, 4)]
    stages = [w.download(np.empty(W * H * W, np.int32))]
    shadow = vrt.World(W, H)  # replays the edits to know each stage's words
    shadow.upload(stages[0])
    for (x, y, z, r) in edits:
        shadow.remove_sphere(x, y, z, r, 1)
        stages.append(shadow.download(np.empty(W * H * W, np.int32)))
    outs, tag = {}, 0
    for stage in range(len(stages)):
        for _ in range(2):
            outs[tag] = (np.zeros(48 * 32 * 4, np.uint8), stage)
            submit_render(srv, wid, u, 48, 32, outs[tag][0], tag)
            tag += 1
        if stage < len(edits):
            submit_edit(srv, wid, edits[stage][:3], edits[stage][3], 1000 + stage)
    done = collect(srv, tag + len(edits))
    assert all(done[t].status == 0 for t in done)
    for t, (img, stage) in outs.items():
        o = oracle.render(stages[stage], W, H, u, 48, 32)
        assert np.array_equal(img.reshape(32, 48, 4), o["rgba"]), f"render {t} after {stage} edits"
    vrt.check(vrt.lib().vrt_server_destroy(srv))


def test_partial_batch_waits_for_company(cuda, worlds):
    """max_wait_us: a partial batch stays queued until it fills up (then it goes at once, as
    one launch) or until its oldest request has waited max_wait_us."""
    import time
    _, b = worlds
    w = make_world(b.words, b.W, b.H)
    u = vrt.Uniforms.from_buffer_copy(b.uniforms)
    u.aspectRatio = 1.0
    alone = gpu_render(w, u, 32, 32)["rgba"]
    srv = make_server(slots=2, max_batch=4, max_wait_us=2_000_000)
    wid = add_world(srv, w)
    imgs = [np.zeros(32 * 32 * 4, np.uint8) for _ in range(5)]
    buf = (vrt.Completion * 16)()
    for i in range(2):
        submit_render(srv, wid, u, 32, 32, imgs[i], i)
    assert vrt.check(vrt.lib().vrt_server_poll(srv, buf, 16)) == 0
    assert vrt.check(vrt.lib().vrt_server_wait(srv, 1000)) == 0  # nothing in flight
    for i in range(2, 4):
        submit_render(srv, wid, u, 32, 32, imgs[i], i)
    assert vrt.check(vrt.lib().vrt_server_poll(srv, buf, 16)) == 0  # launched, not done
    assert vrt.check(vrt.lib().vrt_server_wait(srv, 5_000_000)) == 1
    got = []
    while len(got) < 4:
        got += [buf[i] for i in range(vrt.check(vrt.lib().vrt_server_poll(srv, buf, 16)))]
        if len(got) < 4:
            vrt.check(vrt.lib().vrt_server_wait(srv, 100_000))
    assert len({c.start_ms for c in got}) == 1  # one launch
    vrt.lib().vrt_server_destroy(srv)
    srv = make_server(slots=2, max_batch=4, max_wait_us=30_000)
    wid = add_world(srv, w)
    submit_render(srv, wid, u, 32, 32, imgs[4], 4)
    t0 = time.perf_counter()
    done = collect(srv, 1)
    assert time.perf_counter() - t0 >= 0.025
    assert done[4].start_ms - done[4].submit_ms >= 29.0
    for img in imgs:
        assert np.array_equal(img.reshape(32, 32, 4), alone)
    vrt.lib().vrt_server_destroy(srv)


def test_pixel_cap_splits_launches(cuda, worlds):
    """max_batch_pixels: a launch gathers requests only while their pixels fit the cap (a
    larger request goes alone); every image still equals the one rendered alone."""
    _, b = worlds
    w = make_world(b.words, b.W, b.H)
    u = vrt.Uniforms.from_buffer_copy(b.uniforms)
    u.aspectRatio = 1.0
    sizes = [32, 32, 32, 32, 32, 80, 32]  # 1024-pixel requests and one of 6400
    alone = {n: gpu_render(w, u, n, n)["rgba"] for n in set(sizes)}
    srv = make_server(slots=1, max_batch=8, max_batch_pixels=2 * 32 * 32)
    wid = add_world(srv, w)
    imgs = [np.zeros(n * n * 4, np.uint8) for n in sizes]
    for i, n in enumerate(sizes):
        submit_render(srv, wid, u, n, n, imgs[i], i)
    done = collect(srv, len(sizes))
    launches = {}
    for tag, c in done.items():
        assert c.status == 0
        launches.setdefault(c.start_ms, []).append(sizes[tag])
    for members in launches.values():
        assert sum(m * m for m in members) <= 2 * 32 * 32 or len(members) == 1, launches
    assert any(members == [80] for members in launches.values())
    for i, n in enumerate(sizes):
        assert np.array_equal(imgs[i].reshape(n, n, 4), alone[n]), f"request {i}"
    vrt.lib().vrt_server_destroy(srv)


def test_add_world_while_another_thread_polls(cuda, worlds):
    """vrt_server_add_world may run on another thread while this one submits and polls: the
    world list grows under the server's lock and entries never move, so renders of the
    first world keep their results while worlds are being added."""
    import threading
    a, b = worlds
    w0 = make_world(b.words, b.W, b.H)
    extra = [make_world(b.words, b.W, b.H) for _ in range(24)]
    u = vrt.Uniforms.from_buffer_copy(b.uniforms)
    u.aspectRatio = 1.0
    alone = gpu_render(w0, u, 40, 40)["rgba"]
    srv = make_server(budget=8 << 30, slots=3, max_batch=2)
    wid = add_world(srv, w0)
    ids = []

    def adder():
        for w in extra:
            ids.append(add_world(srv, w))

    t = threading.Thread(target=adder)
    imgs = [np.zeros(40 * 40 * 4, np.uint8) for _ in range(40)]
    buf = (vrt.Completion * 64)()
    got = []
    t.start()
    for i, img in enumerate(imgs):
        submit_render(srv, wid, u, 40, 40, img, i)
        got += [buf[k] for k in range(vrt.check(vrt.lib().vrt_server_poll(srv, buf, 64)))]
    t.join()
    vrt.check(vrt.lib().vrt_server_drain(srv))
    while True:
        k = vrt.check(vrt.lib().vrt_server_poll(srv, buf, 64))
        got += [buf[i] for i in range(k)]
        if k == 0:
            break
    assert sorted(ids) == list(range(1, 25))
    assert len(got) == len(imgs) and all(c.status == 0 for c in got)
    for img in imgs:
        assert np.array_equal(img.reshape(40, 40, 4), alone)
    vrt.lib().vrt_server_destroy(srv)
