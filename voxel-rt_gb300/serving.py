"""Open-loop request driver for the vrt server (vrt_server_*): Poisson arrivals of render
and edit requests over resident worlds, latency percentiles and throughput.

Requests: 90% renders at 640x360, 1280x720 or 1920x1080 with a random surface camera
and 0-16 of the world's lights; 10% edits that remove a sphere of radius 1-8 at a
surface point (removeSphere, level.cpp:30-56).  Arrivals are generated on the host
clock and submitted when due; in between, the driver waits on the server
(vrt_server_wait: until a launch finishes or the next arrival is due) and polls, so
requests that arrive while others run are admitted as slots and memory free up.
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

import scenes
import vrt

RESOLUTIONS = [(640, 360), (1280, 720), (1920, 1080)]


class Server:
    def __init__(self, budget_bytes: int, slots: int = 4, max_batch: int = 8, max_wait_us: int = 0,
                 image_memory: int = 0, max_batch_pixels: int = 0):
        cfg = vrt.ServerConfig(budget_bytes, slots, max_batch, max_wait_us, image_memory, max_batch_pixels)
        self.h = C.c_void_p()
        vrt.check(vrt.lib().vrt_server_create(C.byref(cfg), C.byref(self.h)))
        self._buf = (vrt.Completion * 512)()

    def add_world(self, world: vrt.World) -> int:
        wid = C.c_int32()
        vrt.check(vrt.lib().vrt_server_add_world(self.h, world.handle, C.byref(wid)))
        return wid.value

    def submit(self, req: vrt.Request):
        vrt.check(vrt.lib().vrt_server_submit(self.h, C.byref(req)))

    def poll(self):
        n = vrt.check(vrt.lib().vrt_server_poll(self.h, self._buf, 512))
        return [vrt.Completion.from_buffer_copy(self._buf[i]) for i in range(n)]

    def drain(self):
        vrt.check(vrt.lib().vrt_server_drain(self.h))
        out = []
        while True:
            got = self.poll()
            if not got:
                return out
            out += got

    def wait(self, timeout_us: int) -> bool:
        """True when a launch in flight has finished (poll retires it)."""
        return vrt.check(vrt.lib().vrt_server_wait(self.h, int(timeout_us))) == 1

    def now_ms(self) -> float:
        return vrt.lib().vrt_server_now_ms(self.h)

    def close(self):
        if self.h:
            vrt.lib().vrt_server_destroy(self.h)
            self.h = None


class WorldSpec:
    def __init__(self, scene: scenes.Scene, world: vrt.World):
        self.scene = scene
        self.world = world


def make_requests(specs, rate_hz: float, duration_s: float, seed: int):
    """(arrival_s, kind, world_index, payload) sorted by arrival."""
    rng = scenes.SplitMix64(seed)
    t = 0.0
    out = []
    while True:
        t += -math.log(max(1e-12, 1.0 - rng.uniform())) / rate_hz
        if t >= duration_s:
            return out
        wi = rng.randint(0, len(specs) - 1)
        sc = specs[wi].scene
        if rng.uniform() < 0.9:
            w, h = RESOLUTIONS[rng.randint(0, 2)]
            u = scenes.base_uniforms(w, h, sc.uniforms.maxSteps, 70.0, sc.uniforms.localLightDist)
            scenes.set_lights(u, sc.lights[: rng.randint(0, 16)])
            scenes.aim(u, scenes.surface_camera(rng, sc.W, sc.seed), rng.uniform(0, 360), rng.uniform(-30, 0))
            u.lightPos[:] = list(sc.uniforms.lightPos)
            out.append((t, vrt.REQ_RENDER, wi, (u, w, h)))
        else:
            x, z = rng.randint(0, sc.W - 1), rng.randint(0, sc.W - 1)
            y = vrt.terrain_height(sc.W, sc.seed, x, z) - 1
            out.append((t, vrt.REQ_EDIT, wi, (x, y, z, rng.randint(1, 8))))


def run_open_loop(server: Server, wids, requests, keep_images: bool = False):
    """Submit requests at their arrival times; returns completions and wall seconds."""
    t0 = time.perf_counter()
    done = []
    tags = {}
    i = 0
    n = len(requests)
    while i < n:
        now = time.perf_counter() - t0
        while i < n and requests[i][0] <= now:
            _, kind, wi, payload = requests[i]
            q = vrt.Request()
            q.kind = kind
            q.world_id = wids[wi]
            q.user_tag = i
            if kind == vrt.REQ_RENDER:
                u, w, h = payload
                q.uniforms = u
                q.width, q.height = w, h
                q.host_rgba = None
            else:
                q.cx, q.cy, q.cz, q.radius = payload
            server.submit(q)
            tags[i] = kind
            i += 1
        done += server.poll()
        if i < n:
            wait = requests[i][0] - (time.perf_counter() - t0)
            # until a launch finishes or the next request is due; with nothing in flight,
            # sleep in short steps (a late wake-up then stays small)
            if wait > 0 and not server.wait(min(wait, 0.002) * 1e6):
                left = requests[i][0] - (time.perf_counter() - t0)
                if left > 0.0002:
                    time.sleep(min(left - 0.0001, 0.0005))
    done += server.drain()
    wall = time.perf_counter() - t0
    return done, wall


def summarize(done, wall_s: float):
    lat = np.array([c.done_ms - c.submit_ms for c in done if c.kind == vrt.REQ_RENDER and c.status == 0])
    rays = sum(int(c.rays) for c in done if c.kind == vrt.REQ_RENDER and c.status == 0)
    refused = sum(1 for c in done if c.status != 0)
    if lat.size == 0:
        return {"renders": 0}
    return {
        "renders": int(lat.size),
        "edits": int(sum(1 for c in done if c.kind == vrt.REQ_EDIT)),
        "refused": refused,
        "p50_ms": float(np.percentile(lat, 50)),
        "p99_ms": float(np.percentile(lat, 99)),
        "mrays_per_s": rays / wall_s / 1e6,
        "wall_s": wall_s,
    }
