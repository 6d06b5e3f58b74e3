"""Shared test helpers: golden loading, GPU rendering through the C ABI, comparisons."""
from __future__ import annotations

import json
import os

import numpy as np

import vrt

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# The bar for the shader outputs.  Integer/index work is bit-exact; the north-star
# floating-point bar is RGB within 1/255 per channel, and this build is held to
# exact equality of the light multipliers and of the RGBA8 bytes as well.
RGB_TOL = 1


def load_golden(name: str):
    if name.endswith(".json"):
        with open(os.path.join(GOLDEN, name)) as f:
            return json.load(f)
    return dict(np.load(os.path.join(GOLDEN, name)))


def uniforms_from_dict(d: dict) -> vrt.Uniforms:
    u = vrt.default_uniforms()
    u.camPos[:] = d["camPos"]
    u.lightPos[:] = d["lightPos"]
    u.aspectRatio = d["aspectRatio"]
    u.rotateMatrix[:] = d["rotateMatrix"]
    for i in range(16):
        u.localLights[i][:] = d["localLights"][i]
    u.maxSteps = d["maxSteps"]
    u.localLightDist = d["localLightDist"]
    return u


def fcolor_from_outputs(words, hit, shade, primary_steps=None, depth_view=False):
    """fColor (fshader.glsl:133,144,184-187) rebuilt from hit index and multipliers."""
    hit = np.asarray(hit)
    word = words[np.maximum(hit, 0)]
    ch = np.stack([(word >> 16) & 255, (word >> 8) & 255, word & 255], -1).astype(np.float32)
    col = (ch / np.float32(255.0)) * shade.astype(np.float32)
    col[hit < 0] = np.array([0.6, 0.7, 0.8], np.float32)
    return col


DEBUG_OUTPUTS = ("hit", "cast", "occ", "steps", "primary_steps", "shade")
# the side outputs that leave a launch inexact (no step counts asked for): the launch the
# bench times, with its per-pixel results made visible
INEXACT_OUTPUTS = ("hit", "cast", "occ", "shade")


def gpu_render(world: vrt.World, u: vrt.Uniforms, width: int, height: int, kernel: int = vrt.KERNEL_AUTO,
               tile=None, refill_min: int = 0, renderer: vrt.Renderer | None = None, debug: bool = True,
               exact_steps: int = 0, outputs=None):
    """Render through the C ABI; with debug=True every debug output is requested (which
    makes step accounting exact), with debug=False only the image and the counters;
    outputs (a subset of DEBUG_OUTPUTS) requests just those side outputs."""
    import torch
    dev = torch.device("cuda")
    n = width * height
    rgba = torch.zeros(n * 4, dtype=torch.uint8, device=dev)
    hit = torch.full((n,), -7, dtype=torch.int32, device=dev)
    cast = torch.zeros(n, dtype=torch.int32, device=dev)
    occ = torch.zeros(n, dtype=torch.int32, device=dev)
    steps = torch.zeros(n, dtype=torch.int32, device=dev)
    psteps = torch.zeros(n, dtype=torch.int32, device=dev)
    shade = torch.zeros(n * 3, dtype=torch.float32, device=dev)
    stats = torch.zeros(vrt.STAT_COUNT, dtype=torch.int64, device=dev)
    want = set(DEBUG_OUTPUTS if outputs is None else outputs) if (debug or outputs is not None) else set()
    ptr = {"hit": hit, "cast": cast, "occ": occ, "steps": steps, "primary_steps": psteps, "shade": shade}
    dbg = vrt.DebugOut(*[ptr[k].data_ptr() if k in want else None for k in DEBUG_OUTPUTS]) if want else None
    opts = vrt.RenderOpts()
    opts.kernel = kernel
    opts.exact_steps = exact_steps
    if tile:
        opts.tile_w, opts.tile_h = tile
    opts.refill_min = refill_min
    r = renderer or vrt.Renderer()
    stream = torch.cuda.current_stream().cuda_stream
    r.render(world, u, width, height, rgba.data_ptr(), dbg, stats.data_ptr(), opts, stream)
    torch.cuda.synchronize()
    return {
        "rgba": rgba.cpu().numpy().reshape(height, width, 4),
        "hit": hit.cpu().numpy().reshape(height, width),
        "cast": cast.cpu().numpy().view(np.uint32).reshape(height, width),
        "occ": occ.cpu().numpy().view(np.uint32).reshape(height, width),
        "steps": steps.cpu().numpy().reshape(height, width),
        "primary_steps": psteps.cpu().numpy().reshape(height, width),
        "shade": shade.cpu().numpy().reshape(height, width, 3),
        "stats": stats.cpu().numpy().astype(np.uint64),
    }


def assert_same_frame(o: dict, g: dict, rows=None, outputs=DEBUG_OUTPUTS):
    """Oracle vs GPU: hit index, cast/occlusion bits and step counts bit-exact; light
    multipliers bit-exact; RGBA8 within RGB_TOL (and in practice equal).  outputs names
    the side outputs the GPU render was asked for (the image is always compared)."""
    sel = slice(None) if rows is None else rows
    for key in [k for k in ("hit", "cast", "occ", "steps", "primary_steps") if k in outputs]:
        a, b = np.asarray(o[key])[sel], np.asarray(g[key])[sel]
        bad = np.argwhere(a != b)
        assert bad.size == 0, f"{key}: {len(bad)} mismatches, first at {bad[:3].tolist()}: {a[tuple(bad[0])]} vs {b[tuple(bad[0])]}"
    if "shade" in outputs:
        a = np.asarray(o["shade"])[sel].view(np.uint32)
        b = np.asarray(g["shade"])[sel].view(np.uint32)
        assert np.array_equal(a, b), f"shade: {(a != b).any(-1).sum()} pixels differ"
    da = np.abs(np.asarray(o["rgba"])[sel].astype(np.int32) - np.asarray(g["rgba"])[sel].astype(np.int32))
    assert da.max(initial=0) <= RGB_TOL, f"rgba differs by {da.max()}"
    assert np.array_equal(np.asarray(o["rgba"])[sel], np.asarray(g["rgba"])[sel])


def make_world(words: np.ndarray, W: int, H: int) -> vrt.World:
    w = vrt.World(W, H)
    w.upload(np.ascontiguousarray(words, np.int32))
    return w


_W64 = (np.uint64(1) << np.arange(64, dtype=np.uint64)).reshape(4, 4, 4)  # [dz][dy][dx] -> bit dx+4dy+16dz


def _pack(cells):
    """cells [..., 4(z), 4(y), 4(x)] bool -> uint64 with bit x + 4y + 16z."""
    return (cells.astype(np.uint64) * _W64).sum(axis=(-3, -2, -1), dtype=np.uint64)


def expected_masks(words, W, H):
    """The occupancy hierarchy of a world, in the device's storage order:
    supers[sx + SW*(sy + SH*sz)], regions[super*64 + local], bricks[bx + BWp*(by + BHp*bz)]
    with BWp = 16*SW, BHp = 16*SH; local = x + 4y + 16z of the child inside its parent,
    voxel bit x + 4y + 16z."""
    SW, SH = (W + 63) // 64, (H + 63) // 64
    PW, PH = 64 * SW, 64 * SH
    solid = np.zeros((PW, PH, PW), bool)  # [z][y][x]
    solid[:W, :H, :W] = words.reshape(W, H, W) >= 0
    B = _pack(solid.reshape(PW // 4, 4, PH // 4, 4, PW // 4, 4).transpose(0, 2, 4, 1, 3, 5))  # [bz][by][bx]
    R = _pack((B != 0).reshape(PW // 16, 4, PH // 16, 4, PW // 16, 4).transpose(0, 2, 4, 1, 3, 5))
    S = _pack((R != 0).reshape(SW, 4, SH, 4, SW, 4).transpose(0, 2, 4, 1, 3, 5))
    supers = S.reshape(-1)
    regions = R.reshape(SW, 4, SH, 4, SW, 4).transpose(0, 2, 4, 1, 3, 5).reshape(-1)
    bricks = B.reshape(-1)  # linear: bx + BWp*(by + BHp*bz)
    return bricks, regions, supers


def _first_nonempty_cube(occ, signs, centred, cap=15):
    """For every node of the boolean grid occ [z][y][x]: the smallest k in [0, cap) such
    that the cube of radius k around the node (centred) or from the node k nodes along
    `signs` (+1/-1 per axis x, y, z) holds a non-empty node, else cap.  Counts come from a
    summed-area table, clipped to the grid."""
    nz, ny, nx = occ.shape
    sat = np.zeros((nz + 1, ny + 1, nx + 1), np.int64)
    sat[1:, 1:, 1:] = occ.astype(np.int64).cumsum(0).cumsum(1).cumsum(2)
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    out = np.full(occ.shape, cap, np.uint8)
    done = np.zeros(occ.shape, bool)
    for k in range(cap):
        lo, hi = [], []
        for c, n, sg in ((x, nx, signs[0]), (y, ny, signs[1]), (z, nz, signs[2])):
            a = c - k if (centred or sg < 0) else c
            b = c + k if (centred or sg > 0) else c
            lo.append(np.clip(a, 0, n - 1))
            hi.append(np.clip(b, 0, n - 1) + 1)
        (x0, y0, z0), (x1, y1, z1) = lo, hi
        cnt = (sat[z1, y1, x1] - sat[z0, y1, x1] - sat[z1, y0, x1] - sat[z1, y1, x0] + sat[z0, y0, x1] +
               sat[z0, y1, x0] + sat[z1, y0, x0] - sat[z0, y0, x0])
        new = (cnt > 0) & ~done
        out[new] = k
        done |= new
    return out


def expected_distances(words, W, H):
    """The device's distance fields: (brick_dir, region_dist).  brick_dir holds 8 bytes per
    brick in brick-mask order; byte o is the capped (15) Chebyshev distance to the nearest
    non-empty brick in octant o (bit a of o set: coordinates >= the brick's along axis a).
    region_dist is the capped centred distance of each region, rx + RWp*(ry + RHp*rz)."""
    bricks, regions, _ = expected_masks(words, W, H)
    SW, SH = (W + 63) // 64, (H + 63) // 64
    occ_b = (bricks != 0).reshape(16 * SW, 16 * SH, 16 * SW)  # [bz][by][bx]
    bdir = np.empty(occ_b.shape + (8,), np.uint8)
    for o in range(8):
        signs = tuple(1 if (o >> a) & 1 else -1 for a in range(3))
        bdir[..., o] = _first_nonempty_cube(occ_b, signs, False)
    # regions: super*64 + local -> [rz][ry][rx]
    r = (regions != 0).reshape(SW, SH, SW, 4, 4, 4).transpose(0, 3, 1, 4, 2, 5).reshape(4 * SW, 4 * SH, 4 * SW)
    rdist = _first_nonempty_cube(r, (1, 1, 1), True)
    return bdir.reshape(-1), rdist.reshape(-1)


def expected_distances_brute(words, W, H):
    """Brute-force form of expected_distances (every pair of nodes), for tiny worlds."""
    bricks, regions, _ = expected_masks(words, W, H)
    SW, SH = (W + 63) // 64, (H + 63) // 64
    BW, BH = 16 * SW, 16 * SH
    ne = [(x, y, z) for z in range(BW) for y in range(BH) for x in range(BW) if bricks[x + BW * (y + BH * z)]]
    bdir = np.full(BW * BH * BW * 8, 15, np.uint8)
    for z in range(BW):
        for y in range(BH):
            for x in range(BW):
                for (a, b, c) in ne:
                    d = (a - x, b - y, c - z)
                    o = (d[0] >= 0) | ((d[1] >= 0) << 1) | ((d[2] >= 0) << 2)
                    dist = min(15, max(abs(v) for v in d))
                    # a zero component lies in both half-spaces of its axis
                    for oo in range(8):
                        if all(((oo >> i) & 1) == ((o >> i) & 1) or d[i] == 0 for i in range(3)):
                            j = 8 * (x + BW * (y + BH * z)) + oo
                            bdir[j] = min(bdir[j], dist)
    RW, RH = 4 * SW, 4 * SH
    nr = []
    for i, m in enumerate(regions):
        if m:
            s, l = divmod(i, 64)
            sx, sy, sz = s % SW, (s // SW) % SH, s // (SW * SH)
            nr.append((4 * sx + (l & 3), 4 * sy + ((l >> 2) & 3), 4 * sz + (l >> 4)))
    rdist = np.full(RW * RH * RW, 15, np.uint8)
    for z in range(RW):
        for y in range(RH):
            for x in range(RW):
                for (a, b, c) in nr:
                    j = x + RW * (y + RH * z)
                    rdist[j] = min(rdist[j], min(15, max(abs(a - x), abs(b - y), abs(c - z))))
    return bdir, rdist


def expected_masks_loops(words, W, H):
    """Slow loop form of expected_masks, for checking it on tiny worlds."""
    SW, SH = (W + 63) // 64, (H + 63) // 64
    bricks = np.zeros(64 * 64 * SW * SH * SW, np.uint64)
    regions = np.zeros(64 * SW * SH * SW, np.uint64)
    for z in range(W):
        for y in range(H):
            for x in range(W):
                if words[x + W * y + W * H * z] < 0:
                    continue
                bx, by, bz = x >> 2, y >> 2, z >> 2
                rx, ry, rz = bx >> 2, by >> 2, bz >> 2
                sx, sy, sz = rx >> 2, ry >> 2, rz >> 2
                si = sx + SW * (sy + SH * sz)
                ri = si * 64 + (rx & 3) + 4 * (ry & 3) + 16 * (rz & 3)
                bi = bx + 16 * SW * (by + 16 * SH * bz)
                bricks[bi] |= np.uint64(1) << np.uint64((x & 3) + 4 * (y & 3) + 16 * (z & 3))
                regions[ri] |= np.uint64(1) << np.uint64((bx & 3) + 4 * (by & 3) + 16 * (bz & 3))
    supers = np.zeros(SW * SH * SW, np.uint64)
    for i in range(supers.size):
        for c in range(64):
            if regions[i * 64 + c]:
                supers[i] |= np.uint64(1) << np.uint64(c)
    return bricks, regions, supers
