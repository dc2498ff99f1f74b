"""The benchmarked frame sequences, several consecutive frames, against the
oracle on crops of the configurations' own frame sizes.

The GPU renders whole 1920x1080 frames in the benchmark's pass order (RIS with
visibility and temporal reuse, then the chained unbiased spatial passes, then
shading; reservoir buffers ping-pong as in bench.py's step).  The oracle
evaluates each stage only on the region it needs for the last frame's crop to
be exact, working backwards in time:

  * a spatial pass reads neighbours within R pixels, so the stage before it
    is evaluated on its region grown by R + 1 on every side;
  * temporal reuse reads the previous frame's reservoirs at the reprojected
    pixel (src/shaders/restirOmni.glsl:162-209), so the previous frame's
    final region is the bounding box of the previous-frame pixels that this
    frame's RIS region may read (_reprojection_box).

Every stage of every frame is then compared bit for bit on its region:
reservoir words (sample, light index, p-hat, sum of weights, W, M) and the
shaded image.  The oracle runs on its own outputs from the first frame on;
nothing of the GPU's reservoirs enters it.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_binding as ob
from helpers import crop_mask, mismatch, new_res, image_bits

pytestmark = pytest.mark.gpu


def _grow(region, d, w, h):
    x0, y0, cw, ch = region
    a, b = max(x0 - d, 0), max(y0 - d, 0)
    c, e = min(x0 + cw + d, w), min(y0 + ch + d, h)
    return (a, b, c - a, e - b)


def _reprojection_box(scene, frame, g_cur, g_prev, region):
    """Bounding box (x, y, w, h) of the previous-frame pixels whose reservoirs
    temporal reuse of `frame` may read for the pixels of `region`: the
    reprojected pixel and its 8 neighbours (float rounding of the
    reprojection), kept where the world-position and normal similarity tests
    (src/shaders/restirOmni.glsl:178-184) pass with a margin.  The reservoir is read only
    when those tests pass, so a pixel that reprojects far away (a surface
    nearer than the previous camera's near plane, behind it) costs nothing."""
    w, h = scene.width, scene.height
    m = np.array(scene.uniforms(frame).prev_frame_projection_view[:], np.float64)
    x0, y0, cw, ch = region
    p = g_cur["world_pos"][y0:y0 + ch, x0:x0 + cw, :3].reshape(-1, 3).astype(np.float64)
    n = _normals(g_cur)[y0:y0 + ch, x0:x0 + cw].reshape(-1, 3)
    px = m[0] * p[:, 0] + m[4] * p[:, 1] + m[8] * p[:, 2] + m[12]
    py = m[1] * p[:, 0] + m[5] * p[:, 1] + m[9] * p[:, 2] + m[13]
    pw = m[3] * p[:, 0] + m[7] * p[:, 1] + m[11] * p[:, 2] + m[15]
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        px = (px / pw + 1.0) * 0.5 * w
        py = (py / pw + 1.0) * 0.5 * h
    ok = np.isfinite(px) & np.isfinite(py) & (px > -2) & (py > -2) & (px < w + 2) & (py < h + 2)
    fx0 = np.floor(px[ok]).astype(np.int64)
    fy0 = np.floor(py[ok]).astype(np.int64)
    p, n = p[ok], n[ok]
    wp_prev = g_prev["world_pos"][..., :3].astype(np.float64)
    n_prev = _normals(g_prev)
    xs, ys = [], []
    for a in (-1, 0, 1):
        for b in (-1, 0, 1):
            fx, fy = np.clip(fx0 + a, 0, w - 1), np.clip(fy0 + b, 0, h - 1)
            dp = p - wp_prev[fy, fx]
            keep = (np.sum(dp * dp, axis=1) < 0.0105) & (np.sum(n * n_prev[fy, fx], axis=1) > 0.49)
            xs.append(fx[keep])
            ys.append(fy[keep])
    xs, ys = np.concatenate(xs), np.concatenate(ys)
    if len(xs) == 0:
        return None
    a, b = int(xs.min()), int(ys.min())
    return (a, b, int(xs.max()) + 1 - a, int(ys.max()) + 1 - b)


def _normals(g):
    return g["normal"][..., :3].view(np.float16).astype(np.float64)


def _union(r1, r2):
    if r1 is None:
        return r2
    if r2 is None:
        return r1
    a, b = min(r1[0], r2[0]), min(r1[1], r2[1])
    c, e = max(r1[0] + r1[2], r2[0] + r2[2]), max(r1[1] + r1[3], r2[1] + r2[3])
    return (a, b, c - a, e - b)


def _regions(scene, gs, frames, crop):
    """Per frame: [RIS region, pass 0 region, ..., final region]."""
    w, h = scene.width, scene.height
    halo = int(scene.radius) + 1
    npass = scene.spatial_passes
    out = [None] * frames
    final = crop
    for f in range(frames - 1, -1, -1):
        regs = [_grow(final, halo * (npass - k), w, h) for k in range(npass + 1)]
        out[f] = regs
        if f > 0:
            final = _union(_reprojection_box(scene, f, gs[f], gs[f - 1], regs[0]), crop)
    return out


def _gpu_frames(ctx, scene, dgs, frames, cuda):
    """The benchmark's frame loop (bench.py step) over frames 0..frames-1: per
    frame the reservoirs after every stage and the image."""
    from restir_gb300.passes import reservoirs, reservoirs_to_numpy
    n = scene.width * scene.height
    res = [reservoirs(n), reservoirs(n)]
    tmp = reservoirs(n)
    image = cuda.zeros((scene.height, scene.width, 4), dtype=cuda.float32, device="cuda")
    out = []
    for f in range(frames):
        slot = f % 2
        cur, prev = res[slot], res[1 - slot]
        u = scene.uniforms(f)
        passes = scene.spatial_passes
        first = tmp if passes % 2 == 1 else cur
        ctx.initial_temporal(dgs[f], dgs[f - 1] if f else None, prev, first, u)
        stages = [reservoirs_to_numpy(first)]
        src = first
        for p in range(passes):
            dst = cur if src is tmp else tmp
            ctx.spatial_unbiased(dgs[f], src, dst, u, scene.neighbors, p)
            stages.append(reservoirs_to_numpy(dst))
            src = dst
        assert src is cur
        ctx.shade(dgs[f], cur, scene.lighting_uniforms(f), image)
        out.append((stages, image.cpu().numpy().copy()))
    return out


def _oracle_frames(scene, gs, regions):
    n = scene.width * scene.height
    prev = None
    out = []
    for f, regs in enumerate(regions):
        u = scene.uniforms(f)
        r = new_res(n)
        ob.initial_temporal(scene, gs[f], gs[f - 1] if f else None, prev if f else None, r, u, crop=regs[0])
        stages = [r]
        for p in range(scene.spatial_passes):
            o = new_res(n)
            ob.spatial_unbiased(scene, gs[f], r, o, u, scene.neighbors, p, crop=regs[p + 1])
            r = o
            stages.append(r)
        img = np.zeros((scene.height, scene.width, 4), np.float32)
        ob.shade(scene, gs[f], r, scene.lighting_uniforms(f), img, crop=regs[-1])
        out.append((stages, img))
        prev = r
    return out


def _check_sequence(ctx, scene, dgs, gs, frames, crops, cuda):
    got = _gpu_frames(ctx, scene, dgs, frames, cuda)
    w, h = scene.width, scene.height
    for crop in crops:
        regions = _regions(scene, gs, frames, crop)
        exp = _oracle_frames(scene, gs, regions)
        for f in range(frames):
            for k, region in enumerate(regions[f]):
                mask = crop_mask(w, h, region)
                bad = mismatch(got[f][0][k], exp[f][0][k], mask)
                assert bad == 0, f"crop {crop} frame {f} stage {k} region {region}: {bad} reservoirs differ"
            fin = crop_mask(w, h, regions[f][-1]).reshape(h, w)
            gi, ei = got[f][1][fin], exp[f][1][fin]
            assert np.array_equal(image_bits(gi), image_bits(ei)), f"crop {crop} frame {f}: image differs"
        last = got[frames - 1][0][-1]
        m = crop_mask(w, h, crop)
        assert np.mean(last["w"][m] > 0) > 0.3  # lit, not a trivially empty crop
    # temporal reuse merged history somewhere in every later frame (M above the
    # RIS candidate count); near the frame's edges new content may have none
    for f in range(1, frames):
        assert np.mean(got[f][0][0]["m"] > scene.candidates) > 0.1, f"frame {f}: no temporal reuse"


@pytest.fixture(scope="module")
def cfg3_seq(restir_lib, cuda, ctx):
    from restir_gb300 import scenes
    from restir_gb300.passes import DeviceGBuffer
    s = scenes.config3(frames=4)
    ctx.upload_scene(s)
    dgs = []
    for f in range(s.frames):
        d = DeviceGBuffer(s.width, s.height)
        ctx.trace_gbuffer(s.cameras[f], d)
        dgs.append(d)
    return s, dgs, [d.to_host() for d in dgs]


def test_config3_four_frames_full_sequence_on_crops(ctx, cuda, cfg3_seq):
    """Config 3 (1920x1080, 1,048,588 triangles, 1,048,576 clustered lights):
    frames 0..3 of RIS + visibility + temporal, 3 chained unbiased passes
    (pass indices 0, 1, 2, k = 5, R = 30) and shading, on three 64x64 crops
    (top-left corner, centre, bottom-right corner)."""
    s, dgs, gs = cfg3_seq
    ctx.upload_scene(s)
    _check_sequence(ctx, s, dgs, gs, s.frames, [(0, 0, 64, 64), (928, 508, 64, 64), (1856, 1016, 64, 64)], cuda)


@pytest.fixture(scope="module")
def cfg2_seq(restir_lib, cuda, ctx):
    from restir_gb300 import scenes
    from restir_gb300.passes import DeviceGBuffer
    s = scenes.config2()
    ctx.upload_scene(s)
    dgs = []
    for f in range(s.frames):
        d = DeviceGBuffer(s.width, s.height)
        ctx.trace_gbuffer(s.cameras[f], d)
        dgs.append(d)
    return s, dgs, [d.to_host() for d in dgs]


def test_config2_eight_frames_at_1080p_on_crops(ctx, cuda, cfg2_seq):
    """Config 2 at its own size (1920x1080, 100k triangles, 65,536 lights) for
    its 8 frames: RIS + visibility + temporal, 2 unbiased passes, shading, on
    the centre crop and a corner crop."""
    s, dgs, gs = cfg2_seq
    assert (s.width, s.height, s.frames) == (1920, 1080, 8)
    ctx.upload_scene(s)
    _check_sequence(ctx, s, dgs, gs, s.frames, [(928, 508, 64, 64), (1856, 0, 64, 64)], cuda)
