"""CUDA path against the oracle, through the C ABI, on identical inputs.

Bar: bit-exact.  Visibility bits, selected light indices, W, M, sum of
weights and p-hat of every reservoir and every shaded pixel must equal the
oracle's, because both sides evaluate the same operations in the same order
without FMA contraction, with IEEE division/sqrt and the same PCG32 streams.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_binding as ob
from helpers import crop_mask, mismatch, new_res, oracle_frame, image_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cfg1(restir_lib):
    from restir_gb300 import scenes
    s = scenes.config1()
    return s, scenes.trace_gbuffer_host(s, 0)


@pytest.fixture(scope="module")
def cfg2_small(restir_lib):
    from restir_gb300 import scenes
    s = scenes.config2(width=320, height=180, frames=3)
    return s, [scenes.trace_gbuffer_host(s, f) for f in range(s.frames)]


def _dev(ctx, s, g):
    from restir_gb300.passes import DeviceGBuffer
    ctx.upload_scene(s)
    return DeviceGBuffer.from_host(g)


def test_visibility_batch_bit_exact(ctx, cfg1, cuda):
    s, g = cfg1
    ctx.upload_scene(s)
    rng = np.random.default_rng(5)
    n = 200_000
    wp = g["world_pos"].reshape(-1, 4)
    p1 = wp[rng.integers(0, len(wp), n)].copy()
    p2 = np.zeros_like(p1)
    p2[:, :3] = s.point_lights["pos"][rng.integers(0, len(s.point_lights), n), :3]
    p2[: n // 4, :3] = rng.uniform(-0.1, 1.1, (n // 4, 3))  # arbitrary segments, some leaving the room
    p2[::1000] = p1[::1000]                                 # zero-length segments
    torch = cuda
    d1 = torch.from_numpy(p1).cuda()
    d2 = torch.from_numpy(p2).cuda()
    out = torch.zeros(n, dtype=torch.uint8, device="cuda")
    ctx.stats(reset=True)
    ctx.visibility_batch(d1, d2, out)
    got = out.cpu().numpy()
    exp = np.zeros(n, np.uint8)
    sc, keep = ob.scene_struct(s)
    import ctypes as C
    p1c = np.ascontiguousarray(p1[:, :3])
    p2c = np.ascontiguousarray(p2[:, :3])
    ob.oracle().or_test_visibility_batch(C.byref(sc), n, ob.P(p1c), ob.P(p2c), ob.P(exp), None)
    assert np.array_equal(got, exp), f"{np.count_nonzero(got != exp)} of {n} visibility bits differ"
    assert 0.02 < exp.mean() < 0.98
    st = ctx.stats()
    assert st.rays_traced == n and st.traversal_errors == 0


@pytest.mark.parametrize("name,frames", [("config1", [0]), ("config2", [0, 7]), ("config3", [0, 15])])
def test_gbuffer_gpu_equals_oracle(ctx, cuda, name, frames):
    """k_trace_gbuffer against the oracle's independent primary-ray G-buffer
    (or_trace_gbuffer: gBuffer.frag's planes for one closest-hit ray per
    pixel centre, camera.h's convention), every plane byte for byte, at the
    configurations' own sizes."""
    from restir_gb300 import scenes
    from restir_gb300.passes import DeviceGBuffer
    s = scenes.CONFIGS[name]()
    ctx.upload_scene(s)
    d = DeviceGBuffer(s.width, s.height)
    for f in frames:
        ctx.trace_gbuffer(s.cameras[f], d)
        got = d.to_host()
        exp = ob.trace_gbuffer(s, f)
        for k in exp:
            assert np.array_equal(got[k].reshape(exp[k].shape).view(np.uint8), exp[k].view(np.uint8)), (name, f, k)


def test_config1_frame_bit_exact(ctx, cfg1, cuda):
    """RIS + visibility reuse, biased spatial (2 dispatches), shading."""
    from restir_gb300.passes import reservoirs, reservoirs_from_numpy, reservoirs_to_numpy
    s, g = cfg1
    dg = _dev(ctx, s, g)
    n = s.width * s.height
    stages, img = oracle_frame(s, 0, g, None, None)
    u = s.uniforms(0)
    r0 = reservoirs(n)
    ctx.initial_temporal(dg, None, None, r0, u)
    got0 = reservoirs_to_numpy(r0)
    assert mismatch(got0, stages[0]) == 0
    # the spatial pass from identical inputs
    r1 = reservoirs(n)
    r2 = reservoirs(n)
    ctx.spatial_biased(dg, r0, r1, u, 0)
    ctx.spatial_biased(dg, r1, r2, u, 1)
    got = reservoirs_to_numpy(r2)
    assert mismatch(got, stages[-1]) == 0
    out = cuda.zeros((s.height, s.width, 4), dtype=cuda.float32, device="cuda")
    ctx.shade(dg, r2, s.lighting_uniforms(0), out)
    gi = out.cpu().numpy()
    assert np.array_equal(image_bits(gi), image_bits(img))
    # shading from a reservoir buffer the oracle produced
    out2 = cuda.zeros_like(out)
    ctx.shade(dg, reservoirs_from_numpy(stages[-1]), s.lighting_uniforms(0), out2)
    assert np.array_equal(image_bits(out2.cpu().numpy()), image_bits(img))


def test_frame_sequence_unbiased_temporal_bit_exact(ctx, cfg2_small, cuda):
    """Three frames of config 2's pass order (temporal + 2 unbiased passes, k=5)
    through the frame driver, against the oracle run on the same wiring."""
    from restir_gb300.passes import DeviceGBuffer, reservoirs_to_numpy
    s, gs = cfg2_small
    ctx.upload_scene(s)
    n = s.width * s.height
    dgs = [DeviceGBuffer.from_host(g) for g in gs]
    prev_res = new_res(n)
    for f in range(s.frames):
        stages, img = oracle_frame(s, f, gs[f], gs[f - 1] if f else None, prev_res)
        out = cuda.zeros((s.height, s.width, 4), dtype=cuda.float32, device="cuda")
        ctx.render_frame(dgs[f], dgs[f - 1] if f else None, f % 2, s.frame_params(f), out)
        from restir_gb300.passes import device_view
        got = device_view(ctx.frame_reservoirs_ptr(f % 2), n * 64).cpu().numpy().view(stages[-1].dtype)
        assert mismatch(got, stages[-1]) == 0, f"frame {f}"
        assert np.array_equal(image_bits(out.cpu().numpy()), image_bits(img)), f"frame {f}"
        prev_res = stages[-1]


def test_unbiased_pass_counts_rays(ctx, cfg2_small, cuda):
    from restir_gb300.passes import DeviceGBuffer, reservoirs, reservoirs_from_numpy, reservoirs_to_numpy
    s, gs = cfg2_small
    ctx.upload_scene(s)
    n = s.width * s.height
    g = gs[0]
    u = s.uniforms(0)
    r0 = new_res(n)
    ob.initial_temporal(s, g, None, None, r0, u)
    st = ob.Stats()
    r1 = new_res(n)
    ob.spatial_unbiased(s, g, r0, r1, u, 3, 0, stats=st)  # the reference's NUM_NEIGHBORS
    dg = DeviceGBuffer.from_host(g)
    out = reservoirs(n)
    ctx.set_visibility_cache(False)
    try:
        ctx.stats(reset=True)
        ctx.spatial_unbiased(dg, reservoirs_from_numpy(r0), out, u, 3, 0)
    finally:
        ctx.set_visibility_cache(True)
    assert mismatch(reservoirs_to_numpy(out), r1) == 0
    # every segment whose answer reaches the output is traced; a neighbour's
    # segment whose pixel's own segment is shadowed may be skipped (the count
    # is reset whatever it answers), depending on which finishes first
    got = ctx.stats().rays_traced
    assert st.rays - st.rays_unobservable <= got <= st.rays, (got, st.rays, st.rays_unobservable)
    assert st.rays_unobservable > 0


@pytest.mark.parametrize("crop", [(0, 0, 64, 64), (928, 508, 64, 64), (1856, 1016, 64, 64)])
def test_config3_full_size_crops_bit_exact(ctx, cuda, crop, cfg3_full):
    """1080p, 1,048,588 triangles, 1,048,576 clustered lights: every pass on
    identical inputs; the oracle evaluates only the crop."""
    from restir_gb300.passes import DeviceGBuffer, reservoirs, reservoirs_from_numpy, reservoirs_to_numpy
    s, g0, g1, dg0, dg1 = cfg3_full
    ctx.upload_scene(s)
    n = s.width * s.height
    mask = crop_mask(s.width, s.height, crop)
    # frame 0 on the GPU provides previous reservoirs for frame 1's temporal reuse
    prev = reservoirs(n)
    ctx.initial_temporal(dg0, None, None, prev, s.uniforms(0))
    prev_np = reservoirs_to_numpy(prev)
    u = s.uniforms(1)
    r = reservoirs(n)
    ctx.initial_temporal(dg1, dg0, prev, r, u)
    exp = new_res(n)
    ob.initial_temporal(s, g1, g0, prev_np, exp, u, crop=crop)
    got = reservoirs_to_numpy(r)
    assert mismatch(got, exp, mask) == 0
    # one unbiased pass from the GPU's reservoirs
    o = reservoirs(n)
    ctx.spatial_unbiased(dg1, r, o, u, s.neighbors, 1)
    exp2 = new_res(n)
    ob.spatial_unbiased(s, g1, got, exp2, u, s.neighbors, 1, crop=crop)
    assert mismatch(reservoirs_to_numpy(o), exp2, mask) == 0


@pytest.fixture(scope="module")
def cfg3_full(restir_lib, cuda, ctx):
    from restir_gb300 import scenes
    from restir_gb300.passes import DeviceGBuffer
    s = scenes.config3(frames=2)
    ctx.upload_scene(s)
    dg0 = DeviceGBuffer(s.width, s.height)
    dg1 = DeviceGBuffer(s.width, s.height)
    ctx.trace_gbuffer(s.cameras[0], dg0)
    ctx.trace_gbuffer(s.cameras[1], dg1)
    return s, dg0.to_host(), dg1.to_host(), dg0, dg1


def test_render_frame_host_matches_device(ctx, cfg2_small, cuda):
    from restir_gb300.passes import DeviceGBuffer
    s, gs = cfg2_small
    ctx.upload_scene(s)
    imgs_dev, imgs_host = [], []
    for f in range(2):
        out = cuda.zeros((s.height, s.width, 4), dtype=cuda.float32, device="cuda")
        ctx.render_frame(DeviceGBuffer.from_host(gs[f]), DeviceGBuffer.from_host(gs[f - 1]) if f else None, f % 2,
                         s.frame_params(f), out)
        imgs_dev.append(out.cpu().numpy())
    for f in range(2):
        h = np.zeros((s.height, s.width, 4), np.float32)
        ctx.render_frame_host(gs[f], s.frame_params(f), h)
        imgs_host.append(h)
    for a, b in zip(imgs_dev, imgs_host):
        assert np.array_equal(image_bits(a), image_bits(b))


def test_triangle_light_scene_bit_exact(ctx, cuda):
    """Emissive-triangle lights: pickPointOnTriangle, the |cos| x area pdf, the
    luminance x area alias table, negative light indices in shading and the
    emissive passthrough (restirOmni.glsl:68-71,123-133; lighting.frag:56-71)."""
    from restir_gb300 import scenes
    from restir_gb300.passes import DeviceGBuffer, reservoirs, reservoirs_to_numpy
    s = scenes.config1_triangle_lights()
    g = scenes.trace_gbuffer_host(s, 0)
    assert (g["albedo"][..., 3] == 255).any()
    ctx.upload_scene(s)
    dg = DeviceGBuffer.from_host(g)
    n = s.width * s.height
    stages, img = oracle_frame(s, 0, g, None, None)
    u = s.uniforms(0)
    r0, r1, r2 = reservoirs(n), reservoirs(n), reservoirs(n)
    ctx.initial_temporal(dg, None, None, r0, u)
    assert mismatch(reservoirs_to_numpy(r0), stages[0]) == 0
    ctx.spatial_biased(dg, r0, r1, u, 0)
    ctx.spatial_biased(dg, r1, r2, u, 1)
    got = reservoirs_to_numpy(r2)
    assert mismatch(got, stages[-1]) == 0
    assert (got["light_index"] < 0).mean() > 0.5
    out = cuda.zeros((s.height, s.width, 4), dtype=cuda.float32, device="cuda")
    ctx.shade(dg, r2, s.lighting_uniforms(0), out)
    assert np.array_equal(image_bits(out.cpu().numpy()), image_bits(img))


def test_final_ris_weight_flag_bit_exact(ctx, cfg1, cuda):
    from restir_gb300 import _lib
    from restir_gb300.passes import reservoirs, reservoirs_to_numpy
    s, g = cfg1
    dg = _dev(ctx, s, g)
    n = s.width * s.height
    u = s.uniforms(0)
    u.flags |= _lib.RG_FLAG_FINAL_RIS_WEIGHT
    exp = new_res(n)
    ob.initial_temporal(s, g, None, None, exp, u)
    r = reservoirs(n)
    ctx.initial_temporal(dg, None, None, r, u)
    got = reservoirs_to_numpy(r)
    assert mismatch(got, exp) == 0
    ref_mode = new_res(n)
    ob.initial_temporal(s, g, None, None, ref_mode, s.uniforms(0))
    assert mismatch(got, ref_mode) > 0  # the flag changes W
