"""Frame sizes that do not fill the launch tiles, and degenerate sizes.

Bar: bit-exact against the oracle.  Every pass tiles the frame (RIS 32 x 12,
unbiased spatial 32 x 4, biased spatial and shading 32 x 4 pixels); frames of
1 x 1, 1 x 7, 33 x 5 and 97 x 61 pixels leave partial tiles on both axes and
rows narrower than a warp, and spatial neighbours clamp at every border.
Zero-sized frames are rejected on the host."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import mismatch, new_res, oracle_frame, image_bits

pytestmark = pytest.mark.gpu

SIZES = [(1, 1), (1, 7), (33, 5), (97, 61)]


@pytest.mark.parametrize("w,h", SIZES)
def test_biased_frame_odd_sizes_bit_exact(ctx, cuda, w, h):
    from restir_gb300 import scenes
    from restir_gb300.passes import DeviceGBuffer, reservoirs, reservoirs_to_numpy
    s = scenes.config1(width=w, height=h)
    g = scenes.trace_gbuffer_host(s, 0)
    ctx.upload_scene(s)
    dg = DeviceGBuffer.from_host(g)
    n = w * h
    stages, img = oracle_frame(s, 0, g, None, None)
    u = s.uniforms(0)
    r0 = reservoirs(n)
    ctx.initial_temporal(dg, None, None, r0, u)
    assert mismatch(reservoirs_to_numpy(r0), stages[0]) == 0
    r1, r2 = reservoirs(n), reservoirs(n)
    ctx.spatial_biased(dg, r0, r1, u, 0)
    ctx.spatial_biased(dg, r1, r2, u, 1)
    assert mismatch(reservoirs_to_numpy(r2), stages[-1]) == 0
    out = cuda.zeros((h, w, 4), dtype=cuda.float32, device="cuda")
    ctx.shade(dg, r2, s.lighting_uniforms(0), out)
    assert np.array_equal(image_bits(out.cpu().numpy()), image_bits(img))


@pytest.mark.parametrize("w,h", SIZES)
def test_unbiased_temporal_odd_sizes_bit_exact(ctx, cuda, w, h):
    """Two frames of config 2's pass order (temporal reuse, 2 unbiased passes)
    through the frame driver."""
    from restir_gb300 import scenes
    from restir_gb300.passes import DeviceGBuffer, device_view
    s = scenes.config2(width=w, height=h, n_tris=20_000, n_lights=4096, frames=2)
    gs = [scenes.trace_gbuffer_host(s, f) for f in range(2)]
    ctx.upload_scene(s)
    n = w * h
    dgs = [DeviceGBuffer.from_host(g) for g in gs]
    prev_res = new_res(n)
    for f in range(2):
        stages, img = oracle_frame(s, f, gs[f], gs[f - 1] if f else None, prev_res)
        out = cuda.zeros((h, w, 4), dtype=cuda.float32, device="cuda")
        ctx.render_frame(dgs[f], dgs[f - 1] if f else None, f % 2, s.frame_params(f), out)
        got = device_view(ctx.frame_reservoirs_ptr(f % 2), n * 64).cpu().numpy().view(stages[-1].dtype)
        assert mismatch(got, stages[-1]) == 0, f"frame {f}"
        assert np.array_equal(image_bits(out.cpu().numpy()), image_bits(img)), f"frame {f}"
        prev_res = stages[-1]
    assert ctx.stats().traversal_errors == 0


def test_zero_sized_frame_rejected(ctx, cuda):
    from restir_gb300 import scenes
    from restir_gb300._lib import RestirError
    from restir_gb300.passes import DeviceGBuffer, reservoirs
    s = scenes.config1(width=8, height=8)
    ctx.upload_scene(s)
    g = DeviceGBuffer.from_host(scenes.trace_gbuffer_host(s, 0))
    u = s.uniforms(0)
    u.screen_size[0] = 0
    with pytest.raises(RestirError):
        ctx.initial_temporal(g, None, None, reservoirs(64), u)
