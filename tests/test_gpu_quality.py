"""Image quality of GPU frame sequences against the FP64 judge.

Config 2's scene at 320x180 with a static camera; the running mean of the
frames is compared with the brute-force judge on a 32x32 crop.  Two measured
properties of the reference's algorithm are pinned here:
  - its default per-frame sequence (RIS + visibility + temporal reuse and
    one unbiased spatial pass with NUM_NEIGHBORS = 3, src/app.h:150-174,
    unbiasedReuse.glsl:48) converges to the judge;
  - chaining its unbiased pass darkens the image: the pass adds every
    neighbour's M to the reservoir (unbiasedReuse.glsl:116) but normalises W
    by the visibility-filtered count (:168-182), so a later pass or the next
    frame's temporal merge counts samples the weight does not carry.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_binding as ob

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene_judge(ctx, cuda):
    from restir_gb300 import scenes
    from restir_gb300.passes import DeviceGBuffer
    s = scenes.config2(width=320, height=180, frames=1)
    ctx.upload_scene(s)
    dg = DeviceGBuffer(s.width, s.height)
    ctx.trace_gbuffer(s.cameras[0], dg)
    crop = (144, 74, 32, 32)
    judge = ob.brute_force(s, dg.to_host(), s.cameras[0].basis()[0], crop=crop)
    return s, dg, crop, judge


def _mean_image(ctx, cuda, s, dg, crop, frames, passes, neighbors):
    x0, y0, cw, ch = crop
    acc = np.zeros((ch, cw, 3))
    for f in range(frames):
        fp = s.frame_params(0)
        fp.uniforms.frame = f + 1
        fp.uniforms.flags = 1 | (2 if f > 0 else 0)  # visibility reuse; temporal from frame 2 on
        fp.spatial_iterations = passes
        fp.unbiased_neighbors = neighbors
        out = cuda.zeros((s.height, s.width, 4), dtype=cuda.float32, device="cuda")
        ctx.render_frame(dg, dg, f % 2, fp, out)
        acc += out.cpu().numpy()[y0:y0 + ch, x0:x0 + cw, :3]
    return acc / frames


def _bias(m, judge):
    return float((m.mean() - judge.mean()) / judge.mean())


def test_reference_default_sequence_converges(ctx, cuda, scene_judge):
    s, dg, crop, judge = scene_judge
    ctx.upload_scene(s)
    m = _mean_image(ctx, cuda, s, dg, crop, 64, passes=1, neighbors=3)
    assert np.isfinite(m).all()
    assert abs(_bias(m, judge)) < 0.2, _bias(m, judge)


def test_chained_unbiased_passes_darken(ctx, cuda, scene_judge):
    s, dg, crop, judge = scene_judge
    ctx.upload_scene(s)
    m = _mean_image(ctx, cuda, s, dg, crop, 32, passes=2, neighbors=5)
    assert _bias(m, judge) < -0.5, _bias(m, judge)
