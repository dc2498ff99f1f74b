"""The visibility cache between ray passes (rg_set_visibility_cache).

A pass takes the recorded answer of a segment whose two end points equal a
recorded segment's bit for bit instead of tracing it.  Bar: reservoirs bit
for bit equal to the same sequence with the cache off (which the oracle
tests pin to the reference), fewer segments traced, and no answer carried
over a scene upload.
"""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest

from helpers import mismatch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def seq_scene(restir_lib, ctx):
    from restir_gb300 import scenes
    from restir_gb300.passes import DeviceGBuffer
    s = scenes.config3(width=320, height=180, frames=3)
    ctx.upload_scene(s)
    dgs = []
    for f in range(s.frames):
        d = DeviceGBuffer(s.width, s.height)
        ctx.trace_gbuffer(s.cameras[f], d)
        dgs.append(d)
    return s, dgs


def _sequence(ctx, s, dgs, cache: bool):
    """RIS + temporal, then the configuration's unbiased passes, per frame:
    every pass's output reservoirs and the segments traced."""
    import torch
    from restir_gb300.passes import reservoirs, reservoirs_to_numpy
    n = s.width * s.height
    ctx.set_visibility_cache(cache)
    ctx.upload_scene(s)
    outs, rays = [], 0
    prev = None
    try:
        ctx.stats(reset=True)
        for f in range(s.frames):
            u = s.uniforms(f)
            r = reservoirs(n)
            ctx.initial_temporal(dgs[f], dgs[f - 1] if f else None, prev, r, u)
            outs.append(reservoirs_to_numpy(r))
            for p in range(s.spatial_passes):
                o = reservoirs(n)
                ctx.spatial_unbiased(dgs[f], r, o, u, s.neighbors, p)
                outs.append(reservoirs_to_numpy(o))
                r = o
            prev = r
        torch.cuda.synchronize()
        st = ctx.stats(reset=True)
        assert st.traversal_errors == 0
        rays = int(st.rays_traced)
    finally:
        ctx.set_visibility_cache(True)
    return outs, rays


def test_cache_keeps_every_reservoir_and_saves_rays(ctx, cuda, seq_scene):
    s, dgs = seq_scene
    on, rays_on = _sequence(ctx, s, dgs, True)
    off, rays_off = _sequence(ctx, s, dgs, False)
    assert len(on) == len(off) == s.frames * (1 + s.spatial_passes)
    for k, (a, b) in enumerate(zip(on, off)):
        assert mismatch(a, b) == 0, f"pass {k}"
    print("segments traced: cache on", rays_on, "off", rays_off)
    assert rays_on < 0.9 * rays_off


def test_upload_clears_the_cache(ctx, cuda, seq_scene):
    """The same G-buffer and reservoirs over another scene (the occluders
    moved out of the way): a pass right after the upload must not take the
    first scene's answers for its segments."""
    from restir_gb300.passes import reservoirs, reservoirs_to_numpy
    s, dgs = seq_scene
    n = s.width * s.height
    u = s.uniforms(0)
    moved = s.triangles.copy()
    for k in ("p1", "p2", "p3"):
        moved[k][:, 0] += np.float32(100.0)
    s2 = dataclasses.replace(s, triangles=moved, nodes=s.nodes.copy())
    for k in ("lmin", "lmax", "rmin", "rmax"):
        s2.nodes[k][:, 0] += np.float32(100.0)
    results = []
    for cache in (True, False):
        ctx.set_visibility_cache(cache)
        try:
            ctx.upload_scene(s)
            r = reservoirs(n)
            ctx.initial_temporal(dgs[0], None, None, r, u)
            o = reservoirs(n)
            ctx.spatial_unbiased(dgs[0], r, o, u, s.neighbors, 0)  # fills the cache for scene 1
            ctx.upload_scene(s2)
            o2 = reservoirs(n)
            ctx.spatial_unbiased(dgs[0], o, o2, u, s.neighbors, 1)
            results.append(reservoirs_to_numpy(o2))
        finally:
            ctx.set_visibility_cache(True)
    assert mismatch(results[0], results[1]) == 0
    # the moved scene shadows nothing: every reservoir with a positive p-hat keeps a positive w
    ok = results[1]["p_hat"] > 0
    assert ok.any() and np.all(results[1]["w"][ok] >= 0)


def test_setters_reject_bad_values(ctx, restir_lib):
    L = restir_lib
    assert L.rg_set_visibility_cache(ctx._h, 2) == -1 and b"enable" in L.rg_last_error()
    assert L.rg_set_tree_layout(ctx._h, 3) == -1 and b"tree layout" in L.rg_last_error()
    assert L.rg_set_visibility_cache(None, 1) == -1
    assert L.rg_set_tree_layout(ctx._h, 2) == 0 and L.rg_set_visibility_cache(ctx._h, 1) == 0
