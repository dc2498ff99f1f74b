"""Many views in one launch per pass (rg_batch_*) against the single-view
passes on the same inputs.

Bar: bit-exact.  Every view's reservoirs and shaded image after each run of a
batch equal those of the single-view pass sequence of rg_render_frame
(RIS + visibility + temporal, the spatial chain, shading) for that view and
frame, for every launch-shape tuning, for the unbiased and the biased chains,
and when the run is replayed from a captured CUDA graph; with the learned
proposal; and after the candidate count is chosen by efficiency."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import mismatch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def views5(restir_lib):
    from restir_gb300 import scenes
    base, views = scenes.config5(n_views=6, n_tris=20_000, n_lights=4096, min_size=(40, 30), max_size=(200, 150))
    return base, views


def _make(ctx, cuda, base, views, unbiased=True, learned=False):
    from restir_gb300 import _lib
    from restir_gb300.passes import DeviceGBuffer, reservoirs
    ctx.upload_scene(base)
    out = []
    for i, v in enumerate(views):
        g = DeviceGBuffer(v.width, v.height)
        ctx.trace_gbuffer(v.cameras[0], g)
        n = v.width * v.height
        u = v.uniforms(0)
        u.flags |= 2  # temporal reuse (static camera: the previous G-buffer is the current one)
        u.frame = 7
        if learned:
            u.flags |= _lib.RG_FLAG_LEARNED_PROPOSAL
            u.initial_light_sample_count = (32, 16, 8)[i % 3]
        out.append({"scene": v, "cur": g, "prev": g, "res0": reservoirs(n), "res1": reservoirs(n),
                    "tmp": reservoirs(n),
                    "image": cuda.zeros((v.height, v.width, 4), dtype=cuda.float32, device="cuda"), "uniforms": u})
    fp = base.frame_params(0)
    fp.unbiased = int(unbiased)
    fp.spatial_iterations = 2 if unbiased else 1
    fp.unbiased_neighbors = 5
    return out, fp


def _single(ctx, cuda, vw, fp, parity, frame):
    """rg_render_frame's sequence for one view on the view's own buffers."""
    from restir_gb300.passes import reservoirs
    v = vw["scene"]
    n = v.width * v.height
    u = vw["uniforms"]
    import ctypes as C
    uu = type(u).from_buffer_copy(bytes(u))
    uu.frame = frame
    cur, prev = vw[f"s{parity}"], vw[f"s{1 - parity}"]
    passes = fp.spatial_iterations
    from restir_gb300 import _lib
    if uu.flags & _lib.RG_FLAG_LEARNED_PROPOSAL:
        ctx.proposal_infer(vw["cur"], uu)
    if fp.unbiased:
        first = vw["stmp"] if passes % 2 == 1 else cur
        ctx.initial_temporal(vw["cur"], vw["prev"], prev, first, uu)
        src = first
        for k in range(passes):
            dst = cur if src is vw["stmp"] else vw["stmp"]
            ctx.spatial_unbiased(vw["cur"], src, dst, uu, fp.unbiased_neighbors, k)
            src = dst
    else:
        ctx.initial_temporal(vw["cur"], vw["prev"], prev, cur, uu)
        for j in range(passes):
            ctx.spatial_biased(vw["cur"], cur, prev, uu, 2 * j)
            ctx.spatial_biased(vw["cur"], prev, cur, uu, 2 * j + 1)
    img = cuda.zeros_like(vw["image"])
    lu = v.lighting_uniforms(0)
    ctx.shade(vw["cur"], cur, lu, img)
    return cur, img


def _compare(ctx, cuda, vws, fp, batch, runs, graph=False):
    from restir_gb300.passes import reservoirs, reservoirs_to_numpy
    for vw in vws:
        n = vw["scene"].width * vw["scene"].height
        vw["s0"], vw["s1"], vw["stmp"] = reservoirs(n), reservoirs(n), reservoirs(n)
    graphs = {}
    if graph:
        stream = cuda.cuda.Stream()
        for parity in (0, 1):
            g = cuda.cuda.CUDAGraph()
            with cuda.cuda.graph(g, stream=stream):
                batch.run(parity, stream)
            graphs[parity] = g
        batch.reset_frames()
        for vw in vws:
            for k in ("res0", "res1", "tmp"):
                vw[k].zero_()
        cuda.cuda.synchronize()
    for r in range(runs):
        parity = r & 1
        if graph:
            graphs[parity].replay()
        else:
            batch.run(parity)
        cuda.cuda.synchronize()
        for vw in vws:
            exp_res, exp_img = _single(ctx, cuda, vw, fp, parity, vw["uniforms"].frame + r)
            got = reservoirs_to_numpy(vw[f"res{parity}"])
            assert mismatch(got, reservoirs_to_numpy(exp_res)) == 0, (r, vw["scene"].name)
            assert np.array_equal(vw["image"].cpu().numpy().view(np.uint32), exp_img.cpu().numpy().view(np.uint32))


@pytest.mark.parametrize("tuning", [(4, 32, 0), (1, 8, 0), (2, 16, 2)])
def test_batch_equals_single_views_unbiased(ctx, cuda, views5, tuning):
    from restir_gb300 import _lib
    from restir_gb300.passes import Batch
    base, views = views5
    vws, fp = _make(ctx, cuda, base, views, unbiased=True)
    b = Batch(ctx, vws, fp, _lib.BatchTuning(*tuning))
    _compare(ctx, cuda, vws, fp, b, runs=3)
    b.close()
    assert ctx.stats().traversal_errors == 0


def test_batch_equals_single_views_biased(ctx, cuda, views5):
    from restir_gb300.passes import Batch
    base, views = views5
    vws, fp = _make(ctx, cuda, base, views, unbiased=False)
    b = Batch(ctx, vws, fp)
    _compare(ctx, cuda, vws, fp, b, runs=2)
    b.close()


def test_batch_graph_replay_equals_single_views(ctx, cuda, views5):
    from restir_gb300.passes import Batch
    base, views = views5
    vws, fp = _make(ctx, cuda, base, views, unbiased=True)
    b = Batch(ctx, vws, fp)
    b.run(0)  # first run outside capture: function attributes are set here
    cuda.cuda.synchronize()
    _compare(ctx, cuda, vws, fp, b, runs=3, graph=True)
    b.close()


def test_autotune_keeps_results(ctx, cuda, views5):
    from restir_gb300.passes import Batch
    base, views = views5
    vws, fp = _make(ctx, cuda, base, views, unbiased=True)
    b = Batch(ctx, vws, fp)
    t, ms = b.autotune(repeats=2)
    assert ms > 0 and t.ris_pixels_per_thread in (1, 2, 4) and t.spatial_tile_width in (8, 16, 32)
    b.reset_frames()
    for vw in vws:
        for k in ("res0", "res1", "tmp"):
            vw[k].zero_()
    _compare(ctx, cuda, vws, fp, b, runs=2)
    b.close()


def test_batch_learned_proposal_equals_single_views(ctx, cuda, views5):
    """Learned proposal: one inference launch pair over all views' pixels,
    then the batched passes; every view equals rg_proposal_infer +
    rg_render_frame's sequence for that view (views draw 32, 16 or 8
    candidates), also from a captured graph."""
    from restir_gb300.passes import Batch, cluster_lights
    base, views = views5
    vws, fp = _make(ctx, cuda, base, views, unbiased=True, learned=True)
    cluster_of, _ = cluster_lights(base.point_lights, 256, iterations=4, seed=3)
    ctx.create_proposal(cluster_of, 256, seed=5)
    b = Batch(ctx, vws, fp)
    _compare(ctx, cuda, vws, fp, b, runs=2)
    b.run(0)
    cuda.cuda.synchronize()
    _compare(ctx, cuda, vws, fp, b, runs=2, graph=True)
    b.close()
    assert ctx.stats().mma_timeouts == 0
    assert ctx.stats().traversal_errors == 0


def test_batch_learned_guards(ctx, cuda, views5):
    from restir_gb300 import _lib
    from restir_gb300._lib import RestirError
    from restir_gb300.passes import Batch, cluster_lights
    base, views = views5
    vws, fp = _make(ctx, cuda, base, views[:2], unbiased=True, learned=True)
    ctx.destroy_proposal()
    with pytest.raises(RestirError, match="without a proposal"):
        Batch(ctx, vws, fp)
    cluster_of, _ = cluster_lights(base.point_lights, 256, iterations=2, seed=3)
    ctx.create_proposal(cluster_of, 256, seed=5)
    vws[1]["uniforms"].flags &= ~_lib.RG_FLAG_LEARNED_PROPOSAL
    with pytest.raises(RestirError, match="all views or none"):
        Batch(ctx, vws, fp)
    vws[1]["uniforms"].flags |= _lib.RG_FLAG_LEARNED_PROPOSAL
    b = Batch(ctx, vws, fp)
    ctx.create_proposal(cluster_of, 256, seed=6)  # a new proposal: the batch's tables are stale
    with pytest.raises(RestirError, match="proposal changed"):
        b.run(0)
    b.close()


@pytest.mark.parametrize("learned", [False, True])
def test_candidate_tuning_by_efficiency(ctx, cuda, views5, learned):
    """The tuner times each candidate count, measures the per-pixel variance
    of one frame from two runs that share their history, keeps the most
    efficient count, and leaves it set: afterwards every view equals its
    single-view passes run with that count."""
    from restir_gb300.passes import Batch, cluster_lights
    base, views = views5
    vws, fp = _make(ctx, cuda, base, views, unbiased=True, learned=learned)
    if learned:
        cluster_of, _ = cluster_lights(base.point_lights, 256, iterations=4, seed=3)
        ctx.create_proposal(cluster_of, 256, seed=5)
    b = Batch(ctx, vws, fp)
    best, ms, var = b.autotune_candidates((4, 32), repeats=1)
    assert best in (4, 32)
    assert all(m > 0 for m in ms)
    assert var[0] > var[1] > 0  # more candidates, less noise
    eff = [1.0 / (m * v) for m, v in zip(ms, var)]
    assert best == (4, 32)[int(np.argmax(eff))]
    assert all(vw["uniforms"].initial_light_sample_count == best for vw in vws)
    b.reset_frames()
    for vw in vws:
        for k in ("res0", "res1", "tmp"):
            vw[k].zero_()
    _compare(ctx, cuda, vws, fp, b, runs=2)
    if learned:
        from restir_gb300._lib import RestirError
        with pytest.raises(RestirError, match="out of range"):
            b.autotune_candidates((33,))
    b.close()
