"""The learned light-cluster proposal on the GPU against the oracle.

Bars:
  * inference (tensor-core logits, FP32 accumulation) against the oracle's
    double-precision forward on the same bf16 weights: log-sum-exp within
    2e-3 everywhere (a hidden activation may round to the neighbouring bf16
    value when FP32 and double sums straddle a rounding boundary) and within
    1e-4 for 99% of pixels; the most probable cluster equal for 99%;
  * candidates: uniform-branch lights identical (same PCG stream), learned
    clusters identical for 99.5% (the CDF walk is FP32 on the GPU), q within
    1e-4 relative for 99% of candidates and 1e-2 for all (a logit moves by a
    few 1e-3 when a hidden activation rounds to the neighbouring bf16 value);
  * RIS with the learned candidates: bit-exact against the oracle's pass fed
    the same candidates;
  * gradients: per parameter block, relative L2 error 2e-2 against the
    oracle's double-precision gradient with bf16 rounding at the points where
    the product rounds.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_binding as ob
from helpers import mismatch, mlp_params, new_res

pytestmark = pytest.mark.gpu

# Two networks: a small one (256 clusters: 4 logit chunks of 64) and config
# 4's own (4096 clusters: 64 chunks through the double-buffered tensor-memory
# pipeline, the 32-wide piece search over 4096 columns) on config 2's scene
# with its 65,536 lights and 100k triangles at 320x180.
SETUPS = {
    "small": dict(width=128, height=96, n_tris=20_000, n_lights=4096, clusters=256),
    "config4": dict(width=320, height=180, n_tris=100_000, n_lights=65_536, clusters=4096),
}


@pytest.fixture(scope="module", params=list(SETUPS))
def scene4(request, restir_lib):
    from restir_gb300 import scenes
    from restir_gb300.passes import cluster_lights
    c = SETUPS[request.param]
    s = scenes.config2(width=c["width"], height=c["height"], n_tris=c["n_tris"], n_lights=c["n_lights"], frames=2)
    gs = [scenes.trace_gbuffer_host(s, f) for f in range(s.frames)]
    cluster_of, _ = cluster_lights(s.point_lights, c["clusters"], iterations=6, seed=4)
    return s, gs, cluster_of, c["clusters"]


def _setup(ctx, scene4, seed=1, scale_w4=0.3, lr=1e-3):
    from restir_gb300.passes import DeviceGBuffer
    s, gs, cluster_of, clusters = scene4
    ctx.upload_scene(s)
    ctx.create_proposal(cluster_of, clusters, mix=0.9, batch=4096, seed=seed, learning_rate=lr)
    count = len(ctx.proposal_params())
    params = mlp_params(count, clusters, seed, scale_w4)
    ctx.set_proposal_params(params)
    m = ob.OracleMlp(ctx.proposal_params(), cluster_of, clusters, mix=0.9)
    return s, gs, cluster_of, [DeviceGBuffer.from_host(g) for g in gs], m


def _learned_uniforms(s, f):
    from restir_gb300 import _lib
    u = s.uniforms(f)
    u.flags |= _lib.RG_FLAG_LEARNED_PROPOSAL
    return u


def test_params_round_trip_and_padding(ctx, scene4):
    s, gs, cluster_of, dgs, m = _setup(ctx, scene4)
    p = ctx.proposal_params()
    assert np.all(p[9 * 64:16 * 64] == 0.0)  # padded feature rows of W1 stay zero
    q = p.copy()
    q[9 * 64:16 * 64] = 1.0
    ctx.set_proposal_params(q)
    assert np.all(ctx.proposal_params()[9 * 64:16 * 64] == 0.0)


def test_inference_matches_oracle(ctx, scene4, cuda):
    s, gs, cluster_of, dgs, m = _setup(ctx, scene4)
    u = _learned_uniforms(s, 0)
    ctx.proposal_infer(dgs[0], u)
    n = s.width * s.height
    cand, stat = ctx.proposal_buffers(n)
    lse, amax = m.row_stats(gs[0], s.cameras[0].position)
    d = np.abs(stat[:, 0].astype(np.float64) - lse)
    assert d.max() <= 2e-3, d.max()
    assert np.quantile(d, 0.99) <= 1e-4
    assert np.mean(stat[:, 1].view(np.int32) == amax) >= 0.99
    assert ctx.stats().mma_timeouts == 0


def test_candidates_match_oracle(ctx, scene4, cuda):
    s, gs, cluster_of, dgs, m = _setup(ctx, scene4, seed=2)
    for f in range(2):
        u = _learned_uniforms(s, f)
        ctx.proposal_infer(dgs[f], u)
        n = s.width * s.height
        cand, _ = ctx.proposal_buffers(n)
        keys, qs = m.sample(gs[f], s.cameras[f].position, u.frame, 32, np.arange(n, dtype=np.int32))
        got_k, got_q = cand["key"], cand["q"]
        uni = keys >= 0
        assert np.array_equal(got_k[uni], keys[uni])
        assert np.array_equal(got_k >= 0, uni)
        same = got_k == keys
        assert same[~uni].mean() >= 0.995, same[~uni].mean()
        rel = np.abs(got_q[same] - qs[same]) / np.maximum(qs[same], 1e-30)
        assert rel.max() <= 1e-2, rel.max()
        assert np.quantile(rel, 0.99) <= 1e-4
        assert 0.85 < (~uni).mean() < 0.95


def test_learned_ris_bit_exact(ctx, scene4, cuda):
    """RIS + visibility reuse (+ temporal on the second frame) with the
    learned candidates equals the oracle's pass fed the same candidates."""
    from restir_gb300.passes import reservoirs, reservoirs_to_numpy
    s, gs, cluster_of, dgs, m = _setup(ctx, scene4, seed=3)
    n = s.width * s.height
    prev_gpu = None
    prev_orc = None
    for f in range(2):
        u = _learned_uniforms(s, f)
        if f == 0:
            u.flags &= ~2  # no temporal reuse on the first frame
        ctx.proposal_infer(dgs[f], u)
        cand, _ = ctx.proposal_buffers(n)
        out = reservoirs(n)
        ctx.initial_temporal(dgs[f], dgs[f - 1] if f else None, prev_gpu, out, u)
        got = reservoirs_to_numpy(out)
        exp = new_res(n)
        ob.initial_temporal_learned(s, gs[f], gs[f - 1] if f else None, prev_orc, exp, u, cand, cluster_of,
                                    m.clusters, mix=0.9)
        assert mismatch(got, exp) == 0
        assert np.mean(got["w"] > 0) > 0.05  # lit and unshadowed samples exist
        prev_gpu, prev_orc = out, exp


def test_learned_flag_needs_matching_inference(ctx, scene4, cuda):
    from restir_gb300.passes import reservoirs
    from restir_gb300._lib import RestirError
    s, gs, cluster_of, dgs, m = _setup(ctx, scene4, seed=4)
    u = _learned_uniforms(s, 0)
    u.flags &= ~2
    ctx.proposal_infer(dgs[0], u)
    u.frame += 1  # candidates are for the previous frame
    with pytest.raises(RestirError):
        ctx.initial_temporal(dgs[0], None, None, reservoirs(s.width * s.height), u)


def test_gradients_match_oracle(ctx, scene4, cuda):
    s, gs, cluster_of, dgs, m = _setup(ctx, scene4, seed=5)
    n = 3000
    rng = np.random.default_rng(6)
    rows = rng.integers(0, s.width * s.height, n).astype(np.int32)
    targets = cluster_of[rng.integers(0, len(cluster_of), n)].astype(np.int32)
    targets[::11] = -1
    cam = s.cameras[0].position
    grad, loss = ctx.proposal_gradients(dgs[0], cam, cuda.from_numpy(rows).cuda(), cuda.from_numpy(targets).cuda())
    g_gpu = grad.cpu().numpy().astype(np.float64)
    loss_o, g_orc = m.loss_grad(gs[0], cam, rows, targets, emulate=True)
    assert abs(loss - loss_o) <= 1e-4 * abs(loss_o), (loss, loss_o)
    blocks = {"W1": (0, 1024), "b1": (1024, 1088), "W2": (1088, 5184), "b2": (5184, 5248), "W3": (5248, 9344),
              "b3": (9344, 9408), "W4": (9408, 9408 + 64 * m.clusters), "b4": (9408 + 64 * m.clusters, len(g_orc))}
    for name, (a, b) in blocks.items():
        err = np.linalg.norm(g_gpu[a:b] - g_orc[a:b]) / max(np.linalg.norm(g_orc[a:b]), 1e-30)
        assert err <= 2e-2, (name, err)
    assert ctx.stats().mma_timeouts == 0


def test_training_steps_reduce_loss(ctx, scene4, cuda):
    """Adam steps on one frame's final reservoirs lower the loss on the same
    pixels, and the weights stay finite."""
    s, gs, cluster_of, dgs, m = _setup(ctx, scene4, seed=7, scale_w4=0.05, lr=1e-2)
    from restir_gb300.passes import reservoirs
    u = s.uniforms(0)
    u.flags &= ~2
    n = s.width * s.height
    res = reservoirs(n)
    ctx.initial_temporal(dgs[0], None, None, res, u)
    losses = []
    for step in range(30):
        ctx.proposal_train(dgs[0], u, res.data_ptr())
        losses.append(ctx.proposal_last_loss()[0])
    assert np.all(np.isfinite(ctx.proposal_params()))
    assert losses[-1] < 0.8 * losses[0], losses
