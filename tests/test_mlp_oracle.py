"""The oracle's statement of the learned proposal, on the CPU: its analytic
gradient against central finite differences of its own double-precision loss,
the bf16-emulating gradient against the plain one, its sampling rule against
the softmax it samples, and the host k-means of the C ABI."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import mlp_params


@pytest.fixture(scope="module")
def small_scene(restir_lib):
    from restir_gb300 import scenes
    sc = scenes.config1(width=48, height=40)
    g = scenes.trace_gbuffer_host(sc)
    return sc, g


def _setup(small_scene, clusters=128, seed=5):
    from oracle_binding import OracleMlp, oracle
    from restir_gb300.passes import cluster_lights
    sc, g = small_scene
    cluster_of, _ = cluster_lights(sc.point_lights, clusters, iterations=4, seed=seed)
    count = int(oracle().or_mlp_param_count(clusters))
    m = OracleMlp(mlp_params(count, clusters, seed), cluster_of, clusters)
    return sc, g, m, cluster_of


def _foreground_rows(g, n, seed):
    rng = np.random.default_rng(seed)
    nz = np.flatnonzero(g["normal"].reshape(-1, 4)[:, :3].any(axis=1))
    return rng.choice(nz, n, replace=False).astype(np.int32)


def test_gradient_matches_finite_differences(small_scene):
    sc, g, m, cluster_of = _setup(small_scene)
    cam = sc.cameras[0].position
    rows = _foreground_rows(g, 24, 1)
    rng = np.random.default_rng(2)
    targets = cluster_of[rng.integers(0, len(cluster_of), len(rows))]
    targets[::7] = -1  # rows without a target count in the mean with zero loss
    p64 = m.params.astype(np.float64)
    loss, grad = m.loss_grad(g, cam, rows, targets, emulate=False, params64=p64)
    n = len(rows)
    from oracle_binding import oracle
    count = int(oracle().or_mlp_param_count(m.clusters))
    # parameters from every block: W1 (used rows), b1, W2, b2, W3, b3, W4, b4
    idx = np.concatenate([rng.integers(0, 9 * 64, 8), 1024 + rng.integers(0, 64, 4),
                          1088 + rng.integers(0, 4096, 8), 5184 + rng.integers(0, 64, 4),
                          5248 + rng.integers(0, 4096, 8), 9344 + rng.integers(0, 64, 4),
                          9408 + rng.integers(0, 64 * m.clusters, 12), count - m.clusters + rng.integers(0, m.clusters, 8)])
    h = 1e-6
    for i in idx:
        pp, pm = p64.copy(), p64.copy()
        pp[i] += h
        pm[i] -= h
        lp, _ = m.loss_grad(g, cam, rows, targets, emulate=False, params64=pp)
        lm, _ = m.loss_grad(g, cam, rows, targets, emulate=False, params64=pm)
        fd = (lp - lm) / (2 * h) / n
        assert abs(fd - grad[i]) <= 1e-5 * max(1.0, abs(grad[i])) + 1e-7, (i, fd, grad[i])
    assert np.isfinite(loss) and loss > 0


def test_bf16_emulation_stays_close_to_double(small_scene):
    sc, g, m, cluster_of = _setup(small_scene)
    cam = sc.cameras[0].position
    rows = _foreground_rows(g, 64, 3)
    targets = cluster_of[np.random.default_rng(4).integers(0, len(cluster_of), len(rows))]
    l0, g0 = m.loss_grad(g, cam, rows, targets, emulate=False)
    l1, g1 = m.loss_grad(g, cam, rows, targets, emulate=True)
    assert abs(l1 - l0) <= 0.02 * abs(l0)
    assert np.linalg.norm(g1 - g0) <= 0.06 * np.linalg.norm(g0)


def test_sampling_follows_the_softmax(small_scene):
    """Learned-branch candidates land on clusters with the softmax's
    frequencies; uniform-branch candidates carry q of their light's cluster."""
    sc, g, m, cluster_of = _setup(small_scene, seed=9)
    cam = sc.cameras[0].position
    px = _foreground_rows(g, 1, 5)
    rows = np.repeat(px, 1)
    lse, amax, z = m.row_stats(g, cam, rows, logits=True)
    q = np.exp(z[0] - lse[0])
    assert abs(q.sum() - 1.0) < 1e-9
    counts = np.zeros(m.clusters)
    n_learned = n_uniform = 0
    for frame in range(300):
        keys, qs = m.sample(g, cam, frame, 32, rows)
        for k, qq in zip(keys[0], qs[0]):
            if k < 0:
                counts[-1 - k] += 1
                n_learned += 1
                assert abs(qq - q[-1 - k]) <= 1e-6 * max(1.0, q[-1 - k])
            else:
                n_uniform += 1
                assert abs(qq - q[cluster_of[k]]) <= 1e-6 * max(1.0, q[cluster_of[k]])
    total = n_learned + n_uniform
    assert abs(n_learned / total - 0.9) < 0.02
    expected = q * n_learned
    big = expected > 20
    chi2 = np.sum((counts[big] - expected[big]) ** 2 / expected[big])
    assert chi2 < 3.0 * big.sum() + 30, chi2


def test_cluster_lights_is_seeded_lloyd(restir_lib):
    from restir_gb300 import scenes
    from restir_gb300.passes import cluster_lights
    sc = scenes.config1(width=8, height=8)
    a, ca = cluster_lights(sc.point_lights, 128, iterations=6, seed=3)
    b, cb = cluster_lights(sc.point_lights, 128, iterations=6, seed=3)
    assert np.array_equal(a, b) and np.array_equal(ca, cb)
    assert a.min() >= 0 and a.max() < 128
    pos = sc.point_lights["pos"][:, :3].astype(np.float64)
    # every light sits with its nearest centre (assignment step of Lloyd)
    d = ((pos[:, None, :] - cb[None, :, :].astype(np.float64)) ** 2).sum(-1)
    nearest = d.argmin(1)
    same = d[np.arange(len(pos)), a] <= d[np.arange(len(pos)), nearest] * (1 + 1e-6) + 1e-12
    assert same.mean() > 0.99
