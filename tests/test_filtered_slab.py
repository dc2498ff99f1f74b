"""The shadow-ray walk's filtered slab decision, emulated in float32 numpy,
against the reference's slab test (softwareRaytracing.glsl:9-14: per-slab
division, GLSL min/max, then rmin < 1 && rmax >= rmin && rmax > 0).

The GPU computes t~ = RN(RN(b - o) * RN(1/d)) instead of RN(RN(b - o) / d)
and decides a box only when the reference's three comparisons are out of
reach of that rounding difference (trace_pool.cuh filtered_decision); every
other box goes to the exact test.  Bar: zero wrong decisions on random and
adversarial boxes (segment ends on a face, flat boxes, grazing segments,
segments through a box corner, overflowing and tiny distances), and most
ordinary boxes decided.  The GPU side of the same rule is checked
bit-exactly by tests/test_gpu_visibility.py.
"""
from __future__ import annotations

import numpy as np

f = np.float32
EPS = f(2.0 ** -19)
TINY = f(2.0 ** -90)


def _gmin(x, y):
    return np.where(y < x, y, x)


def _gmax(x, y):
    return np.where(x < y, y, x)


def exact(o, d, bmin, bmax):
    """The reference's test: division per slab, GLSL min/max nesting."""
    with np.errstate(all="ignore"):
        t0 = (bmin - o) / d
        t1 = (bmax - o) / d
    rmin = _gmax(_gmin(t0[:, 0], t1[:, 0]), _gmax(_gmin(t0[:, 1], t1[:, 1]), _gmin(t0[:, 2], t1[:, 2])))
    rmax = _gmin(_gmax(t0[:, 0], t1[:, 0]), _gmin(_gmax(t0[:, 1], t1[:, 1]), _gmax(t0[:, 2], t1[:, 2])))
    return (rmin < f(1)) & (rmax >= rmin) & (rmax > f(0))


def filtered(o, d, bmin, bmax):
    """1 hit, 0 miss, -1 undecided, as the device's fast path decides."""
    with np.errstate(all="ignore"):
        inv = f(1) / d
        t0 = (bmin + (-o)) * inv
        t1 = (bmax + (-o)) * inv
        rmin = np.fmax(np.fmax(np.fmin(t0[:, 0], t1[:, 0]), np.fmin(t0[:, 1], t1[:, 1])), np.fmin(t0[:, 2], t1[:, 2]))
        rmax = np.fmin(np.fmin(np.fmax(t0[:, 0], t1[:, 0]), np.fmax(t0[:, 1], t1[:, 1])), np.fmax(t0[:, 2], t1[:, 2]))
        dd = rmax - rmin
        s = (np.abs(rmin) + np.abs(rmax)).astype(f)
        ss = (np.float64(EPS) * s.astype(np.float64) + np.float64(TINY)).astype(f)  # one rounding, as the FMA
        hit = (rmin < f(1) - EPS) & (rmax > TINY) & (dd > ss)
        miss = (rmin > f(1) + EPS) | (rmax < -TINY) | (dd < -ss)

    ad = np.abs(d)
    fast = np.all((ad >= f(2.0 ** -100)) & (ad <= f(2.0 ** 100)), axis=1)  # ray_inverse
    assert not np.any(fast & hit & miss)
    res = np.full(len(o), -1, np.int8)
    res[fast & miss] = 0
    res[fast & hit] = 1
    return res


def _case(rng, kind, n):
    o = rng.uniform(0, 1, (n, 3)).astype(f)
    d = (rng.uniform(-1, 1, (n, 3)) * rng.choice([1, 1e-3, 1e-6], (n, 1))).astype(f)
    c = rng.uniform(0, 1, (n, 3))
    h = rng.uniform(0, 0.3, (n, 3))
    bmin = (c - h).astype(f)
    bmax = (c + h).astype(f)
    if kind == "zero_component":
        d[rng.random(n) < 0.2, rng.integers(0, 3)] = 0
    elif kind == "end_on_face":
        bmin[:, 0] = o[:, 0] + d[:, 0] * f(1) * f(1 + rng.uniform(-1e-6, 1e-6))
    elif kind == "flat":
        bmax[:, 1] = bmin[:, 1]
        o[::7, 1] = bmin[::7, 1]
    elif kind == "grazing":
        bmin[:, 2] = o[:, 2] + d[:, 2] * f(0.5)
        bmax[:, 0] = o[:, 0] + d[:, 0] * f(0.5)
    elif kind == "huge":
        d[:, rng.integers(0, 3)] *= f(1e-28)
        s = rng.choice([1, 1e6, 1e9, 1e12], (n, 1)).astype(f)
        bmin = (bmin * s).astype(f)
        bmax = (bmax * s).astype(f)
    elif kind == "tiny":
        d = (d * f(1e25)).astype(f)
    elif kind == "behind":
        bmax[:, 0] = (o[:, 0] - d[:, 0] * f(1e-7) * rng.uniform(0, 2, n).astype(f)).astype(f)
    elif kind == "corner":
        t = rng.uniform(0.1, 0.9, (n, 1)).astype(f)
        o = (bmax - d * t).astype(f)
    return o, d, bmin.astype(f), bmax.astype(f)


KINDS = ["plain", "zero_component", "end_on_face", "flat", "grazing", "huge", "tiny", "behind", "corner"]


def test_filtered_decisions_never_wrong():
    rng = np.random.default_rng(2026)
    decided_plain = None
    for kind in KINDS:
        o, d, bmin, bmax = _case(rng, kind, 200_000)
        e = exact(o, d, bmin, bmax)
        r = filtered(o, d, bmin, bmax)
        dec = r >= 0
        wrong = np.count_nonzero(e[dec] != (r[dec] == 1))
        assert wrong == 0, f"{kind}: {wrong} wrong decisions"
        if kind == "plain":
            decided_plain = dec.mean()
    assert decided_plain > 0.999  # ordinary boxes almost never need the exact test


def test_undecided_near_the_thresholds():
    """Boxes whose exact rmin sits within a few ulps of 1 are left undecided
    rather than guessed."""
    rng = np.random.default_rng(7)
    o, d, bmin, bmax = _case(rng, "end_on_face", 100_000)
    r = filtered(o, d, bmin, bmax)
    assert np.count_nonzero(r < 0) > 0
