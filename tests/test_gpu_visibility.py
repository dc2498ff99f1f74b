"""Shadow segments placed where the slab test is hardest to decide, against
the oracle's testVisibility (visibilityTest.glsl:1-29 over
softwareRaytracing.glsl:9-85).

Bar: bit-exact visibility bits.  The GPU walk decides most child boxes with
a reciprocal-direction slab test and falls back to the reference's division
only when that test cannot decide; these segments aim at the fallback:
they end on, or pass through, corners, edges and faces of the tree's own
boxes, run parallel to a box face (a zero direction component), or have
direction components too small or too large for the reciprocal.  A NaN in a
box must disable the reciprocal test for the whole tree, because IEEE
min/max drop NaN operands where the GLSL definitions keep them.
"""
from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np
import pytest

import oracle_binding as ob

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cfg1_scene(restir_lib):
    from restir_gb300 import scenes
    return scenes.config1()


def _boundary_points(s, rng, n):
    """Points on the boundary of random child boxes of the tree: corners,
    points on edges and points on faces, one third each."""
    nodes = s.nodes
    idx = rng.integers(0, len(nodes), n)
    side = rng.integers(0, 2, n).astype(bool)
    bmin = np.where(side[:, None], nodes["rmin"][idx, :3], nodes["lmin"][idx, :3]).astype(np.float32)
    bmax = np.where(side[:, None], nodes["rmax"][idx, :3], nodes["lmax"][idx, :3]).astype(np.float32)
    pick = rng.integers(0, 2, (n, 3)).astype(bool)
    q = np.where(pick, bmax, bmin)
    inner = (bmin + (bmax - bmin) * rng.uniform(0, 1, (n, 3)).astype(np.float32)).astype(np.float32)
    kind = rng.integers(0, 3, n)  # 0 corner, 1 edge (one free axis), 2 face (two free axes)
    ax = rng.integers(0, 3, n)
    rows = np.arange(n)
    free = kind >= 1
    q[rows[free], ax[free]] = inner[rows[free], ax[free]]
    ax2 = (ax + 1) % 3
    face = kind == 2
    q[rows[face], ax2[face]] = inner[rows[face], ax2[face]]
    return q.astype(np.float32), bmin, bmax


def _segments(s, seed=11, n=60_000):
    rng = np.random.default_rng(seed)
    lo = np.minimum(s.nodes["lmin"][0, :3], s.nodes["rmin"][0, :3]) - 0.05
    hi = np.maximum(s.nodes["lmax"][0, :3], s.nodes["rmax"][0, :3]) + 0.05
    q, bmin, bmax = _boundary_points(s, rng, n)
    p1 = (lo + (hi - lo) * rng.uniform(0, 1, (n, 3))).astype(np.float32)
    p2 = np.empty_like(p1)
    kind = rng.integers(0, 5, n)
    # 0: the offset segment ends on the boundary point (testVisibility pulls
    #    both ends in by 0.001 along the segment)
    d = (q - p1).astype(np.float32)
    ln = np.sqrt((d.astype(np.float64) ** 2).sum(1, keepdims=True)).astype(np.float32)
    ln[ln == 0] = 1
    k0 = kind == 0
    p2[k0] = (q + np.float32(0.001) * d / ln)[k0]
    # 1: the segment passes through the boundary point
    k1 = kind == 1
    p2[k1] = (p1 + np.float32(2.0) * d)[k1]
    # 2: parallel to a box face, starting on that face's plane (zero direction
    #    component, b - o = 0 in that slab)
    k2 = np.nonzero(kind == 2)[0]
    ax = np.random.default_rng(seed + 1).integers(0, 3, len(k2))
    p2[k2] = q[k2]
    p1[k2, ax] = bmin[k2, ax]
    p2[k2, ax] = bmin[k2, ax]
    # 3: a direction component below 2^-100 or above the reciprocal's range
    k3 = np.nonzero(kind == 3)[0]
    ax3 = np.random.default_rng(seed + 2).integers(0, 3, len(k3))
    p2[k3] = q[k3]
    p2[k3, ax3] = p1[k3, ax3] + np.float32(1e-35)
    # 4: through an edge point with one nearly-parallel axis (tiny but usable
    #    reciprocal: the filtered test's huge-distance range)
    k4 = np.nonzero(kind == 4)[0]
    ax4 = np.random.default_rng(seed + 3).integers(0, 3, len(k4))
    p2[k4] = (p1 + np.float32(2.0) * d)[k4]
    p2[k4, ax4] = p1[k4, ax4] + np.float32(3e-25)
    p1_4 = np.zeros((n, 4), np.float32)
    p2_4 = np.zeros((n, 4), np.float32)
    p1_4[:, :3], p2_4[:, :3] = p1, p2
    return p1_4, p2_4


def _gpu_vs_oracle(ctx, cuda, s, p1, p2):
    ctx.upload_scene(s)
    n = len(p1)
    out = cuda.zeros(n, dtype=cuda.uint8, device="cuda")
    ctx.stats(reset=True)
    ctx.visibility_batch(cuda.from_numpy(p1).cuda(), cuda.from_numpy(p2).cuda(), out)
    got = out.cpu().numpy()
    exp = np.zeros(n, np.uint8)
    sc, keep = ob.scene_struct(s)
    p1c = np.ascontiguousarray(p1[:, :3])  # named: the oracle reads them through raw pointers
    p2c = np.ascontiguousarray(p2[:, :3])
    ob.oracle().or_test_visibility_batch(C.byref(sc), n, ob.P(p1c), ob.P(p2c), ob.P(exp), None)
    assert ctx.stats().traversal_errors == 0
    return got, exp


@pytest.mark.parametrize("layout", ["binary", "quant"])
def test_grazing_segments_bit_exact(ctx, cuda, cfg1_scene, layout):
    p1, p2 = _segments(cfg1_scene)
    ctx.set_tree_layout(layout)
    try:
        got, exp = _gpu_vs_oracle(ctx, cuda, cfg1_scene, p1, p2)
        assert (ctx.stats().tree_layout == 2) == (layout == "quant")
    finally:
        ctx.set_tree_layout("quant")
    bad = np.nonzero(got != exp)[0]
    assert len(bad) == 0, f"{len(bad)} of {len(got)} visibility bits differ, first at {bad[:8]}"
    assert 0.02 < exp.mean() < 0.98


def test_nan_box_bit_exact(ctx, cuda, cfg1_scene):
    """A NaN in the root's left box: under the GLSL min/max definitions the
    left subtree's slab test never passes, so those triangles never shadow."""
    s = cfg1_scene
    nodes = s.nodes.copy()
    nodes["lmin"][0, 0] = np.float32("nan")
    sn = dataclasses.replace(s, nodes=nodes)
    p1, p2 = _segments(s, seed=12, n=20_000)
    got, exp = _gpu_vs_oracle(ctx, cuda, sn, p1, p2)
    assert np.array_equal(got, exp), f"{np.count_nonzero(got != exp)} of {len(got)} bits differ"
    _, exp_clean = _gpu_vs_oracle(ctx, cuda, s, p1, p2)
    assert np.count_nonzero(exp != exp_clean) > 0  # the NaN changed the answers


@pytest.mark.parametrize("layout", ["wide", "quant"])
def test_wide_copy_on_config3_bit_exact(ctx, cuda, layout):
    """1,048,588 triangles with RG_TREE_WIDE4 or RG_TREE_QUANT4: the upload
    builds the 4-wide copy (exact boxes, every expanded box's children nested
    in it; or 8-bit boxes containing the exact ones over a tree nested
    throughout), and fast-path rays walk it; segments aimed at the boxes of
    the reference's tree (among them the boxes the collapse skips) and
    pixel-to-light style segments equal the oracle's bits."""
    from restir_gb300 import scenes
    s = scenes.config3(width=64, height=64, frames=1)
    p1, p2 = _segments(s, seed=21, n=60_000)
    rng = np.random.default_rng(22)
    m = 200_000
    q1 = np.zeros((m, 4), np.float32)
    q2 = np.zeros((m, 4), np.float32)
    q1[:, :3] = rng.uniform(0.0, 1.0, (m, 3))
    q2[:, :3] = s.point_lights["pos"][rng.integers(0, len(s.point_lights), m), :3]
    p1, p2 = np.concatenate([p1, q1]), np.concatenate([p2, q2])
    ctx.set_tree_layout(layout)
    try:
        got, exp = _gpu_vs_oracle(ctx, cuda, s, p1, p2)
        st = ctx.stats()
        assert st.wide_nodes > 0 and st.tree_layout == ctx.TREE_LAYOUTS[layout]
    finally:
        ctx.set_tree_layout("quant")
    bad = np.nonzero(got != exp)[0]
    assert len(bad) == 0, f"{len(bad)} of {len(got)} visibility bits differ, first at {bad[:8]}"
    assert 0.05 < exp.mean() < 0.95


def test_quant_copy_left_out_when_a_deep_box_is_not_nested(ctx, cuda, cfg1_scene):
    """The quantized copy tests only a triangle's own exact box, which keeps
    the answer only when every box of the tree lies inside its parent's:
    one inner node whose stored box is shrunk below its children's boxes
    (at any depth, where the exact 4-wide copy may not mind) and no
    quantized copy is built; the answers stay exact."""
    s = cfg1_scene
    nodes = s.nodes.copy()
    # a node two levels down whose left child is an inner node: shrink the
    # box it stores for that child
    pick = next(i for i in range(3, len(nodes)) if nodes["left"][i] >= 0)
    nodes["lmax"][pick, :3] -= np.float32(0.05) * (nodes["lmax"][pick, :3] - nodes["lmin"][pick, :3])
    sn = dataclasses.replace(s, nodes=nodes)
    p1, p2 = _segments(s, seed=24, n=30_000)
    ctx.set_tree_layout("quant")
    try:
        got, exp = _gpu_vs_oracle(ctx, cuda, sn, p1, p2)
        assert np.array_equal(got, exp), f"{np.count_nonzero(got != exp)} of {len(got)} bits differ"
        assert ctx.stats().wide_nodes == 0 and ctx.stats().tree_layout == 0
        ctx.upload_scene(s)
        assert ctx.stats().tree_layout == 2
    finally:
        ctx.set_tree_layout("quant")


@pytest.mark.parametrize("layout", ["wide", "quant"])
def test_wide_copy_left_out_when_boxes_are_not_nested(ctx, cuda, cfg1_scene, layout):
    """A tree whose root stores boxes smaller than its children's boxes
    (possible for a tree handed to rg_upload_scene): the collapse must skip
    one of those boxes, which would no longer keep the answer, so no 4-wide
    copy is built and every ray walks the reference's tree."""
    s = cfg1_scene
    nodes = s.nodes.copy()
    nodes["lmax"][0, :3] -= np.float32(0.3)
    nodes["rmax"][0, :3] -= np.float32(0.3)
    sn = dataclasses.replace(s, nodes=nodes)
    p1, p2 = _segments(s, seed=23, n=30_000)
    ctx.set_tree_layout(layout)
    try:
        got, exp = _gpu_vs_oracle(ctx, cuda, sn, p1, p2)
        assert np.array_equal(got, exp), f"{np.count_nonzero(got != exp)} of {len(got)} bits differ"
        assert ctx.stats().wide_nodes == 0
        ctx.upload_scene(s)
        assert ctx.stats().wide_nodes > 0
    finally:
        ctx.set_tree_layout("quant")
