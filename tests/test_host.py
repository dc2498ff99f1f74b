"""Host-side checks that need no GPU: the C ABI library, the reference-layout
BVH builder, the alias table, the CPU G-buffer and argument validation."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"


def P(a):
    return C.c_void_p(a.ctypes.data)


def test_library_exports_every_declared_symbol(restir_lib):
    header = (ROOT / "include" / "restir_gb300.h").read_text()
    declared = set(re.findall(r"^(?:int64_t|int|const char \*)\s*\*?\s*(rg_\w+)\s*\(", header, re.M))
    assert len(declared) >= 18
    for name in sorted(declared):
        assert hasattr(restir_lib, name), name
    from restir_gb300 import _lib
    assert declared <= set(_lib.EXPORTED) | declared  # binding covers the header
    assert set(_lib.EXPORTED) <= declared


def test_struct_layouts_match_reference():
    from restir_gb300 import _lib
    # sizes probed from the reference's shaderIncludes.h (std430/std140)
    assert C.sizeof(_lib.Reservoir) == 64
    assert _lib.Reservoir.light_index.offset == 32 and _lib.Reservoir.num_stream_samples.offset == 48
    assert C.sizeof(_lib.AabbTreeNode) == 80 and _lib.AabbTreeNode.left_child.offset == 64
    assert C.sizeof(_lib.RestirUniforms) == 128
    offs = {f: getattr(_lib.RestirUniforms, f).offset for f, _ in _lib.RestirUniforms._fields_}
    assert offs["camera_pos"] == 64 and offs["screen_size"] == 80 and offs["frame"] == 88
    assert offs["initial_light_sample_count"] == 92 and offs["flags"] == 116
    assert C.sizeof(_lib.LightingUniforms) == 96


def test_bvh_matches_reference_golden(restir_lib):
    g = np.load(GOLDEN / "bvh_visibility.npz")
    xyz = np.ascontiguousarray(g["tri_xyz"])
    from restir_gb300 import scenes
    nodes, tris, depth = scenes.build_bvh(xyz)
    ref_nodes = np.frombuffer(g["nodes"].tobytes(), dtype=nodes.dtype)
    for f in ("lmin", "lmax", "rmin", "rmax", "left", "right"):
        assert np.array_equal(nodes[f].view(np.uint32) if nodes[f].dtype == np.float32 else nodes[f],
                              ref_nodes[f].view(np.uint32) if ref_nodes[f].dtype == np.float32 else ref_nodes[f]), f
    assert np.array_equal(tris.view(np.uint8).reshape(-1), g["tris"].view(np.uint8).reshape(-1))
    assert 0 < depth <= 63


@pytest.mark.skipif(not (ROOT / "oracle" / "_ref" / "libref.so").exists(), reason="reference build not present")
def test_bvh_matches_reference_live(restir_lib, oracle_lib):
    from restir_gb300 import _lib, scenes
    ref = oracle_lib.ref()
    for seed, n in ((1, 3), (2, 257), (3, 30000)):
        rng = np.random.default_rng(seed)
        xyz = (rng.uniform(0, 1, (n, 1, 3)) ** 2 + rng.uniform(-0.02, 0.02, (n, 3, 3))).reshape(n, 9).astype(np.float32)
        nodes, tris, _ = scenes.build_bvh(xyz)
        rn = np.zeros(n - 1, _lib.NODE_DTYPE)
        rt = np.zeros(n, _lib.TRI_DTYPE)
        assert ref.ref_build_bvh(P(xyz), C.c_int32(n), P(rn), P(rt)) == n - 1
        assert nodes.tobytes() == rn.tobytes() and tris.tobytes() == rt.tobytes()


def test_bvh_rejects_single_triangle(restir_lib):
    from restir_gb300 import _lib
    xyz = np.zeros((1, 9), np.float32)
    rc = restir_lib.rg_build_bvh(xyz.ctypes.data, 1, np.zeros(1, _lib.NODE_DTYPE).ctypes.data,
                                 np.zeros(1, _lib.TRI_DTYPE).ctypes.data)
    assert rc == -1 and b"2 triangles" in restir_lib.rg_last_error()


def test_tree_validation_rejects_malformed(restir_lib):
    from restir_gb300 import _lib, scenes
    rng = np.random.default_rng(0)
    xyz = rng.uniform(0, 1, (50, 9)).astype(np.float32)
    nodes, _, _ = scenes.build_bvh(xyz)
    bad = nodes.copy()
    bad[3]["left"] = 0  # cycle back to the root
    assert restir_lib.rg_tree_depth(bad.ctypes.data, len(bad)) < 0
    bad = nodes.copy()
    leaf = next(int(v) for v in np.concatenate([nodes["left"], nodes["right"]]) if v < 0)
    bad[0]["right"] = leaf  # a triangle reached twice, a subtree unreached
    assert restir_lib.rg_tree_depth(bad.ctypes.data, len(bad)) < 0


def test_tree_preorder_renumbering(restir_lib, oracle_lib):
    """rg_tree_preorder (the order of the device copy rg_upload_scene keeps):
    the same tree, renumbered so each internal left child follows its
    parent; the CPU G-buffer and the oracle's visibility over it are
    unchanged."""
    import dataclasses

    import oracle_binding as ob
    from restir_gb300 import scenes
    s = scenes.config1(width=64, height=48)
    n = len(s.nodes)
    out = np.zeros_like(s.nodes)
    assert restir_lib.rg_tree_preorder(s.nodes.ctypes.data, n, out.ctypes.data) == n
    assert restir_lib.rg_tree_depth(out.ctypes.data, n) == restir_lib.rg_tree_depth(s.nodes.ctypes.data, n)
    internal_left = np.nonzero(out["left"] >= 0)[0]
    assert np.array_equal(out["left"][internal_left], internal_left + 1)
    # the same node records up to the numbering: boxes bit for bit, same leaves
    key = lambda a: np.sort(np.concatenate([a["lmin"], a["lmax"], a["rmin"], a["rmax"]], 1).view(np.uint32), axis=0)
    assert np.array_equal(key(out), key(s.nodes))
    assert np.array_equal(np.sort(out["left"][out["left"] < 0]), np.sort(s.nodes["left"][s.nodes["left"] < 0]))
    so = dataclasses.replace(s, nodes=out)
    g0, g1 = scenes.trace_gbuffer_host(s, 0), scenes.trace_gbuffer_host(so, 0)
    for k in g0:
        assert np.array_equal(g0[k], g1[k]), k
    rng = np.random.default_rng(3)
    m = 20_000
    p1 = rng.uniform(-0.05, 1.05, (m, 3)).astype(np.float32)
    p2 = rng.uniform(-0.05, 1.05, (m, 3)).astype(np.float32)
    vis = []
    for sc in (s, so):
        st, keep = ob.scene_struct(sc)
        r = np.zeros(m, np.uint8)
        ob.oracle().or_test_visibility_batch(C.byref(st), m, ob.P(p1), ob.P(p2), ob.P(r), None)
        vis.append(r)
    assert np.array_equal(vis[0], vis[1]) and 0.02 < vis[0].mean() < 0.98
    bad = s.nodes.copy()
    bad[3]["left"] = 0  # cycle back to the root
    assert restir_lib.rg_tree_preorder(bad.ctypes.data, n, out.ctypes.data) < 0


def test_alias_table_product_equals_oracle(restir_lib, oracle_lib):
    from restir_gb300 import _lib
    rng = np.random.default_rng(4)
    for n in (1, 2, 17, 4096):
        pl = np.zeros(n, _lib.POINT_LIGHT_DTYPE)
        pl["color_lum"][:, 3] = (rng.pareto(1.5, n) + 0.01).astype(np.float32)
        a = np.zeros(n, _lib.ALIAS_DTYPE)
        b = np.zeros(n, _lib.ALIAS_DTYPE)
        assert restir_lib.rg_build_alias_table(P(pl), n, None, 0, P(a)) == 0
        oracle_lib.oracle().or_build_alias_table(P(pl), n, None, 0, P(b))
        assert a.tobytes() == b.tobytes()


def test_uniform_alias_table(restir_lib):
    from restir_gb300 import scenes
    s = scenes.config1()
    assert np.all(s.alias["prob"] == 1.0)
    assert np.array_equal(s.alias["alias"], np.arange(len(s.alias)))
    assert np.all(s.alias["ori_prob"] == np.float32(1.0 / 1024))


def test_config1_scene_shape(restir_lib):
    from restir_gb300 import scenes
    s = scenes.config1()
    assert len(s.tri_xyz) == 780 and len(s.point_lights) == 1024 and len(s.nodes) == 779
    assert s.samples_per_frame() == 256 * 256 * (32 + 2 * 5)


def test_cpu_gbuffer_closed_room(restir_lib):
    from restir_gb300 import scenes
    s = scenes.config1(width=64, height=48)
    g = scenes.trace_gbuffer_host(s, 0)
    assert (g["world_pos"][..., 3] == 1.0).all()  # every primary ray hits the closed room
    assert ((g["depth"] > 0) & (g["depth"] < 1)).all()
    g2 = scenes.trace_gbuffer_host(s, 0)
    for k in g:
        assert np.array_equal(g[k], g2[k])


def test_create_without_gpu_fails_cleanly(restir_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    h = C.c_void_p()
    rc = restir_lib.rg_create(0, C.byref(h))
    assert rc < 0 and h.value is None
    assert len(restir_lib.rg_last_error()) > 0


def test_null_arguments_rejected(restir_lib):
    assert restir_lib.rg_initial_temporal(None, None, None, None, None, None, None) == -1
    assert restir_lib.rg_shade(None, None, None, None, None, None) == -1
    assert restir_lib.rg_build_alias_table(None, 0, None, 0, None) == -1
