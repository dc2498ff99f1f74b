"""The GPU tree builder (rg_build_bvh_device) against the host builder, which
is byte-identical to the reference's AabbTree::build.

Bar: bit-exact.  Node and triangle buffers equal rg_build_bvh's byte for
byte, on the configurations' scenes (780 to 1,048,588 triangles) and on
inputs that exercise the median-split fallback (coincident centroids), and
the reference-undefined flag agrees."""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host(tri_xyz):
    from restir_gb300 import _lib
    n = len(tri_xyz)
    nodes = np.zeros(n - 1, _lib.NODE_DTYPE)
    tris = np.zeros(n, _lib.TRI_DTYPE)
    xyz = np.ascontiguousarray(tri_xyz, np.float32)
    rc = _lib.lib().rg_build_bvh(xyz.ctypes.data, n, nodes.ctypes.data, tris.ctypes.data)
    assert rc == n - 1
    return nodes, tris


def _device(ctx, cuda, tri_xyz):
    from restir_gb300 import _lib
    n = len(tri_xyz)
    xyz = cuda.from_numpy(np.ascontiguousarray(tri_xyz, np.float32)).cuda()
    nodes = cuda.zeros((n - 1) * 80, dtype=cuda.uint8, device="cuda")
    tris = cuda.zeros(n * 48, dtype=cuda.uint8, device="cuda")
    undef = C.c_int32(-1)
    cuda.cuda.synchronize()
    t0 = time.perf_counter()
    rc = _lib.lib().rg_build_bvh_device(ctx._h, xyz.data_ptr(), n, nodes.data_ptr(), tris.data_ptr(), C.byref(undef),
                                        None)
    dt = time.perf_counter() - t0
    assert rc == n - 1, _lib.lib().rg_last_error()
    return (nodes.cpu().numpy().view(_lib.NODE_DTYPE), tris.cpu().numpy().view(_lib.TRI_DTYPE), undef.value, dt)


def _compare(ctx, cuda, tri_xyz):
    hn, ht = _host(tri_xyz)
    dn, dt_, undef, sec = _device(ctx, cuda, tri_xyz)
    assert np.array_equal(hn.view(np.uint8), dn.view(np.uint8)), \
        f"{np.count_nonzero(np.any(hn.view(np.uint32).reshape(len(hn), -1) != dn.view(np.uint32).reshape(len(dn), -1), 1))} nodes differ"
    assert np.array_equal(ht.view(np.uint8), dt_.view(np.uint8))
    return undef, sec


@pytest.mark.parametrize("name", ["config1", "config2_small", "config2", "config3"])
def test_gpu_tree_equals_host_tree(ctx, cuda, name):
    from restir_gb300 import scenes
    if name == "config1":
        xyz = scenes.config1().tri_xyz
    elif name == "config2_small":
        xyz = scenes.config2(width=8, height=8, n_tris=20_000, n_lights=16, frames=1).tri_xyz
    elif name == "config2":
        xyz = scenes.config2(width=8, height=8, n_lights=16, frames=1).tri_xyz
    else:
        xyz = scenes.config3(width=8, height=8, frames=1).tri_xyz
    undef, sec = _compare(ctx, cuda, xyz)
    assert undef == 0
    print(f"{name}: {len(xyz)} triangles, GPU build {sec * 1e3:.1f} ms")


def test_gpu_tree_fallback_paths(ctx, cuda):
    rng = np.random.default_rng(3)
    base = rng.uniform(0, 1, (200, 9)).astype(np.float32)
    dup = np.repeat(base[:7], 9, axis=0)            # coincident centroids: median split
    tiny = np.tile(np.float32([0, 0, 0, 1, 0, 0, 0, 1, 0]), (5, 1))  # identical triangles
    neg = -base[:40]                                 # negative coordinates (and -0 from sign flips of 0)
    neg[0, :3] = -0.0
    undefs = [_compare(ctx, cuda, xyz)[0] for xyz in (dup, tiny, neg, base[:2], base[:3], np.concatenate([base, dup]))]
    assert undefs[1] == 1  # identical triangles: every split is the median one
