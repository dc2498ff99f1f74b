"""The oracle's restatement of the reference's tree builder, pinned.

or_build_bvh restates AabbTree::build (src/aabbTreeBuilder.cpp:52-214) so
that runs which must not load the library (the reference arm of bench.py)
still get the reference's tree.  Its node and triangle buffers must equal,
byte for byte, the reference builder's own output: the golden fixture made
by the reference compiled from its sources (tests/golden/bvh_visibility.npz)
and, where that build is present, the reference builder run live on the
configurations' triangle sets (780 to 1,048,588 triangles).  The library's
builder (rg_build_bvh) is held to the same bytes in tests/test_host.py.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def P(a):
    return C.c_void_p(a.ctypes.data)


def test_oracle_tree_equals_reference_golden(oracle_lib):
    g = np.load(GOLDEN / "bvh_visibility.npz")
    nodes, tris, depth = oracle_lib.build_bvh(g["tri_xyz"])
    assert np.array_equal(nodes.view(np.uint8).reshape(-1), g["nodes"].reshape(-1))
    assert np.array_equal(tris.view(np.float32).reshape(-1).view(np.uint32), g["tris"].view(np.uint32))
    assert depth > 5


def test_oracle_tree_equals_reference_live(oracle_lib, restir_lib):
    if not oracle_lib.ref_available():
        pytest.skip("reference build (oracle/_ref/libref.so) not present")
    from restir_gb300 import scenes
    ref = oracle_lib.ref()
    sets = [scenes.config1().tri_xyz, scenes.config2(width=64, height=64, frames=1).tri_xyz,
            scenes.config3(width=64, height=64, frames=1).tri_xyz]
    xyz = sets[0].copy()
    xyz[::5, 0] = -0.0  # the world-matrix product turns -0 into +0
    sets.append(xyz)
    for xyz in sets:
        xyz = np.ascontiguousarray(xyz, np.float32)
        n = len(xyz)
        rn = np.zeros((n - 1) * 20, np.float32)
        rt = np.zeros(n * 12, np.float32)
        assert ref.ref_build_bvh(P(xyz), C.c_int32(n), P(rn), P(rt)) == n - 1
        nodes, tris, _ = oracle_lib.build_bvh(xyz)
        assert np.array_equal(nodes.view(np.uint32).reshape(-1), rn.view(np.uint32)), n
        assert np.array_equal(tris.view(np.uint32).reshape(-1), rt.view(np.uint32)), n


def test_oracle_tree_rejects_what_the_reference_leaves_undefined(oracle_lib):
    xyz = np.tile(np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32), (5, 1))  # 5 identical triangles
    with pytest.raises(RuntimeError):
        oracle_lib.build_bvh(xyz)
    with pytest.raises(RuntimeError):
        oracle_lib.build_bvh(xyz[:1])
