"""Generates tests/golden/*.npz from the reference's own code.

The reference ships no golden vectors or tests, so the fixtures come from
the reference sources compiled on the CPU (oracle/_ref/libref.so, built by
oracle/Makefile from the reference tree): its BVH builder
(src/aabbTreeBuilder.cpp), its p-hat / BRDF (src/shaders/include/
restirUtils.glsl, disneyBRDF.glsl) and its shadow-ray traversal
(src/shaders/include/softwareRaytracing.glsl, visibilityTest.glsl) on seeded
inputs, and its createAliasTable (src/misc.cpp, the function copied
unchanged out of the sources by oracle/Makefile) on seeded light sets.
PCG32 known answers come from the published PCG32 reference output for the
demo seeds (state 42, sequence 54).

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle_binding as ob  # noqa: E402

OUT = Path(__file__).resolve().parent


def P(a):
    return C.c_void_p(a.ctypes.data)


def phat_args(rng, n):
    a = np.zeros((n, 20), np.float32)
    a[:, 0:3] = rng.uniform(0, 1, (n, 3))
    a[:, 3:6] = rng.uniform(0, 1, (n, 3))
    a[:, 6:9] = rng.uniform(0, 1, (n, 3))
    nn = rng.normal(size=(n, 3)); nn /= np.linalg.norm(nn, axis=1, keepdims=True)
    ln = rng.normal(size=(n, 3)); ln /= np.linalg.norm(ln, axis=1, keepdims=True)
    a[:, 9:12] = nn
    a[:, 12:15] = ln
    a[:, 15] = rng.integers(0, 2, n)
    a[:, 16] = rng.uniform(0, 1, n)
    a[:, 17] = rng.uniform(0, 10, n)
    a[:, 18] = rng.uniform(0, 1, n)
    a[:, 19] = (rng.uniform(0, 1, n) < 0.3)
    return a


def tri_lights(seed=7):
    """Triangle lights of the seeded meshes of tests/test_tri_lights.py as the
    reference's nvmath arithmetic computes them (oracle/ref_lights_bridge.cpp)."""
    sys.path.insert(0, str(ROOT / "tests"))
    sys.path.insert(0, str(ROOT / "restir-vulkan_gb300"))
    import test_tri_lights as tt
    arr, keep = tt.instances(seed)
    ref = ob.ref()
    n = ref.ref_collect_tri_lights(C.cast(arr, C.c_void_p), len(arr), None, 0)
    out = np.zeros((n, 20), np.float32)
    ref.ref_collect_tri_lights(C.cast(arr, C.c_void_p), len(arr), C.c_void_p(out.ctypes.data), n)
    np.savez_compressed(OUT / "tri_lights.npz", seed=np.int64(seed), lights=out)


def alias_light_sets(seed=20261204):
    """Seeded light sets for the alias-table pin: (name, point lights as
    (n, 8) float32 records, triangle lights as (n, 20) float32 records).
    Only the luminance (points) or emission luminance x area (triangles)
    enters the table, so the other fields stay zero."""
    rng = np.random.default_rng(seed)

    def points(lum):
        a = np.zeros((len(lum), 8), np.float32)
        a[:, 3] = 1.0
        a[:, 7] = lum
        return a

    sets = [("one_light", points(np.array([3.0], np.float32)), None),
            ("two_equal", points(np.array([1.0, 1.0], np.float32)), None),
            ("uniform_1000", points(np.ones(1000, np.float32)), None),
            ("loguniform_777", points(np.exp(rng.uniform(np.log(0.01), np.log(100), 777)).astype(np.float32)), None),
            ("pareto_5000", points(((1 - rng.uniform(0, 1, 5000)) ** (-1 / 1.5)).astype(np.float32)), None)]
    z = rng.uniform(0, 1, 3000).astype(np.float32)
    z[::3] = 0.0
    sets.append(("with_zero_power_3000", points(z), None))
    dom = np.full(513, 1e-3, np.float32)
    dom[17] = 1e4
    sets.append(("one_dominant_513", points(dom), None))
    tl = np.zeros((600, 20), np.float32)
    tl[:, 15] = rng.uniform(0.1, 5, 600)
    tl[:, 19] = rng.uniform(1e-4, 1e-2, 600)
    sets.append(("triangles_600", None, tl))
    return sets


def alias_tables():
    """The reference's createAliasTable (src/misc.cpp, compiled unchanged by
    oracle/Makefile into _ref/libref_alias.so) on seeded light sets."""
    lib = ob.ref_alias()
    arrays = {}
    for name, pl, tl in alias_light_sets():
        n = len(pl) if pl is not None else len(tl)
        out = np.zeros((n, 4), np.float32)
        k = lib.ref_create_alias_table(P(pl) if pl is not None else None, 0 if pl is None else len(pl),
                                       P(tl) if tl is not None else None, 0 if tl is None else len(tl), P(out))
        assert k == n
        if pl is not None:
            arrays[f"{name}__points"] = pl
        if tl is not None:
            arrays[f"{name}__tris"] = tl
        arrays[f"{name}__table"] = out
    np.savez_compressed(OUT / "alias.npz", **arrays)


def main():
    ob.build(ref=True)
    ref = ob.ref()
    rng = np.random.default_rng(20261203)

    # p-hat (luminance) and p-hat (RGB)
    n = 4096
    a = phat_args(rng, n)
    out = np.zeros(n, np.float32)
    ref.ref_eval_phat_batch(C.c_int32(n), P(a), P(out))
    b = np.zeros((n, 24), np.float32)
    b[:, :16] = a[:, :16]
    b[:, 16:19] = rng.uniform(0, 1, (n, 3))
    b[:, 19:22] = rng.uniform(0, 10, (n, 3))
    b[:, 22:24] = a[:, 18:20]
    out3 = np.zeros(3 * n, np.float32)
    ref.ref_eval_phat_full_batch(C.c_int32(n), P(b), P(out3))
    np.savez_compressed(OUT / "phat.npz", args=a, phat=out, args_full=b, phat_full=out3.reshape(n, 3))

    # ray-box / ray-triangle with axis-aligned and degenerate cases
    r = rng.uniform(-1, 2, (n, 12)).astype(np.float32)
    r[::7, 3] = 0.0
    r[::11, 4] = 0.0
    r[::13, 6] = r[::13, 0]
    r[::29, 3:6] = 0.0
    box = np.zeros(n, np.uint8)
    ref.ref_ray_aabb_batch(C.c_int32(n), P(r), P(box))
    t = rng.uniform(-1, 2, (n, 15)).astype(np.float32)
    t[::5, 9:12] = t[::5, 6:9]  # degenerate (p1 == p2)
    tri = np.zeros(n, np.uint8)
    ref.ref_ray_tri_batch(C.c_int32(n), P(t), P(tri))
    np.savez_compressed(OUT / "intersect.npz", box_args=r, box=box, tri_args=t, tri=tri)

    # BVH of a seeded triangle soup (+ a -0.0 coordinate) and shadow rays on it
    nt = 2000
    centers = rng.uniform(0, 1, (nt, 1, 3))
    xyz = (centers + rng.uniform(-0.04, 0.04, (nt, 3, 3))).reshape(nt, 9).astype(np.float32)
    xyz[::37, 0] = -0.0
    nodes = np.zeros((nt - 1) * 20, np.float32)
    tris = np.zeros(nt * 12, np.float32)
    k = ref.ref_build_bvh(P(xyz), C.c_int32(nt), P(nodes), P(tris))
    assert k == nt - 1
    nr = 8192
    p1 = rng.uniform(0, 1, (nr, 3)).astype(np.float32)
    p2 = rng.uniform(0, 1, (nr, 3)).astype(np.float32)
    p2[::97] = p1[::97]  # zero-length segment
    shadowed = np.zeros(nr, np.uint8)
    rc = ref.ref_test_visibility_batch(P(nodes), C.c_int32(nt - 1), P(tris), C.c_int32(nt), C.c_int32(nr), P(p1),
                                       P(p2), P(shadowed))
    assert rc == 0
    np.savez_compressed(OUT / "bvh_visibility.npz", tri_xyz=xyz, nodes=nodes.view(np.uint8), tris=tris,
                        p1=p1, p2=p2, shadowed=shadowed)
    tri_lights()
    alias_tables()
    print("wrote", sorted(p.name for p in OUT.glob("*.npz")))


if __name__ == "__main__":
    main()
