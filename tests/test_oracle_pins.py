"""The oracle against the reference's own code.

Golden fixtures (tests/golden/*.npz) were produced by the reference's
sources compiled on the CPU (tests/golden/make_golden.py); when the
reference build (oracle/_ref) is present the same checks also run live on
fresh inputs.  Everything here is bit-exact.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def P(a):
    return C.c_void_p(a.ctypes.data)


def test_pcg32_known_answer(oracle_lib):
    # pcg32 demo output (initstate 42, initseq 54); the reference's seedRand
    # (src/shaders/include/rand.glsl:20-28) is pcg32_srandom_r.
    out = np.zeros(6, np.uint32)
    oracle_lib.oracle().or_pcg_stream(42, 54, 6, P(out))
    assert [int(v) for v in out] == [0xa15c02b7, 0x7b47f409, 0xba1d3330, 0x83d2f293, 0xbfa4784b, 0xcbed606e]


def test_rand_float_can_be_one(oracle_lib):
    # randUint / 2^32 in float rounds values >= 2^32-128 up to exactly 1.0
    # (reference quirk, rand.glsl:30-32); check the conversion rule itself.
    u = np.array([0xFFFFFFFF, 0xFFFFFF80, 0xFFFFFF7F], np.uint64)
    f = (u.astype(np.float32) / np.float32(4294967296.0))
    assert f[0] == 1.0 and f[1] == 1.0 and f[2] < 1.0
    r = np.zeros(1000, np.float32)
    oracle_lib.oracle().or_rand_floats(7, 11, 1000, P(r))
    assert (r >= 0).all() and (r <= 1).all()


def test_phat_golden(oracle_lib):
    g = np.load(GOLDEN / "phat.npz")
    a = np.ascontiguousarray(g["args"])
    out = np.zeros(len(a), np.float32)
    oracle_lib.oracle().or_eval_phat_batch(len(a), P(a), P(out))
    assert np.array_equal(out.view(np.uint32), g["phat"].view(np.uint32))
    b = np.ascontiguousarray(g["args_full"])
    out3 = np.zeros(3 * len(b), np.float32)
    oracle_lib.oracle().or_eval_phat_full_batch(len(b), P(b), P(out3))
    assert np.array_equal(out3.view(np.uint32), g["phat_full"].reshape(-1).view(np.uint32))


def test_intersection_golden(oracle_lib):
    g = np.load(GOLDEN / "intersect.npz")
    r = np.ascontiguousarray(g["box_args"])
    out = np.zeros(len(r), np.uint8)
    oracle_lib.oracle().or_ray_aabb_batch(len(r), P(r), P(out))
    assert np.array_equal(out, g["box"])
    t = np.ascontiguousarray(g["tri_args"])
    out = np.zeros(len(t), np.uint8)
    oracle_lib.oracle().or_ray_tri_batch(len(t), P(t), P(out))
    assert np.array_equal(out, g["tri"])


def test_visibility_golden(oracle_lib):
    g = np.load(GOLDEN / "bvh_visibility.npz")
    nodes = np.ascontiguousarray(g["nodes"])
    tris = np.ascontiguousarray(g["tris"])
    nt = len(tris) // 12
    sc = oracle_lib.Scene(nodes.ctypes.data, nt - 1, tris.ctypes.data, nt, None, 0, None, 0, None, 0)
    p1, p2 = np.ascontiguousarray(g["p1"]), np.ascontiguousarray(g["p2"])
    out = np.zeros(len(p1), np.uint8)
    st = oracle_lib.Stats()
    oracle_lib.oracle().or_test_visibility_batch(C.byref(sc), len(p1), P(p1), P(p2), P(out), C.byref(st))
    assert np.array_equal(out, g["shadowed"])
    assert st.stack_overflows == 0 and st.rays == len(p1)


@pytest.mark.skipif(not (Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "libref.so").exists(),
                    reason="reference build (oracle/_ref) not present")
def test_phat_and_traversal_live_against_reference(oracle_lib):
    ref = oracle_lib.ref()
    rng = np.random.default_rng(99)
    from golden.make_golden import phat_args  # noqa
    a = phat_args(rng, 50000)
    o1 = np.zeros(len(a), np.float32)
    o2 = np.zeros(len(a), np.float32)
    oracle_lib.oracle().or_eval_phat_batch(len(a), P(a), P(o1))
    ref.ref_eval_phat_batch(C.c_int32(len(a)), P(a), P(o2))
    assert np.array_equal(o1.view(np.uint32), o2.view(np.uint32))
    # traversal on a deeper, clustered soup
    nt = 20000
    xyz = (rng.uniform(0, 1, (nt, 1, 3)) ** 3 + rng.uniform(-0.01, 0.01, (nt, 3, 3))).reshape(nt, 9).astype(np.float32)
    nodes = np.zeros((nt - 1) * 20, np.float32)
    tris = np.zeros(nt * 12, np.float32)
    assert ref.ref_build_bvh(P(xyz), C.c_int32(nt), P(nodes), P(tris)) == nt - 1
    n = 40000
    p1 = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    p2 = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    r1 = np.zeros(n, np.uint8)
    r2 = np.zeros(n, np.uint8)
    assert ref.ref_test_visibility_batch(P(nodes), C.c_int32(nt - 1), P(tris), C.c_int32(nt), C.c_int32(n), P(p1),
                                         P(p2), P(r2)) == 0
    sc = oracle_lib.Scene(nodes.ctypes.data, nt - 1, tris.ctypes.data, nt, None, 0, None, 0, None, 0)
    oracle_lib.oracle().or_test_visibility_batch(C.byref(sc), n, P(p1), P(p2), P(r1), None)
    assert np.array_equal(r1, r2)
    assert 0.05 < r1.mean() < 0.95


def test_sincos_accuracy(oracle_lib):
    # the spatial passes' project-defined sin/cos: within 2 ulp-ish of the
    # exact value on the domain used (angle in [0, 2*pi], plus radians(25)).
    x = np.concatenate([np.linspace(0, 2 * math.pi, 200001, dtype=np.float32),
                        np.array([np.float32(25.0) * np.float32(0.0174532923847436905)], np.float32)])
    s = np.zeros_like(x)
    c = np.zeros_like(x)
    oracle_lib.oracle().or_sincos_batch(len(x), P(x), P(s), P(c))
    xd = x.astype(np.float64)
    assert np.max(np.abs(s - np.sin(xd))) < 3e-7
    assert np.max(np.abs(c - np.cos(xd))) < 3e-7


def test_alias_table_is_vose(oracle_lib):
    # the table reproduces the normalised weights exactly in expectation
    rng = np.random.default_rng(3)
    n = 1000
    from restir_gb300 import _lib
    pl = np.zeros(n, _lib.POINT_LIGHT_DTYPE)
    pl["color_lum"][:, 3] = rng.pareto(1.5, n).astype(np.float32) + 0.01
    tab = np.zeros(n, _lib.ALIAS_DTYPE)
    oracle_lib.oracle().or_build_alias_table(P(pl), n, None, 0, P(tab))
    mass = tab["prob"].astype(np.float64) / n
    np.add.at(mass, tab["alias"], (1.0 - tab["prob"].astype(np.float64)) / n)
    w = pl["color_lum"][:, 3].astype(np.float64)
    assert np.allclose(mass, w / w.sum(), rtol=1e-4, atol=1e-7)
    assert np.allclose(tab["ori_prob"], w / w.sum(), rtol=1e-5)
