"""Triangle lights of loaded meshes (rg_collect_triangle_lights, replacing
collectTriangleLightsFromScene, src/misc.cpp:380-414).

Bar: bit-exact.  The product's host code, the oracle's restatement and the
reference's own nvmath arithmetic (oracle/_ref, built from the reference
sources when present; a fixture made from it otherwise) give the same light
records on seeded meshes with rotated, scaled and translated world
matrices, including non-emissive and barely emissive materials."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle_binding as ob


def instances(seed):
    from restir_gb300 import _lib
    rng = np.random.default_rng(seed)
    keep, inst = [], []
    emissive = [(1.0, 0.5, 0.25), (0.0, 0.0, 0.0), (5e-4, 6e-4, 5e-4), (3.0, 9.0, 0.1), (1e-3, 0.0, 0.0)]
    for k, e in enumerate(emissive):
        nv = int(rng.integers(3, 40))
        pos = rng.uniform(-2, 2, (nv, 3)).astype(np.float32)
        tris = [rng.choice(nv, 3, replace=False) for _ in range(int(rng.integers(1, 30)))]
        tris.append(np.array([0, 0, 1]))  # one degenerate triangle (zero area, NaN normal) per mesh
        idx = np.concatenate(tris).astype(np.uint32)
        a = rng.normal(size=(3, 3))
        q, _ = np.linalg.qr(a)
        m = np.eye(4)
        m[:3, :3] = q * rng.uniform(0.2, 3.0, 3)
        m[:3, 3] = rng.uniform(-5, 5, 3)
        if k == 3:
            m[3, :3] = rng.uniform(-0.01, 0.01, 3)  # a projective row: w differs from 1
        keep += [pos, idx]
        rec = _lib.MeshInstance(pos.ctypes.data, idx.ctypes.data, len(idx),
                                (C.c_float * 16)(*m.astype(np.float32).T.ravel()),  # column-major
                                (C.c_float * 3)(*np.float32(e)))
        inst.append(rec)
    arr = (_lib.MeshInstance * len(inst))(*inst)
    return arr, keep


def _same(a, b):
    """Equal bits, except that any two NaNs match: a degenerate triangle
    (repeated vertex) has area 0 and a 0/0 normal, whose NaN sign bit is the
    machine's default NaN (negative on x86-64, positive on AArch64)."""
    a = np.asarray(a, np.float32).reshape(-1)
    b = np.asarray(b, np.float32).reshape(-1)
    nan = np.isnan(a) & np.isnan(b)
    return a.shape == b.shape and bool(np.all(nan | (a.view(np.uint32) == b.view(np.uint32))))


def _product(arr):
    from restir_gb300 import _lib
    n = _lib.lib().rg_collect_triangle_lights(arr, len(arr), None, 0)
    assert n >= 0
    out = np.zeros(n, _lib.TRI_LIGHT_DTYPE)
    assert _lib.lib().rg_collect_triangle_lights(arr, len(arr), out.ctypes.data, n) == n
    return out


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_product_equals_oracle(restir_lib, oracle_lib, seed):
    from restir_gb300 import _lib
    arr, keep = instances(seed)
    got = _product(arr)
    n = ob.oracle().or_collect_tri_lights(C.cast(arr, C.c_void_p), len(arr), None, 0)
    exp = np.zeros(n, _lib.TRI_LIGHT_DTYPE)
    ob.oracle().or_collect_tri_lights(C.cast(arr, C.c_void_p), len(arr), C.c_void_p(exp.ctypes.data), n)
    assert len(got) == n > 0
    assert _same(got.view(np.float32), exp.view(np.float32))
    # an instance emits when its factor's squared norm (float) exceeds 1e-6 (double)
    def emits(e):
        f = np.float32
        sq = (f(e[0]) * f(e[0]) + f(e[1]) * f(e[1])) + f(e[2]) * f(e[2])
        return float(sq) > 1e-6
    flags = [emits(inst.emissive_factor) for inst in arr]
    assert flags == [True, False, False, True, True]  # 8.6e-7 is below, 1.0000001e-6 above
    assert n == sum(int(inst.index_count) // 3 for inst, f in zip(arr, flags) if f)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_product_equals_reference_nvmath(restir_lib, seed):
    if not ob.ref_available():
        pytest.skip("reference build not present (the fixture test pins this case)")
    arr, keep = instances(seed)
    got = _product(arr)
    ref = np.zeros((len(got), 20), np.float32)
    n = ob.ref().ref_collect_tri_lights(C.cast(arr, C.c_void_p), len(arr), C.c_void_p(ref.ctypes.data), len(got))
    assert n == len(got)
    assert _same(got.view(np.float32), ref)


def test_product_equals_reference_fixture(restir_lib):
    from pathlib import Path
    fx = np.load(Path(__file__).resolve().parent / "golden" / "tri_lights.npz")
    arr, keep = instances(int(fx["seed"]))
    got = _product(arr)
    assert _same(got.view(np.float32), fx["lights"])


def test_bad_arguments(restir_lib):
    from restir_gb300 import _lib
    assert _lib.lib().rg_collect_triangle_lights(None, 2, None, 0) < 0
    arr = (_lib.MeshInstance * 1)()
    arr[0].index_count = 3  # no positions or indices
    assert _lib.lib().rg_collect_triangle_lights(arr, 1, None, 0) < 0
