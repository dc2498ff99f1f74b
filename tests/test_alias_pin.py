"""createAliasTable pinned against the reference's own code.

Both restatements of the reference's Vose alias-table build
(src/misc.cpp:416-497) -- the library's rg_build_alias_table (host.cpp) and
the oracle's or_build_alias_table -- must equal the reference's function bit
for bit: prob, alias, oriProb and aliasOriProb of every column.  The golden
fixture (tests/golden/alias.npz, tests/golden/make_golden.py) holds the
reference's output on seeded light sets, so the pin also runs where the
reference sources are absent; where oracle/_ref/libref_alias.so is built (the
function copied unchanged from the sources by oracle/Makefile) the same
check runs live on the configurations' own light sets, 1,048,576 lights
included.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def P(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _product(restir_lib, pl, tl):
    n = len(pl) if pl is not None else len(tl)
    out = np.zeros((n, 4), np.float32)
    rc = restir_lib.rg_build_alias_table(P(pl), 0 if pl is None else len(pl), P(tl), 0 if tl is None else len(tl),
                                         P(out))
    assert rc == 0
    return out


def _oracle(oracle_lib, pl, tl):
    n = len(pl) if pl is not None else len(tl)
    out = np.zeros((n, 4), np.float32)
    oracle_lib.oracle().or_build_alias_table(P(pl), 0 if pl is None else len(pl), P(tl), 0 if tl is None else len(tl),
                                             P(out))
    return out


def _sets_from_golden():
    g = np.load(GOLDEN / "alias.npz")
    names = sorted({k.split("__")[0] for k in g.files})
    for name in names:
        pl = np.ascontiguousarray(g[f"{name}__points"]) if f"{name}__points" in g.files else None
        tl = np.ascontiguousarray(g[f"{name}__tris"]) if f"{name}__tris" in g.files else None
        yield name, pl, tl, g[f"{name}__table"]


def test_alias_tables_equal_reference_golden(restir_lib, oracle_lib):
    count = 0
    for name, pl, tl, ref in _sets_from_golden():
        for who, got in (("library", _product(restir_lib, pl, tl)), ("oracle", _oracle(oracle_lib, pl, tl))):
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), f"{who} differs on {name}"
        count += 1
    assert count >= 8


def test_alias_tables_equal_reference_live(restir_lib, oracle_lib):
    lib = oracle_lib.ref_alias()
    if lib is None:
        pytest.skip("reference build (oracle/_ref/libref_alias.so) not present")
    from restir_gb300 import scenes
    sets = [("config1 (uniform weights)", scenes.config1().point_lights.copy()),
            ("config2", scenes.config2(width=64, height=64, frames=1).point_lights),
            ("config3", scenes.config3(width=64, height=64, frames=1).point_lights)]
    sets[0][1]["color_lum"][:, 3] = 1.0  # the uniform source pdf's table
    for name, pl in sets:
        pl = np.ascontiguousarray(pl)
        ref = np.zeros((len(pl), 4), np.float32)
        assert lib.ref_create_alias_table(P(pl), len(pl), None, 0, P(ref)) == len(pl)
        for who, got in (("library", _product(restir_lib, pl, None)), ("oracle", _oracle(oracle_lib, pl, None))):
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), f"{who} differs on {name}"
    tl = np.ascontiguousarray(scenes.config1_triangle_lights().tri_lights)
    ref = np.zeros((len(tl), 4), np.float32)
    assert lib.ref_create_alias_table(None, 0, P(tl), len(tl), P(ref)) == len(tl)
    assert np.array_equal(_product(restir_lib, None, tl).view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(_oracle(oracle_lib, None, tl).view(np.uint32), ref.view(np.uint32))
