"""RESERVOIR_SIZE > 1 and UNBIASED_MIS (restirStructs.glsl:16-17): the
oracle's variant builds against the reference's own reservoir.glsl compiled
for the same variant (oracle/_ref/libref_res_*.so), on scripted sequences of
addSampleToReservoir and combineReservoirs with seeded PCG streams.

Bar: bit-exact, including the reference's swapped (w, sumPHat) arguments in
combineReservoirs under UNBIASED_MIS (reservoir.glsl:55-60), which the oracle
keeps unless RG_FLAG_MIS_SWAP_FIX / swap_fix asks for the declared order."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle_binding as ob

VARIANTS = [(1, 0), (2, 0), (1, 1), (2, 1)]


def _script_inputs(rng, rs, mis):
    n = int(rng.integers(1, 40))
    cand = np.zeros((n, 12), np.float32)
    cand[:, 0:3] = rng.uniform(-1, 1, (n, 3))
    cand[:, 3:7] = rng.uniform(-1, 1, (n, 4))
    cand[:, 7] = rng.uniform(0, 10, n)
    cand[:, 8] = rng.integers(-5, 1000, n).astype(np.int32).view(np.float32)
    cand[:, 9] = np.where(rng.uniform(0, 1, n) < 0.1, 0.0, rng.exponential(1.0, n))
    cand[:, 10] = rng.uniform(0.01, 2.0, n)
    other = np.zeros(1, ob.reservoir_dtype(rs, mis))
    s = other["s"][0]
    s["pos_lum"] = rng.uniform(-1, 1, (rs, 4))
    s["normal"] = rng.uniform(-1, 1, (rs, 4))
    s["light_index"] = rng.integers(0, 100, rs)
    s["p_hat"] = rng.uniform(0, 2, rs)
    s["sum_weights"] = rng.uniform(0, 5, rs)
    s["w"] = np.where(rng.uniform(0, 1, rs) < 0.3, 0.0, rng.uniform(0, 3, rs))
    if mis:
        s["sum_phat"] = rng.uniform(0, 4, rs)
    other["s"][0] = s
    other["m"] = rng.integers(0, 50)
    phat = np.where(rng.uniform(0, 1, rs) < 0.2, 0.0, rng.uniform(0, 3, rs)).astype(np.float32)
    return cand, other, phat


@pytest.mark.parametrize("rs,mis", VARIANTS)
def test_oracle_variant_matches_reference_reservoir_ops(rs, mis):
    ref = ob.ref_reservoir(rs, mis)
    if ref is None:
        pytest.skip("reference build (oracle/_ref) not present")
    o = ob.oracle_variant(rs, mis)
    m = C.c_int32()
    assert ref.ref_reservoir_size(C.byref(m)) == rs and m.value == mis
    rng = np.random.default_rng(rs * 10 + mis)
    for trial in range(300):
        cand, other, phat = _script_inputs(rng, rs, mis)
        use_other = trial % 4 != 0
        seed, seq = int(rng.integers(0, 2**40)), int(rng.integers(0, 2**40))
        got = np.zeros(1, ob.reservoir_dtype(rs, mis))
        o.or_reservoir_script(ob.P(cand), C.c_int32(len(cand)), ob.P(other) if use_other else None, ob.P(phat),
                              C.c_uint64(seed), C.c_uint64(seq), C.c_int32(0), ob.P(got))
        exp = np.zeros(16 * rs + 4, np.float32)
        of = ob.to_flat(other, rs)
        ref.ref_reservoir_script(ob.P(cand), C.c_int32(len(cand)), ob.P(of) if use_other else None, ob.P(phat),
                                 C.c_uint64(seed), C.c_uint64(seq), ob.P(exp))
        assert np.array_equal(ob.to_flat(got, rs)[0].view(np.uint32), exp.view(np.uint32)), trial


def test_mis_swap_fix_changes_the_merge():
    rs, mis = 1, 1
    o = ob.oracle_variant(rs, mis)
    rng = np.random.default_rng(9)
    differ = 0
    for trial in range(100):
        cand, other, phat = _script_inputs(rng, rs, mis)
        outs = []
        for fix in (0, 1):
            got = np.zeros(1, ob.reservoir_dtype(rs, mis))
            o.or_reservoir_script(ob.P(cand), C.c_int32(len(cand)), ob.P(other), ob.P(phat), C.c_uint64(1),
                                  C.c_uint64(trial), C.c_int32(fix), ob.P(got))
            outs.append(ob.to_flat(got, rs))
        differ += not np.array_equal(outs[0].view(np.uint32), outs[1].view(np.uint32))
    assert differ > 10


def test_default_build_is_the_single_sample_layout():
    o = ob.oracle_variant(1, 0)
    from restir_gb300 import _lib
    assert ob.reservoir_dtype(1, 0).itemsize == _lib.RESERVOIR_DTYPE.itemsize == 64
    assert ob.reservoir_dtype(2, 0).itemsize == 112 and ob.reservoir_dtype(1, 1).itemsize == 80
    assert ob.reservoir_dtype(2, 1).itemsize == 144
