"""The reservoir formats RESERVOIR_SIZE = 2 and UNBIASED_MIS
(rg_set_reservoir_format) on the GPU against the oracle built for the same
variant (whose reservoir operations are pinned to the reference's own
reservoir.glsl in tests/test_reservoir_variants.py).

Bar: bit-exact reservoirs and images through RIS + visibility reuse +
temporal reuse, the biased spatial pass, the unbiased spatial pass chain and
shading, with the reference's swapped combineReservoirs arguments and with
RG_FLAG_MIS_SWAP_FIX."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle_binding as ob

pytestmark = pytest.mark.gpu

FORMATS = [(2, 0), (1, 1), (2, 1)]


@pytest.fixture(scope="module")
def cfg1(restir_lib):
    from restir_gb300 import scenes
    s = scenes.config1(width=96, height=64)
    return s, scenes.trace_gbuffer_host(s, 0)


@pytest.fixture(scope="module")
def cfg2(restir_lib):
    from restir_gb300 import scenes
    s = scenes.config2(width=128, height=72, n_tris=20_000, n_lights=4096, frames=2)
    return s, [scenes.trace_gbuffer_host(s, f) for f in range(2)]


def _bytes(t):
    return t.cpu().numpy().view(np.uint8).reshape(-1)


def _orc(lib, name, scene, *args):
    s, keep = ob.scene_struct(scene)
    rc = getattr(lib, name)(C.byref(s), *args)
    assert rc == 0, (name, rc)


def _set(ctx, rs, mis):
    ctx.set_reservoir_format(rs, mis)
    nb = ctx.reservoir_bytes()
    assert nb == ob.reservoir_dtype(rs, mis).itemsize
    return nb


@pytest.mark.parametrize("rs,mis", FORMATS)
def test_biased_frame_variant_bit_exact(ctx, cuda, cfg1, rs, mis):
    from restir_gb300.passes import DeviceGBuffer, reservoirs
    s, g = cfg1
    ctx.upload_scene(s)
    try:
        nb = _set(ctx, rs, mis)
        lib = ob.oracle_variant(rs, mis)
        dg = DeviceGBuffer.from_host(g)
        n = s.width * s.height
        dt = ob.reservoir_dtype(rs, mis)
        u = s.uniforms(0)
        gg = ob.gbuffer_struct(g)
        exp0 = np.zeros(n, dt)
        _orc(lib, "or_initial_temporal", s, C.byref(gg), None, None, ob.P(exp0), C.byref(u), None, None)
        r0 = reservoirs(n, nbytes=nb)
        ctx.initial_temporal(dg, None, None, r0, u)
        assert np.array_equal(_bytes(r0), exp0.view(np.uint8))
        exp1, exp2 = np.zeros(n, dt), np.zeros(n, dt)
        _orc(lib, "or_spatial_biased", s, C.byref(gg), ob.P(exp0), ob.P(exp1), C.byref(u), C.c_int32(0), None)
        _orc(lib, "or_spatial_biased", s, C.byref(gg), ob.P(exp1), ob.P(exp2), C.byref(u), C.c_int32(1), None)
        r1, r2 = reservoirs(n, nbytes=nb), reservoirs(n, nbytes=nb)
        ctx.spatial_biased(dg, r0, r1, u, 0)
        ctx.spatial_biased(dg, r1, r2, u, 1)
        assert np.array_equal(_bytes(r2), exp2.view(np.uint8))
        img = np.zeros((s.height, s.width, 4), np.float32)
        lu = s.lighting_uniforms(0)
        _orc(lib, "or_shade", s, C.byref(gg), ob.P(exp2), C.byref(lu), ob.P(img), None)
        out = cuda.zeros((s.height, s.width, 4), dtype=cuda.float32, device="cuda")
        ctx.shade(dg, r2, lu, out)
        assert np.array_equal(out.cpu().numpy().view(np.uint32), img.view(np.uint32))
        assert np.mean(exp2["s"]["w"] > 0) > 0.2
    finally:
        ctx.set_reservoir_format(1, 0)


@pytest.mark.parametrize("rs,mis,fix", [(2, 0, 0), (1, 1, 0), (2, 1, 0), (2, 1, 1)])
def test_unbiased_temporal_sequence_variant_bit_exact(ctx, cuda, cfg2, rs, mis, fix):
    """Two frames: RIS + visibility (+ temporal on frame 2) and two chained
    unbiased passes (k = 5), then shading, on the variant's layout."""
    from restir_gb300 import _lib
    from restir_gb300.passes import DeviceGBuffer, reservoirs
    s, gs = cfg2
    ctx.upload_scene(s)
    try:
        nb = _set(ctx, rs, mis)
        lib = ob.oracle_variant(rs, mis)
        n = s.width * s.height
        dt = ob.reservoir_dtype(rs, mis)
        dgs = [DeviceGBuffer.from_host(g) for g in gs]
        prev_exp, prev_got = None, None
        for f in range(2):
            u = s.uniforms(f)
            if fix:
                u.flags |= _lib.RG_FLAG_MIS_SWAP_FIX
            gg = ob.gbuffer_struct(gs[f])
            gp = ob.gbuffer_struct(gs[f - 1]) if f else None
            exp = np.zeros(n, dt)
            _orc(lib, "or_initial_temporal", s, C.byref(gg), C.byref(gp) if gp else None,
                 ob.P(prev_exp) if f else None, ob.P(exp), C.byref(u), None, None)
            got = reservoirs(n, nbytes=nb)
            ctx.initial_temporal(dgs[f], dgs[f - 1] if f else None, prev_got if f else None, got, u)
            assert np.array_equal(_bytes(got), exp.view(np.uint8)), f
            for p in range(2):
                e2 = np.zeros(n, dt)
                _orc(lib, "or_spatial_unbiased", s, C.byref(gg), ob.P(exp), ob.P(e2), C.byref(u), C.c_int32(5),
                     C.c_int32(p), None, None)
                g2 = reservoirs(n, nbytes=nb)
                ctx.spatial_unbiased(dgs[f], got, g2, u, 5, p)
                assert np.array_equal(_bytes(g2), e2.view(np.uint8)), (f, p)
                exp, got = e2, g2
            img = np.zeros((s.height, s.width, 4), np.float32)
            lu = s.lighting_uniforms(f)
            _orc(lib, "or_shade", s, C.byref(gg), ob.P(exp), C.byref(lu), ob.P(img), None)
            out = cuda.zeros((s.height, s.width, 4), dtype=cuda.float32, device="cuda")
            ctx.shade(dgs[f], got, lu, out)
            assert np.array_equal(out.cpu().numpy().view(np.uint32), img.view(np.uint32))
            prev_exp, prev_got = exp, got
        assert ctx.stats().traversal_errors == 0
    finally:
        ctx.set_reservoir_format(1, 0)


def test_frame_driver_and_guards_with_a_variant(ctx, cuda, cfg2):
    from restir_gb300.passes import Batch, DeviceGBuffer
    from restir_gb300._lib import RestirError
    s, gs = cfg2
    ctx.upload_scene(s)
    try:
        ctx.set_reservoir_format(2, 1)
        dg = DeviceGBuffer.from_host(gs[0])
        out = cuda.zeros((s.height, s.width, 4), dtype=cuda.float32, device="cuda")
        ctx.render_frame(dg, dg, 0, s.frame_params(0), out)
        assert np.isfinite(out.cpu().numpy()).all()
        n = s.width * s.height
        nb = ctx.reservoir_bytes()
        from restir_gb300.passes import reservoirs
        view = {"cur": dg, "prev": dg, "res0": reservoirs(n, nbytes=nb), "res1": reservoirs(n, nbytes=nb),
                "tmp": reservoirs(n, nbytes=nb), "image": out, "uniforms": s.uniforms(0)}
        with pytest.raises(RestirError, match="default reservoir format"):
            Batch(ctx, [view], s.frame_params(0))
    finally:
        ctx.set_reservoir_format(1, 0)
