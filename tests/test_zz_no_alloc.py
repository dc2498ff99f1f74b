"""rg_spatial_unbiased_chain_noalloc: the chain of unbiased spatial passes
for callers that cannot allocate device memory mid-frame, checked through
the C ABI against the same chain built from rg_spatial_unbiased with a
caller-allocated temporary buffer.

The parity bar is the one every GPU test here uses: bit-exact reservoirs.
Two calls are made in a row with different inputs and pass counts, so a
second call that picked up anything the first left in the library's
built-in buffer would show.  This file is collected last on purpose.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import mismatch

pytestmark = pytest.mark.gpu

MAX_PIXELS = 512 * 512


@pytest.fixture(scope="module")
def chain_inputs(ctx, cuda):
    from restir_gb300 import scenes
    from restir_gb300.passes import DeviceGBuffer, reservoirs
    s = scenes.config2(width=320, height=180, frames=2)
    ctx.upload_scene(s)
    g = [DeviceGBuffer(s.width, s.height) for _ in range(2)]
    for f in range(2):
        ctx.trace_gbuffer(s.cameras[f], g[f])
    n = s.width * s.height
    ris = [reservoirs(n), reservoirs(n)]
    ctx.initial_temporal(g[0], None, None, ris[0], s.uniforms(0))
    ctx.initial_temporal(g[1], g[0], ris[0], ris[1], s.uniforms(1))
    cuda.cuda.synchronize()
    return s, g, ris


def _chain_with_temporary(ctx, g, res_in, u, neighbors, passes):
    from restir_gb300.passes import reservoirs
    n = g.width * g.height
    bufs = [reservoirs(n), reservoirs(n)]
    src = res_in
    for k in range(passes):
        dst = bufs[k % 2]
        ctx.spatial_unbiased(g, src, dst, u, neighbors, k)
        src = dst
    return src


def _chain_noalloc(restir_lib, ctx, g, res_in, out, u, neighbors, passes, cuda):
    from restir_gb300 import _lib
    gs = g.struct()
    stream = cuda.cuda.current_stream().cuda_stream
    return restir_lib.rg_spatial_unbiased_chain_noalloc(ctx._h, C.byref(gs), _lib.ptr(res_in), _lib.ptr(out),
                                                        C.byref(u), neighbors, passes, stream)


def test_noalloc_chain_equals_chained_passes_twice(ctx, cuda, restir_lib, chain_inputs):
    from restir_gb300.passes import reservoirs, reservoirs_to_numpy
    s, g, ris = chain_inputs
    n = s.width * s.height
    assert n <= MAX_PIXELS
    # call 1: frame 1, three passes; call 2: frame 0, two passes, other neighbour count
    for frame, passes, k in ((1, 3, 5), (0, 2, 3)):
        u = s.uniforms(frame)
        expected = reservoirs_to_numpy(_chain_with_temporary(ctx, g[frame], ris[frame], u, k, passes))
        out = reservoirs(n)
        rc = _chain_noalloc(restir_lib, ctx, g[frame], ris[frame], out, u, k, passes, cuda)
        assert rc == 0, restir_lib.rg_last_error()
        got = reservoirs_to_numpy(out)
        assert mismatch(got, expected) == 0, f"frame {frame}: {mismatch(got, expected)} reservoirs differ"
        assert np.count_nonzero(got["m"]) > 0


def test_noalloc_chain_at_its_exact_limit(ctx, cuda, restir_lib):
    """A 512 x 512 frame fills the built-in buffer exactly; two calls in a row
    (three passes, then two) against the chain with a temporary buffer."""
    from restir_gb300 import scenes
    from restir_gb300.passes import DeviceGBuffer, reservoirs, reservoirs_to_numpy
    s = scenes.config2(width=512, height=512, frames=1)
    ctx.upload_scene(s)
    g = DeviceGBuffer(s.width, s.height)
    ctx.trace_gbuffer(s.cameras[0], g)
    n = s.width * s.height
    assert n == MAX_PIXELS
    ris = reservoirs(n)
    u = s.uniforms(0)
    ctx.initial_temporal(g, None, None, ris, u)
    for passes, k in ((3, 5), (2, 4)):
        expected = reservoirs_to_numpy(_chain_with_temporary(ctx, g, ris, u, k, passes))
        out = reservoirs(n)
        rc = _chain_noalloc(restir_lib, ctx, g, ris, out, u, k, passes, cuda)
        assert rc == 0, restir_lib.rg_last_error()
        got = reservoirs_to_numpy(out)
        assert mismatch(got, expected) == 0, f"{passes} passes: {mismatch(got, expected)} reservoirs differ"
    # one row more than the buffer holds
    gs = g.struct()
    gs.height = 513
    u.screen_size[1] = 513
    rc = restir_lib.rg_spatial_unbiased_chain_noalloc(ctx._h, C.byref(gs), _lib_ptr(ris), _lib_ptr(out),
                                                      C.byref(u), 5, 2, None)
    assert rc == -1
    assert b"262144" in restir_lib.rg_last_error()


def _lib_ptr(t):
    from restir_gb300 import _lib
    return _lib.ptr(t)


def _call(restir_lib, ctx, gs, a, b, u, neighbors=5, passes=2):
    return restir_lib.rg_spatial_unbiased_chain_noalloc(ctx._h, C.byref(gs) if gs is not None else None, a, b,
                                                        C.byref(u), neighbors, passes, None)


def test_noalloc_chain_rejects_bad_arguments_before_any_launch(ctx, cuda, restir_lib, chain_inputs):
    """Every rejection returns its code on the host; nothing is launched
    (the reservoirs passed in stay as they were)."""
    s, g, ris = chain_inputs
    ctx.upload_scene(s)
    u = s.uniforms(0)
    before = ris[1].clone()
    a, b = _lib_ptr(ris[0]), _lib_ptr(ris[1])
    gs = g[0].struct()
    # frames above the limit
    big = g[0].struct()
    big.width, big.height = 1024, 1024
    ub = s.uniforms(0)
    ub.screen_size[0], ub.screen_size[1] = 1024, 1024
    assert _call(restir_lib, ctx, big, a, b, ub) == -1
    assert b"262144" in restir_lib.rg_last_error()
    # pass counts outside 1..64, neighbour counts outside 0..16
    for passes in (0, 65):
        assert _call(restir_lib, ctx, gs, a, b, u, passes=passes) == -1
        assert b"num_passes" in restir_lib.rg_last_error()
    assert _call(restir_lib, ctx, gs, a, b, u, neighbors=17) == -1
    # in == out
    assert _call(restir_lib, ctx, gs, a, a, u) == -1
    assert b"differ" in restir_lib.rg_last_error()
    # a misaligned albedo plane (the kernel reads it as 32-bit words)
    off = g[0].struct()
    off.albedo = g[0].planes["albedo"].data_ptr() + 1
    assert _call(restir_lib, ctx, off, a, b, u) == -1
    assert b"misaligned" in restir_lib.rg_last_error()
    # a G-buffer whose size differs from the uniforms
    small = g[0].struct()
    small.width = s.width - 1
    assert _call(restir_lib, ctx, small, a, b, u) == -1
    # misaligned reservoir buffers
    assert _call(restir_lib, ctx, gs, a + 4, b, u) == -1
    # a reservoir format other than the default (its scratch stride is 64 bytes)
    for samples, mis in ((2, 0), (1, 1)):
        ctx.set_reservoir_format(samples, mis)
        try:
            assert _call(restir_lib, ctx, gs, a, b, u) == -6  # RG_ERR_UNSUPPORTED
            assert b"default reservoir format" in restir_lib.rg_last_error()
        finally:
            ctx.set_reservoir_format(1, 0)
    cuda.cuda.synchronize()
    assert cuda.equal(ris[1], before)
