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


def test_noalloc_chain_rejects_frames_above_its_limit(ctx, cuda, restir_lib, chain_inputs):
    from restir_gb300 import _lib
    s, g, ris = chain_inputs
    gs = g[0].struct()
    gs.width, gs.height = 1024, 1024
    u = s.uniforms(0)
    u.screen_size[0], u.screen_size[1] = 1024, 1024
    rc = restir_lib.rg_spatial_unbiased_chain_noalloc(ctx._h, C.byref(gs), _lib.ptr(ris[0]), _lib.ptr(ris[1]),
                                                      C.byref(u), 5, 2, None)
    assert rc == -1
    assert b"262144" in restir_lib.rg_last_error()
