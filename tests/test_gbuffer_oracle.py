"""The primary-ray G-buffer against the oracle's independent statement of it.

The oracle (or_trace_gbuffer) restates the planes the reference's raster
G-buffer pass writes (src/shaders/gBuffer.frag:27-79, camera of
src/camera.h:25-50) for one closest-hit ray per pixel centre, with its own
conservative double-precision walk of the tree.  The library's CPU tracer
(rg_trace_gbuffer_host) must produce the same bytes in every plane here; the
GPU tracer (k_trace_gbuffer) is checked against the oracle in
tests/test_gpu_parity.py.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_binding as ob


def _differing_pixels(a: dict, b: dict) -> dict:
    out = {}
    for k in a:
        x, y = a[k], b[k]
        d = (x.view(np.uint8) != y.view(np.uint8)).reshape(x.shape[0], x.shape[1], -1).any(-1)
        out[k] = int(np.count_nonzero(d))
    return out


@pytest.mark.parametrize("name,frames", [("config1", [0]), ("config2", [0, 7]), ("config3", [0, 15])])
def test_library_tracer_equals_oracle(restir_lib, oracle_lib, name, frames):
    from restir_gb300 import scenes
    s = scenes.CONFIGS[name]()
    for f in frames:
        a = scenes.trace_gbuffer_host(s, f)
        b = ob.trace_gbuffer(s, f)
        bad = _differing_pixels(a, b)
        assert all(v == 0 for v in bad.values()), (name, f, bad)
        assert (b["depth"] < 1.0).mean() > 0.99  # the closed room: every ray hits


def test_oracle_tracer_crop_and_half_rounding(oracle_lib):
    from restir_gb300 import scenes
    s = scenes.config1(width=64, height=48)
    full = ob.trace_gbuffer(s, 0)
    crop = ob.trace_gbuffer(s, 0, crop=(10, 7, 20, 13))
    for k in full:
        assert np.array_equal(full[k][7:20, 10:30], crop[k][7:20, 10:30])
        outside = crop[k].copy()
        outside[7:20, 10:30] = 0
        assert not outside.any()
    # binary16 conversion, round to nearest even, against numpy's
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-1, 1, 20000), rng.uniform(-1e-4, 1e-4, 5000),
                        np.array([0.0, -0.0, 6.1035e-05, 5.9604645e-08, 2.98e-08, 65504.0, 65519.0, 65520.0])])
    x = x.astype(np.float32)
    got = np.array([oracle_lib.oracle().or_float_to_half(float(v)) for v in x], np.uint16)
    assert np.array_equal(got, x.astype(np.float16).view(np.uint16))
