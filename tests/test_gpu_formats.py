"""The reference's G-buffer attachment formats at the boundary.

The reference picks, per attachment, the first format its device supports
(GBuffer::Formats::initialize, src/passes/gBufferPass.cpp:75-101):
  normal          R16G16B16_SNORM, R16G16B16_SFLOAT, R16G16B16A16_SNORM,
                  R16G16B16A16_SFLOAT, R32G32B32_SFLOAT
  world position  R32G32B32_SFLOAT, R32G32B32A32_SFLOAT
  depth           D32_SFLOAT, D32_SFLOAT_S8_UINT, D24_UNORM_S8_UINT
Each is accepted through rg_gbuffer's format fields.  The planes here are the
traced G-buffer re-encoded into each format (so the decoded values differ
from the default planes'), and every pass that reads them -- RIS with
visibility and temporal reuse, the unbiased and the biased spatial passes
(the latter reads depth), shading -- must equal the oracle fed the same planes
bit for bit.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle_binding as ob
from helpers import image_bits, mismatch, new_res

pytestmark = pytest.mark.gpu

F = {"RGB16_SNORM": 85, "RGB16F": 90, "RGBA16_SNORM": 92, "RGBA16F": 97, "RGB32F": 106, "RGBA32F": 109,
     "D32F": 126, "D24S8": 129, "D32FS8": 130}


def encode(g: dict, nf: int, pf: int, df: int, seed: int = 0) -> dict:
    """The default planes of g re-encoded into the given formats (host)."""
    rng = np.random.default_rng(seed)
    n = g["normal"][..., :3].view(np.float16).astype(np.float32)
    out = {"albedo": g["albedo"], "material": g["material"], "formats": (nf, pf, df)}
    snorm = np.round(np.clip(n, -1.0, 1.0) * 32767.0).astype(np.int16).view(np.uint16)
    if nf in (0, F["RGBA16F"]):
        out["normal"] = g["normal"]
    elif nf == F["RGB16_SNORM"]:
        out["normal"] = np.ascontiguousarray(snorm)
    elif nf == F["RGBA16_SNORM"]:
        out["normal"] = np.ascontiguousarray(np.concatenate([snorm, np.zeros_like(snorm[..., :1])], -1))
    elif nf == F["RGB16F"]:
        out["normal"] = np.ascontiguousarray(g["normal"][..., :3])
    elif nf == F["RGB32F"]:
        out["normal"] = np.ascontiguousarray(n)
    out["world_pos"] = g["world_pos"] if pf in (0, F["RGBA32F"]) else np.ascontiguousarray(g["world_pos"][..., :3])
    if df == F["D24S8"]:
        d24 = np.round(np.clip(g["depth"], 0.0, 1.0).astype(np.float64) * 16777215.0).astype(np.uint32)
        out["depth"] = d24 | (rng.integers(0, 256, d24.shape, dtype=np.uint32) << 24)  # stencil bits: ignored
    else:
        out["depth"] = g["depth"]
    return out


class FormattedGBuffer:
    """Device planes of an encoded G-buffer with its rg_gbuffer record."""

    def __init__(self, e: dict, torch):
        self.height, self.width = e["depth"].shape[:2]
        conv = {np.uint8: np.uint8, np.uint16: np.int16, np.uint32: np.int32, np.float32: np.float32}
        self.planes = {k: torch.from_numpy(np.ascontiguousarray(e[k]).view(conv[e[k].dtype.type])).cuda()
                       for k in ("albedo", "normal", "material", "world_pos", "depth")}
        self.formats = e["formats"]

    def struct(self):
        from restir_gb300 import _lib
        p = self.planes
        return _lib.GBuffer(self.width, self.height, p["albedo"].data_ptr(), p["normal"].data_ptr(),
                            p["material"].data_ptr(), p["world_pos"].data_ptr(), p["depth"].data_ptr(),
                            *self.formats, 0)


COMBOS = [("RGB16_SNORM", 0, 0), ("RGB16F", 0, 0), ("RGBA16_SNORM", 0, 0), ("RGBA16F", "RGBA32F", "D32F"),
          ("RGB32F", 0, 0), (0, "RGB32F", 0), (0, 0, "D32FS8"), (0, 0, "D24S8"), ("RGB16_SNORM", "RGB32F", "D24S8")]


def _fmt(x):
    return F[x] if isinstance(x, str) else x


@pytest.fixture(scope="module")
def scenes_fmt(restir_lib, cuda, ctx):
    from restir_gb300 import scenes
    from restir_gb300.passes import DeviceGBuffer
    out = {}
    for name, s in (("unbiased", scenes.config2(width=160, height=96, frames=2)),
                    ("biased", scenes.config2(width=128, height=96, frames=1))):
        ctx.upload_scene(s)
        gs = []
        for f in range(s.frames):
            d = DeviceGBuffer(s.width, s.height)
            ctx.trace_gbuffer(s.cameras[f], d)
            gs.append(d.to_host())
        out[name] = (s, gs)
    return out


@pytest.mark.parametrize("combo", COMBOS, ids=lambda c: "-".join(str(x) for x in c))
def test_passes_read_every_reference_format(ctx, cuda, scenes_fmt, combo):
    from restir_gb300.passes import reservoirs, reservoirs_to_numpy
    nf, pf, df = (_fmt(x) for x in combo)
    # unbiased sequence: two frames, temporal reuse from the second on
    s, gs = scenes_fmt["unbiased"]
    ctx.upload_scene(s)
    n = s.width * s.height
    enc = [encode(g, nf, pf, df, seed=f) for f, g in enumerate(gs)]
    dev = [FormattedGBuffer(e, cuda) for e in enc]
    prev_gpu = prev_orc = None
    for f in range(s.frames):
        u = s.uniforms(f)
        r = reservoirs(n)
        ctx.initial_temporal(dev[f], dev[f - 1] if f else None, prev_gpu, r, u)
        exp = new_res(n)
        ob.initial_temporal(s, enc[f], enc[f - 1] if f else None, prev_orc, exp, u)
        assert mismatch(reservoirs_to_numpy(r), exp) == 0, f"RIS/temporal frame {f}"
        o = reservoirs(n)
        ctx.spatial_unbiased(dev[f], r, o, u, s.neighbors, 0)
        exp2 = new_res(n)
        ob.spatial_unbiased(s, enc[f], exp, exp2, u, s.neighbors, 0)
        assert mismatch(reservoirs_to_numpy(o), exp2) == 0, f"unbiased pass frame {f}"
        img = cuda.zeros((s.height, s.width, 4), dtype=cuda.float32, device="cuda")
        ctx.shade(dev[f], o, s.lighting_uniforms(f), img)
        ei = np.zeros((s.height, s.width, 4), np.float32)
        ob.shade(s, enc[f], exp2, s.lighting_uniforms(f), ei)
        assert np.array_equal(image_bits(img.cpu().numpy()), image_bits(ei)), f"shading frame {f}"
        prev_gpu, prev_orc = o, exp2
    # biased spatial reuse (reads depth and the neighbours' normals)
    s, gs = scenes_fmt["biased"]
    ctx.upload_scene(s)
    n = s.width * s.height
    e = encode(gs[0], nf, pf, df)
    d = FormattedGBuffer(e, cuda)
    u = s.uniforms(0)
    r0, r1, r2 = reservoirs(n), reservoirs(n), reservoirs(n)
    ctx.initial_temporal(d, None, None, r0, u)
    ctx.spatial_biased(d, r0, r1, u, 0)
    ctx.spatial_biased(d, r1, r2, u, 1)
    e0, e1, e2 = new_res(n), new_res(n), new_res(n)
    ob.initial_temporal(s, e, None, None, e0, u)
    ob.spatial_biased(s, e, e0, e1, u, 0)
    ob.spatial_biased(s, e, e1, e2, u, 1)
    got = reservoirs_to_numpy(r2)
    assert mismatch(got, e2) == 0, "biased passes"
    assert np.mean(got["w"] > 0) > 0.2


def test_formats_change_the_decoded_values(scenes_fmt):
    """The re-encoded planes are not the default ones in disguise: the SNORM
    normals decode to other floats than the default planes for most pixels,
    the D24 depth for some (so the bit-exact runs above exercise each
    decoder)."""
    s, gs = scenes_fmt["biased"]
    g = gs[0]
    e = encode(g, F["RGB16_SNORM"], 0, F["D24S8"])
    n_half = g["normal"][..., :3].view(np.float16).astype(np.float32)
    n_snorm = np.maximum(e["normal"].view(np.int16).astype(np.float32) / np.float32(32767.0), -1.0)
    assert np.mean(np.any(n_half != n_snorm, -1)) > 0.5
    d24 = (e["depth"] & 0xFFFFFF).astype(np.float32) / np.float32(16777215.0)
    assert np.mean(d24 != g["depth"]) > 0.01  # z/w near 1 is mostly on the 24-bit grid already


def test_unknown_or_misaligned_formats_are_rejected(ctx, cuda, scenes_fmt, restir_lib):
    from restir_gb300.passes import reservoirs
    s, gs = scenes_fmt["biased"]
    ctx.upload_scene(s)
    n = s.width * s.height
    u = s.uniforms(0)
    e = encode(gs[0], F["RGB32F"], 0, 0)
    d = FormattedGBuffer(e, cuda)
    r0, r1 = reservoirs(n), reservoirs(n)
    L = restir_lib
    for bad in ((97 + 1, 0, 0), (0, 107, 0), (0, 0, 125)):
        st = d.struct()
        st.normal_format, st.world_pos_format, st.depth_format = bad
        rc = L.rg_spatial_biased(ctx._h, C.byref(st), r0.data_ptr(), r1.data_ptr(), C.byref(u), 0, None)
        assert rc == -6 and b"not one of the reference's" in L.rg_last_error()
    st = d.struct()
    st.normal = st.normal + 2  # R32G32B32_SFLOAT needs 4-byte alignment
    rc = L.rg_spatial_biased(ctx._h, C.byref(st), r0.data_ptr(), r1.data_ptr(), C.byref(u), 0, None)
    assert rc == -1 and b"misaligned" in L.rg_last_error()
