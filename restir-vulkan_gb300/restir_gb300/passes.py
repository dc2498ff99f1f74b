"""Python mirror of the reference's pass interface over the C ABI.

A `Context` owns one rg_context (one GPU).  Its methods are the reference's
passes (RestirPass, SpatialReusePass, UnbiasedReusePass, LightingPass; see
src/passes/*.h) taking device buffers; `render_frame` is the reference's
per-frame command sequence (App::_recordMainCommandBuffers, src/app.h:212-262).
Device memory is held in torch tensors, used only as allocations; all compute
runs in librestir_gb300.so.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, lib

PLANES = {  # name: (dtype, channels)
    "albedo": (np.uint8, 4),
    "normal": (np.uint16, 4),
    "material": (np.uint16, 2),
    "world_pos": (np.float32, 4),
    "depth": (np.float32, 1),
}


def _torch():
    import torch
    return torch


def _stream_handle(stream) -> int | None:
    if stream is None:
        torch = _torch()
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class DeviceGBuffer:
    """G-buffer planes resident on the GPU (torch tensors)."""

    def __init__(self, width: int, height: int, device="cuda"):
        torch = _torch()
        tmap = {np.uint8: torch.uint8, np.uint16: torch.int16, np.float32: torch.float32}
        self.width, self.height = width, height
        self.planes = {}
        for name, (dt, ch) in PLANES.items():
            shape = (height, width, ch) if ch > 1 else (height, width)
            self.planes[name] = torch.zeros(shape, dtype=tmap[dt], device=device)

    @classmethod
    def from_host(cls, g: dict, device="cuda"):
        h, w = g["depth"].shape
        d = cls(w, h, device)
        d.upload(g)
        return d

    def upload(self, g: dict):
        torch = _torch()
        for name, t in self.planes.items():
            src = np.ascontiguousarray(g[name])
            if src.dtype == np.uint16:
                src = src.view(np.int16)
            t.copy_(torch.from_numpy(src))

    def to_host(self) -> dict:
        out = {}
        for name, t in self.planes.items():
            a = t.cpu().numpy()
            if a.dtype == np.int16:
                a = a.view(np.uint16)
            out[name] = a
        return out

    def struct(self) -> _lib.GBuffer:
        p = self.planes
        return _lib.GBuffer(self.width, self.height, p["albedo"].data_ptr(), p["normal"].data_ptr(),
                            p["material"].data_ptr(), p["world_pos"].data_ptr(), p["depth"].data_ptr())

    def out_struct(self) -> _lib.GBufferOut:
        p = self.planes
        return _lib.GBufferOut(self.width, self.height, p["albedo"].data_ptr(), p["normal"].data_ptr(),
                               p["material"].data_ptr(), p["world_pos"].data_ptr(), p["depth"].data_ptr())


def reservoirs(n: int, device="cuda", nbytes: int = 64):
    """Zero-filled device reservoir buffer (nbytes per pixel: 64 for the
    default format, Context.reservoir_bytes() for the others)."""
    return _torch().zeros((n, nbytes // 4), dtype=_torch().int32, device=device)


class _DeviceSpan:
    def __init__(self, ptr: int, nbytes: int):
        self.__cuda_array_interface__ = {"shape": (nbytes,), "typestr": "|u1", "data": (ptr, False), "version": 3}


def device_view(ptr: int, nbytes: int):
    """A torch uint8 tensor aliasing `nbytes` of device memory at `ptr`
    (for buffers the library owns, e.g. the frame driver's reservoirs)."""
    return _torch().as_tensor(_DeviceSpan(ptr, nbytes), device="cuda")


def reservoirs_to_numpy(t) -> np.ndarray:
    return t.cpu().numpy().view(_lib.RESERVOIR_DTYPE).reshape(-1)


def reservoirs_from_numpy(a: np.ndarray, device="cuda"):
    return _torch().from_numpy(np.ascontiguousarray(a).view(np.int32).reshape(-1, 16)).to(device)


class Context:
    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        check(lib().rg_create(device, C.byref(self._h)))
        self.device = device
        self.scene = None

    def close(self):
        if self._h:
            lib().rg_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload_scene(self, scene):
        self.scene = scene
        d = scene.desc()
        check(lib().rg_upload_scene(self._h, C.byref(d)))

    # ---- passes
    def initial_temporal(self, cur: DeviceGBuffer, prev: DeviceGBuffer | None, prev_res, out, uniforms, stream=None):
        cs = cur.struct()
        ps = prev.struct() if prev is not None else None
        check(lib().rg_initial_temporal(self._h, C.byref(cs), C.byref(ps) if ps is not None else None,
                                        _lib.ptr(prev_res), _lib.ptr(out), C.byref(uniforms), _stream_handle(stream)))

    def spatial_biased(self, g: DeviceGBuffer, res_in, res_out, uniforms, iteration: int, stream=None):
        gs = g.struct()
        check(lib().rg_spatial_biased(self._h, C.byref(gs), _lib.ptr(res_in), _lib.ptr(res_out), C.byref(uniforms),
                                      iteration, _stream_handle(stream)))

    def spatial_unbiased(self, g: DeviceGBuffer, res_in, res_out, uniforms, neighbors: int = 3, pass_index: int = 0,
                         stream=None):
        gs = g.struct()
        check(lib().rg_spatial_unbiased(self._h, C.byref(gs), _lib.ptr(res_in), _lib.ptr(res_out),
                                        C.byref(uniforms), neighbors, pass_index, _stream_handle(stream)))

    def shade(self, g: DeviceGBuffer, res, lighting_uniforms, out_rgba, stream=None):
        gs = g.struct()
        check(lib().rg_shade(self._h, C.byref(gs), _lib.ptr(res), C.byref(lighting_uniforms), _lib.ptr(out_rgba),
                             _stream_handle(stream)))

    def visibility_batch(self, p1, p2, out, stream=None):
        n = p1.shape[0]
        check(lib().rg_visibility_batch(self._h, _lib.ptr(p1), _lib.ptr(p2), _lib.ptr(out), n,
                                        _stream_handle(stream)))

    def trace_gbuffer(self, camera, out: DeviceGBuffer, stream=None):
        cam = camera.to_c()
        os_ = out.out_struct()
        check(lib().rg_trace_gbuffer(self._h, C.byref(cam), C.byref(os_), _stream_handle(stream)))

    def render_frame(self, cur: DeviceGBuffer, prev: DeviceGBuffer | None, slot: int, params, out_rgba=None,
                     stream=None):
        cs = cur.struct()
        ps = (prev if prev is not None else cur).struct()
        check(lib().rg_render_frame(self._h, C.byref(cs), C.byref(ps), slot, C.byref(params), _lib.ptr(out_rgba),
                                    _stream_handle(stream)))

    def frame_reservoirs_ptr(self, slot: int) -> int:
        p = C.c_void_p()
        check(lib().rg_frame_reservoirs(self._h, slot, C.byref(p)))
        return p.value

    def render_frame_host(self, g: dict, params, out_rgba: np.ndarray, stream=None):
        h, w = g["depth"].shape
        check(lib().rg_render_frame_host(self._h, w, h, _lib.ptr(g["albedo"]), _lib.ptr(g["normal"]),
                                         _lib.ptr(g["material"]), _lib.ptr(g["world_pos"]), _lib.ptr(g["depth"]),
                                         C.byref(params), _lib.ptr(out_rgba), _stream_handle(stream)))

    def set_reservoir_format(self, samples: int, unbiased_mis: int):
        check(lib().rg_set_reservoir_format(self._h, samples, unbiased_mis))

    TREE_LAYOUTS = {"binary": 0, "wide": 1, "quant": 2}

    def set_tree_layout(self, layout):
        """The shadow-ray tree from the next upload: "binary" (RG_TREE_BINARY),
        "wide" (RG_TREE_WIDE4) or "quant" (RG_TREE_QUANT4); True / False mean
        "wide" / "binary"."""
        if isinstance(layout, bool):
            layout = "wide" if layout else "binary"
        check(lib().rg_set_tree_layout(self._h, self.TREE_LAYOUTS[layout]))

    def set_visibility_cache(self, enable: bool):
        """rg_set_visibility_cache: reuse own-segment answers between ray passes."""
        check(lib().rg_set_visibility_cache(self._h, 1 if enable else 0))

    def reservoir_bytes(self) -> int:
        return check(lib().rg_reservoir_bytes(self._h))

    def stats(self, reset: bool = False) -> _lib.Stats:
        s = _lib.Stats()
        check(lib().rg_get_stats(self._h, C.byref(s), int(reset)))
        return s

    # ---- learned light-cluster proposal
    def create_proposal(self, cluster_of: np.ndarray, clusters: int, *, mix: float = 0.9,
                        learning_rate: float = 1e-3, batch: int = 65536, box_min=(0.0, 0.0, 0.0),
                        box_max=(1.0, 1.0, 1.0), seed: int = 1):
        pl = self.scene.point_lights
        cfg = _lib.ProposalConfig(clusters, mix, learning_rate, batch, (C.c_float * 3)(*box_min),
                                  (C.c_float * 3)(*box_max), seed)
        co = np.ascontiguousarray(cluster_of, np.int32)
        check(lib().rg_proposal_create(self._h, C.byref(cfg), _lib.ptr(pl), len(pl), _lib.ptr(co)))
        self.proposal_clusters = clusters

    def destroy_proposal(self):
        check(lib().rg_proposal_destroy(self._h))
        self.proposal_clusters = 0

    def proposal_params(self) -> np.ndarray:
        n = lib().rg_proposal_param_count(self.proposal_clusters)
        out = np.empty(n, np.float32)
        check(lib().rg_proposal_get_params(self._h, _lib.ptr(out), n))
        return out

    def set_proposal_params(self, params: np.ndarray):
        p = np.ascontiguousarray(params, np.float32)
        check(lib().rg_proposal_set_params(self._h, _lib.ptr(p), p.size))

    def proposal_infer(self, g: DeviceGBuffer, uniforms, stream=None):
        gs = g.struct()
        check(lib().rg_proposal_infer(self._h, C.byref(gs), C.byref(uniforms), _stream_handle(stream)))

    def proposal_buffers(self, n_pixels: int):
        """(candidates [n_pixels x 32] as CANDIDATE_DTYPE, row stats [n_pixels x 4] float32), copied to host."""
        torch = _torch()
        cp, sp = C.c_void_p(), C.c_void_p()
        check(lib().rg_proposal_buffers(self._h, C.byref(cp), C.byref(sp)))
        torch.cuda.synchronize()
        cand = torch.as_tensor(device_view(cp.value, n_pixels * 32 * 8), device="cuda").cpu().numpy()
        stat = torch.as_tensor(device_view(sp.value, n_pixels * 16), device="cuda").cpu().numpy()
        return cand.view(_lib.CANDIDATE_DTYPE).reshape(n_pixels, 32), stat.view(np.float32).reshape(n_pixels, 4)

    def proposal_gradients(self, g: DeviceGBuffer, camera_pos, rows, targets):
        """(gradient as a float32 device tensor, summed loss) for device int32 tensors rows, targets."""
        torch = _torch()
        n = lib().rg_proposal_param_count(self.proposal_clusters)
        grad = torch.zeros(n, dtype=torch.float32, device="cuda")
        cam = (C.c_float * 3)(*camera_pos)
        loss = C.c_double()
        gs = g.struct()
        check(lib().rg_proposal_gradients(self._h, C.byref(gs), cam, _lib.ptr(rows), _lib.ptr(targets),
                                          rows.shape[0], _lib.ptr(grad), C.byref(loss), None))
        return grad, loss.value

    def proposal_train(self, g: DeviceGBuffer, uniforms, final_res_ptr: int, stream=None):
        gs = g.struct()
        check(lib().rg_proposal_train(self._h, C.byref(gs), C.byref(uniforms), final_res_ptr,
                                      _stream_handle(stream)))

    def proposal_last_loss(self):
        loss, cnt = C.c_double(), C.c_int64()
        check(lib().rg_proposal_last_loss(self._h, C.byref(loss), C.byref(cnt)))
        return loss.value, cnt.value


class Batch:
    """Many views through the passes with one launch per pass (rg_batch_*).

    views: list of dicts with keys cur, prev (DeviceGBuffer), res0, res1, tmp
    (reservoir tensors), image (float4 tensor) and uniforms (RestirUniforms);
    params: FrameParams (unbiased, spatial_iterations, unbiased_neighbors, gamma)."""

    def __init__(self, ctx: "Context", views: list, params, tuning: _lib.BatchTuning | None = None):
        arr = (_lib.View * len(views))()
        self._keep = views
        for i, v in enumerate(views):
            arr[i].cur = v["cur"].struct()
            arr[i].prev = v["prev"].struct()
            arr[i].reservoirs[0] = _lib.ptr(v["res0"])
            arr[i].reservoirs[1] = _lib.ptr(v["res1"])
            arr[i].tmp = _lib.ptr(v["tmp"])
            arr[i].rgba_out = _lib.ptr(v["image"])
            arr[i].uniforms = v["uniforms"]
        self._h = C.c_void_p()
        check(lib().rg_batch_create(ctx._h, arr, len(views), C.byref(params),
                                    C.byref(tuning) if tuning is not None else None, C.byref(self._h)))

    def run(self, parity: int, stream=None):
        check(lib().rg_batch_run(self._h, parity, _stream_handle(stream)))

    def reset_frames(self, stream=None):
        check(lib().rg_batch_reset_frames(self._h, _stream_handle(stream)))

    def set_tuning(self, ris_pixels_per_thread: int, spatial_tile_width: int, ctas_per_sm: int = 0):
        t = _lib.BatchTuning(ris_pixels_per_thread, spatial_tile_width, ctas_per_sm)
        check(lib().rg_batch_set_tuning(self._h, C.byref(t)))

    def tuning(self) -> _lib.BatchTuning:
        t = _lib.BatchTuning()
        check(lib().rg_batch_get_tuning(self._h, C.byref(t)))
        return t

    def autotune(self, repeats: int = 3, stream=None):
        t = _lib.BatchTuning()
        ms = C.c_float()
        check(lib().rg_batch_autotune(self._h, repeats, C.byref(t), C.byref(ms), _stream_handle(stream)))
        return t, ms.value

    def autotune_candidates(self, counts=(8, 16, 32), repeats: int = 1, stream=None):
        """Chooses the views' RIS candidate count by Monte Carlo efficiency
        (rg_batch_autotune_candidates): (chosen count, ms per run, per-pixel
        variance of log(1 + luminance)) for every count tried."""
        n = len(counts)
        c_arr = (C.c_int32 * n)(*counts)
        ms = (C.c_float * n)()
        var = (C.c_double * n)()
        best = C.c_int32()
        check(lib().rg_batch_autotune_candidates(self._h, c_arr, n, repeats, C.byref(best), ms, var,
                                                 _stream_handle(stream)))
        for v in self._keep:
            v["uniforms"].initial_light_sample_count = best.value
        return best.value, list(ms), list(var)

    def close(self):
        if self._h:
            lib().rg_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cluster_lights(point_lights: np.ndarray, k: int, iterations: int = 10, seed: int = 1):
    """Seeded k-means of the point lights (host): (cluster_of int32 [n], centers float32 [k x 3])."""
    n = len(point_lights)
    cluster_of = np.empty(n, np.int32)
    centers = np.empty((k, 3), np.float32)
    pl = np.ascontiguousarray(point_lights)
    check(lib().rg_cluster_lights(_lib.ptr(pl), n, k, iterations, seed, _lib.ptr(cluster_of), _lib.ptr(centers)))
    return cluster_of, centers
