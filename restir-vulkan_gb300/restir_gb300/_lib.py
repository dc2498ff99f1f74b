"""ctypes binding of include/restir_gb300.h (librestir_gb300.so).

The structures below mirror the C ABI byte for byte; the reservoir, node,
triangle, light and alias-column layouts are the reference's std430 layouts.
Loading fails loudly if the shared library has not been built: there is no
fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG_ROOT = Path(__file__).resolve().parent.parent
# RESTIR_GB300_LIB selects another build of the library (e.g. one compiled
# with different tuning constants); the default is the in-tree build.
LIB_PATH = Path(os.environ.get("RESTIR_GB300_LIB", str(PKG_ROOT / "librestir_gb300.so")))

RG_OK = 0
RG_FLAG_VISIBILITY_REUSE = 1
RG_FLAG_TEMPORAL_REUSE = 2
RG_FLAG_FINAL_RIS_WEIGHT = 256
RG_FLAG_LEARNED_PROPOSAL = 512
RG_FLAG_LEARNED_TRAIN = 1024
RG_FLAG_MIS_SWAP_FIX = 2048
RG_MAX_TREE_DEPTH = 63

F4 = C.c_float * 4


class Reservoir(C.Structure):
    _fields_ = [("position_emission_lum", F4), ("normal", F4), ("light_index", C.c_int32), ("p_hat", C.c_float),
                ("sum_weights", C.c_float), ("w", C.c_float), ("num_stream_samples", C.c_uint32),
                ("_pad", C.c_uint32 * 3)]


class AabbTreeNode(C.Structure):
    _fields_ = [("left_aabb_min", F4), ("left_aabb_max", F4), ("right_aabb_min", F4), ("right_aabb_max", F4),
                ("left_child", C.c_int32), ("right_child", C.c_int32), ("_pad", C.c_int32 * 2)]


class RestirUniforms(C.Structure):
    _fields_ = [("prev_frame_projection_view", C.c_float * 16), ("camera_pos", F4), ("screen_size", C.c_uint32 * 2),
                ("frame", C.c_uint32), ("initial_light_sample_count", C.c_uint32),
                ("temporal_sample_count_multiplier", C.c_uint32), ("spatial_pos_threshold", C.c_float),
                ("spatial_normal_threshold", C.c_float), ("spatial_neighbors", C.c_uint32),
                ("spatial_radius", C.c_float), ("flags", C.c_int32), ("_pad", C.c_uint32 * 2)]


class LightingUniforms(C.Structure):
    _fields_ = [("prev_frame_projection_view", C.c_float * 16), ("camera_pos", F4), ("buffer_size", C.c_uint32 * 2),
                ("debug_mode", C.c_int32), ("gamma", C.c_float)]


# G-buffer formats (VkFormat numbers of the reference's candidates; 0 = default)
FORMAT_DEFAULT = 0
FORMAT_R16G16B16_SNORM = 85
FORMAT_R16G16B16_SFLOAT = 90
FORMAT_R16G16B16A16_SNORM = 92
FORMAT_R16G16B16A16_SFLOAT = 97
FORMAT_R32G32B32_SFLOAT = 106
FORMAT_R32G32B32A32_SFLOAT = 109
FORMAT_D32_SFLOAT = 126
FORMAT_D24_UNORM_S8_UINT = 129
FORMAT_D32_SFLOAT_S8_UINT = 130


class GBuffer(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("albedo", C.c_void_p), ("normal", C.c_void_p),
                ("material", C.c_void_p), ("world_pos", C.c_void_p), ("depth", C.c_void_p),
                ("normal_format", C.c_int32), ("world_pos_format", C.c_int32), ("depth_format", C.c_int32),
                ("_reserved", C.c_int32)]


class GBufferOut(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("albedo", C.c_void_p), ("normal", C.c_void_p),
                ("material", C.c_void_p), ("world_pos", C.c_void_p), ("depth", C.c_void_p)]


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("right", C.c_float * 3), ("up", C.c_float * 3),
                ("forward", C.c_float * 3), ("tan_half_fov_y", C.c_float), ("aspect", C.c_float),
                ("projection_view", C.c_float * 16)]


class SceneDesc(C.Structure):
    _fields_ = [("nodes", C.c_void_p), ("n_nodes", C.c_int32), ("triangles", C.c_void_p), ("n_triangles", C.c_int32),
                ("point_lights", C.c_void_p), ("n_point_lights", C.c_int32), ("tri_lights", C.c_void_p),
                ("n_tri_lights", C.c_int32), ("alias_table", C.c_void_p), ("n_alias", C.c_int32),
                ("materials", C.c_void_p), ("n_materials", C.c_int32)]


class FrameParams(C.Structure):
    _fields_ = [("uniforms", RestirUniforms), ("unbiased", C.c_int32), ("spatial_iterations", C.c_int32),
                ("unbiased_neighbors", C.c_int32), ("gamma", C.c_float)]


class Stats(C.Structure):
    _fields_ = [("rays_traced", C.c_uint64), ("traversal_errors", C.c_uint64), ("node_visits", C.c_uint64),
                ("triangle_tests", C.c_uint64), ("mma_timeouts", C.c_uint64), ("wide_nodes", C.c_uint64),
                ("tree_layout", C.c_uint64)]


class View(C.Structure):
    _fields_ = [("cur", GBuffer), ("prev", GBuffer), ("reservoirs", C.c_void_p * 2), ("tmp", C.c_void_p),
                ("rgba_out", C.c_void_p), ("uniforms", RestirUniforms)]


class MeshInstance(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("indices", C.c_void_p), ("index_count", C.c_uint32),
                ("world_matrix", C.c_float * 16), ("emissive_factor", C.c_float * 3)]


class BatchTuning(C.Structure):
    _fields_ = [("ris_pixels_per_thread", C.c_int32), ("spatial_tile_width", C.c_int32), ("ctas_per_sm", C.c_int32)]


class ProposalConfig(C.Structure):
    _fields_ = [("clusters", C.c_int32), ("mix", C.c_float), ("learning_rate", C.c_float), ("batch", C.c_int32),
                ("box_min", C.c_float * 3), ("box_max", C.c_float * 3), ("seed", C.c_uint64)]


assert C.sizeof(ProposalConfig) == 48
assert C.sizeof(Reservoir) == 64 and C.sizeof(AabbTreeNode) == 80
assert C.sizeof(RestirUniforms) == 128 and C.sizeof(LightingUniforms) == 96

# numpy views of the same layouts
RESERVOIR_DTYPE = np.dtype([("pos_lum", "<f4", 4), ("normal", "<f4", 4), ("light_index", "<i4"), ("p_hat", "<f4"),
                            ("sum_weights", "<f4"), ("w", "<f4"), ("m", "<u4"), ("pad", "<u4", 3)])
NODE_DTYPE = np.dtype([("lmin", "<f4", 4), ("lmax", "<f4", 4), ("rmin", "<f4", 4), ("rmax", "<f4", 4),
                       ("left", "<i4"), ("right", "<i4"), ("pad", "<i4", 2)])
TRI_DTYPE = np.dtype([("p1", "<f4", 4), ("p2", "<f4", 4), ("p3", "<f4", 4)])
POINT_LIGHT_DTYPE = np.dtype([("pos", "<f4", 4), ("color_lum", "<f4", 4)])
TRI_LIGHT_DTYPE = np.dtype([("p1", "<f4", 4), ("p2", "<f4", 4), ("p3", "<f4", 4), ("emission_lum", "<f4", 4),
                            ("normal_area", "<f4", 4)])
ALIAS_DTYPE = np.dtype([("prob", "<f4"), ("alias", "<i4"), ("ori_prob", "<f4"), ("alias_ori_prob", "<f4")])
CANDIDATE_DTYPE = np.dtype([("key", "<i4"), ("q", "<f4")])
MATERIAL_DTYPE = np.dtype([("albedo", "u1", 4), ("roughness", "<u2"), ("metallic", "<u2")])
assert RESERVOIR_DTYPE.itemsize == 64 and NODE_DTYPE.itemsize == 80 and TRI_DTYPE.itemsize == 48
assert POINT_LIGHT_DTYPE.itemsize == 32 and TRI_LIGHT_DTYPE.itemsize == 80 and ALIAS_DTYPE.itemsize == 16


class RestirError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"restir_gb300 error {code}: {msg}")
        self.code = code


_lib = None

_SIGNATURES = {
    "rg_create": (C.c_int, [C.c_int32, C.POINTER(C.c_void_p)]),
    "rg_destroy": (C.c_int, [C.c_void_p]),
    "rg_last_error": (C.c_char_p, []),
    "rg_get_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats), C.c_int32]),
    "rg_build_bvh": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "rg_tree_depth": (C.c_int, [C.c_void_p, C.c_int32]),
    "rg_tree_preorder": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "rg_build_alias_table": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]),
    "rg_trace_gbuffer_host": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(Camera), C.c_int32, C.c_int32, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rg_upload_scene": (C.c_int, [C.c_void_p, C.POINTER(SceneDesc)]),
    "rg_initial_temporal": (C.c_int, [C.c_void_p, C.POINTER(GBuffer), C.POINTER(GBuffer), C.c_void_p, C.c_void_p,
                                      C.POINTER(RestirUniforms), C.c_void_p]),
    "rg_spatial_biased": (C.c_int, [C.c_void_p, C.POINTER(GBuffer), C.c_void_p, C.c_void_p, C.POINTER(RestirUniforms),
                                    C.c_int32, C.c_void_p]),
    "rg_spatial_unbiased": (C.c_int, [C.c_void_p, C.POINTER(GBuffer), C.c_void_p, C.c_void_p,
                                      C.POINTER(RestirUniforms), C.c_int32, C.c_int32, C.c_void_p]),
    "rg_shade": (C.c_int, [C.c_void_p, C.POINTER(GBuffer), C.c_void_p, C.POINTER(LightingUniforms), C.c_void_p,
                           C.c_void_p]),
    "rg_visibility_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "rg_trace_gbuffer": (C.c_int, [C.c_void_p, C.POINTER(Camera), C.POINTER(GBufferOut), C.c_void_p]),
    "rg_render_frame": (C.c_int, [C.c_void_p, C.POINTER(GBuffer), C.POINTER(GBuffer), C.c_int32,
                                  C.POINTER(FrameParams), C.c_void_p, C.c_void_p]),
    "rg_frame_reservoirs": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "rg_render_frame_host": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.POINTER(FrameParams), C.c_void_p, C.c_void_p]),
    "rg_gemm_bf16": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_int32, C.c_void_p,
                               C.c_int32, C.c_int64, C.c_int64, C.c_int32, C.c_int32, C.c_void_p, C.c_int64,
                               C.c_int32, C.c_float, C.c_int32, C.c_void_p]),
    "rg_spatial_unbiased_chain_noalloc": (C.c_int, [C.c_void_p, C.POINTER(GBuffer), C.c_void_p, C.c_void_p,
                                                    C.POINTER(RestirUniforms), C.c_int32, C.c_int32, C.c_void_p]),
    "rg_set_reservoir_format": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "rg_set_tree_layout": (C.c_int, [C.c_void_p, C.c_int32]),
    "rg_set_visibility_cache": (C.c_int, [C.c_void_p, C.c_int32]),
    "rg_reservoir_bytes": (C.c_int, [C.c_void_p]),
    "rg_build_bvh_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                      C.POINTER(C.c_int32), C.c_void_p]),
    "rg_batch_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(FrameParams),
                                  C.POINTER(BatchTuning), C.POINTER(C.c_void_p)]),
    "rg_batch_run": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "rg_batch_reset_frames": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rg_batch_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(BatchTuning)]),
    "rg_batch_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(BatchTuning)]),
    "rg_batch_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(BatchTuning), C.POINTER(C.c_float),
                                    C.c_void_p]),
    "rg_batch_autotune_candidates": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.c_int32, C.c_int32,
                                               C.POINTER(C.c_int32), C.POINTER(C.c_float), C.POINTER(C.c_double),
                                               C.c_void_p]),
    "rg_batch_destroy": (C.c_int, [C.c_void_p]),
    "rg_collect_triangle_lights": (C.c_int64, [C.POINTER(MeshInstance), C.c_int32, C.c_void_p, C.c_int64]),
    "rg_cluster_lights": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.c_void_p,
                                    C.c_void_p]),
    "rg_proposal_param_count": (C.c_int64, [C.c_int32]),
    "rg_proposal_create": (C.c_int, [C.c_void_p, C.POINTER(ProposalConfig), C.c_void_p, C.c_int32, C.c_void_p]),
    "rg_proposal_destroy": (C.c_int, [C.c_void_p]),
    "rg_proposal_set_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "rg_proposal_get_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "rg_proposal_infer": (C.c_int, [C.c_void_p, C.POINTER(GBuffer), C.POINTER(RestirUniforms), C.c_void_p]),
    "rg_proposal_buffers": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "rg_proposal_gradients": (C.c_int, [C.c_void_p, C.POINTER(GBuffer), C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_int32, C.c_void_p, C.POINTER(C.c_double), C.c_void_p]),
    "rg_proposal_train": (C.c_int, [C.c_void_p, C.POINTER(GBuffer), C.POINTER(RestirUniforms), C.c_void_p,
                                    C.c_void_p]),
    "rg_proposal_last_loss": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
}

EXPORTED = tuple(_SIGNATURES)


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RestirError(-100, f"{LIB_PATH} is missing: run __graft_entry__.build() (or build.py) first")
        handle = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def check(rc: int) -> int:
    if rc < 0:
        raise RestirError(rc, lib().rg_last_error().decode(errors="replace"))
    return rc


def ptr(a) -> int | None:
    """Address of a numpy array or torch tensor (None for None)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()
