"""ctypes binding of the CPU oracle (liboracle.so) and of the reference build
(_ref/libref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker; never by the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref.so"
# The reference project's sources: $RESTIR_REFERENCE, else a checkout named
# "reference" beside this repository.
REFERENCE_ROOT = Path(os.environ.get("RESTIR_REFERENCE") or (HERE.parent.parent / "reference")).resolve()


def build(ref: bool | None = None) -> None:
    """Builds liboracle.so and, when the reference sources exist, _ref/libref.so."""
    env = dict(os.environ)
    r = subprocess.run(["make", "-C", str(HERE), "all"], capture_output=True, text=True, env=env)
    if r.returncode != 0:  # retry without OpenMP (toolchains without libgomp)
        r = subprocess.run(["make", "-C", str(HERE), "all", "OMP="], capture_output=True, text=True, env=env)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    if ref is None:
        ref = (REFERENCE_ROOT / "src" / "aabbTreeBuilder.cpp").exists()
    if ref:
        r = subprocess.run(["make", "-C", str(HERE), "ref", f"REF={REFERENCE_ROOT}"], capture_output=True, text=True,
                           env=env)
        if r.returncode != 0:
            raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")


class Scene(C.Structure):
    _fields_ = [("nodes", C.c_void_p), ("n_nodes", C.c_int32), ("tris", C.c_void_p), ("n_tris", C.c_int32),
                ("point_lights", C.c_void_p), ("n_point_lights", C.c_int32), ("tri_lights", C.c_void_p),
                ("n_tri_lights", C.c_int32), ("alias", C.c_void_p), ("n_alias", C.c_int32)]


class GBuffer(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("albedo", C.c_void_p), ("normal", C.c_void_p),
                ("material", C.c_void_p), ("world_pos", C.c_void_p), ("depth", C.c_void_p),
                ("normal_format", C.c_int32), ("world_pos_format", C.c_int32), ("depth_format", C.c_int32),
                ("reserved", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("node_visits", C.c_uint64), ("box_tests", C.c_uint64),
                ("tri_tests", C.c_uint64), ("stack_overflows", C.c_uint64), ("rays_unobservable", C.c_uint64)]


_oracle = None
_ref = None


def oracle():
    global _oracle
    if _oracle is None:
        if not LIB.exists():
            build(ref=False)
        _oracle = C.CDLL(str(LIB))
        _oracle.or_half_to_float.restype = C.c_float
        _oracle.or_half_to_float.argtypes = [C.c_uint16]
        _oracle.or_pcg_stream.argtypes = [C.c_uint64, C.c_uint64, C.c_int32, C.c_void_p]
        _oracle.or_rand_floats.argtypes = [C.c_uint64, C.c_uint64, C.c_int32, C.c_void_p]
        for name in ("or_initial_temporal", "or_spatial_biased", "or_spatial_unbiased", "or_shade",
                     "or_brute_force_fp64", "or_trace_gbuffer"):
            getattr(_oracle, name).restype = C.c_int
        _oracle.or_float_to_half.restype = C.c_uint16
        _oracle.or_float_to_half.argtypes = [C.c_float]
        _oracle.or_collect_tri_lights.restype = C.c_int64
        _oracle.or_collect_tri_lights.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64]
    return _oracle


def ref_available() -> bool:
    return REF_LIB.exists()


def ref():
    global _ref
    if _ref is None:
        _ref = C.CDLL(str(REF_LIB))
        _ref.ref_collect_tri_lights.restype = C.c_int64
        _ref.ref_collect_tri_lights.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64]
    return _ref


_ref_alias = None


def ref_alias():
    """The reference's own createAliasTable (_ref/libref_alias.so), or None."""
    global _ref_alias
    if _ref_alias is None:
        p = HERE / "_ref" / "libref_alias.so"
        if not p.exists():
            return None
        _ref_alias = C.CDLL(str(p))
        _ref_alias.ref_create_alias_table.restype = C.c_int32
        _ref_alias.ref_create_alias_table.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]
    return _ref_alias


def P(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def scene_struct(scene) -> tuple[Scene, list]:
    """Oracle view of a restir_gb300 Scene (keeps the arrays alive)."""
    tl = getattr(scene, "tri_lights", None)
    has_tri = tl is not None and len(tl) > 0
    keep = [scene.nodes, scene.triangles, scene.point_lights, scene.alias, tl]
    s = Scene(scene.nodes.ctypes.data, len(scene.nodes), scene.triangles.ctypes.data, len(scene.triangles),
              scene.point_lights.ctypes.data if len(scene.point_lights) else None, len(scene.point_lights),
              tl.ctypes.data if has_tri else None, len(tl) if has_tri else 0, scene.alias.ctypes.data,
              len(scene.alias))
    return s, keep


def gbuffer_struct(g: dict) -> GBuffer:
    """Planes of a G-buffer dict; an optional "formats" entry holds the
    (normal, world position, depth) VkFormat numbers (0 = default)."""
    h, w = g["depth"].shape[:2]
    nf, pf, df = g.get("formats", (0, 0, 0))
    return GBuffer(w, h, g["albedo"].ctypes.data, g["normal"].ctypes.data, g["material"].ctypes.data,
                   g["world_pos"].ctypes.data, g["depth"].ctypes.data, nf, pf, df, 0)


def crop_arg(crop):
    return None if crop is None else (C.c_int32 * 4)(*crop)


def check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed: {rc}")


def initial_temporal(scene, g_cur, g_prev, prev_res, out, uniforms, crop=None, stats=None):
    s, keep = scene_struct(scene)
    gc = gbuffer_struct(g_cur)
    gp = gbuffer_struct(g_prev) if g_prev is not None else None
    check(oracle().or_initial_temporal(C.byref(s), C.byref(gc), C.byref(gp) if gp else None, P(prev_res), P(out),
                                       C.byref(uniforms), crop_arg(crop), C.byref(stats) if stats else None),
          "initial_temporal")


def spatial_biased(scene, g, res_in, res_out, uniforms, iteration, crop=None):
    s, keep = scene_struct(scene)
    gg = gbuffer_struct(g)
    check(oracle().or_spatial_biased(C.byref(s), C.byref(gg), P(res_in), P(res_out), C.byref(uniforms),
                                     C.c_int32(iteration), crop_arg(crop)), "spatial_biased")


def spatial_unbiased(scene, g, res_in, res_out, uniforms, neighbors, pass_index=0, crop=None, stats=None):
    """pass_index p seeds the pass with frame*17 + p (p = 0 is the reference)."""
    s, keep = scene_struct(scene)
    gg = gbuffer_struct(g)
    check(oracle().or_spatial_unbiased(C.byref(s), C.byref(gg), P(res_in), P(res_out), C.byref(uniforms),
                                       C.c_int32(neighbors), C.c_int32(pass_index), crop_arg(crop),
                                       C.byref(stats) if stats else None),
          "spatial_unbiased")


def shade(scene, g, res, lighting_uniforms, out_rgba, crop=None):
    s, keep = scene_struct(scene)
    gg = gbuffer_struct(g)
    check(oracle().or_shade(C.byref(s), C.byref(gg), P(res), C.byref(lighting_uniforms), P(out_rgba),
                            crop_arg(crop)), "shade")


def brute_force(scene, g, camera_pos3, crop=None):
    s, keep = scene_struct(scene)
    gg = gbuffer_struct(g)
    h, w = g["depth"].shape
    cw, ch = (w, h) if crop is None else (crop[2], crop[3])
    out = np.zeros((ch, cw, 3), np.float64)
    cam = np.asarray(camera_pos3, np.float32)
    check(oracle().or_brute_force_fp64(C.byref(s), C.byref(gg), P(cam), P(out), crop_arg(crop)), "brute_force")
    return out


# ---------------------------------------------------------------- host preprocessing
NODE_DTYPE = np.dtype([("lmin", "<f4", 4), ("lmax", "<f4", 4), ("rmin", "<f4", 4), ("rmax", "<f4", 4),
                       ("left", "<i4"), ("right", "<i4"), ("pad", "<i4", 2)])                 # 80 B
TRI_DTYPE = np.dtype([("p1", "<f4", 4), ("p2", "<f4", 4), ("p3", "<f4", 4)])              # 48 B
ALIAS_DTYPE = np.dtype([("prob", "<f4"), ("alias", "<i4"), ("ori_prob", "<f4"), ("alias_ori_prob", "<f4")])


def tree_depth(nodes) -> int:
    """Levels of the tree (root = 1), breadth first over the child links."""
    left = np.asarray(nodes["left"]).astype(np.int64)
    right = np.asarray(nodes["right"]).astype(np.int64)
    level, depth = np.array([0], np.int64), 0
    while len(level):
        depth += 1
        kids = np.concatenate([left[level], right[level]])
        level = kids[kids >= 0]
    return depth


def build_bvh(tri_xyz):
    """The oracle's restatement of the reference's AabbTree::build: (nodes,
    triangles, depth) in the reference's layouts."""
    xyz = np.ascontiguousarray(tri_xyz, np.float32).reshape(-1, 9)
    n = len(xyz)
    nodes = np.zeros(max(n - 1, 1), NODE_DTYPE)
    tris = np.zeros(n, TRI_DTYPE)
    o = oracle()
    o.or_build_bvh.restype = C.c_int32
    rc = o.or_build_bvh(P(xyz), C.c_int32(n), P(nodes), P(tris))
    if rc != n - 1:
        raise RuntimeError(f"oracle tree build failed: {rc}")
    return nodes, tris, tree_depth(nodes)


def build_alias_table(point_lights):
    """The oracle's restatement of createAliasTable over point lights."""
    pl = np.ascontiguousarray(point_lights)
    out = np.zeros(len(pl), ALIAS_DTYPE)
    oracle().or_build_alias_table(P(pl), C.c_int32(len(pl)), None, C.c_int32(0), P(out))
    return out


# ---------------------------------------------------------------- primary-ray G-buffer
class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("right", C.c_float * 3), ("up", C.c_float * 3),
                ("forward", C.c_float * 3), ("tan_half_fov_y", C.c_float), ("aspect", C.c_float),
                ("projection_view", C.c_float * 16)]


def camera_struct(cam) -> Camera:
    """The oracle's camera record of a CameraModel (src/camera.h:25-50 basis,
    float32 values as the model computes them)."""
    import math
    pos, right, up, fwd = cam.basis()
    c = Camera()
    c.position[:] = [float(v) for v in pos]
    c.right[:] = [float(v) for v in right]
    c.up[:] = [float(v) for v in up]
    c.forward[:] = [float(v) for v in fwd]
    c.tan_half_fov_y = float(np.float32(math.tan(0.5 * cam.fov_y)))
    c.aspect = float(np.float32(cam.aspect))
    c.projection_view[:] = [float(v) for v in cam.projection_view_colmajor()]
    return c


def has_gbuffer_tracer() -> bool:
    return hasattr(oracle(), "or_trace_gbuffer")


def trace_gbuffer(scene, frame_index: int = 0, crop=None, camera=None) -> dict:
    """The oracle's primary-ray G-buffer of one frame (dict of numpy planes in
    the library's formats); with `crop` only that region is traced, the rest
    stays zero."""
    w, h = scene.width, scene.height
    g = {"albedo": np.zeros((h, w, 4), np.uint8), "normal": np.zeros((h, w, 4), np.uint16),
         "material": np.zeros((h, w, 2), np.uint16), "world_pos": np.zeros((h, w, 4), np.float32),
         "depth": np.zeros((h, w), np.float32)}
    s, keep = scene_struct(scene)
    cam = camera_struct(camera if camera is not None else scene.cameras[frame_index])
    mats = np.ascontiguousarray(scene.materials)
    check(oracle().or_trace_gbuffer(C.byref(s), P(mats), C.c_int32(len(mats)), C.byref(cam), C.c_int32(w),
                                    C.c_int32(h), crop_arg(crop), P(g["albedo"]), P(g["normal"]), P(g["material"]),
                                    P(g["world_pos"]), P(g["depth"])), "trace_gbuffer")
    return g


# ---------------------------------------------------------------- learned proposal
class Mlp(C.Structure):
    _fields_ = [("clusters", C.c_int32), ("mix", C.c_float), ("n_lights", C.c_int32),
                ("box_center", C.c_float * 3), ("box_inv_half", C.c_float * 3), ("params", C.c_void_p),
                ("cluster_valid", C.c_void_p), ("cluster_of", C.c_void_p)]


class OracleMlp:
    """The oracle's statement of the learned proposal for given FP32 parameters,
    clusters and normalisation box (the same float arithmetic as the product's
    box centre and inverse half-extent)."""

    def __init__(self, params, cluster_of, clusters, mix=0.9, box_min=(0, 0, 0), box_max=(1, 1, 1)):
        self.params = np.ascontiguousarray(params, np.float32)
        self.cluster_of = np.ascontiguousarray(cluster_of, np.int32)
        self.clusters = clusters
        self.valid = np.zeros(clusters, np.uint8)
        self.valid[np.unique(self.cluster_of)] = 1
        bmin, bmax = np.asarray(box_min, np.float32), np.asarray(box_max, np.float32)
        center = np.float32(0.5) * (bmin + bmax)
        inv_half = np.float32(2.0) / (bmax - bmin)
        self.s = Mlp(clusters, mix, len(self.cluster_of), (C.c_float * 3)(*center), (C.c_float * 3)(*inv_half),
                     self.params.ctypes.data, self.valid.ctypes.data, self.cluster_of.ctypes.data)
        o = oracle()
        o.or_mlp_loss_grad.restype = C.c_double
        o.or_bf16_round.restype = C.c_float
        o.or_bf16_round.argtypes = [C.c_float]

    def set_params(self, params):
        self.params = np.ascontiguousarray(params, np.float32)
        self.s.params = self.params.ctypes.data

    def row_stats(self, g, cam, rows=None, logits=False):
        gg = gbuffer_struct(g)
        n = len(rows) if rows is not None else g["depth"].size
        rows_a = None if rows is None else np.ascontiguousarray(rows, np.int32)
        lse = np.zeros(n, np.float64)
        amax = np.zeros(n, np.int32)
        z = np.zeros((n, self.clusters), np.float64) if logits else None
        cam_a = np.asarray(cam, np.float32)
        oracle().or_mlp_row_stats(C.byref(self.s), C.byref(gg), P(cam_a), C.c_int32(n), P(rows_a), P(lse), P(amax),
                                  P(z))
        return (lse, amax, z) if logits else (lse, amax)

    def sample(self, g, cam, frame, n_cand, rows):
        gg = gbuffer_struct(g)
        rows_a = np.ascontiguousarray(rows, np.int32)
        n = len(rows_a)
        keys = np.zeros((n, n_cand), np.int32)
        qs = np.zeros((n, n_cand), np.float32)
        cam_a = np.asarray(cam, np.float32)
        oracle().or_mlp_sample(C.byref(self.s), C.byref(gg), P(cam_a), C.c_uint32(frame), C.c_int32(n_cand),
                               C.c_int32(n), P(rows_a), P(keys), P(qs))
        return keys, qs

    def loss_grad(self, g, cam, rows, targets, emulate=True, params64=None):
        gg = gbuffer_struct(g)
        rows_a = np.ascontiguousarray(rows, np.int32)
        tg = np.ascontiguousarray(targets, np.int32)
        grad = np.zeros(len(self.params), np.float64)
        p64 = None if params64 is None else np.ascontiguousarray(params64, np.float64)
        cam_a = np.asarray(cam, np.float32)
        loss = oracle().or_mlp_loss_grad(C.byref(self.s), P(p64), C.byref(gg), P(cam_a), C.c_int32(len(rows_a)),
                                         P(rows_a), P(tg), C.c_int32(1 if emulate else 0), P(grad))
        return loss, grad


class Learned(C.Structure):
    _fields_ = [("cand", C.c_void_p), ("order", C.c_void_p), ("offset", C.c_void_p), ("col", C.c_void_p),
                ("within", C.c_void_p), ("mix", C.c_float), ("uniform_pdf", C.c_float)]


def cluster_tables(point_lights, cluster_of, clusters):
    """(order, offset, col, within) of the oracle's per-cluster alias tables."""
    n = len(point_lights)
    order = np.zeros(n, np.int32)
    offset = np.zeros(clusters + 1, np.int32)
    col = np.zeros(n, np.dtype([("prob", "<f4"), ("alias", "<i4"), ("ori_prob", "<f4"), ("alias_ori_prob", "<f4")]))
    within = np.zeros(n, np.float32)
    co = np.ascontiguousarray(cluster_of, np.int32)
    check(oracle().or_cluster_tables(P(point_lights), C.c_int32(n), P(co), C.c_int32(clusters), P(order), P(offset),
                                     P(col), P(within)), "cluster_tables")
    return order, offset, col, within


def initial_temporal_learned(scene, g_cur, g_prev, prev_res, out, uniforms, candidates, cluster_of, clusters,
                             mix=0.9, crop=None, stats=None):
    """The pass with the learned proposal's candidates (structured array with
    fields key, q; 32 per pixel) as the candidate source."""
    s, keep = scene_struct(scene)
    gc = gbuffer_struct(g_cur)
    gp = gbuffer_struct(g_prev) if g_prev is not None else None
    order, offset, col, within = cluster_tables(scene.point_lights, cluster_of, clusters)
    cand = np.ascontiguousarray(candidates)
    upd = np.float32(np.float32(1.0) - np.float32(mix)) / np.float32(len(scene.point_lights))
    lrn = Learned(cand.ctypes.data, order.ctypes.data, offset.ctypes.data, col.ctypes.data, within.ctypes.data,
                  mix, float(upd))
    check(oracle().or_initial_temporal_learned(C.byref(s), C.byref(gc), C.byref(gp) if gp else None, P(prev_res),
                                               P(out), C.byref(uniforms), C.byref(lrn), crop_arg(crop),
                                               C.byref(stats) if stats else None),
          "initial_temporal_learned")


# ---------------------------------------------------------------- reservoir variants
VARIANT_LIBS = {(1, 0): "liboracle.so", (2, 0): "liboracle_rs2.so", (1, 1): "liboracle_mis.so",
                (2, 1): "liboracle_rs2_mis.so"}
_variant_handles = {}


def reservoir_dtype(rs: int, mis: int) -> np.dtype:
    """std430 Reservoir with RESERVOIR_SIZE rs and UNBIASED_MIS mis."""
    sample = [("pos_lum", "<f4", 4), ("normal", "<f4", 4), ("light_index", "<i4"), ("p_hat", "<f4"),
              ("sum_weights", "<f4"), ("w", "<f4")]
    if mis:
        sample += [("sum_phat", "<f4"), ("pad_s", "<f4", 3)]
    return np.dtype([("s", np.dtype(sample), (rs,)), ("m", "<u4"), ("pad", "<u4", 3)])


def oracle_variant(rs: int, mis: int):
    """The oracle built for RESERVOIR_SIZE rs / UNBIASED_MIS mis (same symbols as oracle())."""
    key = (rs, mis)
    if key not in _variant_handles:
        path = HERE / VARIANT_LIBS[key]
        if not path.exists():
            build(ref=False)
        h = C.CDLL(str(path))
        for name in ("or_initial_temporal", "or_spatial_biased", "or_spatial_unbiased", "or_shade"):
            getattr(h, name).restype = C.c_int
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        h.or_reservoir_layout(C.byref(a), C.byref(b), C.byref(c))
        assert (a.value, b.value) == key and c.value == reservoir_dtype(rs, mis).itemsize
        _variant_handles[key] = h
    return _variant_handles[key]


def ref_reservoir(rs: int, mis: int):
    """The reference's own reservoir.glsl compiled for the variant (None if not built)."""
    p = HERE / "_ref" / f"libref_res_rs{rs}_mis{mis}.so"
    return C.CDLL(str(p)) if p.exists() else None


def to_flat(res: np.ndarray, rs: int) -> np.ndarray:
    """Reservoirs of a variant dtype -> the interchange layout of the reference bridge."""
    out = np.zeros((len(res), 16 * rs + 4), np.float32)
    for i in range(rs):
        s = res["s"][:, i]
        out[:, 16 * i:16 * i + 4] = s["pos_lum"]
        out[:, 16 * i + 4:16 * i + 8] = s["normal"]
        out[:, 16 * i + 8] = s["light_index"].view(np.float32)
        out[:, 16 * i + 9] = s["p_hat"]
        out[:, 16 * i + 10] = s["sum_weights"]
        out[:, 16 * i + 11] = s["w"]
        if "sum_phat" in s.dtype.names:
            out[:, 16 * i + 12] = s["sum_phat"]
    out[:, 16 * rs] = res["m"].view(np.float32)
    return out
