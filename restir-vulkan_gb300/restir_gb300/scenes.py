"""Seeded synthetic scenes for the benchmark configurations.

The reference renders glTF demo scenes; the workloads here are procedural,
fully determined by a seed (numpy PCG64), and built into the reference's
buffers with this package's own host preprocessing: the binned-SAH tree
(rg_build_bvh, the reference's AabbTree::build) and the Vose alias table
(rg_build_alias_table, the reference's createAliasTable).

  config 1  256x256, unit box room (12 tris) + 64 cube occluders (768 tris),
            Lambertian albedo U[0.2,0.9], 1024 point lights uniform in the box,
            RGB intensity log-uniform [0.1,10], uniform source pdf, C=32,
            biased spatial reuse k=5, R=30, 1 iteration, 1 frame.
  config 2  1920x1080, 100k random triangles (edge log-uniform [1e-3,0.1]) in
            the room, roughness U[0.05,1], metallic Bernoulli(0.2); 65,536
            point lights, intensity log-uniform [0.01,100]; alias table by
            power; 8 frames, camera moving 0.01/frame; C=32; temporal (M clamp
            20) + 2 unbiased spatial passes, k=5, R=30.
  config 3  1920x1080, 2^16 jittered-grid rocks of 16 triangles + room
            (1,048,588 tris); 1,048,576 point lights with Pareto(1.5) power in
            4096 Gaussian clusters (sigma 0.02); alias table by power; 16
            frames; temporal + 3 unbiased spatial passes, k=5, R=30.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field, replace

import numpy as np

from . import _lib
from .camera import CameraModel


@dataclass
class Scene:
    name: str
    tri_xyz: np.ndarray          # (n, 9) float32, scene order
    nodes: np.ndarray            # NODE_DTYPE
    triangles: np.ndarray        # TRI_DTYPE (scene order)
    materials: np.ndarray        # MATERIAL_DTYPE per triangle
    point_lights: np.ndarray     # POINT_LIGHT_DTYPE
    alias: np.ndarray            # ALIAS_DTYPE
    width: int
    height: int
    cameras: list                # CameraModel per frame
    candidates: int = 32
    unbiased: bool = False
    spatial_passes: int = 1
    neighbors: int = 5
    radius: float = 30.0
    temporal: bool = False
    temporal_mult: int = 20
    pos_threshold: float = 0.1
    normal_threshold: float = 25.0
    source_pdf: str = "power"
    tree_depth: int = 0
    tri_lights: np.ndarray | None = None  # TRI_LIGHT_DTYPE; used when point_lights is empty
    extra: dict = field(default_factory=dict)

    @property
    def frames(self) -> int:
        return len(self.cameras)

    def desc(self) -> _lib.SceneDesc:
        d = _lib.SceneDesc()
        d.nodes = self.nodes.ctypes.data
        d.n_nodes = len(self.nodes)
        d.triangles = self.triangles.ctypes.data
        d.n_triangles = len(self.triangles)
        d.point_lights = self.point_lights.ctypes.data if len(self.point_lights) else None
        d.n_point_lights = len(self.point_lights)
        has_tri = self.tri_lights is not None and len(self.tri_lights) > 0
        d.tri_lights = self.tri_lights.ctypes.data if has_tri else None
        d.n_tri_lights = len(self.tri_lights) if has_tri else 0
        d.alias_table = self.alias.ctypes.data
        d.n_alias = len(self.alias)
        d.materials = self.materials.ctypes.data
        d.n_materials = len(self.materials)
        return d

    def uniforms(self, frame_index: int) -> _lib.RestirUniforms:
        """RestirUniforms of frame `frame_index` (0-based); the reference's
        counter is incremented before the first submit (app.cpp:420,776)."""
        u = _lib.RestirUniforms()
        cam = self.cameras[frame_index]
        prev = self.cameras[frame_index - 1] if frame_index > 0 else cam
        u.prev_frame_projection_view[:] = [float(v) for v in prev.projection_view_colmajor()]
        u.camera_pos[:] = [float(v) for v in cam.basis()[0]] + [1.0]
        u.screen_size[:] = [self.width, self.height]
        u.frame = frame_index + 1
        u.initial_light_sample_count = self.candidates
        u.temporal_sample_count_multiplier = self.temporal_mult
        u.spatial_pos_threshold = self.pos_threshold
        u.spatial_normal_threshold = self.normal_threshold
        u.spatial_neighbors = self.neighbors
        u.spatial_radius = self.radius
        flags = _lib.RG_FLAG_VISIBILITY_REUSE
        if self.temporal and frame_index > 0:
            flags |= _lib.RG_FLAG_TEMPORAL_REUSE
        u.flags = flags
        return u

    def lighting_uniforms(self, frame_index: int, gamma: float = 1.0) -> _lib.LightingUniforms:
        lu = _lib.LightingUniforms()
        cam = self.cameras[frame_index]
        lu.camera_pos[:] = [float(v) for v in cam.basis()[0]] + [1.0]
        lu.buffer_size[:] = [self.width, self.height]
        lu.debug_mode = 0
        lu.gamma = gamma
        return lu

    def view(self, camera, width: int, height: int, name: str | None = None) -> "Scene":
        """The same scene seen by another camera at another resolution (arrays shared)."""
        return replace(self, name=name or self.name, width=width, height=height, cameras=[camera])

    def frame_params(self, frame_index: int) -> _lib.FrameParams:
        fp = _lib.FrameParams()
        fp.uniforms = self.uniforms(frame_index)
        fp.unbiased = int(self.unbiased)
        fp.spatial_iterations = self.spatial_passes
        fp.unbiased_neighbors = self.neighbors
        fp.gamma = 1.0
        return fp

    def samples_per_frame(self, frame_index: int = 1) -> int:
        """Reservoir samples of one frame: RIS candidates + temporal merges +
        spatial neighbour merges (per pixel, times the pixel count)."""
        temporal = 1 if (self.temporal and frame_index > 0) else 0
        if self.unbiased:
            spatial = self.spatial_passes * self.neighbors
        else:
            spatial = 2 * self.spatial_passes * self.neighbors
        return self.width * self.height * (self.candidates + temporal + spatial)

    def nominal_rays_per_frame(self) -> int:
        per_px = 1 + (self.spatial_passes * (self.neighbors + 1) if self.unbiased else 0)
        return self.width * self.height * per_px


# ------------------------------------------------------------------ geometry helpers
def room_triangles(lo=0.0, hi=1.0) -> np.ndarray:
    c = np.array([[x, y, z] for x in (lo, hi) for y in (lo, hi) for z in (lo, hi)], np.float32)
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    tris = []
    for a, b, cc, d in quads:
        tris.append(np.concatenate([c[a], c[b], c[cc]]))
        tris.append(np.concatenate([c[a], c[cc], c[d]]))
    return np.array(tris, np.float32)


def cube_triangles(center, edge) -> np.ndarray:
    h = 0.5 * edge
    room = room_triangles(-1.0, 1.0).reshape(-1, 3, 3)
    return (room * np.float32(h) + np.asarray(center, np.float32)).reshape(-1, 9).astype(np.float32)


def rock_mesh(rng, n_instances: int):
    """Octagonal bipyramid (16 triangles) per instance, jittered vertices."""
    ang = np.arange(8) * (2 * math.pi / 8)
    ring = np.stack([np.cos(ang), np.zeros(8), np.sin(ang)], 1)  # (8,3)
    jitter = rng.uniform(0.7, 1.3, (n_instances, 8, 1))
    ring_v = ring[None] * jitter
    top = np.zeros((n_instances, 1, 3)); top[..., 1] = rng.uniform(0.6, 1.2, (n_instances, 1))
    bot = np.zeros((n_instances, 1, 3)); bot[..., 1] = -rng.uniform(0.6, 1.2, (n_instances, 1))
    verts = np.concatenate([ring_v, top, bot], 1)  # (n, 10, 3)
    faces = []
    for k in range(8):
        faces.append((k, (k + 1) % 8, 8))
        faces.append(((k + 1) % 8, k, 9))
    faces = np.array(faces)
    return verts, faces


def random_rotations(rng, n):
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    r = np.empty((n, 3, 3))
    r[:, 0, 0] = 1 - 2 * (y * y + z * z); r[:, 0, 1] = 2 * (x * y - z * w); r[:, 0, 2] = 2 * (x * z + y * w)
    r[:, 1, 0] = 2 * (x * y + z * w); r[:, 1, 1] = 1 - 2 * (x * x + z * z); r[:, 1, 2] = 2 * (y * z - x * w)
    r[:, 2, 0] = 2 * (x * z - y * w); r[:, 2, 1] = 2 * (y * z + x * w); r[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return r


def srgb_encode_u8(lin: np.ndarray) -> np.ndarray:
    lin = np.clip(lin, 0.0, 1.0)
    s = np.where(lin <= 0.0031308, lin * 12.92, 1.055 * np.power(lin, 1.0 / 2.4) - 0.055)
    return np.clip(np.rint(s * 255.0), 0, 255).astype(np.uint8)


def luminance_f32(r, g, b):
    f = np.float32
    r, g, b = (np.asarray(v, f) for v in (r, g, b))
    return (f(0.2126) * r + f(0.7152) * g) + f(0.0722) * b  # common.glsl:7-9, left to right


def make_point_lights(pos: np.ndarray, rgb: np.ndarray) -> np.ndarray:
    n = len(pos)
    pl = np.zeros(n, _lib.POINT_LIGHT_DTYPE)
    pl["pos"][:, :3] = pos.astype(np.float32)
    pl["pos"][:, 3] = 1.0
    rgb = rgb.astype(np.float32)
    pl["color_lum"][:, :3] = rgb
    pl["color_lum"][:, 3] = luminance_f32(rgb[:, 0], rgb[:, 1], rgb[:, 2])
    return pl


def make_materials(albedo_lin: np.ndarray, roughness: np.ndarray, metallic: np.ndarray) -> np.ndarray:
    n = len(albedo_lin)
    m = np.zeros(n, _lib.MATERIAL_DTYPE)
    m["albedo"][:, :3] = srgb_encode_u8(albedo_lin)
    m["albedo"][:, 3] = 0
    m["roughness"] = np.clip(np.rint(np.asarray(roughness) * 65535.0), 0, 65535).astype(np.uint16)
    m["metallic"] = np.clip(np.rint(np.asarray(metallic) * 65535.0), 0, 65535).astype(np.uint16)
    return m


# ------------------------------------------------------------------ host preprocessing through the C ABI
# The tree and alias-table builds the scenes use: the library's (rg_build_bvh,
# rg_build_alias_table) unless set_preprocessing replaced them, e.g. with
# another implementation of the same reference functions for a run that must
# not load the library.
_PREPROCESS = {}


def set_preprocessing(bvh=None, alias=None):
    """bvh(tri_xyz) -> (nodes, triangles, depth) and alias(point_lights) ->
    alias table, in the reference's layouts; None restores the library's."""
    _PREPROCESS.clear()
    if bvh is not None:
        _PREPROCESS["bvh"] = bvh
    if alias is not None:
        _PREPROCESS["alias"] = alias


def build_bvh(tri_xyz: np.ndarray):
    tri_xyz = np.ascontiguousarray(tri_xyz, np.float32)
    if "bvh" in _PREPROCESS:
        nodes, tris, depth = _PREPROCESS["bvh"](tri_xyz)
        return nodes.view(_lib.NODE_DTYPE), tris.view(_lib.TRI_DTYPE), depth
    n = len(tri_xyz)
    nodes = np.zeros(max(n - 1, 1), _lib.NODE_DTYPE)
    tris = np.zeros(n, _lib.TRI_DTYPE)
    L = _lib.lib()
    _lib.check(L.rg_build_bvh(tri_xyz.ctypes.data, n, nodes.ctypes.data, tris.ctypes.data))
    depth = _lib.check(L.rg_tree_depth(nodes.ctypes.data, len(nodes)))
    return nodes, tris, depth


def build_alias(point_lights: np.ndarray, uniform: bool = False) -> np.ndarray:
    src = point_lights.copy()
    if uniform:  # equal weights give the uniform source pdf through the same table
        src["color_lum"][:, 3] = 1.0
    if "alias" in _PREPROCESS:
        return _PREPROCESS["alias"](src).view(_lib.ALIAS_DTYPE)
    out = np.zeros(len(src), _lib.ALIAS_DTYPE)
    _lib.check(_lib.lib().rg_build_alias_table(src.ctypes.data, len(src), None, 0, out.ctypes.data))
    return out


def _finish(name, tri_xyz, mats, lights, width, height, cameras, uniform_pdf, **kw) -> Scene:
    nodes, tris, depth = build_bvh(tri_xyz)
    alias = build_alias(lights, uniform=uniform_pdf)
    return Scene(name=name, tri_xyz=tri_xyz, nodes=nodes, triangles=tris, materials=mats, point_lights=lights,
                 alias=alias, width=width, height=height, cameras=cameras, tree_depth=depth,
                 source_pdf="uniform" if uniform_pdf else "power", **kw)


def camera_path(rng, frames: int, aspect: float, step: float = 0.01):
    """Seeded camera path inside the unit room: a straight spline moving
    `step` per frame, looking at a fixed seeded target."""
    start = rng.uniform(0.25, 0.75, 3)
    target = rng.uniform(0.2, 0.8, 3)
    while np.linalg.norm(target - start) < 0.3:
        target = rng.uniform(0.2, 0.8, 3)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    cams = []
    for f in range(frames):
        pos = start + d * step * f
        cams.append(CameraModel(position=pos.astype(np.float32), look_at=target.astype(np.float32), aspect=aspect))
    return cams


def config1(seed: int = 1, width: int = 256, height: int = 256) -> Scene:
    rng = np.random.default_rng(seed)
    room = room_triangles()
    cubes, albedo = [], []
    albedo.append(np.repeat(rng.uniform(0.2, 0.9, (1, 3)), 12, 0))
    for _ in range(64):
        e = rng.uniform(0.02, 0.15)
        c = rng.uniform(0.0, 1.0, 3)
        cubes.append(cube_triangles(c, e))
        albedo.append(np.repeat(rng.uniform(0.2, 0.9, (1, 3)), 12, 0))
    tri_xyz = np.concatenate([room] + cubes).astype(np.float32)
    albedo = np.concatenate(albedo)
    n = len(tri_xyz)
    mats = make_materials(albedo, np.ones(n), np.zeros(n))  # Lambertian: roughness 1, metallic 0
    lpos = rng.uniform(0.0, 1.0, (1024, 3))
    rgb = np.exp(rng.uniform(math.log(0.1), math.log(10.0), (1024, 3)))
    lights = make_point_lights(lpos, rgb)
    cams = camera_path(rng, 1, width / height)
    return _finish("config1", tri_xyz, mats, lights, width, height, cams, uniform_pdf=True, candidates=32,
                   unbiased=False, spatial_passes=1, neighbors=5, radius=30.0, temporal=False)


def config2(seed: int = 2, width: int = 1920, height: int = 1080, n_tris: int = 100_000, n_lights: int = 65_536,
            frames: int = 8) -> Scene:
    rng = np.random.default_rng(seed)
    room = room_triangles()
    centers = rng.uniform(0.0, 1.0, (n_tris, 1, 3))
    edge = np.exp(rng.uniform(math.log(1e-3), math.log(0.1), (n_tris, 1, 1)))
    verts = centers + edge * rng.uniform(-0.5, 0.5, (n_tris, 3, 3))
    tri_xyz = np.concatenate([room, verts.reshape(n_tris, 9)]).astype(np.float32)
    n = len(tri_xyz)
    albedo = rng.uniform(0.2, 0.9, (n, 3))
    rough = rng.uniform(0.05, 1.0, n)
    metal = (rng.uniform(0, 1, n) < 0.2).astype(np.float64)
    mats = make_materials(albedo, rough, metal)
    lpos = rng.uniform(0.0, 1.0, (n_lights, 3))
    rgb = np.exp(rng.uniform(math.log(0.01), math.log(100.0), (n_lights, 3)))
    lights = make_point_lights(lpos, rgb)
    cams = camera_path(rng, frames, width / height)
    return _finish("config2", tri_xyz, mats, lights, width, height, cams, uniform_pdf=False, candidates=32,
                   unbiased=True, spatial_passes=2, neighbors=5, radius=30.0, temporal=True, temporal_mult=20)


def config3(seed: int = 3, width: int = 1920, height: int = 1080, grid=(64, 32, 32), n_lights: int = 1_048_576,
            n_clusters: int = 4096, frames: int = 16) -> Scene:
    rng = np.random.default_rng(seed)
    room = room_triangles()
    gx, gy, gz = grid
    n_rocks = gx * gy * gz
    ii, jj, kk = np.meshgrid(np.arange(gx), np.arange(gy), np.arange(gz), indexing="ij")
    cell = np.array([1.0 / gx, 1.0 / gy, 1.0 / gz])
    centers = (np.stack([ii, jj, kk], -1).reshape(-1, 3) + rng.uniform(0.25, 0.75, (n_rocks, 3))) * cell
    verts, faces = rock_mesh(rng, n_rocks)
    rot = random_rotations(rng, n_rocks)
    scale = rng.uniform(0.15, 0.35, (n_rocks, 1, 1)) * cell.min()
    world = np.einsum("nij,nvj->nvi", rot, verts) * scale + centers[:, None, :]
    rock_tris = world[:, faces, :].reshape(n_rocks * 16, 9)
    tri_xyz = np.concatenate([room, rock_tris]).astype(np.float32)
    n = len(tri_xyz)
    albedo = np.repeat(rng.uniform(0.2, 0.9, (n_rocks + 1, 3)), [12] + [16] * n_rocks, axis=0)
    rough = np.repeat(rng.uniform(0.05, 1.0, n_rocks + 1), [12] + [16] * n_rocks)
    metal = np.repeat((rng.uniform(0, 1, n_rocks + 1) < 0.2).astype(np.float64), [12] + [16] * n_rocks)
    mats = make_materials(albedo, rough, metal)
    cl = rng.uniform(0.05, 0.95, (n_clusters, 3))
    which = rng.integers(0, n_clusters, n_lights)
    lpos = np.clip(cl[which] + rng.normal(0.0, 0.02, (n_lights, 3)), 0.001, 0.999)
    power = (1.0 - rng.uniform(0.0, 1.0, n_lights)) ** (-1.0 / 1.5)  # Pareto(alpha = 1.5, x_m = 1)
    tint = rng.uniform(0.5, 1.0, (n_lights, 3))
    rgb = tint / luminance_f32(tint[:, 0], tint[:, 1], tint[:, 2])[:, None] * power[:, None] * 0.05
    lights = make_point_lights(lpos, rgb)
    cams = camera_path(rng, frames, width / height)
    # the Gaussian cluster of each light: a light clustering for the learned
    # proposal at this scale (k-means over 1M lights is slow on the host)
    return _finish("config3", tri_xyz, mats, lights, width, height, cams, uniform_pdf=False, candidates=32,
                   unbiased=True, spatial_passes=3, neighbors=5, radius=30.0, temporal=True, temporal_mult=20,
                   extra={"light_cluster": which.astype(np.int32)})


def config5(seed: int = 5, n_views: int = 64, n_tris: int = 100_000, n_lights: int = 65_536,
            min_size=(320, 240), max_size=(1920, 1080)):
    """Batched multi-view workload: config 2's scene seen by n_views seeded
    cameras whose widths and heights are each log-uniform between min_size and
    max_size.  Returns (scene, views), every view a Scene sharing its arrays."""
    base = config2(width=min_size[0], height=min_size[1], n_tris=n_tris, n_lights=n_lights, frames=1)
    rng = np.random.default_rng(seed)
    views = []
    for v in range(n_views):
        w = int(round(math.exp(rng.uniform(math.log(min_size[0]), math.log(max_size[0])))))
        h = int(round(math.exp(rng.uniform(math.log(min_size[1]), math.log(max_size[1])))))
        pos = rng.uniform(0.15, 0.85, 3)
        target = rng.uniform(0.15, 0.85, 3)
        while np.linalg.norm(target - pos) < 0.3:
            target = rng.uniform(0.15, 0.85, 3)
        cam = CameraModel(position=pos.astype(np.float32), look_at=target.astype(np.float32), aspect=w / h)
        views.append(base.view(cam, w, h, name=f"config5_view{v}"))
    return base, views


def make_tri_lights(tri_xyz: np.ndarray, emission_rgb: np.ndarray) -> np.ndarray:
    """triLight records of emissive triangles, collected by the library
    (rg_collect_triangle_lights, the reference's collectTriangleLightsFromScene,
    src/misc.cpp:380-414): one instance per triangle with an identity world
    matrix and the triangle's emission as its emissive factor."""
    t = np.ascontiguousarray(tri_xyz.reshape(-1, 3, 3), np.float32)
    e = np.ascontiguousarray(emission_rgb, np.float32)
    idx = np.arange(3, dtype=np.uint32)
    eye = (C.c_float * 16)(*np.eye(4, dtype=np.float32).ravel())
    inst = (_lib.MeshInstance * len(t))()
    for i in range(len(t)):
        inst[i] = _lib.MeshInstance(t[i].ctypes.data, idx.ctypes.data, 3, eye, (C.c_float * 3)(*e[i]))
    out = np.zeros(len(t), _lib.TRI_LIGHT_DTYPE)
    n = _lib.lib().rg_collect_triangle_lights(inst, len(t), out.ctypes.data, len(out))
    _lib.check(n if n < 0 else 0)
    return out[:n]


def config1_triangle_lights(seed: int = 11, width: int = 128, height: int = 128, n_quads: int = 12) -> Scene:
    """Config 1's room and cubes lit by emissive quads under the ceiling instead
    of point lights: exercises triangle-light sampling (pickPointOnTriangle,
    restirOmni.glsl:68-71,123-133), the alias table by luminance x area, and
    negative light indices in shading (lighting.frag:56-58)."""
    base = config1(seed=seed, width=width, height=height)
    rng = np.random.default_rng(seed + 1000)
    quads, emis = [], []
    for _ in range(n_quads):
        cx, cz = rng.uniform(0.15, 0.85, 2)
        h = rng.uniform(0.02, 0.06)
        y = 0.97
        a, b, c, d = ([cx - h, y, cz - h], [cx + h, y, cz - h], [cx + h, y, cz + h], [cx - h, y, cz + h])
        quads.append(np.array([a + b + c, a + c + d], np.float32))  # facing down
        e = np.exp(rng.uniform(np.log(2.0), np.log(40.0), 3))
        emis.append(np.repeat(e[None], 2, 0))
    quad_xyz = np.concatenate(quads).astype(np.float32)
    tri_xyz = np.concatenate([base.tri_xyz, quad_xyz]).astype(np.float32)
    emis = np.concatenate(emis)
    tl = make_tri_lights(quad_xyz, emis)
    n_geo = len(base.tri_xyz)
    mats = np.concatenate([base.materials, make_materials(np.clip(emis, 0, 1), np.ones(len(quad_xyz)),
                                                          np.zeros(len(quad_xyz)))])
    mats["albedo"][n_geo:, 3] = 255  # emissive flag (gBuffer.frag:73-79)
    nodes, tris, depth = build_bvh(tri_xyz)
    alias = np.zeros(len(tl), _lib.ALIAS_DTYPE)
    _lib.check(_lib.lib().rg_build_alias_table(None, 0, tl.ctypes.data, len(tl), alias.ctypes.data))
    # looking up from below the middle of the room, so the emitters are in view
    cams = [CameraModel(position=np.array([0.5, 0.35, 0.2], np.float32),
                        look_at=np.array([0.5, 0.9, 0.6], np.float32), aspect=width / height)]
    return Scene(name="config1_triangle_lights", tri_xyz=tri_xyz, nodes=nodes, triangles=tris, materials=mats,
                 point_lights=np.zeros(0, _lib.POINT_LIGHT_DTYPE), alias=alias, width=width, height=height,
                 cameras=cams, tree_depth=depth, candidates=32, unbiased=False, spatial_passes=1,
                 neighbors=5, radius=30.0, temporal=False, tri_lights=tl, source_pdf="power")


CONFIGS = {"config1": config1, "config2": config2, "config3": config3}


def trace_gbuffer_host(scene: Scene, frame_index: int = 0):
    """CPU primary-ray G-buffer of one frame (dict of numpy planes)."""
    w, h = scene.width, scene.height
    g = {
        "albedo": np.zeros((h, w, 4), np.uint8),
        "normal": np.zeros((h, w, 4), np.uint16),
        "material": np.zeros((h, w, 2), np.uint16),
        "world_pos": np.zeros((h, w, 4), np.float32),
        "depth": np.zeros((h, w), np.float32),
    }
    cam = scene.cameras[frame_index].to_c()
    d = scene.desc()
    _lib.check(_lib.lib().rg_trace_gbuffer_host(C.byref(d), C.byref(cam), w, h, g["albedo"].ctypes.data,
                                                g["normal"].ctypes.data, g["material"].ctypes.data,
                                                g["world_pos"].ctypes.data, g["depth"].ctypes.data))
    return g
