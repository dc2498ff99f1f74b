"""Shared helpers for the parity tests (oracle sequences, comparisons)."""
from __future__ import annotations

import numpy as np

import oracle_binding as ob
from restir_gb300 import _lib


def new_res(n):
    return np.zeros(n, _lib.RESERVOIR_DTYPE)


# Float words of a reservoir (pos_lum, normal, p-hat, sum of weights, W); word 8
# is the light index and word 12 M.
_FLOAT_WORDS = np.array([0, 1, 2, 3, 4, 5, 6, 7, 9, 10, 11])
QNAN = np.uint32(0x7FC00000)


def canonical_nan(bits: np.ndarray) -> np.ndarray:
    """32-bit float patterns with every NaN replaced by one quiet NaN: where
    the reference's arithmetic yields NaN (0/0 in the unbiased pass's W for a
    reservoir without a sample), the GPU writes 0x7fffffff and the CPU
    0x7fc00000; parity compares NaN with NaN."""
    b = bits.copy()
    nan = ((b & np.uint32(0x7F800000)) == np.uint32(0x7F800000)) & ((b & np.uint32(0x007FFFFF)) != 0)
    b[nan] = QNAN
    return b


def res_bits(a: np.ndarray) -> np.ndarray:
    """Reservoirs as raw 32-bit words without the padding lanes (float words
    with canonical NaN)."""
    w = a.view(np.uint32).reshape(-1, 16)[:, :13].copy()
    w[:, _FLOAT_WORDS] = canonical_nan(w[:, _FLOAT_WORDS])
    return w


def image_bits(img: np.ndarray) -> np.ndarray:
    """Image floats as 32-bit patterns with canonical NaN."""
    return canonical_nan(np.ascontiguousarray(img, np.float32).view(np.uint32))


def mismatch(a: np.ndarray, b: np.ndarray, mask=None) -> int:
    x, y = res_bits(a), res_bits(b)
    if mask is not None:
        x, y = x[mask], y[mask]
    return int(np.count_nonzero(np.any(x != y, axis=1)))


def crop_mask(w, h, crop):
    m = np.zeros((h, w), bool)
    x0, y0, cw, ch = crop
    m[y0:y0 + ch, x0:x0 + cw] = True
    return m.reshape(-1)


def oracle_frame(scene, frame_index, g_cur, g_prev, prev_res, crop=None):
    """The reference's pass sequence for one frame on the oracle.  Returns
    (reservoirs of every stage, image)."""
    n = scene.width * scene.height
    u = scene.uniforms(frame_index)
    stages = []
    r = new_res(n)
    ob.initial_temporal(scene, g_cur, g_prev, prev_res, r, u, crop=crop)
    stages.append(r.copy())
    if scene.unbiased:
        for k in range(scene.spatial_passes):
            o = new_res(n)
            ob.spatial_unbiased(scene, g_cur, r, o, u, scene.neighbors, k, crop=crop)
            r = o
            stages.append(r.copy())
    else:
        for j in range(scene.spatial_passes):
            o = new_res(n)
            ob.spatial_biased(scene, g_cur, r, o, u, 2 * j, crop=crop)
            o2 = new_res(n)
            ob.spatial_biased(scene, g_cur, o, o2, u, 2 * j + 1, crop=crop)
            r = o2
            stages.append(r.copy())
    img = np.zeros((scene.height, scene.width, 4), np.float32)
    ob.shade(scene, g_cur, r, scene.lighting_uniforms(frame_index), img, crop=crop)
    return stages, img


def mlp_params(count, clusters, seed, scale_w4=0.3):
    """Seeded parameters of the learned proposal's network (packed layout:
    W1 16x64 with rows 9..15 zero, b1, W2, b2, W3, b3, W4 64xC, b4)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(count, np.float32)
    o = 0
    for rows, cols, used in ((16, 64, 9), (64, 64, 64), (64, 64, 64)):
        w = rng.uniform(-1, 1, (rows, cols)) * np.sqrt(6.0 / used)
        w[used:] = 0.0
        p[o:o + rows * cols] = w.ravel()
        o += rows * cols
        p[o:o + cols] = rng.uniform(-0.1, 0.1, cols)
        o += cols
    p[o:o + 64 * clusters] = rng.uniform(-scale_w4, scale_w4, 64 * clusters)
    o += 64 * clusters
    p[o:o + clusters] = rng.uniform(-1, 1, clusters)
    o += clusters
    assert o == count
    return p
