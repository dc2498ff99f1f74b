"""Generates the FP64 judge's estimates for the benchmarked frames' crops.

The judge (oracle `or_brute_force_fp64`) sums every point light at every
pixel in double precision with an exact double-precision shadow test; on
config 3 (1,048,576 lights, 1,048,588 triangles) that is about two billion
shadow rays for one 64x64 crop, far too slow for a test run, so its result is
computed once here and committed:

  judge_config3.npz  config 3, frame index 15 (the last of its 16-frame
                     camera path), the 64x64 crop centred in the 1920x1080
                     frame (x 928..991, y 508..571);
  judge_config2.npz  config 2, frame index 7 (the last of its 8 frames), the
                     same centred crop.

Each file holds the judge's linear RGB (float64, crop rows x cols x 3), the
crop, the frame index, and a SHA-256 of every G-buffer plane over the crop,
so a consumer can check that its G-buffer is the one that was judged.  The
G-buffer comes from the primary-ray tracer of the oracle when it is built
with one (`or_trace_gbuffer`), else from the library's CPU tracer; both
produce identical planes (tests check this).

Run from the repository root:  python tests/golden/make_judge.py [config2|config3 ...]
"""
from __future__ import annotations

import hashlib
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
for p in (ROOT / "oracle", ROOT / "restir-vulkan_gb300"):
    sys.path.insert(0, str(p))

import oracle_binding as ob  # noqa: E402

OUT = Path(__file__).resolve().parent
JUDGED = {"config3": 15, "config2": 7}   # frame index judged per configuration
CROP = (928, 508, 64, 64)                # centred in 1920 x 1080


def crop_digest(g: dict, crop) -> dict:
    x0, y0, cw, ch = crop
    return {k: hashlib.sha256(np.ascontiguousarray(v[y0:y0 + ch, x0:x0 + cw]).tobytes()).hexdigest()
            for k, v in sorted(g.items())}


def gbuffer(scene, frame: int) -> dict:
    if hasattr(ob, "trace_gbuffer") and ob.has_gbuffer_tracer():
        return ob.trace_gbuffer(scene, frame)
    from restir_gb300 import scenes
    return scenes.trace_gbuffer_host(scene, frame)


def judge(name: str) -> Path:
    from restir_gb300 import scenes
    frame = JUDGED[name]
    s = scenes.CONFIGS[name]()
    g = gbuffer(s, frame)
    t0 = time.perf_counter()
    rgb = ob.brute_force(s, g, s.cameras[frame].position, crop=CROP)
    secs = time.perf_counter() - t0
    dig = crop_digest(g, CROP)
    out = OUT / f"judge_{name}.npz"
    np.savez_compressed(out, rgb=rgb, crop=np.array(CROP, np.int32), frame=np.int32(frame),
                        digest_keys=np.array(list(dig.keys())), digest_values=np.array(list(dig.values())),
                        seconds=np.float64(secs), threads=np.int32(ob.oracle().or_max_threads()))
    print(f"{out.name}: {name} frame {frame} crop {CROP}, {secs:.0f} s on {ob.oracle().or_max_threads()} threads, "
          f"mean {rgb.mean(axis=(0, 1))}", flush=True)
    return out


if __name__ == "__main__":
    for name in (sys.argv[1:] or ["config2", "config3"]):
        judge(name)
