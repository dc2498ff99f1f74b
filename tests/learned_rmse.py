"""RMSE against the FP64 judge versus GPU time: the learned light-cluster
proposal against the plain alias-table proposal.

Both arms run the same per-frame estimator on a static camera: initial RIS
(32 candidates) with visibility reuse and the final RIS weight
(RG_FLAG_FINAL_RIS_WEIGHT, so each frame is an unbiased estimate), then
shading; the image estimate is the running mean of the frames.  The learned
arm also runs the proposal's inference before RIS and its Adam steps on the
frame's final reservoirs after shading, all inside its timed region.  GPU time
is measured with CUDA events around each frame's work.  The FP64 brute-force
judge (every light, exact visibility) gives the reference on a crop.

Result: each arm's RMSE after every frame and its cumulative GPU time; "GPU
time to equal RMSE" is the learned arm's time to reach the plain arm's final
RMSE, as a fraction of the plain arm's time.

Run as a script to produce the record at full size:
    python tests/learned_rmse.py --width 1920 --height 1080 --frames 64
(tests/test_gpu_learned_gain.py runs a small case.)  Test infrastructure: it
uses the oracle's judge, it is not the product.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT / "restir-vulkan_gb300", ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def _arm(ctx, s, dg, res, image, crop, judge, frames, learned, steps_per_frame, candidates=32, cam=0, mask=None):
    import torch
    from restir_gb300 import _lib
    x0, y0, cw, ch = crop
    acc = torch.zeros((ch, cw, 3), dtype=torch.float64, device="cuda")
    jt = torch.from_numpy(judge).cuda()
    mt = torch.from_numpy(np.ones(judge.shape[:2], bool) if mask is None else mask).cuda()
    lu = s.lighting_uniforms(cam)
    stream = torch.cuda.current_stream()
    cum_ms, rmse, loss = [], [], []
    total = 0.0
    for f in range(1, frames + 1):
        u = s.uniforms(cam)
        u.frame = f
        u.flags = _lib.RG_FLAG_VISIBILITY_REUSE | _lib.RG_FLAG_FINAL_RIS_WEIGHT
        if learned:
            u.flags |= _lib.RG_FLAG_LEARNED_PROPOSAL
            u.initial_light_sample_count = candidates
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        if learned:
            ctx.proposal_infer(dg, u, stream)
        ctx.initial_temporal(dg, None, None, res, u, stream)
        ctx.shade(dg, res, lu, image, stream)
        if learned:
            for k in range(steps_per_frame):
                ut = s.uniforms(cam)
                ut.frame = f * steps_per_frame + k
                ctx.proposal_train(dg, ut, res.data_ptr(), stream)
        e1.record(stream)
        torch.cuda.synchronize()
        total += e0.elapsed_time(e1)
        acc += image[y0:y0 + ch, x0:x0 + cw, :3].double()
        err = acc / f - jt
        cum_ms.append(total)
        rmse.append(float(torch.sqrt((err[mt] ** 2).mean())))
        if learned:
            loss.append(ctx.proposal_last_loss()[0])
    return cum_ms, rmse, loss


def run(width=1920, height=1080, frames=64, clusters=4096, n_tris=100_000, n_lights=65_536, crop_size=64,
        lr=3e-3, steps_per_frame=1, batch=65_536, kmeans_iters=8, seed=4, log=print, learned_candidates=32,
        zero_w4=False, scene=None, cam=0, judge=None, crop=None, cluster_of=None, judge_check=None, mask=None):
    """scene (default: config 2's at width x height), the static camera index
    cam, and optionally a precomputed judge of that view on crop (with
    judge_check(host G-buffer) raising if it was judged on other planes) and
    a light clustering (default: k-means); mask selects the crop pixels the
    RMSE is taken over (default: all)."""
    import torch

    from restir_gb300 import scenes
    from restir_gb300.passes import Context, DeviceGBuffer, cluster_lights, reservoirs

    t0 = time.perf_counter()
    s = scene if scene is not None else scenes.config2(width=width, height=height, n_tris=n_tris,
                                                         n_lights=n_lights, frames=1)
    width, height = s.width, s.height
    ctx = Context(0)
    ctx.upload_scene(s)
    dg = DeviceGBuffer(s.width, s.height)
    ctx.trace_gbuffer(s.cameras[cam], dg)
    if judge_check is not None:  # the precomputed judge must be of this G-buffer
        judge_check(dg.to_host())
    if judge is None:
        import oracle_binding as ob
        crop = ((width - crop_size) // 2, (height - crop_size) // 2, crop_size, crop_size)
        judge = ob.brute_force(s, dg.to_host(), s.cameras[cam].basis()[0], crop=crop)
    crop_size = crop[2]
    t_judge = time.perf_counter() - t0
    log(f"scene + judge {t_judge:.1f}s")
    t1 = time.perf_counter()
    if cluster_of is None:
        cluster_of, _ = cluster_lights(s.point_lights, clusters, iterations=kmeans_iters, seed=seed)
    t_kmeans = time.perf_counter() - t1
    n = s.width * s.height
    res = reservoirs(n)
    image = torch.zeros((s.height, s.width, 4), dtype=torch.float32, device="cuda")
    # warm both paths (module load, first-launch attributes), then start fresh
    ctx.create_proposal(cluster_of, clusters, mix=0.9, learning_rate=lr, batch=batch, seed=seed)
    _arm(ctx, s, dg, res, image, crop, judge, 2, True, 1, cam=cam, mask=mask)
    _arm(ctx, s, dg, res, image, crop, judge, 2, False, 1, cam=cam, mask=mask)
    plain_ms, plain_rmse, _ = _arm(ctx, s, dg, res, image, crop, judge, frames, False, 1, cam=cam, mask=mask)
    ctx.create_proposal(cluster_of, clusters, mix=0.9, learning_rate=lr, batch=batch, seed=seed)
    if zero_w4:  # the untrained proposal is then exactly the power-proportional one (plus the mixture)
        params = ctx.proposal_params()
        n123 = 16 * 64 + 64 + 2 * (64 * 64 + 64)
        params[n123:n123 + 64 * clusters] = 0.0
        ctx.set_proposal_params(params)
    lrn_ms, lrn_rmse, loss = _arm(ctx, s, dg, res, image, crop, judge, frames, True, steps_per_frame,
                                  learned_candidates, cam=cam, mask=mask)
    st = ctx.stats()
    ctx.close()
    # the plain arm's final error, taken as its lowest over the last quarter of
    # its frames, so that a late spike of its running mean (heavy-tailed
    # estimates) does not make the target easier to reach
    target = min(plain_rmse[-max(1, frames // 4):])
    hit = next((i for i, r in enumerate(lrn_rmse) if r <= target), None)
    frac = (lrn_ms[hit] / plain_ms[-1]) if hit is not None else None
    judge_mean = float(judge[mask].mean()) if mask is not None else float(judge.mean())
    every = max(1, frames // 16)
    return {
        "workload": f"{s.name} scene {width}x{height}, {len(s.triangles):,} triangles, {len(s.point_lights):,} point "
                    f"lights, {clusters} light clusters, static camera {cam}, {frames} frames",
        "estimator": f"RIS (plain 32, learned {learned_candidates} candidates) + visibility reuse + final RIS weight, "
                     "shaded; running mean of frames",
        "judge": f"FP64 brute force (every light, exact visibility) on a {crop_size}x{crop_size} crop at {crop[:2]}",
        "judge_mean_radiance": judge_mean,
        "plain": {"ms_per_frame": plain_ms[-1] / frames, "final_rmse": plain_rmse[-1], "target_rmse": target,
                  "final_rel_rmse": plain_rmse[-1] / judge_mean, "target_rel_rmse": target / judge_mean,
                  "rmse_every": plain_rmse[::every], "cum_ms_every": plain_ms[::every]},
        "learned": {"ms_per_frame": lrn_ms[-1] / frames, "final_rmse": lrn_rmse[-1],
                    "final_rel_rmse": lrn_rmse[-1] / judge_mean,
                    "rmse_every": lrn_rmse[::every], "cum_ms_every": lrn_ms[::every],
                    "loss_every": loss[::every], "adam_steps_per_frame": steps_per_frame, "learning_rate": lr,
                    "batch": batch, "mix": 0.9},
        "equal_rmse": {"learned_frame": None if hit is None else hit + 1,
                       "learned_ms": None if hit is None else lrn_ms[hit], "plain_ms": plain_ms[-1],
                       "time_fraction": frac},
        "rmse_ratio_at_equal_frames": lrn_rmse[-1] / plain_rmse[-1],
        "kmeans_seconds_host": t_kmeans,
        "mma_timeouts": int(st.mma_timeouts),
    }


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--frames", type=int, default=64)
    ap.add_argument("--clusters", type=int, default=4096)
    ap.add_argument("--lights", type=int, default=65_536)
    ap.add_argument("--tris", type=int, default=100_000)
    ap.add_argument("--crop", type=int, default=64)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--steps-per-frame", type=int, default=1)
    ap.add_argument("--batch", type=int, default=65_536)
    ap.add_argument("--learned-candidates", type=int, default=32, help="RIS candidates of the learned arm")
    ap.add_argument("--zero-w4", action="store_true", help="start the learned arm with W4 = 0")
    ap.add_argument("--out", default=None, help="also write the JSON here")
    a = ap.parse_args(argv)
    r = run(a.width, a.height, a.frames, a.clusters, a.tris, a.lights, a.crop, a.lr, a.steps_per_frame, a.batch,
            log=lambda *x: print(*x, file=sys.stderr, flush=True), learned_candidates=a.learned_candidates,
            zero_w4=a.zero_w4)
    txt = json.dumps(r)
    print(txt, flush=True)
    if a.out:
        Path(a.out).write_text(txt + "\n")


if __name__ == "__main__":
    main()
