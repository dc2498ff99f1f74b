"""What the trained proposal gains over the plain one: the same unbiased
per-frame estimator (RIS + visibility reuse + final RIS weight) with the
learned candidates, trained online on the frames' own final reservoirs,
reaches a lower RMSE against the FP64 judge than the alias-table proposal
after the same number of frames (config 2's scene at 320x180, 4096 lights in
256 k-means clusters, 64 frames, 32x32 crop).  Both estimators are unbiased,
so the gain is variance: the network learns which clusters are bright and
unoccluded at each pixel."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu


def test_trained_proposal_lowers_rmse(restir_lib, oracle_lib, cuda):
    import learned_rmse  # makes its own context
    r = learned_rmse.run(width=320, height=180, frames=64, clusters=256, n_tris=20_000, n_lights=4096, crop_size=32,
                         lr=1e-2, steps_per_frame=4, batch=16384, log=lambda *a: None)
    assert r["mma_timeouts"] == 0
    assert r["rmse_ratio_at_equal_frames"] < 0.9, r
    assert r["learned"]["loss_every"][-1] < r["learned"]["loss_every"][0]
