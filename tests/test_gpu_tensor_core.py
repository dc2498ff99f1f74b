"""The tcgen05 tensor-core GEMM (rg_gemm_bf16) against float64 products of
the same bf16-rounded operands.  FP32 accumulation in tensor memory differs
from the float64 sum only by accumulation rounding: the bar is a relative
error of 2e-5 of the row x column magnitude sum."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16(x: np.ndarray) -> np.ndarray:
    import torch
    return torch.from_numpy(np.ascontiguousarray(x, np.float32)).to(torch.bfloat16).to(torch.float32).numpy()


def _gemm(ctx, restir_lib, cuda, a, a_rs, a_ks, m, b, b_rs, b_ks, n, k, d, accumulate=0, alpha=1.0, splits=1):
    from restir_gb300 import _lib
    rc = restir_lib.rg_gemm_bf16(ctx._h, a.data_ptr(), 1 if a.dtype == cuda.float32 else 0, a_rs, a_ks, m,
                                 b.data_ptr(), 1 if b.dtype == cuda.float32 else 0, b_rs, b_ks, n, k, d.data_ptr(),
                                 d.shape[1], accumulate, alpha, splits, None)
    assert rc == 0, restir_lib.rg_last_error()
    cuda.cuda.synchronize()


def _check(got, ref, a_abs, b_abs):
    bound = 2e-5 * (a_abs @ b_abs.T) + 1e-30
    err = np.abs(got - ref)
    assert np.all(err <= bound), f"max err {err.max()}, max rel {(err / bound).max()}"


@pytest.mark.parametrize("m,n,k", [(300, 200, 96), (128, 256, 64), (129, 64, 200), (50, 33, 17)])
def test_gemm_row_major(ctx, restir_lib, cuda, m, n, k):
    rng = np.random.default_rng(m * 1000 + n)
    a = rng.normal(size=(m, k)).astype(np.float32)
    b = rng.normal(size=(n, k)).astype(np.float32)
    ta, tb = cuda.from_numpy(a).cuda(), cuda.from_numpy(b).cuda()
    d = cuda.zeros((m, n), dtype=cuda.float32, device="cuda")
    _gemm(ctx, restir_lib, cuda, ta, k, 1, m, tb, k, 1, n, k, d)
    ab, bb = _bf16(a).astype(np.float64), _bf16(b).astype(np.float64)
    _check(d.cpu().numpy(), ab @ bb.T, np.abs(ab), np.abs(bb))


def test_gemm_bf16_sources_and_alpha(ctx, restir_lib, cuda):
    rng = np.random.default_rng(7)
    m, n, k = 256, 300, 128
    a = cuda.from_numpy(rng.normal(size=(m, k)).astype(np.float32)).cuda().to(cuda.bfloat16)
    b = cuda.from_numpy(rng.normal(size=(n, k)).astype(np.float32)).cuda().to(cuda.bfloat16)
    d = cuda.zeros((m, n), dtype=cuda.float32, device="cuda")
    _gemm(ctx, restir_lib, cuda, a, k, 1, m, b, k, 1, n, k, d, alpha=0.5)
    ab, bb = a.float().cpu().numpy().astype(np.float64), b.float().cpu().numpy().astype(np.float64)
    _check(d.cpu().numpy(), 0.5 * ab @ bb.T, 0.5 * np.abs(ab), np.abs(bb))


def test_gemm_transposed_split_k_accumulate(ctx, restir_lib, cuda):
    """dW = h^T . dz over a batch: both operands read transposed, K split over
    4 CTAs with an atomic epilogue, accumulated onto an existing D."""
    rng = np.random.default_rng(11)
    batch, f, c = 1000, 64, 130
    h = rng.normal(size=(batch, f)).astype(np.float32)
    z = rng.normal(size=(batch, c)).astype(np.float32)
    d0 = rng.normal(size=(f, c)).astype(np.float32)
    th, tz = cuda.from_numpy(h).cuda(), cuda.from_numpy(z).cuda()
    d = cuda.from_numpy(d0.copy()).cuda()
    _gemm(ctx, restir_lib, cuda, th, 1, f, f, tz, 1, c, c, batch, d, accumulate=1, splits=4)
    hb, zb = _bf16(h).astype(np.float64), _bf16(z).astype(np.float64)
    ref = d0 + hb.T @ zb
    bound = 2e-5 * (np.abs(hb).T @ np.abs(zb)) + 1e-5 * np.abs(d0) + 1e-6
    assert np.all(np.abs(d.cpu().numpy() - ref) <= bound)
    assert ctx.stats().mma_timeouts == 0
