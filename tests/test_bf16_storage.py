"""BF16 storage of the per-view stacks (cfg.bf16_storage, IBR_gradient): the views arrive in BF16, the view
gradients and weights are stored in BF16, every accumulation stays FP32 and the CG's dot products and energy
FP64. The result is stated against the FP64 oracle (the same solve on the FP32 views): its PSNR to the ground
truth must be within 0.05 dB of the oracle's, and the per-pixel difference bounded by the BF16 rounding of the
inputs (2^-9 relative) carried through the weighted averages.
"""
from __future__ import annotations

import numpy as np
import pytest

import lfrv
import pyoracle
from scenes import gradient_config, warped

pytestmark = pytest.mark.gpu


def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_bf16_storage_rejected_where_unsupported(ctx):
    sc, tau, dpart, _ = warped(1, 32)
    cfg = gradient_config(sc, bf16_storage=1)
    with pytest.raises(lfrv.LfrvError):
        ctx.ibr_gradient(cfg, sc.views, tau, dpart)  # host buffers: FP32 only


@pytest.mark.parametrize("preset,w", [(1, 48), (2, 32)])
@pytest.mark.parametrize("faithful", [0, 1])
def test_bf16_storage_vs_fp64_oracle(ctx, preset, w, faithful):
    torch = _cuda()
    sc, tau, dpart, _ = warped(preset, w)
    cfg32 = gradient_config(sc, faithful=faithful, cg_gap_tol=1e-6)
    ref, _ = pyoracle.ibr_gradient(cfg32, sc.views, tau, dpart, prec=0)
    cfg = gradient_config(sc, faithful=faithful, cg_gap_tol=1e-6, bf16_storage=1)
    H, W = cfg.h * cfg.dsf, cfg.w * cfg.dsf
    views_bf16 = torch.from_numpy(np.ascontiguousarray(sc.views, np.float32)).cuda().to(torch.bfloat16)
    d_tau = torch.from_numpy(np.ascontiguousarray(tau, np.float32)).cuda()
    d_dp = torch.from_numpy(np.ascontiguousarray(dpart, np.float32)).cuda()
    out = torch.zeros((3, H, W), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    st = ctx.solve_dev(1, cfg, views_bf16.data_ptr(), d_tau.data_ptr(), tau.shape[1], d_dp.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.all(np.isfinite(got))
    p_ref = lfrv.psnr(ref.astype(np.float32), sc.gt)
    p_got = lfrv.psnr(got, sc.gt)
    assert abs(p_got - p_ref) <= 0.05, (p_got, p_ref)
    # BF16 inputs (relative rounding 2^-9) through normalised weighted averages and the CG
    assert np.max(np.abs(got - ref)) <= 2e-2
    assert np.mean(np.abs(got - ref)) <= 2e-3
    if not faithful:
        assert st.gap <= 1e-6


def test_bf16_storage_warm_start_runs(ctx):
    """The warm-start path reads the same BF16 stacks (network input from BF16 views and weights)."""
    torch = _cuda()
    from scenes import scene

    sc = scene(1, 64, seed=77)
    cfg = gradient_config(sc, cg_gap_tol=1e-6, bf16_storage=1)
    cfg32 = gradient_config(sc, cg_gap_tol=1e-6)
    views = torch.from_numpy(sc.views).cuda()
    depth = torch.from_numpy(sc.depth).cuda()
    vb = views.to(torch.bfloat16)
    a = torch.zeros((3, 64, 64), dtype=torch.float32, device="cuda")
    b = torch.zeros_like(a)
    net = lfrv.WarmStart(ctx, seed=3)
    try:
        torch.cuda.synchronize()
        ctx.render_view_dev(cfg32, 1, views.data_ptr(), depth.data_ptr(), sc.cams, sc.target, a.data_ptr())
        st = net.render_view_dev(cfg, vb.data_ptr(), depth.data_ptr(), sc.cams, sc.target, b.data_ptr())
        torch.cuda.synchronize()
    finally:
        net.close()
    assert st.gap <= 1e-6
    assert abs(lfrv.psnr(b.cpu().numpy(), sc.gt) - lfrv.psnr(a.cpu().numpy(), sc.gt)) <= 0.05
