"""lfrv_render_view / lfrv_render_view_dev: the one-call depth-to-view pipeline (warp stage + solve).

The host-buffer call uploads its inputs on a second stream in view chunks that overlap the warp stage;
its result must equal the device-pointer call's bit for bit, and both must equal the warp and the solve
composed from separate calls (lfrv_warp then lfrv_ibr_color / lfrv_ibr_gradient).
"""
import numpy as np
import pytest

import lfrv
from scenes import color_config, gradient_config, scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = lfrv.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("algorithm,preset,w,views", [(1, 2, 32, None), (0, 1, 48, None), (1, 1, 40, 5)])
def test_render_view_matches_composed_calls(ctx, algorithm, preset, w, views):
    import torch

    sc = scene(preset, w)
    V = sc.views.shape[0] if views is None else views  # 5 views: chunks of unequal size
    imgs, depth, cams = sc.views[:V].copy(), sc.depth[:V].copy(), sc.cams[:V]
    cfg = (gradient_config(sc, cg_gap_tol=1e-6) if algorithm == 1 else color_config(sc, niter=6))
    cfg.nviews = V
    out_host, st = ctx.render_view(cfg, algorithm, imgs, depth, cams, sc.target)
    assert st.kernel_launches > 0

    d_views = torch.from_numpy(imgs).cuda()
    d_depth = torch.from_numpy(depth).cuda()
    d_out = torch.empty(out_host.shape, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ctx.render_view_dev(cfg, algorithm, d_views.data_ptr(), d_depth.data_ptr(), cams, sc.target, d_out.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out_host, d_out.cpu().numpy())

    tau, dpart, _ = ctx.warp(depth, cams, sc.target)
    solve = ctx.ibr_gradient if algorithm == 1 else ctx.ibr_color
    want, _ = solve(cfg, imgs, tau, dpart)
    np.testing.assert_array_equal(out_host, want)


def test_render_view_repeated_calls_are_identical(ctx):
    sc = scene(2, 32)
    cfg = gradient_config(sc, cg_gap_tol=1e-6)
    a, _ = ctx.render_view(cfg, 1, sc.views, sc.depth, sc.cams, sc.target)
    b, _ = ctx.render_view(cfg, 1, sc.views, sc.depth, sc.cams, sc.target)
    np.testing.assert_array_equal(a, b)
