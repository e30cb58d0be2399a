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


def test_render_view_dev_graph_replay(ctx):
    """Repeated identical lfrv_render_view_dev calls are captured once and replayed as a CUDA graph: every call
    gives the uncaptured call's result bit for bit and the same statistics, new input contents behind the same
    pointers are picked up, and changed arguments fall back to an uncaptured run."""
    import torch

    sc = scene(2, 32)
    cfg = gradient_config(sc, cg_gap_tol=1e-6, faithful=0)
    d_views = torch.from_numpy(sc.views.copy()).cuda()
    d_depth = torch.from_numpy(sc.depth.copy()).cuda()
    H, W = sc.target.height, sc.target.width
    d_out = torch.empty((3, H, W), dtype=torch.float32, device="cuda")

    def run(c, cams=sc.cams):
        torch.cuda.synchronize()
        st = c.render_view_dev(cfg, 1, d_views.data_ptr(), d_depth.data_ptr(), cams, sc.target, d_out.data_ptr())
        torch.cuda.synchronize()
        return d_out.cpu().numpy().copy(), st

    with lfrv.Context(0) as fresh:
        want, st0 = run(fresh)
    outs = [run(ctx) for _ in range(4)]  # uncaptured, captured + replayed, replayed, replayed
    for out, st in outs:
        np.testing.assert_array_equal(out, want)
        assert st.outer_iterations == st0.outer_iterations
        assert st.hole_fill_iterations == st0.hole_fill_iterations
        assert st.gap == st0.gap
        assert st.kernel_launches == st0.kernel_launches

    # new view contents behind the same pointers: the replay reads them
    d_views.mul_(0.5)
    got, _ = run(ctx)
    with lfrv.Context(0) as fresh:
        want2, _ = run(fresh)
    np.testing.assert_array_equal(got, want2)
    assert not np.array_equal(want2, want)

    # different cameras: a new key, run uncaptured
    cams2 = [c for c in sc.cams]
    cams2[0], cams2[1] = cams2[1], cams2[0]
    got3, _ = run(ctx, cams2)
    with lfrv.Context(0) as fresh:
        want3, _ = run(fresh, cams2)
    np.testing.assert_array_equal(got3, want3)


def test_render_view_host_graph_replay(ctx):
    """The host-buffer call from pinned memory replays its captured graph (uploads, solve and download): every
    repeated call returns the uncaptured result bit for bit, and new contents of the same host buffers are used."""
    import torch

    sc = scene(2, 32)
    cfg = gradient_config(sc, cg_gap_tol=1e-6, faithful=0)
    hv = torch.from_numpy(sc.views.copy()).pin_memory()
    hd = torch.from_numpy(sc.depth.copy()).pin_memory()
    H, W = sc.target.height, sc.target.width
    ho = torch.empty((3, H, W), dtype=torch.float32).pin_memory()

    def run(c):
        _, st = c.render_view(cfg, 1, hv.data_ptr(), hd.data_ptr(), sc.cams, sc.target, ho.data_ptr())
        return ho.numpy().copy(), st

    with lfrv.Context(0) as fresh:
        want, st0 = run(fresh)
    for _ in range(4):
        out, st = run(ctx)
        np.testing.assert_array_equal(out, want)
        assert st.outer_iterations == st0.outer_iterations and st.gap == st0.gap
    hv.mul_(0.5)
    got, _ = run(ctx)
    with lfrv.Context(0) as fresh:
        want2, _ = run(fresh)
    np.testing.assert_array_equal(got, want2)
