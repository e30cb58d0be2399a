"""lfrv_render_views_dev: many targets per call; IBR_gradient jobs share one persistent CG launch.

Each job of a batch must give what the same job gives alone through lfrv_render_view_dev. Batched CG sums the
dot products over a different block partition, so outputs agree to float rounding rather than bit for bit,
and with the same iteration counts.
"""
import numpy as np
import pytest

import lfrv
from scenes import color_config, gradient_config, scene

pytestmark = pytest.mark.gpu


def _job(torch, sc, cfg, algorithm):
    H, W = cfg.h * cfg.dsf, cfg.w * cfg.dsf
    return dict(cfg=cfg, algorithm=algorithm, views=torch.from_numpy(sc.views).cuda(),
                depth=torch.from_numpy(sc.depth).cuda(), out=torch.zeros((3, H, W), device="cuda"),
                cams=sc.cams, target=sc.target)


def test_batch_matches_single_targets():
    import torch

    specs = [(2, 32, 1, {}), (1, 48, 1, {}), (2, 24, 0, dict(niter=5)), (1, 40, 1, dict(faithful=1)),
             (2, 40, 1, dict(cg_gap_tol=1e-6)), (1, 48, 0, dict(faithful=0, niter=60, cg_gap_tol=1e-4)),
             (2, 32, 0, dict(faithful=0, niter=6, cg_gap_tol=0.0)), (2, 512, 1, {})]
    # the 1024^2 job has more 64 x 16 tiles than the batched CG has resident blocks: it runs the single-target CG
    jobs = []
    for preset, w, alg, kw in specs:
        sc = scene(preset, w)
        cfg = (gradient_config(sc, **kw) if alg == 1 else color_config(sc, **kw))
        jobs.append(_job(torch, sc, cfg, alg))
    with lfrv.Context(0) as ctx:
        torch.cuda.synchronize()
        stats = ctx.render_views_dev([dict(cfg=j["cfg"], algorithm=j["algorithm"], d_views=j["views"].data_ptr(),
                                           d_depth=j["depth"].data_ptr(), cams=j["cams"], target=j["target"],
                                           d_out=j["out"].data_ptr()) for j in jobs])
        torch.cuda.synchronize()
        for j, st in zip(jobs, stats):
            single = torch.zeros_like(j["out"])
            st1 = ctx.render_view_dev(j["cfg"], j["algorithm"], j["views"].data_ptr(), j["depth"].data_ptr(),
                                      j["cams"], j["target"], single.data_ptr())
            torch.cuda.synchronize()
            got, want = j["out"].cpu().numpy(), single.cpu().numpy()
            if j["algorithm"] == 1 and not j["cfg"].faithful:
                assert st.outer_iterations == st1.outer_iterations
                assert st.hole_fill_iterations == st1.hole_fill_iterations
                assert abs(st.gap - st1.gap) <= 1e-6 * max(st1.gap, 1e-12) + 1e-9
                assert np.max(np.abs(got - want)) < 1e-5
            else:
                np.testing.assert_array_equal(got, want)


def test_batch_jobs_match_fp64_oracle():
    """Every job of a batch (IBR_gradient with the batched CG, IBR_color run in the same call) against the FP64 CPU
    oracle on the warps the GPU computed, at a fixed iteration count: 1e-4 max relative error per pixel (floor
    1e-2), and the batched CG's energy trace against the oracle's to 1e-4 relative."""
    import torch

    import pyoracle
    from scenes import rel_err

    specs = [(2, 32, 1, dict(cg_gap_tol=0.0, cg_max_iter=12)), (1, 48, 1, dict(cg_gap_tol=0.0, cg_max_iter=9)),
             (2, 24, 0, dict(niter=5)), (1, 40, 1, dict(cg_gap_tol=0.0, cg_max_iter=15)),
             (1, 48, 0, dict(faithful=0, niter=5, cg_gap_tol=0.0))]
    jobs, scenes = [], []
    for preset, w, alg, kw in specs:
        sc = scene(preset, w)
        cfg = (gradient_config(sc, **kw) if alg == 1 else color_config(sc, **kw))
        jobs.append(_job(torch, sc, cfg, alg))
        scenes.append(sc)
    with lfrv.Context(0) as ctx:
        torch.cuda.synchronize()
        stats = ctx.render_views_dev([dict(cfg=j["cfg"], algorithm=j["algorithm"], d_views=j["views"].data_ptr(),
                                           d_depth=j["depth"].data_ptr(), cams=j["cams"], target=j["target"],
                                           d_out=j["out"].data_ptr()) for j in jobs], trace=32)
        torch.cuda.synchronize()
        for j, st, sc in zip(jobs, stats, scenes):
            tau, dpart, _ = ctx.warp(sc.depth, sc.cams, sc.target)
            solve = pyoracle.ibr_gradient if j["algorithm"] == 1 else pyoracle.ibr_color
            ref, rst = solve(j["cfg"], sc.views, tau, dpart, prec=0, trace=32)
            assert st.outer_iterations == rst.outer_iterations
            assert rel_err(j["out"].cpu().numpy(), ref) <= 1e-4
            tr, rtr = st.trace(), rst.trace()
            # one entry per iteration; the corrected IBR_color trace also holds the starting point's energy
            extra = 1 if (j["algorithm"] == 0 and not j["cfg"].faithful) else 0
            assert len(tr) == len(rtr) == st.outer_iterations + extra
            assert np.max(np.abs(tr - rtr) / np.abs(rtr)) <= 1e-4


def test_host_buffer_batch_equals_device_batch():
    """lfrv_render_views (host buffers, shared inputs uploaded once) gives lfrv_render_views_dev's outputs bit for
    bit; two targets share one light field."""
    import copy

    import torch

    sc = scene(2, 32)
    cfg = gradient_config(sc, cg_gap_tol=1e-6)
    t2 = copy.copy(sc.target)
    t2.t[0] += 0.01
    H, W = cfg.h * cfg.dsf, cfg.w * cfg.dsf
    views = np.ascontiguousarray(sc.views)
    depth = np.ascontiguousarray(sc.depth)
    outs = [np.zeros((3, H, W), np.float32) for _ in range(2)]
    dv, dd = torch.from_numpy(views).cuda(), torch.from_numpy(depth).cuda()
    douts = [torch.zeros((3, H, W), device="cuda") for _ in range(2)]
    with lfrv.Context(0) as ctx:
        st_h = ctx.render_views([dict(cfg=cfg, algorithm=1, d_views=views.ctypes.data, d_depth=depth.ctypes.data,
                                      cams=sc.cams, target=t, d_out=o.ctypes.data) for t, o in zip((sc.target, t2), outs)])
        torch.cuda.synchronize()
        st_d = ctx.render_views_dev([dict(cfg=cfg, algorithm=1, d_views=dv.data_ptr(), d_depth=dd.data_ptr(),
                                          cams=sc.cams, target=t, d_out=o.data_ptr())
                                     for t, o in zip((sc.target, t2), douts)])
        torch.cuda.synchronize()
    for o, d, a, b in zip(outs, douts, st_h, st_d):
        np.testing.assert_array_equal(o, d.cpu().numpy())
        assert a.outer_iterations == b.outer_iterations
    assert not np.array_equal(outs[0], outs[1])


def test_host_buffer_batch_pinned_outputs():
    """Pinned host outputs take the early download (each IBR_gradient job's output leaves for the host as soon as its
    CG is done, while the next jobs run) and the colour views upload while the warp stage runs: the outputs equal
    lfrv_render_views_dev's bit for bit, with a 1024^2 job on the single-target CG, a job with a pageable output and
    a corrected IBR_color job (downloaded at the end) in the same call."""
    import torch

    specs = [(2, 32, 1, {}), (2, 512, 1, {}), (1, 48, 1, {}), (1, 48, 0, dict(faithful=0, niter=60, cg_gap_tol=1e-4))]
    jobs = []
    for preset, w, alg, kw in specs:
        sc = scene(preset, w)
        cfg = gradient_config(sc, **kw) if alg == 1 else color_config(sc, **kw)
        H, W = cfg.h * cfg.dsf, cfg.w * cfg.dsf
        jobs.append(dict(sc=sc, cfg=cfg, alg=alg, views=np.ascontiguousarray(sc.views),
                         depth=np.ascontiguousarray(sc.depth), dout=torch.zeros((3, H, W), device="cuda"),
                         dv=torch.from_numpy(sc.views).cuda(), dd=torch.from_numpy(sc.depth).cuda()))
    pinned = [True, True, False, True]
    for j, pin in zip(jobs, pinned):
        H, W = j["cfg"].h * j["cfg"].dsf, j["cfg"].w * j["cfg"].dsf
        j["hout"] = (torch.zeros((3, H, W)).pin_memory() if pin else torch.zeros((3, H, W)))
    with lfrv.Context(0) as ctx:
        for _ in range(2):  # the second call reuses the pool and the copy stream
            for j in jobs:
                j["hout"].fill_(-1.0)
            st_h = ctx.render_views([dict(cfg=j["cfg"], algorithm=j["alg"], d_views=j["views"].ctypes.data,
                                          d_depth=j["depth"].ctypes.data, cams=j["sc"].cams, target=j["sc"].target,
                                          d_out=j["hout"].data_ptr()) for j in jobs])
        torch.cuda.synchronize()
        st_d = ctx.render_views_dev([dict(cfg=j["cfg"], algorithm=j["alg"], d_views=j["dv"].data_ptr(),
                                          d_depth=j["dd"].data_ptr(), cams=j["sc"].cams, target=j["sc"].target,
                                          d_out=j["dout"].data_ptr()) for j in jobs])
        torch.cuda.synchronize()
    for j, a, b in zip(jobs, st_h, st_d):
        np.testing.assert_array_equal(j["hout"].numpy(), j["dout"].cpu().numpy())
        assert a.outer_iterations == b.outer_iterations


def test_batches_of_both_lane_counts_in_one_context():
    """A batch with a target of 2^21 pixels or more prepares its jobs on two lanes, a batch of small targets on four:
    alternating them in one context gives each job what it gives alone, with the same statistics."""
    import torch

    big = scene(1, 1456)
    small = [scene(2, 32), scene(1, 48)]
    with lfrv.Context(0) as ctx:
        for specs in ([big, small[0]], small, [big]):
            jobs = [_job(torch, sc, gradient_config(sc), 1) for sc in specs]
            torch.cuda.synchronize()
            stats = ctx.render_views_dev([dict(cfg=j["cfg"], algorithm=1, d_views=j["views"].data_ptr(),
                                               d_depth=j["depth"].data_ptr(), cams=j["cams"], target=j["target"],
                                               d_out=j["out"].data_ptr()) for j in jobs])
            torch.cuda.synchronize()
            for j, st in zip(jobs, stats):
                single = torch.zeros_like(j["out"])
                st1 = ctx.render_view_dev(j["cfg"], 1, j["views"].data_ptr(), j["depth"].data_ptr(), j["cams"],
                                          j["target"], single.data_ptr())
                torch.cuda.synchronize()
                assert st.outer_iterations == st1.outer_iterations
                assert st.hole_fill_iterations == st1.hole_fill_iterations
                assert np.max(np.abs(j["out"].cpu().numpy() - single.cpu().numpy())) < 1e-5
