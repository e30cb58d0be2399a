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
             (2, 40, 1, dict(cg_gap_tol=1e-6))]
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
