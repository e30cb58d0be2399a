"""The device scene generator (lfrv_synth_scene_dev) against the host one (lfrv_synth_scene): same tracing code in
double precision; the device's exp, log and cos may differ from the host library's in the last bit, so the final
floats agree except in rare pixels, and there only by a float rounding."""
import numpy as np
import pytest

import lfrv

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("preset,kw", [(1, dict(w=96, h=80)),
                                       (2, dict(w=64, h=64, nbumps=20, bump_amp=0.1, bump_sigma_px=30.0)),
                                       (1, dict(w=64, h=64, grid=9, seed=7, nbumps=5, bump_amp=0.1,
                                                bump_sigma_px=10.0))])
def test_device_scene_matches_host(preset, kw):
    import torch

    p = lfrv.scene_params(preset, **kw)
    sc = lfrv.synth_scene(p)
    V = sc.views.shape[0]
    H, W = sc.gt.shape[1:]
    dv = torch.zeros((V, 3, p.h, p.w), device="cuda")
    dd = torch.zeros_like(dv)
    dg = torch.zeros((3, H, W), device="cuda")
    with lfrv.Context(0) as ctx:
        torch.cuda.synchronize()
        cams, target = ctx.synth_scene_dev(p, dv.data_ptr(), dd.data_ptr(), dg.data_ptr())
        torch.cuda.synchronize()
    for got, want in ((dv.cpu().numpy(), sc.views), (dd.cpu().numpy(), sc.depth), (dg.cpu().numpy(), sc.gt)):
        diff = np.abs(got - want)
        assert np.max(diff / np.maximum(np.abs(want), 1.0)) < 1e-6
        assert np.mean(diff > 0) < 1e-3
    for a, b in zip(cams + [target], sc.cams + [sc.target]):
        assert list(a.K) == list(b.K) and list(a.t) == list(b.t) and a.width == b.width
