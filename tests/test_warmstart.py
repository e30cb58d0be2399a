"""The learned warm start: tensor-core convolutions and the network's gradients against the CPU oracle
(oracle/warmstart_oracle.py), training on the GPU, and what the trained network gains over the plain start.

The oracle is pinned by finite differences of its own FP64 loss (the network has no reference counterpart).
GPU convolutions take BF16 operands and accumulate in FP32: against the oracle's FP64 sums of the same BF16
values the error bound is 1e-5 of the sum of absolute products. Whole-network gradients also see BF16 rounding of
intermediate activations and gradients, where a value on a rounding boundary may round the other way. Per layer,
the relative L2 distance of the GPU gradient to the BF16 oracle must stay below max(2e-2, 1.5 s) and to the
FP64 oracle below max(2e-2, 2 s), s = the distance between the BF16 and the FP64 oracle (the rounding noise of
BF16 training itself, up to ~8 % at the 2 x 2 bottleneck of a 16 x 16 image).
"""
from __future__ import annotations

import numpy as np
import pytest

import lfrv
import warmstart_oracle as wo
from scenes import gradient_config, scene


def test_param_count_matches_oracle():
    assert lfrv.warmstart_param_count() == wo.param_count() == 1229315


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(5)
    th = wo.init_params(11).astype(np.float64)
    x = rng.random((1, 16, 16, 48))
    u0 = rng.random((1, 3, 16, 16))
    tg = rng.random((1, 3, 16, 16))
    _, loss, g = wo.forward_backward(th, x, u0, tg, bf16_mode=False)
    idx = list(rng.choice(th.size, 12, replace=False))
    idx += [s[0].start + 5 for s in wo.layer_slices()] + [s[1].start for s in wo.layer_slices()]
    eps = 1e-6
    for i in idx:
        tp, tm = th.copy(), th.copy()
        tp[i] += eps
        tm[i] -= eps
        fd = (wo.forward_backward(tp, x, u0, tg, False)[1] - wo.forward_backward(tm, x, u0, tg, False)[1]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 1e-30], np.float32)
    r = wo.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5
    assert abs(r[4] - 1e-30) < 1e-32


# ------------------------------------------------------------------ GPU
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _bf16_dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda().to(torch.bfloat16).contiguous()


def _f32_dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


CONV_CASES = [
    # Cin, Cout, ks, stride, batch, H, W
    (48, 32, 3, 1, 2, 16, 24),
    (32, 64, 3, 2, 1, 16, 16),
    (64, 128, 3, 2, 2, 24, 16),
    (256, 256, 3, 1, 1, 8, 8),
    (256, 128, 1, 1, 2, 8, 8),
    (32, 16, 3, 1, 1, 24, 16),
    (64, 64, 3, 1, 1, 20, 12),
    (128, 256, 3, 2, 2, 16, 16),
    # rows of 128 pixels: stride-1 3 x 3 forward and data gradient take the resident-tile kernel
    (48, 32, 3, 1, 1, 8, 128),
    (32, 32, 3, 1, 2, 4, 256),
    (64, 64, 3, 1, 1, 6, 128),
    (128, 128, 3, 1, 1, 4, 128),
    (32, 16, 3, 1, 1, 4, 128),
    (16, 32, 3, 1, 1, 2, 128),
    # patches of 128 pixels over several rows (W < 128): the TMA kernel, stride 1 and 2, 3 x 3 and 1 x 1
    (32, 64, 3, 2, 1, 32, 32),
    (64, 128, 3, 2, 1, 64, 32),
    (256, 128, 1, 1, 1, 16, 8),
    (128, 32, 3, 1, 2, 16, 8),
    (16, 32, 3, 1, 1, 32, 4),
]


@pytest.fixture(params=[0, 1, 2], ids=["tma", "tile", "gather"])
def conv_kernel(request):
    lfrv.set_conv_kernel(request.param)
    yield request.param
    lfrv.set_conv_kernel(0)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CONV_CASES)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_conv_matches_oracle(ctx, case, mode, conv_kernel):
    torch = _cuda()
    Cin, Cout, ks, s, B, H, W = case
    if mode == 1 and Cin not in (16, 32, 64, 128, 256):
        pytest.skip("data gradient output width")
    rng = np.random.default_rng(hash(case) % 2 ** 32 + mode)
    taps = ks * ks
    x = wo.bf16(rng.normal(size=(B, H, W, Cin)))
    w = rng.normal(0, 0.2, size=(Cout, taps, Cin)).astype(np.float32)
    wq = wo.bf16(w)
    dy = wo.bf16(rng.normal(size=(B, H // s, W // s, Cout)))
    if mode == 0:
        ref = wo.conv(x, wq, None, ks, s)
        bound = wo.conv(np.abs(x), np.abs(wq), None, ks, s)
        shape = (B, H // s, W // s, Cout)
    elif mode == 1:
        ref = wo.conv_dgrad(dy, wq, (B, H, W, Cin), ks, s)
        bound = wo.conv_dgrad(np.abs(dy), np.abs(wq), (B, H, W, Cin), ks, s)
        shape = (B, H, W, Cin)
    else:
        ref = wo.conv_wgrad(x, dy, ks, s)
        bound = wo.conv_wgrad(np.abs(x), np.abs(dy), ks, s)
        shape = (Cout, taps, Cin)
    dx, ddy, dw = _bf16_dev(torch, x), _bf16_dev(torch, dy), _f32_dev(torch, w)
    out = torch.full(shape, float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ctx.conv_bf16_dev(mode, B, H, W, Cin, Cout, ks, s, dx.data_ptr(), ddy.data_ptr(), dw.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    got = out.cpu().numpy().astype(np.float64).reshape(ref.shape)
    err = np.abs(got - ref)
    assert np.all(np.isfinite(got))
    assert np.all(err <= 1e-5 * bound + 1e-6), float(np.max(err / (bound + 1e-12)))


@pytest.fixture(scope="module")
def net(ctx):
    n = lfrv.WarmStart(ctx, seed=7)
    yield n
    n.close()


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.gpu
@pytest.mark.parametrize("B,H,W", [(2, 16, 16), (1, 24, 32), (1, 8, 128), (1, 32, 64)])
def test_network_gradients_match_oracle(net, B, H, W, conv_kernel):
    torch = _cuda()
    rng = np.random.default_rng(B * 100 + H)
    theta = wo.init_params(3)
    net.set_params(theta)
    assert np.array_equal(net.get_params(), theta)
    x = rng.random((B, H, W, 48))
    x[..., 41:] = 0.0
    u0 = rng.random((B, 3, H, W)).astype(np.float32)
    tg = (u0 + 0.1 * rng.normal(size=u0.shape)).astype(np.float32)
    pred_ref, loss_ref, g_ref = wo.forward_backward(theta.astype(np.float64), x, u0.astype(np.float64),
                                                    tg.astype(np.float64), bf16_mode=True)
    dx, du0, dtg = _bf16_dev(torch, x), _f32_dev(torch, u0), _f32_dev(torch, tg)
    pred = torch.zeros((B, 3, H, W), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    net.forward_dev(B, H, W, dx.data_ptr(), du0.data_ptr(), pred.data_ptr())
    torch.cuda.synchronize()
    assert np.max(np.abs(pred.cpu().numpy() - pred_ref)) < 2e-2 * max(1.0, np.abs(pred_ref - u0).max())
    loss, g = net.gradients_dev(B, H, W, dx.data_ptr(), du0.data_ptr(), dtg.data_ptr())
    assert abs(loss - loss_ref) <= 1e-2 * loss_ref
    # the FP64 truth on the same BF16 input: the oracle's own BF16 spread sets each layer's tolerance
    _, _, g64 = wo.forward_backward(theta.astype(np.float64), wo.bf16(x), u0.astype(np.float64),
                                    tg.astype(np.float64), bf16_mode=False)
    for l, (sw, sb) in enumerate(wo.layer_slices()):
        for part, sl in (("weights", sw), ("bias", sb)):
            spread = _rel_l2(g_ref[sl], g64[sl])
            e_ref, e_64 = _rel_l2(g[sl], g_ref[sl]), _rel_l2(g[sl], g64[sl])
            assert e_ref < max(2e-2, 1.5 * spread), (l, part, e_ref, spread)
            assert e_64 < max(2e-2, 2.0 * spread), (l, part, e_64, spread)


def _features(ctx, torch, seed, w=64):
    """Network input, anchor u0 and the converged plain solution (gap 1e-6) of a seeded 3 x 3 scene."""
    sc = scene(1, w, seed=seed)
    cfg = gradient_config(sc, cg_gap_tol=1e-6, cg_max_iter=500)
    H, W = sc.params.h * sc.params.dsf, sc.params.w * sc.params.dsf
    views, depth = _f32_dev(torch, sc.views), _f32_dev(torch, sc.depth)
    inp = torch.zeros((H, W, 48), dtype=torch.bfloat16, device="cuda")
    u0 = torch.zeros((3, H, W), dtype=torch.float32, device="cuda")
    sol = torch.zeros((3, H, W), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()  # the library works on its own stream
    ctx.warmstart_features_dev(cfg, views.data_ptr(), depth.data_ptr(), sc.cams, sc.target, inp.data_ptr(),
                               u0.data_ptr(), sol.data_ptr())
    torch.cuda.synchronize()
    return sc, views, depth, inp, u0, sol


@pytest.mark.gpu
def test_features_anchor_is_the_plain_start(ctx):
    """u0 from the features call equals the plain solver's start, and its solution the plain solver's output."""
    torch = _cuda()
    sc, views, depth, inp, u0, sol = _features(ctx, torch, seed=41)
    cfg = gradient_config(sc, cg_gap_tol=1e-6, cg_max_iter=500)
    out = torch.zeros_like(sol)
    torch.cuda.synchronize()
    ctx.render_view_dev(cfg, 1, views.data_ptr(), depth.data_ptr(), sc.cams, sc.target, out.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), sol.cpu().numpy())
    x = inp.float().cpu().numpy()
    np.testing.assert_allclose(x[..., 0:3].transpose(2, 0, 1), u0.cpu().numpy(), rtol=1e-2, atol=1e-2)
    assert np.all(x[..., 41:] == 0)
    assert np.all(x[:, -1, 3] == 0) and np.all(x[-1, :, 4] == 0)
    assert np.all(np.abs(x[..., 3:5]) <= 1) and np.all((x[..., 5] == 0) | (x[..., 5] == 1))
    share = x[..., 30:38].sum(-1)
    assert np.all((np.abs(share - 1) < 3e-2) | (share == 0))


@pytest.mark.gpu
def test_untrained_warm_start_keeps_the_solution(ctx, net):
    """Whatever the seed, the anchor keeps the problem: the warm-started solve converges to the plain solution."""
    torch = _cuda()
    net.set_params(wo.init_params(9))
    sc, views, depth, inp, u0, sol = _features(ctx, torch, seed=42)
    cfg = gradient_config(sc, cg_gap_tol=1e-6, cg_max_iter=500)
    out = torch.zeros_like(sol)
    torch.cuda.synchronize()
    st = net.render_view_dev(cfg, views.data_ptr(), depth.data_ptr(), sc.cams, sc.target, out.data_ptr())
    torch.cuda.synchronize()
    assert st.gap <= 1e-6
    assert lfrv.psnr(out.cpu().numpy(), sol.cpu().numpy()) > 50.0


@pytest.mark.gpu
def test_training_gain_over_plain_start(ctx):
    """Train on 48 seeded scenes (1500 Adam steps of 8 images), test on 4 held-out ones: the prediction is at least
    4x closer (mean squared error) to the converged solution than the plain start, and the CG needs fewer
    iterations to the gap 1e-4 from it (the operator lambda I - Delta is well conditioned, so the saving is a
    fraction of the plain solver's few iterations)."""
    torch = _cuda()
    net = lfrv.WarmStart(ctx, seed=1)
    try:
        train = [_features(ctx, torch, seed=100 + i) for i in range(48)]
        test = [_features(ctx, torch, seed=900 + i) for i in range(4)]
        X = torch.stack([t[3] for t in train])
        U0 = torch.stack([t[4] for t in train])
        S = torch.stack([t[5] for t in train])
        H, W = X.shape[1], X.shape[2]
        g = torch.Generator(device="cpu").manual_seed(0)
        losses = []
        for step in range(1500):
            idx = torch.randperm(len(train), generator=g)[:8].cuda()
            xb, ub, sb = X[idx].contiguous(), U0[idx].contiguous(), S[idx].contiguous()
            torch.cuda.synchronize()
            lr = 5e-4
            losses.append(net.train_step_dev(8, H, W, xb.data_ptr(), ub.data_ptr(), sb.data_ptr(), lr))
        assert np.mean(losses[-20:]) < 0.5 * np.mean(losses[:5])
        err_plain = err_warm = 0.0
        it_plain = it_warm = 0
        for sc, views, depth, inp, u0, sol in test:
            pred = torch.zeros_like(u0)
            torch.cuda.synchronize()
            net.forward_dev(1, H, W, inp.data_ptr(), u0.data_ptr(), pred.data_ptr())
            torch.cuda.synchronize()
            s = sol.cpu().numpy()
            err_plain += float(np.mean((u0.cpu().numpy() - s) ** 2))
            err_warm += float(np.mean((pred.cpu().numpy() - s) ** 2))
            cfg = gradient_config(sc, cg_gap_tol=1e-4, cg_max_iter=500)
            a, b = torch.zeros_like(u0), torch.zeros_like(u0)
            torch.cuda.synchronize()
            sp = ctx.render_view_dev(cfg, 1, views.data_ptr(), depth.data_ptr(), sc.cams, sc.target, a.data_ptr())
            sw = net.render_view_dev(cfg, views.data_ptr(), depth.data_ptr(), sc.cams, sc.target, b.data_ptr())
            torch.cuda.synchronize()
            assert sp.gap <= 1e-4 and sw.gap <= 1e-4
            it_plain += sp.outer_iterations
            it_warm += sw.outer_iterations
            assert lfrv.psnr(b.cpu().numpy(), s) > 40.0
        assert err_warm < 0.25 * err_plain, (err_warm, err_plain)
        assert it_warm < it_plain, (it_warm, it_plain)
    finally:
        net.close()


@pytest.mark.gpu
def test_batched_warm_start_matches_single_targets(ctx, net):
    """lfrv_render_views_warm_dev: seeded jobs converge like the one-target warm call; a target that is not a
    multiple of 8 runs unseeded, as in the plain batch; the 1024^2 target fills the GPU and runs the single-target
    CG from its seed."""
    torch = _cuda()
    net.set_params(wo.init_params(4))
    jobs, keep, singles = [], [], []
    for seed, w in ((50, 64), (51, 40), (52, 36), (53, 1024)):
        sc = scene(1, w, seed=seed)
        cfg = gradient_config(sc, cg_gap_tol=1e-6, cg_max_iter=500)
        views, depth = _f32_dev(torch, sc.views), _f32_dev(torch, sc.depth)
        out = torch.zeros((3, w, w), dtype=torch.float32, device="cuda")
        ref = torch.zeros_like(out)
        keep += [views, depth, out, ref, cfg]
        torch.cuda.synchronize()
        if w % 8 == 0:
            st = net.render_view_dev(cfg, views.data_ptr(), depth.data_ptr(), sc.cams, sc.target, ref.data_ptr())
        else:
            st = ctx.render_view_dev(cfg, 1, views.data_ptr(), depth.data_ptr(), sc.cams, sc.target, ref.data_ptr())
        singles.append((ref, st))
        jobs.append(dict(cfg=cfg, algorithm=1, d_views=views.data_ptr(), d_depth=depth.data_ptr(), cams=sc.cams,
                         target=sc.target, d_out=out.data_ptr()))
    torch.cuda.synchronize()
    stats = ctx.render_views_dev(jobs, net)
    torch.cuda.synchronize()
    for k, (ref, st1) in enumerate(singles):
        out = keep[5 * k + 2]
        assert stats[k].gap <= 1e-6 and st1.gap <= 1e-6
        assert lfrv.psnr(out.cpu().numpy(), ref.cpu().numpy()) > 60.0
        assert abs(stats[k].outer_iterations - st1.outer_iterations) <= 1



@pytest.mark.gpu
def test_learned_input_views_match_oracle(ctx):
    """The per-view channels of the network input on a 24-view light field (views past the first 8 end each bucket's
    scan): view v splatted alone equals the FP64 oracle's weighted average of view v on the same warps and weights,
    and its share of the splat weight the oracle's weight sums, to BF16 rounding."""
    import pyoracle

    torch = _cuda()
    sc = scene(2, 32, seed=43)
    cfg = gradient_config(sc, cg_gap_tol=1e-6, cg_max_iter=500)
    H, W = sc.params.h * sc.params.dsf, sc.params.w * sc.params.dsf
    views, depth = _f32_dev(torch, sc.views), _f32_dev(torch, sc.depth)
    inp = torch.zeros((H, W, 48), dtype=torch.bfloat16, device="cuda")
    u0 = torch.zeros((3, H, W), dtype=torch.float32, device="cuda")
    sol = torch.zeros((3, H, W), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ctx.warmstart_features_dev(cfg, views.data_ptr(), depth.data_ptr(), sc.cams, sc.target, inp.data_ptr(),
                               u0.data_ptr(), sol.data_ptr())
    torch.cuda.synchronize()
    x = inp.float().cpu().numpy()
    assert sc.views.shape[0] > 8
    tau, dpart, _ = ctx.warp(sc.depth, sc.cams, sc.target)
    zero = np.zeros((H, W), np.float32)
    _, _, wgt = pyoracle.stage_weights(cfg, sc.views, tau, dpart, np.zeros((3, H, W), np.float32),
                                       np.zeros((H, W), np.uint8), zero, zero, prec=0)
    cfg1 = gradient_config(sc, cg_gap_tol=1e-6, cg_max_iter=500)
    cfg1.nviews = 1
    norms = []
    for v in range(8):
        Uv, nv = pyoracle.stage_initial_image(cfg1, sc.views[v:v + 1], tau[v:v + 1], wgt[v:v + 1], prec=0)
        got = x[..., 6 + 3 * v:9 + 3 * v].transpose(2, 0, 1)
        want = np.where(nv > 0, Uv, 0.0)
        np.testing.assert_allclose(got, want, rtol=8e-3, atol=2e-3)
        norms.append(nv)
    norms = np.array(norms, np.float64)
    total = norms.sum(0)
    share = np.where(total > 0, norms / np.where(total > 0, total, 1), 0.0)
    np.testing.assert_allclose(x[..., 30:38].transpose(2, 0, 1), share, rtol=8e-3, atol=2e-3)
