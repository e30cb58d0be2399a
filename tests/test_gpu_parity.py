"""GPU parity: every CUDA stage and both solvers against the CPU oracle on the same seeded inputs.

Tolerances (stated per test):
  * stage kernels vs the FP32 mirror of the reference arithmetic: relative 1e-5 (floor 1e-2) -- the only
    differences are float summation order and FMA contraction;
  * full solves vs the FP64 oracle after a fixed iteration count: max relative error per pixel <= 1e-4
    (floor 1e-2 on the denominator), the parity bar of the plain path;
  * warp stage vs the FP64 oracle: the GPU evaluates the projections in float, so tau agrees to 2e-3 px and
    the discrete occlusion / coverage decisions may differ at a small fraction of pixels on depth edges.
"""
import numpy as np
import pytest

import lfrv
import pyoracle
from scenes import color_config, gradient_config, rel_err, scene, warped

pytestmark = pytest.mark.gpu


# ------------------------------------------------------------------ warp stage
@pytest.mark.parametrize("preset,w", [(1, 64), (2, 48)])
def test_warp_vs_oracle(ctx, preset, w):
    sc = scene(preset, w)
    tau, dpart, zb = ctx.warp(sc.depth, sc.cams, sc.target)
    rtau, rdpart, rzb = pyoracle.warp(sc.depth, sc.cams, sc.target)
    # z-buffer: identical coverage almost everywhere, same depth where both cover. Overlapping quads of one
    # surface tie in depth; float and double rasterisation may keep different ones, whose centre depths differ
    # by the surface's depth change across a pixel (the value only feeds the 0.10 occlusion tolerance).
    both = (zb > 0) & (rzb > 0)
    assert np.mean((zb > 0) != (rzb > 0)) < 0.01
    assert np.mean(np.abs(zb[both] - rzb[both]) > 1e-4) < 0.03
    assert np.mean(np.abs(zb[both] - rzb[both]) > 2e-2) < 0.005
    # tau codes
    code = np.where(tau[:, 0] < 0, tau[:, 0], 0)
    rcode = np.where(rtau[:, 0] < 0, rtau[:, 0], 0)
    assert np.mean(code != rcode) < 0.01
    ok = (code == 0) & (rcode == 0)
    assert np.max(np.abs(tau[:, :2][:, :, ][np.stack([ok, ok], 1)] - rtau[:, :2][np.stack([ok, ok], 1)])) < 2e-3
    assert rel_err(tau[:, 2][ok], rtau[:, 2][ok]) < 1e-3
    assert rel_err(dpart, rdpart) < 1e-3


# ------------------------------------------------------------------ IBR_color stages
@pytest.mark.parametrize("preset,w", [(1, 64), (2, 32)])
def test_visibility(ctx, preset, w):
    sc, tau, dpart, _ = warped(preset, w)
    cfg = color_config(sc)
    cov, vis = ctx.stage_visibility(cfg, tau)
    rcov, rvis = pyoracle.stage_visibility(cfg, tau, prec=1)
    assert np.max(np.abs(cov - rcov)) < 1e-5
    ambiguous = np.abs(rcov - 1.0) < 1e-5
    assert np.array_equal(vis[~ambiguous], rvis[~ambiguous])


@pytest.mark.parametrize("preset,w", [(1, 64), (2, 32)])
def test_weights(ctx, preset, w):
    sc, tau, dpart, _ = warped(preset, w)
    cfg = color_config(sc)
    rng = np.random.default_rng(0)
    N = (w * sc.params.dsf) ** 2
    H = W = w * sc.params.dsf
    U = rng.uniform(0, 1, (3, H, W)).astype(np.float32)
    _, vis = pyoracle.stage_visibility(cfg, tau, prec=1)
    gx0 = rng.normal(0, 0.1, (H, W)).astype(np.float32)  # prior content kept where the Sobel does not write
    gy0 = rng.normal(0, 0.1, (H, W)).astype(np.float32)
    gx, gy, wg = ctx.stage_weights(cfg, sc.views, tau, dpart, U, vis, gx0, gy0)
    rgx, rgy, rwg = pyoracle.stage_weights(cfg, sc.views, tau, dpart, U, vis, gx0, gy0, prec=1)
    assert np.max(np.abs(gx - rgx)) < 1e-5 and np.max(np.abs(gy - rgy)) < 1e-5
    # w = 1/(sg^2 + sigma^2) with sg = (A grad) . dpart: on random-noise U the two products of sg cancel by up
    # to ~1e3, so a one-ulp difference in the gathered gradient (FMA contraction) reaches ~2e-4 in w.
    assert rel_err(wg, rwg, floor=1.0) < 5e-4
    assert N > 0


# (dt_alpha, dt_beta, gw_type): intensities only; with the gradient term (vtv_sr_dataterm_gradients)
# unweighted and weighted; the gradient term alone
TERMS = [(1.0, 0.0, 0), (1.0, 0.5, 0), (1.0, 0.5, 1), (0.0, 1.0, 1)]


@pytest.mark.parametrize("preset,w", [(1, 64), (2, 32)])
@pytest.mark.parametrize("alpha,beta,gw", TERMS)
def test_dataterm(ctx, preset, w, alpha, beta, gw):
    sc, tau, dpart, _ = warped(preset, w)
    cfg = color_config(sc, dt_alpha=alpha, dt_beta=beta, gw_type=gw, gradient_step=0.25)
    H = W = w * sc.params.dsf
    rng = np.random.default_rng(1)
    U = rng.uniform(0.2, 0.8, (3, H, W)).astype(np.float32)
    wg = rng.uniform(0.5e4, 1e4, sc.views.shape[0:1] + sc.views.shape[2:]).astype(np.float32)
    G, F = ctx.stage_dataterm(cfg, sc.views, tau, wg, U)
    rG, rF = pyoracle.stage_dataterm(cfg, sc.views, tau, wg, U, prec=1)
    assert np.max(np.abs(G - rG)) < 2e-5 * max(1.0, float(np.abs(rG).max()))
    assert np.max(np.abs(F - rF)) < 1e-5


def test_rof_vs_fp64(ctx):
    rng = np.random.default_rng(2)
    H, W = 40, 56
    F = rng.uniform(0, 1, (3, H, W)).astype(np.float32)
    g = rng.uniform(0.05, 5, (H, W)).astype(np.float32)
    U = F.copy()
    P = rng.normal(0, 0.1, (6, H, W)).astype(np.float32)
    tau = sigma = np.float32(0.3 / np.sqrt(8.0))
    U1, P1 = ctx.stage_rof(25, tau, sigma, 0.05, F, g, U, P)
    rU, rP = pyoracle.stage_rof(25, tau, sigma, 0.05, F, g, U, P, prec=0)
    assert np.max(np.abs(U1 - rU)) < 1e-5
    assert np.max(np.abs(P1 - rP)) < 1e-5


@pytest.mark.parametrize("preset,w", [(1, 64), (2, 32)])
@pytest.mark.parametrize("beta,gw", [(0.0, 0), (0.5, 0), (0.5, 1)])
def test_energy(ctx, preset, w, beta, gw):
    sc, tau, dpart, _ = warped(preset, w)
    cfg = color_config(sc, dt_beta=beta, gw_type=gw)
    H = W = w * sc.params.dsf
    rng = np.random.default_rng(3)
    U = rng.uniform(0.2, 0.8, (3, H, W)).astype(np.float32)
    wg = rng.uniform(0.5e4, 1e4, sc.views.shape[0:1] + sc.views.shape[2:]).astype(np.float32)
    _, vis = pyoracle.stage_visibility(cfg, tau, prec=0)
    e, et, ed = ctx.stage_energy(cfg, sc.views, tau, wg, U, vis)
    re, ret, red = pyoracle.stage_energy(cfg, sc.views, tau, wg, U, vis, prec=0)
    assert abs(et - ret) <= 1e-5 * abs(ret)
    assert abs(ed - red) <= 1e-5 * abs(red)
    assert abs(e - re) <= 1e-5 * abs(re)


@pytest.mark.parametrize("preset,w", [(1, 64), (2, 32)])
def test_regularizer(ctx, preset, w):
    sc, tau, dpart, _ = warped(preset, w)
    cfg = color_config(sc)
    rng = np.random.default_rng(4)
    wg = rng.uniform(0.5e4, 1e4, sc.views.shape[0:1] + sc.views.shape[2:]).astype(np.float32)
    cov, _ = pyoracle.stage_visibility(cfg, tau, prec=1)
    for prior in (None, cov):
        n, g = ctx.stage_regularizer(cfg, tau, wg, prior)
        rn, rg = pyoracle.stage_regularizer(cfg, tau, wg, prior, prec=1)
        assert np.max(np.abs(n - rn)) < 1e-4
        assert rel_err(g, rg, floor=1e-2) < 1e-5


@pytest.mark.parametrize("preset,w", [(1, 64), (2, 32)])
def test_initial_image(ctx, preset, w):
    sc, tau, dpart, _ = warped(preset, w)
    cfg = color_config(sc)
    rng = np.random.default_rng(5)
    wg = rng.uniform(0.5e4, 1e4, sc.views.shape[0:1] + sc.views.shape[2:]).astype(np.float32)
    U, norm = ctx.stage_initial_image(cfg, sc.views, tau, wg)
    rU, rnorm = pyoracle.stage_initial_image(cfg, sc.views, tau, wg, prec=1)
    assert rel_err(norm, rnorm, floor=1.0) < 1e-5
    assert np.max(np.abs(U - rU)) < 1e-5


@pytest.mark.parametrize("faithful", [True, False])
@pytest.mark.parametrize("shape", [(64, 64), (48, 80), (1024, 1024)])
def test_push_pull(ctx, faithful, shape):
    H, W = shape
    rng = np.random.default_rng(6)
    U = rng.uniform(0.1, 0.9, (3, H, W)).astype(np.float32)
    vis = (rng.uniform(0, 1, (H, W)) > 0.3).astype(np.uint8)
    vis[H // 4: H // 2, W // 4: W // 2] = 0  # a large hole
    U[:, vis == 0] = 0.0
    out = ctx.stage_push_pull(U, vis, faithful)
    ref = pyoracle.stage_push_pull(U, vis, faithful, prec=1)
    assert np.max(np.abs(out - ref)) < 2e-6


# ------------------------------------------------------------------ IBR_gradient stages
@pytest.mark.parametrize("preset,w", [(1, 64), (2, 32)])
def test_gradient_visibility(ctx, preset, w):
    sc, tau, _, _ = warped(preset, w)
    cfg = gradient_config(sc)
    assert np.array_equal(ctx.stage_gradient_visibility(cfg, tau), pyoracle.stage_gradient_visibility(cfg, tau, prec=1))


# 868 holes take the single-block shared-memory kernel; 6000 (one region) and about 9000 (scattered, so that many
# neighbours sit in another block's share) the cluster of shared-memory blocks; 38000 the grid-wide persistent one
@pytest.mark.parametrize("case", ["block", "cluster", "cluster_scattered", "grid"])
def test_hole_fill(ctx, case):
    rng = np.random.default_rng(7)
    H, W = {"block": (64, 72), "cluster": (96, 128), "cluster_scattered": (150, 150), "grid": (256, 256)}[case]
    U = rng.uniform(0.1, 0.9, (3, H, W)).astype(np.float32)
    vis = np.ones((H, W), np.uint8)
    if case == "block":
        vis[10:30, 5:40] = 0
        vis[50:64, 60:72] = 0
    elif case == "cluster":
        vis[20:80, 10:110] = 0
    elif case == "cluster_scattered":
        vis[rng.uniform(size=(H, W)) < 0.4] = 0
    else:
        vis[20:220, 10:200] = 0
    U[:, vis == 0] = 0.0
    out, it = ctx.stage_hole_fill(U, vis, 500)
    ref, rit = pyoracle.stage_hole_fill(U, vis, 500, prec=1)
    if case == "grid":
        # the reference sums the stop test's energy sequentially in float over every pixel; the grid-wide kernel
        # sums it in FP64. With 38000 terms the two roundings can put the stop a few iterations apart, near
        # convergence, where an iteration changes the image little
        assert abs(it - rit) <= 3, (it, rit)
        assert np.max(np.abs(out - ref)) < 1e-3, np.max(np.abs(out - ref))
    else:
        assert it == rit
        assert np.max(np.abs(out - ref)) < 1e-5


@pytest.mark.parametrize("preset,w", [(1, 64), (2, 32)])
def test_u_gradient(ctx, preset, w):
    sc, tau, dpart, _ = warped(preset, w)
    cfg = gradient_config(sc)
    rng = np.random.default_rng(8)
    wg = rng.uniform(0.5e4, 1e4, sc.views.shape[0:1] + sc.views.shape[2:]).astype(np.float32)
    gx, gy, m = ctx.stage_u_gradient(cfg, sc.views, tau, wg)
    rgx, rgy, rm = pyoracle.stage_u_gradient(cfg, sc.views, tau, wg, prec=1)
    assert np.max(np.abs(gx - rgx)) < 1e-6 and np.max(np.abs(gy - rgy)) < 1e-6
    assert rel_err(m, rm, floor=1e-2) < 1e-5


@pytest.mark.parametrize("faithful", [True, False])
@pytest.mark.parametrize("H,W", [(48, 64), (37, 53)])  # W % 4 == 0 takes the TMA tile path, 53 the plain one
def test_cg(ctx, faithful, H, W):
    rng = np.random.default_rng(9)
    U = rng.uniform(0, 1, (3, H, W)).astype(np.float32)
    gx = rng.normal(0, 0.05, (H, W)).astype(np.float32)
    gy = rng.normal(0, 0.05, (H, W)).astype(np.float32)
    out, it, gap = ctx.stage_cg(gx, gy, U, faithful, 500, 1e-8)
    ref, rit, rgap = pyoracle.stage_cg(gx, gy, U, faithful, 500, 1e-8, prec=0)
    if faithful:
        assert it == rit == 5
        assert np.max(np.abs(out - ref)) < 1e-4
    else:
        assert abs(it - rit) <= 1
        assert np.max(np.abs(out - ref)) < 1e-4
        assert gap <= 1e-8


# ------------------------------------------------------------------ full solves (fixed iteration counts)
@pytest.mark.parametrize("preset,w,niter", [(1, 48, 12), (2, 24, 8)])
def test_ibr_color_vs_fp64(ctx, preset, w, niter):
    sc, tau, dpart, _ = warped(preset, w)
    cfg = color_config(sc, niter=niter, early_exit=0)
    out, st = ctx.ibr_color(cfg, sc.views, tau, dpart)
    ref, rst = pyoracle.ibr_color(cfg, sc.views, tau, dpart, prec=0)
    assert st.outer_iterations == rst.outer_iterations == niter
    assert rel_err(out, ref) <= 1e-4
    assert abs(st.energy - rst.energy) <= 1e-4 * abs(rst.energy)


@pytest.mark.parametrize("gw", [0, 1])
def test_ibr_color_gradient_term_vs_fp64(ctx, gw):
    sc, tau, dpart, _ = warped(1, 48)
    cfg = color_config(sc, niter=8, early_exit=0, dt_beta=0.5, gw_type=gw, gradient_step=0.25)
    out, st = ctx.ibr_color(cfg, sc.views, tau, dpart)
    ref, rst = pyoracle.ibr_color(cfg, sc.views, tau, dpart, prec=0)
    assert rel_err(out, ref) <= 1e-4
    assert abs(st.energy - rst.energy) <= 1e-4 * abs(rst.energy)


def test_ibr_color_early_exit(ctx):
    sc, tau, dpart, _ = warped(1, 48)
    cfg = color_config(sc, niter=40, nmeta_iter=2, early_exit=1)
    out, st = ctx.ibr_color(cfg, sc.views, tau, dpart)
    ref, rst = pyoracle.ibr_color(cfg, sc.views, tau, dpart, prec=1)
    assert st.outer_iterations == rst.outer_iterations
    assert st.stop_reason == rst.stop_reason
    assert rel_err(out, ref) <= 1e-4


@pytest.mark.parametrize("preset,w,niter", [(1, 48, 6), (2, 24, 4)])
def test_ibr_color_corrected_mode(ctx, preset, w, niter):
    """Corrected IBR_color (the TV_F objective by FISTA + FGP, kernels_tv.cu) against the FP64 oracle after a fixed
    number of outer iterations (gap stop off): 1e-4 max relative error per pixel and per energy-trace entry. The
    certified gap is a difference of nearly equal sums (J_g(u) - <grad u, p> and the box term), so float iterates
    move it by more: 1e-2 relative."""
    sc, tau, dpart, _ = warped(preset, w)
    cfg = color_config(sc, niter=niter, faithful=0, cg_gap_tol=0.0)
    out, st = ctx.ibr_color(cfg, sc.views, tau, dpart, trace=16)
    ref, rst = pyoracle.ibr_color(cfg, sc.views, tau, dpart, prec=0, trace=16)
    assert st.outer_iterations == rst.outer_iterations == niter
    assert rel_err(out, ref) <= 1e-4
    tr, rtr = st.trace(), rst.trace()
    assert len(tr) == len(rtr) == niter + 1
    assert np.max(np.abs(tr - rtr) / np.abs(rtr)) <= 1e-4
    assert abs(st.gap - rst.gap) <= 1e-2 * rst.gap + 1e-7


def test_ibr_color_corrected_certified_gap(ctx):
    """The corrected solve stops at a certified relative gap of 1e-4, and the certificate holds: its energy is
    within gap * E of the FP64 oracle's optimum (solved to a certified 1e-7)."""
    sc, tau, dpart, _ = warped(1, 64)
    cfg = color_config(sc, niter=400, faithful=0, cg_gap_tol=1e-4)
    out, st = ctx.ibr_color(cfg, sc.views, tau, dpart, trace=512)
    assert st.stop_reason == 4 and st.gap <= 1e-4
    ref_cfg = color_config(sc, niter=2000, faithful=0, cg_gap_tol=1e-7)
    _, rst = pyoracle.ibr_color(ref_cfg, sc.views, tau, dpart, prec=0)
    assert rst.gap <= 1e-7
    e_star = rst.energy
    assert st.energy - e_star <= st.gap * st.energy + 1e-6 * e_star
    assert st.energy >= e_star * (1 - 1e-6)
    tr = st.trace()
    assert len(tr) == st.outer_iterations + 1 and tr[-1] == st.energy


@pytest.mark.parametrize("preset,w", [(1, 48), (2, 32)])
@pytest.mark.parametrize("faithful", [0, 1])
def test_ibr_gradient_vs_fp64(ctx, preset, w, faithful):
    sc, tau, dpart, _ = warped(preset, w)
    cfg = gradient_config(sc, faithful=faithful)
    out, st = ctx.ibr_gradient(cfg, sc.views, tau, dpart)
    ref, rst = pyoracle.ibr_gradient(cfg, sc.views, tau, dpart, prec=0)
    assert st.hole_fill_iterations == rst.hole_fill_iterations
    assert abs(st.outer_iterations - rst.outer_iterations) <= 1
    assert rel_err(out, ref) <= 1e-4


def test_solve_is_deterministic(ctx):
    sc, tau, dpart, _ = warped(2, 32)
    cfg = color_config(sc, niter=6)
    a, _ = ctx.ibr_color(cfg, sc.views, tau, dpart)
    b, _ = ctx.ibr_color(cfg, sc.views, tau, dpart)
    assert np.array_equal(a, b)


def test_inverse_map_more_than_64_views(ctx):
    """A 9x9 light field (80 input views, two 64-bit view-mask words per bucket of the inverse footprint map):
    IBR_gradient against the FP64 oracle at a fixed CG iteration count, and IBR_color's data term."""
    import lfrv

    p = lfrv.scene_params(2, w=24, h=24, grid=9, seed=4)
    sc = lfrv.synth_scene(p)
    assert sc.views.shape[0] == 80
    tau, dpart, _ = pyoracle.warp(sc.depth, sc.cams, sc.target)
    cfg = gradient_config(sc, cg_gap_tol=0.0, cg_max_iter=10)
    out, st = ctx.ibr_gradient(cfg, sc.views, tau, dpart)
    ref, rst = pyoracle.ibr_gradient(cfg, sc.views, tau, dpart, prec=0)
    assert st.outer_iterations == rst.outer_iterations == 10
    assert rel_err(out, ref) <= 1e-4
    ccfg = color_config(sc)
    rng = np.random.default_rng(3)
    H = W = 24 * p.dsf
    U = rng.uniform(0, 1, (3, H, W)).astype(np.float32)
    wg = rng.uniform(0.5e4, 1e4, (80, 24, 24)).astype(np.float32)
    G, F = ctx.stage_dataterm(ccfg, sc.views, tau, wg, U)
    rG, rF = pyoracle.stage_dataterm(ccfg, sc.views, tau, wg, U, prec=1)
    assert rel_err(G, rG, floor=1e-2) < 1e-4


@pytest.mark.parametrize("H,W,iters", [(48, 64, 200), (37, 53, 13), (200, 296, 200)])
def test_poisson_jacobi(ctx, H, W, iters):
    """poisson_jacobi (sources/gradientIBR.cu:923-1013) on the GPU: bit for bit against the FP32 mirror (which is
    pinned to the reference's kernels), and within 1e-5 of the FP64 oracle; odd sweep counts end mid super-step."""
    rng = np.random.default_rng(13)
    U = rng.uniform(0.1, 0.9, (3, H, W)).astype(np.float32)
    gx = rng.normal(0, 0.05, (H, W)).astype(np.float32)
    gy = rng.normal(0, 0.05, (H, W)).astype(np.float32)
    mask = rng.uniform(0, 1.5, (H, W)).astype(np.float32)
    mask[H // 4:H // 2, W // 8:W // 2] = 0.0
    out = ctx.stage_poisson_jacobi(gx, gy, mask, U, iters)
    ref32 = pyoracle.stage_poisson_jacobi(gx, gy, mask, U, iters, prec=1)
    ref64 = pyoracle.stage_poisson_jacobi(gx, gy, mask, U, iters, prec=0)
    np.testing.assert_array_equal(out, ref32)
    assert np.max(np.abs(out - ref64)) < 1e-5
