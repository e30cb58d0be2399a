"""Pins the CPU oracle against the reference's own kernels compiled for the CPU (oracle/_ref).

The reference has no golden vectors or fixtures for this path, so its kernel sources are compiled with g++
(oracle/build_ref.sh) and composed (oracle/pyref.py) in the order its host code launches them
(sources/optimization.cu, sources/gradientIBR.cu). The oracle's FP32 mirror must agree BIT FOR BIT: both
evaluate the same float operations in the same order (splats run over one segment in index order).
Skipped where oracle/_ref was not built (the reference tree is absent); tests/golden/ carries fixtures
recorded from these compositions for such machines (tests/test_golden.py).
"""
import numpy as np
import pytest

import pyoracle
import pyref
from scenes import color_config, gradient_config, warped

pytestmark = pytest.mark.skipif(not pyref.available(), reason="oracle/_ref not built (reference tree absent)")

CASES = [(1, 32), (2, 24)]


def geo(sc):
    p = sc.params
    return p.w, p.h, p.dsf


@pytest.mark.parametrize("preset,w", CASES)
def test_visibility_bitexact(preset, w):
    sc, tau, _, _ = warped(preset, w)
    cov, vis = pyref.visibility(tau, *geo(sc))
    ocov, ovis = pyoracle.stage_visibility(color_config(sc), tau, prec=1)
    assert np.array_equal(cov, ocov) and np.array_equal(vis, ovis)


@pytest.mark.parametrize("preset,w", CASES)
def test_weights_bitexact(preset, w):
    sc, tau, dpart, _ = warped(preset, w)
    cfg = color_config(sc)
    H = W = w * sc.params.dsf
    rng = np.random.default_rng(0)
    U = rng.uniform(0, 1, (3, H, W)).astype(np.float32)
    _, vis = pyoracle.stage_visibility(cfg, tau, prec=1)
    gx0 = rng.normal(0, 0.1, (H, W)).astype(np.float32)
    gy0 = rng.normal(0, 0.1, (H, W)).astype(np.float32)
    gx, gy, wr = pyref.weights(sc.views, tau, dpart, U, vis, gx0, gy0, *geo(sc), cfg.sigma_sensor,
                               cfg.ugrad_threshold)
    ogx, ogy, ow = pyoracle.stage_weights(cfg, sc.views, tau, dpart, U, vis, gx0, gy0, prec=1)
    assert np.array_equal(gx, ogx) and np.array_equal(gy, ogy) and np.array_equal(wr, ow)


# (dt_alpha, dt_beta, gw_type): the intensity term alone, plus the gradient term (vtv_sr_dataterm_gradients)
# unweighted and weighted, and the gradient term alone
TERMS = [(1.0, 0.0, 0), (1.0, 0.5, 0), (1.0, 0.5, 1), (0.0, 1.0, 1)]


@pytest.mark.parametrize("preset,w", CASES)
@pytest.mark.parametrize("alpha,beta,gw", TERMS)
def test_dataterm_bitexact(preset, w, alpha, beta, gw):
    sc, tau, _, _ = warped(preset, w)
    cfg = color_config(sc, dt_alpha=alpha, dt_beta=beta, gw_type=gw, gradient_step=0.25)
    p = sc.params
    H = W = w * p.dsf
    rng = np.random.default_rng(1)
    U = rng.uniform(0.2, 0.8, (3, H, W)).astype(np.float32)
    wg = rng.uniform(0.5e4, 1e4, (len(sc.views), p.h, p.w)).astype(np.float32)
    G, F = pyref.dataterm(sc.views, tau, wg, U, *geo(sc), cfg.sigma_sensor, cfg.dt_alpha, cfg.lambda_,
                          beta=cfg.dt_beta, gw_type=gw, gradient_step=cfg.gradient_step)
    oG, oF = pyoracle.stage_dataterm(cfg, sc.views, tau, wg, U, prec=1)
    assert np.array_equal(G, oG) and np.array_equal(F, oF)


def test_rof_bitexact():
    rng = np.random.default_rng(2)
    H, W = 24, 40
    F = rng.uniform(0, 1, (3, H, W)).astype(np.float32)
    g = rng.uniform(0.05, 5, (H, W)).astype(np.float32)
    P = rng.normal(0, 0.1, (6, H, W)).astype(np.float32)
    tau = sigma = np.float32(0.3 / np.sqrt(8.0))
    u, pp = pyref.rof(7, tau, sigma, np.float32(0.05), F, g, F, P)
    oU, oP = pyoracle.stage_rof(7, tau, sigma, 0.05, F, g, F, P, prec=1)
    assert np.array_equal(u, oU) and np.array_equal(pp, oP)


@pytest.mark.parametrize("preset,w", CASES)
def test_initial_image_and_regularizer_bitexact(preset, w):
    sc, tau, _, _ = warped(preset, w)
    cfg = color_config(sc)
    p = sc.params
    rng = np.random.default_rng(3)
    wg = rng.uniform(0.5e4, 1e4, (len(sc.views), p.h, p.w)).astype(np.float32)
    U, norm = pyref.initial_image(sc.views, tau, wg, *geo(sc))
    oU, onorm = pyoracle.stage_initial_image(cfg, sc.views, tau, wg, prec=1)
    assert np.array_equal(U, oU) and np.array_equal(norm, onorm)
    # prior coverage content = the initial image's weight sum (never cleared, optimization.cu:2262-2300)
    nm, g0 = pyref.regularizer_g0(tau, wg, norm, *geo(sc), cfg.sigma_sensor, cfg.lambda_, cfg.lambda_max_factor)
    onm, og = pyoracle.stage_regularizer(cfg, tau, wg, norm, prec=1)
    assert np.array_equal(nm, onm)
    assert np.array_equal(pyoracle.gaussian_blur(g0, prec=1), og)


def test_push_pull_bitexact():
    rng = np.random.default_rng(4)
    H = W = 64
    U = rng.uniform(0.1, 0.9, (3, H, W)).astype(np.float32)
    vis = (rng.uniform(0, 1, (H, W)) > 0.3).astype(np.uint8)
    vis[10:30, 20:50] = 0
    U[:, vis == 0] = 0.0
    assert np.array_equal(pyref.push_pull(U, vis), pyoracle.stage_push_pull(U, vis, True, prec=1))


@pytest.mark.parametrize("preset,w", CASES)
def test_gradient_ibr_pieces_bitexact(preset, w):
    sc, tau, _, _ = warped(preset, w)
    cfg = gradient_config(sc)
    p = sc.params
    assert np.array_equal(pyref.gradient_visibility(tau, *geo(sc)), pyoracle.stage_gradient_visibility(cfg, tau, prec=1))
    rng = np.random.default_rng(5)
    wg = rng.uniform(0.5e4, 1e4, (len(sc.views), p.h, p.w)).astype(np.float32)
    gx, gy, m = pyref.u_gradient(sc.views, tau, wg, *geo(sc), cfg.sigma_sensor)
    ogx, ogy, om = pyoracle.stage_u_gradient(cfg, sc.views, tau, wg, prec=1)
    assert np.array_equal(gx, ogx) and np.array_equal(gy, ogy) and np.array_equal(m, om)


def test_hole_fill_bitexact():
    rng = np.random.default_rng(6)
    H, W = 40, 48
    U = rng.uniform(0.1, 0.9, (3, H, W)).astype(np.float32)
    vis = np.ones((H, W), np.uint8)
    vis[5:20, 10:30] = 0
    U[:, vis == 0] = 0.0
    u, it = pyref.hole_fill(U, vis)
    out, oit = pyoracle.stage_hole_fill(U, vis, 500, prec=1)
    assert oit == it and np.array_equal(u, out)


def test_poisson_jacobi_bitexact():
    """The Jacobi variant of the Poisson integration (poisson_jacobi, sources/gradientIBR.cu:923-1013)."""
    rng = np.random.default_rng(12)
    H, W = 37, 52
    U = rng.uniform(0.1, 0.9, (3, H, W)).astype(np.float32)
    gx = rng.normal(0, 0.05, (H, W)).astype(np.float32)
    gy = rng.normal(0, 0.05, (H, W)).astype(np.float32)
    mask = rng.uniform(0, 1.5, (H, W)).astype(np.float32)
    mask[10:20, 5:25] = 0.0
    ref = pyref.poisson_jacobi(gx, gy, mask, U, iters=40)
    out = pyoracle.stage_poisson_jacobi(gx, gy, mask, U, iters=40, prec=1)
    assert np.array_equal(ref, out)
