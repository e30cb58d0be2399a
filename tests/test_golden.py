"""Golden vectors recorded from the reference's own kernels (tests/golden/make_golden.py).

CPU: the oracle's FP32 mirror reproduces every fixture bit for bit (the pin of the oracle on machines
without the reference tree). GPU: the CUDA kernels reproduce them within the stage tolerances of
tests/test_gpu_parity.py (relative 1e-5, floor 1e-2, unless stated).
"""
from pathlib import Path

import numpy as np
import pytest

import lfrv
import pyoracle
from scenes import rel_err

GOLD = Path(__file__).resolve().parent / "golden"
CASES = ["c1_32", "c2_24"]


def load(name):
    return dict(np.load(GOLD / f"{name}.npz"))


def cfg_of(d, gradient=False):
    w, h, dsf = (int(x) for x in d["geo"])
    return lfrv.default_config(w=w, h=h, dsf=dsf, nviews=d["views"].shape[0], nchannels=3,
                               sigma_sensor=float(d["gsigma"] if gradient else d["sigma"]), ugrad_threshold=1.0,
                               lambda_=0.05, lambda_max_factor=100.0, niter=10, nmeta_iter=1, early_exit=0,
                               faithful=0 if gradient else 1)


# ------------------------------------------------------------------ CPU: oracle == reference kernels
@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_golden(name):
    d = load(name)
    cfg, gcfg = cfg_of(d), cfg_of(d, True)
    cov, vis = pyoracle.stage_visibility(cfg, d["tau"], prec=1)
    assert np.array_equal(cov, d["cov"]) and np.array_equal(vis, d["vis"])
    gx, gy, wg = pyoracle.stage_weights(cfg, d["views"], d["tau"], d["dpart"], d["U"], d["vis"], d["gx0"], d["gy0"],
                                        prec=1)
    assert np.array_equal(gx, d["gx"]) and np.array_equal(gy, d["gy"]) and np.array_equal(wg, d["weights"])
    G, F = pyoracle.stage_dataterm(cfg, d["views"], d["tau"], d["wg"], d["U"], prec=1)
    assert np.array_equal(G, d["G"]) and np.array_equal(F, d["F"])
    U0, n0 = pyoracle.stage_initial_image(cfg, d["views"], d["tau"], d["wg"], prec=1)
    assert np.array_equal(U0, d["U0"]) and np.array_equal(n0, d["norm0"])
    nm, g = pyoracle.stage_regularizer(cfg, d["tau"], d["wg"], d["norm0"], prec=1)
    assert np.array_equal(nm, d["norm_reg"])
    assert np.array_equal(g, pyoracle.gaussian_blur(d["g0"], prec=1))
    assert np.array_equal(pyoracle.stage_gradient_visibility(gcfg, d["tau"], prec=1), d["gvis"])
    ugx, ugy, um = pyoracle.stage_u_gradient(gcfg, d["views"], d["tau"], d["wg"], prec=1)
    assert np.array_equal(ugx, d["ugx"]) and np.array_equal(ugy, d["ugy"]) and np.array_equal(um, d["umask"])


def test_oracle_reproduces_small_golden():
    d = load("small")
    tau = float(d["rof_tau"])
    U, P = pyoracle.stage_rof(7, tau, tau, 0.05, d["rof_F"], d["rof_g"], d["rof_F"], d["rof_P"], prec=1)
    assert np.array_equal(U, d["rof_U_out"]) and np.array_equal(P, d["rof_P_out"])
    assert np.array_equal(pyoracle.stage_push_pull(d["pp_U"], d["pp_vis"], True, prec=1), d["pp_out"])
    hf, it = pyoracle.stage_hole_fill(d["hf_U"], d["hf_vis"], 500, prec=1)
    assert it == int(d["hf_iter"]) and np.array_equal(hf, d["hf_out"])


def test_fp64_oracle_close_to_golden():
    d = load("c1_32")
    cfg = cfg_of(d)
    G, F = pyoracle.stage_dataterm(cfg, d["views"], d["tau"], d["wg"], d["U"], prec=0)
    assert np.max(np.abs(F - d["F"])) < 1e-5
    assert np.max(np.abs(G - d["G"])) < 1e-4 * max(1.0, float(np.abs(d["G"]).max()))


# ------------------------------------------------------------------ GPU: kernels vs reference kernels
@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_golden(ctx, name):
    d = load(name)
    cfg, gcfg = cfg_of(d), cfg_of(d, True)
    cov, vis = ctx.stage_visibility(cfg, d["tau"])
    assert np.max(np.abs(cov - d["cov"])) < 1e-5
    amb = np.abs(d["cov"] - 1.0) < 1e-5
    assert np.array_equal(vis[~amb], d["vis"][~amb])
    gx, gy, wg = ctx.stage_weights(cfg, d["views"], d["tau"], d["dpart"], d["U"], d["vis"], d["gx0"], d["gy0"])
    assert np.max(np.abs(gx - d["gx"])) < 1e-5 and np.max(np.abs(gy - d["gy"])) < 1e-5
    assert rel_err(wg, d["weights"], floor=1.0) < 1e-4
    G, F = ctx.stage_dataterm(cfg, d["views"], d["tau"], d["wg"], d["U"])
    assert np.max(np.abs(G - d["G"])) < 2e-5 * max(1.0, float(np.abs(d["G"]).max()))
    assert np.max(np.abs(F - d["F"])) < 1e-5
    U0, n0 = ctx.stage_initial_image(cfg, d["views"], d["tau"], d["wg"])
    assert np.max(np.abs(U0 - d["U0"])) < 1e-5 and rel_err(n0, d["norm0"], floor=1.0) < 1e-5
    nm, g = ctx.stage_regularizer(cfg, d["tau"], d["wg"], d["norm0"])
    assert rel_err(nm, d["norm_reg"], floor=1.0) < 1e-5
    assert rel_err(g, pyoracle.gaussian_blur(d["g0"], prec=1)) < 1e-5
    assert np.array_equal(ctx.stage_gradient_visibility(gcfg, d["tau"]), d["gvis"])
    ugx, ugy, um = ctx.stage_u_gradient(gcfg, d["views"], d["tau"], d["wg"])
    assert np.max(np.abs(ugx - d["ugx"])) < 1e-6 and np.max(np.abs(ugy - d["ugy"])) < 1e-6
    assert rel_err(um, d["umask"]) < 1e-5


@pytest.mark.gpu
def test_gpu_matches_small_golden(ctx):
    d = load("small")
    tau = float(d["rof_tau"])
    U, P = ctx.stage_rof(7, tau, tau, 0.05, d["rof_F"], d["rof_g"], d["rof_F"], d["rof_P"])
    assert np.max(np.abs(U - d["rof_U_out"])) < 1e-5 and np.max(np.abs(P - d["rof_P_out"])) < 1e-5
    assert np.max(np.abs(ctx.stage_push_pull(d["pp_U"], d["pp_vis"], True) - d["pp_out"])) < 2e-6
    hf, it = ctx.stage_hole_fill(d["hf_U"], d["hf_vis"], 500)
    assert it == int(d["hf_iter"]) and np.max(np.abs(hf - d["hf_out"])) < 1e-5
