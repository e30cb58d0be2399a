"""Records golden vectors of the reference's own kernels (compiled for the CPU by oracle/build_ref.sh).

Run from the repository root on a machine with the reference tree:
    python light-field-remote-vision_gb300/build.py && python tests/golden/make_golden.py
Writes tests/golden/*.npz: seeded inputs (synthetic light fields, random solver states) and the outputs of
the reference's kernels composed as its host code launches them (oracle/pyref.py). tests/test_golden.py checks
the CPU oracle (bit for bit) and the GPU kernels (within stated tolerances) against these files on machines
where the reference is absent.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "light-field-remote-vision_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "tests"))

import pyoracle  # noqa: E402
import pyref  # noqa: E402
from scenes import color_config, gradient_config, scene  # noqa: E402

OUT = Path(__file__).resolve().parent


def cams_array(cams):
    return np.array([[*c.K, *c.R, *c.t, c.width, c.height] for c in cams], np.float64)


def record_scene(preset: int, w: int, name: str) -> None:
    sc = scene(preset, w)
    tau, dpart, zbuf = pyoracle.warp(sc.depth, sc.cams, sc.target)
    p = sc.params
    cfg = color_config(sc)
    gcfg = gradient_config(sc)
    H = W = w * p.dsf
    rng = np.random.default_rng(100 + preset)
    U = rng.uniform(0.2, 0.8, (3, H, W)).astype(np.float32)
    wg = rng.uniform(0.5e4, 1e4, (len(sc.views), p.h, p.w)).astype(np.float32)
    gx0 = rng.normal(0, 0.1, (H, W)).astype(np.float32)
    gy0 = rng.normal(0, 0.1, (H, W)).astype(np.float32)
    geo = (p.w, p.h, p.dsf)
    cov, vis = pyref.visibility(tau, *geo)
    gx, gy, wr = pyref.weights(sc.views, tau, dpart, U, vis, gx0, gy0, *geo, cfg.sigma_sensor, cfg.ugrad_threshold)
    G, F = pyref.dataterm(sc.views, tau, wg, U, *geo, cfg.sigma_sensor, cfg.dt_alpha, cfg.lambda_)
    U0, norm0 = pyref.initial_image(sc.views, tau, wg, *geo)
    nm, g0 = pyref.regularizer_g0(tau, wg, norm0, *geo, cfg.sigma_sensor, cfg.lambda_, cfg.lambda_max_factor)
    gvis = pyref.gradient_visibility(tau, *geo)
    ugx, ugy, umask = pyref.u_gradient(sc.views, tau, wg, *geo, gcfg.sigma_sensor)
    np.savez_compressed(
        OUT / f"{name}.npz", views=sc.views, depth=sc.depth, cams=cams_array(sc.cams + [sc.target]), gt=sc.gt,
        tau=tau, dpart=dpart, zbuf=zbuf, geo=np.array(geo), sigma=np.float32(cfg.sigma_sensor),
        gsigma=np.float32(gcfg.sigma_sensor), U=U, wg=wg, gx0=gx0, gy0=gy0, cov=cov, vis=vis, gx=gx, gy=gy,
        weights=wr, G=G, F=F, U0=U0, norm0=norm0, norm_reg=nm, g0=g0, gvis=gvis, ugx=ugx, ugy=ugy, umask=umask)


def record_small() -> None:
    rng = np.random.default_rng(7)
    H, W = 24, 40
    F = rng.uniform(0, 1, (3, H, W)).astype(np.float32)
    g = rng.uniform(0.05, 5, (H, W)).astype(np.float32)
    P = rng.normal(0, 0.1, (6, H, W)).astype(np.float32)
    tau = np.float32(0.3 / np.sqrt(8.0))
    rU, rP = pyref.rof(7, tau, tau, np.float32(0.05), F, g, F, P)
    H2 = W2 = 64
    Upp = rng.uniform(0.1, 0.9, (3, H2, W2)).astype(np.float32)
    vpp = (rng.uniform(0, 1, (H2, W2)) > 0.3).astype(np.uint8)
    vpp[10:30, 20:50] = 0
    Upp[:, vpp == 0] = 0.0
    pp = pyref.push_pull(Upp, vpp)
    H3, W3 = 40, 48
    Uh = rng.uniform(0.1, 0.9, (3, H3, W3)).astype(np.float32)
    vh = np.ones((H3, W3), np.uint8)
    vh[5:20, 10:30] = 0
    Uh[:, vh == 0] = 0.0
    hf, hit = pyref.hole_fill(Uh, vh)
    np.savez_compressed(OUT / "small.npz", rof_F=F, rof_g=g, rof_P=P, rof_tau=tau, rof_U_out=rU, rof_P_out=rP,
                        pp_U=Upp, pp_vis=vpp, pp_out=pp, hf_U=Uh, hf_vis=vh, hf_out=hf, hf_iter=np.int32(hit))


if __name__ == "__main__":
    if not pyref.available():
        sys.exit("oracle/_ref/libref_kernels.so missing: run oracle/build_ref.sh <reference root> first")
    record_scene(1, 32, "c1_32")
    record_scene(2, 24, "c2_24")
    record_small()
    print("golden fixtures written to", OUT)
