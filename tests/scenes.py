"""Small seeded inputs shared by the tests (synthetic light fields of the benchmark configs' shape)."""
from __future__ import annotations

import functools

import numpy as np

import lfrv
import pyoracle


@functools.lru_cache(maxsize=None)
def scene(preset: int, w: int, seed: int = 1, **kw):
    p = lfrv.scene_params(preset, w=w, h=w, seed=seed, **kw)
    return lfrv.synth_scene(p)


@functools.lru_cache(maxsize=None)
def warped(preset: int, w: int, seed: int = 1):
    """Scene plus tau / dpart from the FP64 oracle's warp (identical inputs for both solvers)."""
    sc = scene(preset, w, seed)
    tau, dpart, zbuf = pyoracle.warp(sc.depth, sc.cams, sc.target)
    return sc, tau, dpart, zbuf


def color_config(sc, **kw) -> lfrv.Config:
    p = sc.params
    base = dict(w=p.w, h=p.h, dsf=p.dsf, nviews=sc.views.shape[0], nchannels=3, sigma_sensor=0.01,
                ugrad_threshold=1.0, lambda_=0.05, lambda_max_factor=100.0, niter=10, nmeta_iter=1, early_exit=0)
    base.update(kw)
    return lfrv.default_config(**base)


def gradient_config(sc, **kw) -> lfrv.Config:
    p = sc.params
    base = dict(w=p.w, h=p.h, dsf=p.dsf, nviews=sc.views.shape[0], nchannels=3, sigma_sensor=0.005, lambda_=0.05,
                faithful=0, cg_gap_tol=1e-6, cg_max_iter=500)
    base.update(kw)
    return lfrv.default_config(**base)


def rel_err(a: np.ndarray, b: np.ndarray, floor: float = 1e-2) -> float:
    """Max over pixels of |a - b| / max(|b|, floor)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))
