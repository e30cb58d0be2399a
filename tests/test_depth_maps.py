"""Radial to orthographic depth (fromRadial2Ortho.frag:10-23) in the oracle and on the GPU.

The oracle is checked by a round trip: orthographic depth maps of a synthetic scene are turned into radial ones
analytically (z_r = z_o d, dz_r/dx = dz_o/dx d + z_o (X . K^-1 column 0) / d), and the conversion must give
the orthographic maps back.
"""
import numpy as np
import pytest

import lfrv
import pyoracle
from scenes import scene


def to_radial(depth, cams):
    V, _, h, w = depth.shape
    out = np.empty_like(depth, dtype=np.float64)
    ys, xs = np.mgrid[0:h, 0:w]
    for v in range(V):
        Ki = np.linalg.inv(np.array(cams[v].K, np.float64).reshape(3, 3))
        X = np.einsum("ij,jyx->iyx", Ki, np.stack([xs + 0.5, ys + 0.5, np.ones_like(xs, np.float64)]))
        d = np.sqrt((X ** 2).sum(0))
        c0 = np.einsum("iyx,i->yx", X, Ki[:, 0])
        c1 = np.einsum("iyx,i->yx", X, Ki[:, 1])
        z, zx, zy = (depth[v, k].astype(np.float64) for k in range(3))
        out[v, 0] = z * d
        out[v, 1] = zx * d + z * c0 / d
        out[v, 2] = zy * d + z * c1 / d
    return out.astype(np.float32)


@pytest.mark.parametrize("preset,w", [(1, 48), (2, 40)])
def test_oracle_round_trip(preset, w):
    sc = scene(preset, w)
    radial = to_radial(sc.depth, sc.cams)
    back = pyoracle.depth_radial_to_ortho(radial, sc.cams)
    # per channel: float rounding of the radial maps (2e-6 relative) plus an absolute floor for derivative
    # channels that vanish on fronto-parallel planes
    tol = 2e-6 * np.abs(sc.depth).max(axis=(0, 2, 3), keepdims=True) + 1e-8
    assert np.all(np.abs(back - sc.depth) <= tol)


@pytest.mark.gpu
@pytest.mark.parametrize("preset,w", [(1, 48), (2, 40)])
def test_gpu_matches_oracle(preset, w):
    sc = scene(preset, w)
    radial = to_radial(sc.depth, sc.cams)
    want = pyoracle.depth_radial_to_ortho(radial, sc.cams)
    with lfrv.Context(0) as ctx:
        got = ctx.depth_radial_to_ortho(radial, sc.cams)
    tol = 2e-6 * np.abs(want).max(axis=(0, 2, 3), keepdims=True) + 1e-8
    assert np.all(np.abs(got - want) <= tol)


# ------------------------------------------------------------------ warps from depth maps (import.cpp:243-450)
def _holey_depth(sc):
    d = sc.depth.copy()
    d[0, 0, :3, :] = 0.0      # below 1/INVALID_DEPTH: no warp
    d[1, 0, 5, 5] = 2000.0    # above INVALID_DEPTH
    return d


@pytest.mark.parametrize("preset,w", [(1, 48), (2, 40)])
def test_oracle_warp_from_depth_matches_projection(preset, w):
    """Pass 1 is the projection the GL path computes; invalid depths give (-w, -h)."""
    sc = scene(preset, w)
    d = _holey_depth(sc)
    tau = pyoracle.warp_from_depth(d, sc.cams, sc.target, sc.params.dsf, faithful=1)
    gl, _, _ = pyoracle.warp(sc.depth, sc.cams, sc.target)
    ok = (tau[:, 0] >= 0) & (gl[:, 0] >= 0)
    assert ok.mean() > 0.9
    assert np.max(np.abs(tau[:, 0][ok] - gl[:, 0][ok])) < 1e-4
    assert np.max(np.abs(tau[:, 1][ok] - gl[:, 1][ok])) < 1e-4
    assert np.all(tau[0, 0, :3, :] == -w) and np.all(tau[0, 1, :3, :] == -w)
    assert tau[1, 0, 5, 5] == -w
    assert np.array_equal(tau[:, 1], tau[:, 2])  # written as (tau_x, tau_y, tau_y)


@pytest.mark.gpu
@pytest.mark.parametrize("preset,w", [(1, 48), (2, 40)])
@pytest.mark.parametrize("faithful", [1, 0])
def test_gpu_warp_from_depth_matches_oracle(preset, w, faithful):
    sc = scene(preset, w)
    d = _holey_depth(sc)
    want = pyoracle.warp_from_depth(d, sc.cams, sc.target, sc.params.dsf, faithful=faithful)
    with lfrv.Context(0) as ctx:
        got = ctx.warp_from_depth(d, sc.cams, sc.target, sc.params.dsf, faithful=bool(faithful))
    code = np.where(got[:, 0] < 0, got[:, 0], 0)
    rcode = np.where(want[:, 0] < 0, want[:, 0], 0)
    assert np.mean(code != rcode) < 1e-3
    ok = (code == 0) & (rcode == 0)
    assert np.max(np.abs(got[:, :2][np.stack([ok, ok], 1)] - want[:, :2][np.stack([ok, ok], 1)])) < 1e-4
