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
