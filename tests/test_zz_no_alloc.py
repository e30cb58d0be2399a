"""lfrv_cg_solve_static: the allocation-free corrected CG, against lfrv_stage_cg (faithful = 0).

The file name sorts last so the GPU test also runs after every other test in the same process. It must
pass there and when run alone.
"""
import numpy as np
import pytest

import lfrv


def test_static_cg_rejects_oversized_images():
    # the size check comes before any device work, so it needs no GPU
    side = int(np.sqrt(lfrv.CG_STATIC_MAX_PIXELS)) + 1
    with pytest.raises(lfrv.LfrvError) as e:
        lfrv.cg_solve_static(0, side, side, 10, 1e-6, 1, 1, 1)
    assert e.value.status == lfrv.E_ARG and "LFRV_CG_STATIC_MAX_PIXELS" in str(e.value)
    with pytest.raises(lfrv.LfrvError) as e:
        lfrv.cg_solve_static(0, 64, 64, 10, 1e-6, 0, 1, 1)
    assert e.value.status == lfrv.E_ARG


# (H, W) and the kernel the call takes: 200 x 296 fits the shared-memory resident CG; images narrower than 30
# pixels do not (their partial 64 x 16 tiles cannot hold the published borders), so 8192 x 28 runs the TMA-fed
# streaming kernel (W a multiple of 4) and 8192 x 26 the streaming kernel with plain loads.
SHAPES = [(200, 296, "resident"), (8192, 28, "streaming, TMA"), (8192, 26, "streaming, plain loads")]


@pytest.mark.gpu
@pytest.mark.parametrize("H,W,path", SHAPES)
def test_static_cg_matches_stage_cg_twice(H, W, path):
    import torch

    rng = np.random.default_rng(21)
    U0 = rng.uniform(0, 1, (3, H, W)).astype(np.float32)
    gx = rng.normal(0, 0.05, (H, W)).astype(np.float32)
    gy = rng.normal(0, 0.05, (H, W)).astype(np.float32)
    with lfrv.Context(0) as ctx:
        want, wit, wgap = ctx.stage_cg(gx, gy, U0, False, 500, 1e-7)
    stream = torch.cuda.Stream()
    d_gx = torch.from_numpy(gx).cuda()
    d_gy = torch.from_numpy(gy).cuda()
    torch.cuda.synchronize()
    for _ in range(2):  # the second call reuses the cached scratch address and re-clears the barrier words
        d_U = torch.from_numpy(U0).cuda()
        torch.cuda.synchronize()
        it, gap = lfrv.cg_solve_static(stream.cuda_stream, W, H, 500, 1e-7, d_gx.data_ptr(), d_gy.data_ptr(),
                                       d_U.data_ptr())
        got = d_U.cpu().numpy()
        assert it == wit and 0 < gap <= 1e-7
        assert abs(gap - wgap) <= 1e-12 + 1e-6 * wgap
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-6)
    # without iterations / gap the call only enqueues its work on the stream; the caller synchronises. A warmed-up
    # call leaves the device's free memory unchanged: it allocates nothing.
    d_U = torch.from_numpy(U0).cuda()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    lfrv.cg_solve_static(stream.cuda_stream, W, H, 500, 1e-7, d_gx.data_ptr(), d_gy.data_ptr(), d_U.data_ptr(),
                         want_stats=False)
    stream.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    np.testing.assert_allclose(d_U.cpu().numpy(), want, rtol=0, atol=1e-6)
