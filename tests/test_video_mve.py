"""The real-data front end and the IBR_video chain: MVE depth / normal maps (InputView::importMVEIFile and
setDepthAndNormals, sources/openGL/view.cpp:279-325, 607-635), the moving target camera of IBR_video
(TargetView::move, sources/openGL/view.cpp:1744-1759) and the batched video render (sources/main.cpp:359-403)."""
import numpy as np
import pytest

import lfrv
from scenes import gradient_config, scene


def _write_mvei(path, img):
    """An MVE image file: a header line, width, height, channels, type (uint32), interleaved float32 pixels."""
    c, h, w = img.shape
    with open(path, "wb") as f:
        f.write(b"MVE_IMAGE\n")
        np.array([w, h, c, 9], "<u4").tofile(f)
        np.ascontiguousarray(img.transpose(1, 2, 0), "<f4").tofile(f)


def test_mvei_read(tmp_path):
    rng = np.random.default_rng(1)
    img = rng.normal(size=(3, 7, 11)).astype(np.float32)
    _write_mvei(tmp_path / "n.mvei", img)
    np.testing.assert_array_equal(lfrv.mvei_read(tmp_path / "n.mvei"), img)
    (tmp_path / "bad.mvei").write_bytes(b"MVE_IMAGE\n\x01\x00")
    with pytest.raises(lfrv.LfrvError) as e:
        lfrv.mvei_read(tmp_path / "bad.mvei")
    assert e.value.status == lfrv.E_FORMAT


def test_depth_from_mve_matches_restatement():
    """Depth plane + first two normal planes, nearest-neighbour upsampling, all-zero pixels -> (invalid, 0, 0)."""
    rng = np.random.default_rng(2)
    h0, w0, f = 9, 13, 3
    depth = rng.uniform(1, 3, (h0, w0)).astype(np.float32)
    normal = rng.normal(size=(3, h0, w0)).astype(np.float32)
    depth[2, 3] = 0.0
    normal[:2, 2, 3] = 0.0  # all three channels zero: an empty pixel
    depth[4, 5] = 0.0  # depth zero alone is kept as it is
    out = lfrv.depth_from_mve(depth, normal[:2], f, 1000.0)
    want = np.stack([depth, normal[0], normal[1]]).repeat(f, axis=1).repeat(f, axis=2)
    empty = np.all(want == 0, axis=0)
    want[0][empty] = 1000.0
    np.testing.assert_array_equal(out, want)
    assert out[0, 2 * f, 3 * f] == 1000.0 and out[0, 4 * f, 5 * f] == 0.0


def test_video_camera_matches_restatement():
    """TargetView::move in float: C = C_a + frame (C_b - C_a) / 1000, R = R_y(frame * 0.0003) R_a, t = -R C."""
    sc = scene(2, 24)
    a, b = sc.cams[5], sc.cams[3]
    Ra, Rb = (np.array(c.R, np.float32).reshape(3, 3) for c in (a, b))
    Ca = -Ra.T @ np.array(a.t, np.float32)
    Cb = -Rb.T @ np.array(b.t, np.float32)
    for frame in (0, 1, 57, 299):
        cam = lfrv.video_camera(a, b, sc.target, frame)
        C = Ca + np.float32(frame) * (Cb - Ca) / np.float32(1000)
        ang = np.float32(frame) * np.float32(0.0003)
        Ry = np.array([[np.cos(ang), 0, np.sin(ang)], [0, 1, 0], [-np.sin(ang), 0, np.cos(ang)]], np.float32)
        R = Ry @ Ra
        np.testing.assert_allclose(np.array(cam.R).reshape(3, 3), R, atol=1e-6)
        np.testing.assert_allclose(np.array(cam.t), -R @ C, atol=1e-6)
        assert list(cam.K) == list(sc.target.K) and cam.width == sc.target.width


@pytest.mark.gpu
def test_render_video_matches_single_frames():
    """Frames of the IBR_video chain rendered as one batch equal the same frames rendered one at a time."""
    import torch

    sc = scene(2, 32)
    cfg = gradient_config(sc, cg_gap_tol=1e-6)
    H, W = sc.gt.shape[1:]
    nf = 4
    dv, dd = torch.from_numpy(sc.views).cuda(), torch.from_numpy(sc.depth).cuda()
    out = torch.zeros((nf, 3, H, W), device="cuda")
    one = torch.zeros((3, H, W), device="cuda")
    with lfrv.Context(0) as ctx:
        torch.cuda.synchronize()
        stats = ctx.render_video_dev(cfg, 1, dv.data_ptr(), dd.data_ptr(), sc.cams, 5, 3, sc.target, 100, nf,
                                     out.data_ptr())
        torch.cuda.synchronize()
        for f in range(nf):
            cam = lfrv.video_camera(sc.cams[5], sc.cams[3], sc.target, 100 + f)
            st = ctx.render_view_dev(cfg, 1, dv.data_ptr(), dd.data_ptr(), sc.cams, cam, one.data_ptr())
            torch.cuda.synchronize()
            assert stats[f].outer_iterations == st.outer_iterations
            assert np.max(np.abs(out[f].cpu().numpy() - one.cpu().numpy())) < 1e-5
    assert not torch.equal(out[0], out[nf - 1])
