"""8-bit PNG light-field I/O and the `ulf` command-line front end.

PNG conversion follows gsl_image_from_qimage / gsl_image_to_qimage (cocolib/cocolib/common/gsl_image.cpp:539-620):
value / 255 on read, clamp(int(v * 255), 0, 255) on write. The decoder is checked against PNGs written here by
a few lines of Python (zlib + every scanline filter), independent of the library's own writer.
"""
import struct
import subprocess
import zlib
from pathlib import Path

import numpy as np
import pytest

import lfrv

ROOT = Path(__file__).resolve().parents[1]
ULF = ROOT / "light-field-remote-vision_gb300" / "bin" / "ulf"


def _chunk(kind: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)


def _paeth(a: int, b: int, c: int) -> int:
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def write_png_py(path: Path, pix: np.ndarray, ctype: int, filters) -> None:
    """pix: h x w x chans uint8. Row y uses filters[y % len(filters)]."""
    h, w, ch = pix.shape
    raw = bytearray()
    prev = np.zeros(w * ch, np.int64)
    for y in range(h):
        cur = pix[y].reshape(-1).astype(np.int64)
        f = filters[y % len(filters)]
        out = np.zeros_like(cur)
        for i in range(cur.size):
            a = cur[i - ch] if i >= ch else 0
            b = prev[i]
            c = prev[i - ch] if i >= ch else 0
            pred = [0, a, b, (a + b) // 2, _paeth(a, b, c)][f]
            out[i] = (cur[i] - pred) & 0xFF
        raw += bytes([f]) + bytes(out.astype(np.uint8))
        prev = cur
    ihdr = struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)
    data = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr)
    z = zlib.compress(bytes(raw))
    data += _chunk(b"IDAT", z[: len(z) // 2]) + _chunk(b"IDAT", z[len(z) // 2:]) + _chunk(b"IEND", b"")
    path.write_bytes(data)


def png_supported() -> bool:
    try:
        lfrv.png_read("/nonexistent.png")
    except lfrv.LfrvError as e:
        return "zlib" not in str(e)
    return True


needs_png = pytest.mark.skipif(not png_supported(), reason="library built without zlib")


@needs_png
@pytest.mark.parametrize("ctype,chans", [(2, 3), (6, 4), (0, 1), (4, 2)])
def test_png_decoder_every_filter(tmp_path, ctype, chans):
    rng = np.random.default_rng(7 + ctype)
    pix = rng.integers(0, 256, size=(9, 13, chans), dtype=np.uint8)
    p = tmp_path / "in.png"
    write_png_py(p, pix, ctype, filters=[0, 1, 2, 3, 4])
    img = lfrv.png_read(p)
    assert img.shape == (3, 9, 13)
    rgb = pix[..., :3] if chans >= 3 else np.repeat(pix[..., :1], 3, axis=2)
    want = (rgb.transpose(2, 0, 1).astype(np.float64) / 255.0).astype(np.float32)
    np.testing.assert_array_equal(img, want)


@needs_png
def test_png_write_quantisation_and_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    img = rng.uniform(-0.2, 1.2, size=(3, 6, 11)).astype(np.float32)
    p = tmp_path / "out.png"
    lfrv.png_write(p, img)
    back = lfrv.png_read(p)
    q = np.clip((img.astype(np.float64) * 255.0).astype(np.int64), 0, 255)  # int() truncates toward zero
    np.testing.assert_array_equal(back, (q / 255.0).astype(np.float32))
    lfrv.png_write(p, back)
    np.testing.assert_array_equal(lfrv.png_read(p), back)  # k/255 -> int(k/255*255) = k


@needs_png
def test_png_errors(tmp_path):
    bad = tmp_path / "bad.png"
    bad.write_bytes(b"not a png at all, just some bytes to read")
    with pytest.raises(lfrv.LfrvError) as e:
        lfrv.png_read(bad)
    assert e.value.status == lfrv.E_FORMAT
    p16 = tmp_path / "deep.png"
    ihdr = struct.pack(">IIBBBBB", 2, 2, 16, 2, 0, 0, 0)
    p16.write_bytes(b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr) + _chunk(b"IDAT", zlib.compress(bytes(26)))
                    + _chunk(b"IEND", b""))
    with pytest.raises(lfrv.LfrvError) as e:
        lfrv.png_read(p16)
    assert e.value.status == lfrv.E_FORMAT
    with pytest.raises(lfrv.LfrvError) as e:
        lfrv.png_read(tmp_path / "missing.png")
    assert e.value.status == lfrv.E_IO


def test_ulf_rejects_incomplete_configs(tmp_path):
    if not ULF.exists():
        pytest.skip("ulf not built")
    cfg = tmp_path / "c.cfg"
    cfg.write_text("algorithm IBR_gradient\n")
    r = subprocess.run([str(ULF), "-config", str(cfg)], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "s_min" in r.stderr
    r = subprocess.run([str(ULF), "-config", str(cfg), "-algorithm", "IBR_video"], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode != 0 and "not part of this path" in r.stderr
    cfg.write_text("s_min 0\ns_max 1\nlf_name " + str(tmp_path / "v_%02i.pfm") + "\n")
    r = subprocess.run([str(ULF), "-config", str(cfg)], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "v_00.pfm" in r.stderr


@pytest.mark.gpu
def test_ulf_matches_library_call(tmp_path):
    """The command-line front end, fed PFM files, reproduces lfrv_ibr_gradient on the same arrays bit for bit."""
    from scenes import gradient_config, warped

    sc, tau, dpart, _ = warped(2, 24)
    V = sc.views.shape[0]
    for s in range(V):
        lfrv.pfm_write(tmp_path / f"v_{s:02d}.pfm", sc.views[s])
        lfrv.pfm_write(tmp_path / f"tau_{s:02d}.pfm", tau[s])
        lfrv.pfm_write(tmp_path / f"dpart_{s:02d}.pfm", dpart[s])
    cfg = gradient_config(sc, cg_gap_tol=1e-5, cg_max_iter=200)
    (tmp_path / "run.cfg").write_text(
        "algorithm IBR_gradient\n"
        f"s_min 0\ns_max {V}\ns_rmv {V}\ndsf {cfg.dsf}\n"
        f"sigma_sensor {cfg.sigma_sensor}\nlambda {cfg.lambda_}\n"
        f"lf_name {tmp_path}/v_%02i.pfm\ntau_name {tmp_path}/tau_%02i.pfm\ndpart_name {tmp_path}/dpart_%02i.pfm\n"
        f"outdir {tmp_path}\noutfile result.png\n")
    r = subprocess.run([str(ULF), "-config", str(tmp_path / "run.cfg"), "-faithful", "0", "-cg_gap_tol", "1e-5",
                        "-cg_max_iter", "200"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = lfrv.pfm_read(tmp_path / "output.pfm")
    # the file's keys go through the reference's conventions (sigma_sensor is divided by 255 on parse)
    fcfg = lfrv.parse_config(tmp_path / "run.cfg")
    fcfg.w, fcfg.h, fcfg.nviews, fcfg.nchannels = cfg.w, cfg.h, V, 3
    fcfg.faithful, fcfg.cg_gap_tol, fcfg.cg_max_iter = 0, 1e-5, 200
    assert abs(fcfg.sigma_sensor - cfg.sigma_sensor / 255.0) < 1e-9
    with lfrv.Context(0) as ctx:
        want, _ = ctx.ibr_gradient(fcfg, sc.views, tau, dpart)
    np.testing.assert_array_equal(got, want)
    png = lfrv.png_read(tmp_path / "result.png")
    q = np.clip((want.astype(np.float64) * 255.0).astype(np.int64), 0, 255)
    np.testing.assert_array_equal(png, (q / 255.0).astype(np.float32))
