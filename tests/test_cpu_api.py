"""Host-side API: exported symbols, config files, PFM I/O, error codes, synthetic scenes (no GPU needed)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import lfrv

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "lfrv.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lfrv_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    names = declared_functions()
    assert len(names) >= 35
    missing = [n for n in names if not hasattr(lfrv.LIB, n)]
    assert not missing, missing
    assert sorted(names) == sorted(lfrv.EXPORTED)


def test_no_device_is_reported_cleanly():
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(lfrv.LfrvError) as e:
        lfrv.Context(0)
    assert e.value.status == lfrv.E_NODEVICE


def test_config_defaults_match_config_data():
    cfg = lfrv.default_config()
    # Config_data::Config_data (sources/config.cpp:11-64)
    assert cfg.nmeta_iter == 1 and cfg.niter == 0 and cfg.dsf == 0
    assert cfg.dt_alpha == 1.0 and cfg.dt_beta == 0.0
    assert cfg.sigma_sensor == pytest.approx(1.0 / 255.0)
    assert cfg.gradient_step == pytest.approx(0.1)
    assert cfg.faithful == 1 and cfg.early_exit == 1


def test_config_file_syntax(tmp_path):
    common = tmp_path / "common_parameters"
    common.write_text("nchannels\t\t3\nlambda\t   \t   \t0.001\nlambda_max_factor  \t100.0\nniter\t\t   \t100\n"
                      "nmeta_iter\t\t10\ngradient_step\t\t0.1\nugrad_threshold\t\t1.\nsigma_sensor\t\t1.\n"
                      "dw_type\t\t\t0\ngw_type \t\t1\t\n")
    top = tmp_path / "buddha"
    top.write_text(f"config \t\t\t{common}\n\n# light field configuration\n"
                   "lf_name\t\t\t./in/lf/v_%02i.png\ntau_name\t\t./in/lf/tau_%02i.pfm\n"
                   "s_min\t\t\t0\ns_max\t\t\t8\ns_rmv\t\t\t4\n\ndsf\t\t\t3\nlambda\t\t\t0.05\n"
                   "#niter 7\noutdir\t\t\t./out/sr/buddha\noutfile\t\t\tbuddha.png\n")
    cfg = lfrv.parse_config(str(top))
    assert cfg.nchannels == 3 and cfg.dsf == 3 and cfg.nviews == 8
    assert cfg.lambda_ == pytest.approx(0.05)            # later line overrides the included one
    assert cfg.niter == 100 and cfg.nmeta_iter == 10     # commented line ignored
    assert cfg.sigma_sensor == pytest.approx(1.0 / 255)  # divided by 255 (sources/config.cpp:119)
    assert cfg.gw_type == 1 and cfg.lambda_max_factor == pytest.approx(100.0)
    assert lfrv.config_string("tau_name") == "./in/lf/tau_%02i.pfm"
    assert lfrv.config_string("outfile") == "buddha.png"


def test_config_missing_file():
    with pytest.raises(lfrv.LfrvError) as e:
        lfrv.parse_config("/nonexistent/config")
    assert e.value.status == lfrv.E_IO


def test_pfm_roundtrip_and_flip(tmp_path):
    rng = np.random.default_rng(0)
    img = rng.normal(size=(3, 5, 7)).astype(np.float32)
    p = tmp_path / "a.pfm"
    lfrv.pfm_write(str(p), img)
    raw = p.read_bytes()
    assert raw.startswith(b"PF\n7 5\n-1.0\n")
    data = np.frombuffer(raw[len(b"PF\n7 5\n-1.0\n"):], np.float32).reshape(5, 7, 3)
    # first stored row is the image's bottom row (write_pfm_image_signed, cuda_helper.cu:355-363)
    assert np.array_equal(data[0], img[:, 4, :].T)
    assert np.array_equal(lfrv.pfm_read(str(p)), img)
    g = rng.normal(size=(1, 4, 6)).astype(np.float32)
    lfrv.pfm_write(str(tmp_path / "g.pfm"), g)
    assert np.array_equal(lfrv.pfm_read(str(tmp_path / "g.pfm")), g)


def test_pfm_corrupt(tmp_path):
    p = tmp_path / "bad.pfm"
    p.write_bytes(b"P6\n2 2\n255\n")
    with pytest.raises(lfrv.LfrvError) as e:
        lfrv.pfm_read(str(p))
    assert e.value.status == lfrv.E_FORMAT
    p.write_bytes(b"PF\n4 4\n-1.0\n" + b"\0" * 10)
    with pytest.raises(lfrv.LfrvError) as e:
        lfrv.pfm_read(str(p))
    assert e.value.status == lfrv.E_FORMAT


def test_null_arguments_are_rejected():
    assert lfrv.LIB.lfrv_config_default(None) == lfrv.E_ARG
    assert lfrv.LIB.lfrv_ibr_color(None, None, None, None, 2, None, None, None, None) == lfrv.E_ARG
    assert b"context" in lfrv.LIB.lfrv_last_error()


def test_synthetic_scene_properties():
    sc = lfrv.synth_scene(lfrv.scene_params(1, w=32, h=32, seed=5))
    assert sc.views.shape == (8, 3, 32, 32) and sc.gt.shape == (3, 32, 32)
    assert np.isfinite(sc.views).all() and np.isfinite(sc.depth).all()
    z = sc.depth[:, 0]
    assert z.min() >= 1.0 - 1e-6 and z.max() <= 2.5 + 1e-6     # plane depths 1.0 / 1.5 / 2.5
    assert np.allclose(sc.depth[:, 1:], 0.0)                   # fronto-parallel planes: flat depth
    assert 0.0 <= sc.gt.min() and sc.gt.max() <= 1.0           # texture in [0, 1] by construction
    again = lfrv.synth_scene(lfrv.scene_params(1, w=32, h=32, seed=5))
    assert np.array_equal(sc.views, again.views)               # seeded, deterministic
    other = lfrv.synth_scene(lfrv.scene_params(1, w=32, h=32, seed=6))
    assert not np.array_equal(sc.views, other.views)
    sc2 = lfrv.synth_scene(lfrv.scene_params(2, w=16, h=16))
    assert sc2.views.shape == (24, 3, 16, 16) and sc2.gt.shape == (3, 32, 32)
    assert np.abs(sc2.depth[:, 1:]).max() > 0                  # bumps give non-zero dz/dx, dz/dy
    assert sc.target.width == 32 and sc2.target.width == 32


def test_psnr_border():
    a = np.zeros((3, 10, 10), np.float32)
    b = a.copy()
    b[:, 0, :] = 1.0  # only in the excluded 2-pixel border
    assert lfrv.psnr(a, b) > 1e200
    b[:, 5, 5] = 0.1
    mse = (0.01 * 3 / 3) / 36.0
    assert lfrv.psnr(a, b) == pytest.approx(10 * np.log10(1.0 / mse))


def test_stats_layout_matches_header():
    """lfrv_stats as ctypes sees it is the C struct of include/lfrv.h (the trace fields sit at the end)."""
    import ctypes as C

    import lfrv

    assert C.sizeof(lfrv.Stats) == 64
    assert lfrv.Stats.energy_trace.offset == 48 and lfrv.Stats.trace_length.offset == 60


def test_oracle_energy_traces():
    """The oracle records one energy per outer iteration: the reference energy after each FISTA iteration
    (IBR_color), the quadratic energy after each CG iteration (IBR_gradient, both CG modes)."""
    import numpy as np

    import pyoracle
    from scenes import color_config, gradient_config, scene

    sc = scene(1, 32)
    tau, dpart, _ = pyoracle.warp(sc.depth, sc.cams, sc.target)
    cfg = color_config(sc, niter=5, early_exit=0)
    _, st = pyoracle.ibr_color(cfg, sc.views, tau, dpart, prec=0, trace=8)
    assert st.trace_length == 5 and st.trace()[-1] == st.energy
    _, st = pyoracle.ibr_color(cfg, sc.views, tau, dpart, prec=0, trace=3)  # a shorter buffer keeps the first 3
    assert st.trace_length == 3
    g = gradient_config(sc, faithful=0, cg_gap_tol=1e-8)
    _, st = pyoracle.ibr_gradient(g, sc.views, tau, dpart, prec=0, trace=200)
    tr = st.trace()
    assert st.trace_length == st.outer_iterations > 3
    assert np.all(np.diff(tr) <= 1e-12 * abs(tr[0]))  # CG lowers the energy at every step
    g = gradient_config(sc, faithful=1)
    _, st = pyoracle.ibr_gradient(g, sc.views, tau, dpart, prec=0, trace=10)
    assert st.trace_length == 5
