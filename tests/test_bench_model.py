"""bench.py's bookkeeping on the CPU: the algorithmic byte model the roofline divides by, and the clock record a
run is judged by (median SM clock under load, the throttle reasons seen)."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def test_solver_byte_model_per_pixel():
    """The per-pixel figures of the measurement contract: 72 B per CG iteration (x, r, d read and written once),
    88 B per ROF inner iteration (U, p, F, g read; p, U written), 216 B per FGP iteration (FP64 p and q read and
    written, F, lambda / D, 1/L, g read)."""
    N = 2048 * 2048
    assert bench.algorithmic_bytes("cg_persistent", 80, 1024 * 1024, N, 3, cg_iters=7) == 7 * 72 * N
    assert bench.algorithmic_bytes("rof_persistent", 8, 256 * 256, 256 * 256, 2, rof_iters=300) == 300 * 88 * 256 * 256
    assert bench.algorithmic_bytes("tv_fgp_df", 8, 256 * 256, 256 * 256, 2) == 200 * 216 * 256 * 256
    assert bench.algorithmic_bytes("hole_fill_iter", 8, 1, 1, 2) is None
    assert bench.algorithmic_bytes("no such kernel", 8, 1, 1, 2) is None


def test_warp_byte_model_scales_with_views_and_targets():
    """The warp-stage kernels' bytes are linear in the views' pixels (V n) plus the target's (N)."""
    for kernel in ("zbuffer_splat", "tau", "weights", "sobel", "gradient_setup"):
        b = lambda V, n, N: bench.algorithmic_bytes(kernel, V, n, N, 3)  # noqa: E731
        base = b(8, 1000, 4000)
        assert b(16, 1000, 4000) - base == b(8, 1000, 4000) - b(0, 1000, 4000)
        assert b(8, 1000, 8000) - base == b(8, 1000, 4000) - b(8, 1000, 0)
    # depth (z, dz/dx, dz/dy) read once and one 64-bit key per target pixel
    assert bench.algorithmic_bytes("zbuffer_splat", 80, 1 << 20, 1 << 22, 3) == 12 * 80 * (1 << 20) + 8 * (1 << 22)


def test_clock_summary(tmp_path):
    """Median SM clock and the maximum over the samples; reasons collected from their columns; malformed lines
    skipped; a missing file gives no samples."""
    rows = [
        "0, 2070, 2070, 900.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 1965, 2070, 1400.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1100.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
        "0, [N/A], 2070, 1100.0, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    path = tmp_path / "clocks.csv"
    path.write_text("\n".join(rows) + "\n")
    got = bench.summarize_clocks(str(path))
    assert got == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    thermal = tmp_path / "thermal.csv"
    thermal.write_text("0, 1500, 2070, 1300.0, 0x40, Not Active, Active, Not Active, Not Active\n")
    assert bench.summarize_clocks(str(thermal))["reasons"] == ["hw_thermal_slowdown"]
    assert bench.summarize_clocks(str(tmp_path / "absent.csv"))["samples"] == 0
