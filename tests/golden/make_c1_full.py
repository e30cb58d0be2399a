"""Records the FP64 oracle's full-length IBR_color solve of the 3x3, 256^2 light field (reference-faithful:
300 FISTA iterations of 300 ROF iterations each, nmeta_iter 1, early exits off, lambda 0.05, sigma 0.01).

Run from the repository root (the CPU oracle must be built):
    python light-field-remote-vision_gb300/build.py && python tests/golden/make_c1_full.py
Writes tests/golden/c1_256_full.npz: the solution (3 x 256 x 256), the energy after every FISTA iteration, and
checksums of the oracle's warps of the scene (which the GPU test recomputes with the same FP64 oracle instead of
storing 12 MB of warps). The solve takes a few minutes on 8 cores; the GPU test then compares the CUDA solver run
on the same warps with this file.
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "light-field-remote-vision_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "tests"))

import pyoracle  # noqa: E402
from scenes import color_config, scene  # noqa: E402

OUT = Path(__file__).resolve().parent / "c1_256_full.npz"
NITER = 300


def warp_checksums(tau: np.ndarray, dpart: np.ndarray) -> np.ndarray:
    """Size-independent fingerprints of the warps: code counts and sums over the valid pixels."""
    code = np.where(tau[:, 0] < 0, tau[:, 0], 0)
    ok = code == 0
    return np.array([np.sum(code == -2), np.sum(code == -1), np.sum(ok),
                     float(np.sum(tau[:, 0][ok], dtype=np.float64)), float(np.sum(tau[:, 1][ok], dtype=np.float64)),
                     float(np.sum(np.abs(dpart), dtype=np.float64))], np.float64)


def main() -> None:
    sc = scene(1, 256)
    tau, dpart, _ = pyoracle.warp(sc.depth, sc.cams, sc.target)
    cfg = color_config(sc, niter=NITER, nmeta_iter=1, early_exit=0, faithful=1)
    t0 = time.time()
    out, st = pyoracle.ibr_color(cfg, sc.views, tau, dpart, prec=0, trace=NITER)
    print(f"FP64 oracle, {NITER} x {NITER} iterations at 256^2: {time.time() - t0:.1f} s, "
          f"energy {st.energy:.9g}, trace {st.trace_length}")
    np.savez_compressed(OUT, out=out, trace=st.trace(), energy=np.float64(st.energy), niter=np.int32(NITER),
                        warp_checksums=warp_checksums(tau, dpart))


if __name__ == "__main__":
    main()
