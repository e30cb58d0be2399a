"""In-tree build of liblfrv.so (CUDA, sm_103a), the `ulf` command-line front end and the CPU oracle.

Usage: python light-field-remote-vision_gb300/build.py [--force] [--verbose]

Outputs (git-ignored, built on whichever machine runs this):
  light-field-remote-vision_gb300/liblfrv.so        the product library (C ABI in include/lfrv.h)
  light-field-remote-vision_gb300/bin/ulf           config-driven command-line front end
  oracle/liblfrv_oracle.so                          CPU restatement used only by tests and the CPU baseline
  oracle/_ref/libref_kernels.so                     reference kernels compiled for the CPU (only where the
                                                    reference tree is present; see oracle/build_ref.sh)
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"
LIB = PKG / "liblfrv.so"
ULF = PKG / "bin" / "ulf"
ORACLE_SRC = ROOT / "oracle" / "lfrv_oracle.cpp"
ORACLE_LIB = ROOT / "oracle" / "liblfrv_oracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-std=c++17", "-O3", "-lineinfo", f"-I{INCLUDE}", f"-I{CSRC}",
               "-Xcompiler", "-fPIC,-ffp-contract=off,-fopenmp"]
LIB_SOURCES = ["errors.cpp", "io.cpp", "png.cpp", "synth.cu", "host.cpp", "learn.cpp",
               "kernels_solver.cu", "kernels_tv.cu", "kernels_warp.cu", "kernels_pushpull.cu", "kernels_cg.cu", "kernels_learn.cu"]


def _have_zlib() -> bool:
    """True when zlib's header and library are present (PNG light fields need it)."""
    probe = BUILD / "zprobe.c"
    probe.write_text("#include <zlib.h>\nint main(void){return (int)zlibVersion()[0] == 0;}\n")
    res = subprocess.run(["gcc", str(probe), "-o", str(BUILD / "zprobe"), "-lz"], capture_output=True)
    return res.returncode == 0


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose and (res.stdout or res.stderr):
        print(res.stdout + res.stderr, flush=True)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build_library(force: bool = False, verbose: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    zlib = _have_zlib()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [INCLUDE / "lfrv.h"]
    jobs = []
    objs = []
    for src in LIB_SOURCES:
        s = CSRC / src
        o = BUILD / (s.name + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            extra = ["-Xptxas", "-v"] if (verbose and s.suffix == ".cu") else []
            if zlib and s.name == "png.cpp":
                extra.append("-DLFRV_HAVE_ZLIB")
            if s.name == "synth.cu":
                extra.append("--fmad=false")  # the scene generator's device code rounds as its host code
            jobs.append([nvcc, *ARCH, *NVCC_COMMON, *extra, "-c", str(s), "-o", str(o)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda c: _run(c, verbose), jobs))
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-Xcompiler", "-fopenmp", "-lgomp",
              *(["-lz"] if zlib else [])], verbose)
    main_src = CSRC / "ulf_main.cpp"
    if main_src.exists() and (force or _stale(ULF, [main_src, LIB])):
        ULF.parent.mkdir(exist_ok=True)
        _run(["g++", "-std=c++17", "-O2", f"-I{INCLUDE}", str(main_src), "-o", str(ULF),
              f"-L{PKG}", "-llfrv", f"-Wl,-rpath,{PKG}"], verbose)
    return LIB


def build_oracle(force: bool = False, verbose: bool = False) -> Path:
    if force or _stale(ORACLE_LIB, [ORACLE_SRC, INCLUDE / "lfrv.h"]):
        _run(["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
              f"-I{INCLUDE}", str(ORACLE_SRC), "-o", str(ORACLE_LIB)], verbose)
    return ORACLE_LIB


def build_reference_kernels(verbose: bool = False) -> Path | None:
    """Builds oracle/_ref from the reference tree when the recipe finds one (oracle/build_ref.sh --probe prints
    its location; LFRV_REFERENCE_ROOT overrides the recipe's default)."""
    script = ROOT / "oracle" / "build_ref.sh"
    if not script.exists():
        return None
    probe = subprocess.run(["bash", str(script), "--probe"], capture_output=True, text=True)
    if probe.returncode != 0:
        return None  # no reference tree on this machine
    _run(["bash", str(script)], verbose)
    out = ROOT / "oracle" / "_ref" / "libref_kernels.so"
    return out if out.exists() else None


def build_all(force: bool = False, verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_library, force, verbose)
        f2 = ex.submit(build_oracle, force, verbose)
        f1.result()
        f2.result()
    build_reference_kernels(verbose)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args()
    build_all(a.force, a.verbose)
    print(f"built {LIB}", file=sys.stderr)
