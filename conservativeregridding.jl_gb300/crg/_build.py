"""Compile the CUDA C-ABI library ``libcrg_gb300.so`` for sm_103a.

The library is built in-tree under ``conservativeregridding.jl_gb300/_build``
with nvcc (one translation unit per process, linked with ``-shared``).  A
stamp records the host machine so that a checkout copied to another
architecture rebuilds instead of loading a foreign binary.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # conservativeregridding.jl_gb300/
REPO_ROOT = PKG_ROOT.parent
CSRC = PKG_ROOT / "csrc"
INCLUDE = REPO_ROOT / "include"
BUILD_DIR = PKG_ROOT / "_build"
LIB_PATH = BUILD_DIR / "libcrg_gb300.so"

# the FP64 peak probe of the build's roofline: its own library, not part of the ABI
PEAKS_SOURCE = "crg_peaks.cu"
PEAKS_LIB_PATH = BUILD_DIR / "libcrg_peaks.so"
SOURCES = ["crg_scan.cu", "crg_build.cu", "crg_layout.cu", "crg_apply.cu", "crg_grad.cu", "crg_batch.cu", "crg_se.cu", "crg_tune.cu", "crg_api.cu"]
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: only explicit fma() fuses, so the FP64 geometry follows the
# exact operation order that the CPU oracle restates.
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcrg_gb300.so")
    return cand


def _stamp() -> str:
    return f"{platform.machine()}\n"


def _inputs() -> list[Path]:
    return [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + [INCLUDE / "crg.h"]


def is_stale() -> bool:
    stamp = BUILD_DIR / "stamp"
    if not LIB_PATH.exists() or not PEAKS_LIB_PATH.exists() or not stamp.exists() or stamp.read_text() != _stamp():
        return True
    t = min(LIB_PATH.stat().st_mtime, PEAKS_LIB_PATH.stat().st_mtime)
    return any(p.stat().st_mtime > t for p in _inputs() + [CSRC / PEAKS_SOURCE])


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile (if stale) and return the path of the shared library."""
    if not force and not is_stale():
        return LIB_PATH
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    objs = []

    def compile_one(src: str) -> Path:
        obj = BUILD_DIR / (Path(src).stem + ".o")
        cmd = [nvcc, *NVCC_FLAGS, *ARCH_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    def compile_peaks() -> None:
        tmp = BUILD_DIR / "libcrg_peaks.so.tmp"
        cmd = [nvcc, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", *ARCH_FLAGS, "-shared",
               str(CSRC / PEAKS_SOURCE), "-o", str(tmp)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {PEAKS_SOURCE}:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, PEAKS_LIB_PATH)

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES) + 1) as ex:
        peaks = ex.submit(compile_peaks)
        objs = list(ex.map(compile_one, SOURCES))
        peaks.result()
    tmp = BUILD_DIR / "libcrg_gb300.so.tmp"
    cmd = [nvcc, "-shared", *ARCH_FLAGS, "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    (BUILD_DIR / "stamp").write_text(_stamp())
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
