"""Build the in-tree CUDA library ``libgeoflood_gb300.so`` for sm_103a.

Each translation unit under ``csrc/`` is compiled by nvcc in parallel into
``_build/`` and linked into ``geoflood_gb300/libgeoflood_gb300.so``. No CMake,
no torch extension machinery: the library is a plain C-ABI shared object.
"""
from __future__ import annotations

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
LIB = PKG / "libgeoflood_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no FMA contraction (gcc contracts by default on aarch64), so
# the host-side hydrograph and controller arithmetic matches the oracle bits
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
          f"-I{ROOT / 'include'}", f"-I{CSRC}", "-diag-suppress", "550"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build geoflood_gb300")


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


# Per-file flags: the parity build of the patch kernel runs without
# floating-point contraction.
PER_FILE = {"gf_kernels_exact.cu": ["-fmad=false"],
            # refinement tags, transfers and the served time-step controller
            # must match the oracle bit for bit: no contraction
            "gf_amr.cu": ["-fmad=false"],
            "gf_qad.cu": ["-fmad=false"],
            "gf_served.cu": ["-fmad=false"],
            "gf_forest_kernels.cu": ["-fmad=false"],
            "gf_topo_kernels.cu": ["-fmad=false"]}


def _compile(src: Path, extra: list[str]) -> Path:
    obj = BUILD / (src.stem + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *PER_FILE.get(src.name, []), *extra, "-c", str(src),
           "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd[1:1] = ["-x", "cu"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stderr}")
    return obj


def _stale(srcs: list[Path]) -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = srcs + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, extra: list[str] | None = None, verbose: bool = False) -> Path:
    """Compile every CUDA/C++ source and link the shared library."""
    srcs = sources()
    if not force and not _stale(srcs):
        return LIB
    BUILD.mkdir(exist_ok=True)
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *map(str, objs), "-o", str(tmp),
           "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
