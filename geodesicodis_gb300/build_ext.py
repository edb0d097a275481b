"""Build libodis_gpu.so in-tree with nvcc for sm_103a (GB300).

Every translation unit of csrc/ is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a`` and linked into
``geodesicodis_gb300/lib/libodis_gpu.so``.  No cmake, no torch extension
machinery: the library is plain C ABI (include/odis_gpu.h).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "lib" / "libodis_gpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without floating-point contraction: the mesh geometry
# (acos-based arc lengths, spherical excess) is ill-conditioned, and fused
# multiply-adds (the aarch64 default) would change the TRiSK coefficients in
# the 12th digit relative to the reference's unfused evaluation.
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-fopenmp,-O3,-ffp-contract=off", "-I", str(ROOT / "include")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libodis_gpu.so")


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


# Per-file device flags.  The setup kernels (grid generation, mesh build) run
# with unfused multiply-adds, as the host code does, so that their sums and
# products round as the host's.
FILE_FLAGS = {"odis_mesh_dev.cu": ["-fmad=false"]}


def _compile(src: Path, nvcc: str, extra: list[str]) -> Path:
    obj = BUILD / (src.name + ".o")
    deps = [src] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "odis_gpu.h"]
    if obj.exists() and obj.stat().st_mtime > max(d.stat().st_mtime for d in deps):
        return obj
    lang = [] if src.suffix == ".cu" else ["-x", "cu"]
    cmd = [nvcc, *ARCH, *NVCC_FLAGS, *FILE_FLAGS.get(src.name, []), *extra, *lang, "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile and link libodis_gpu.so; returns its path."""
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    LIB.parent.mkdir(exist_ok=True)
    extra = list(extra or [])
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc, extra), srcs))
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        cmd = [nvcc, *ARCH, "-shared", "-Xcompiler", "-fopenmp", "-o", str(LIB), *map(str, objs), "-lgomp"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    _build_cli()
    if verbose:
        print(f"built {LIB}")
    return LIB


CLI_SRC = PKG / "cli" / "odis_run.cpp"
CLI = PKG / "bin" / "odis_run"


def _build_cli() -> None:
    """The run driver: host C++ over the C ABI, linked against the in-tree library."""
    if not CLI_SRC.exists():
        return
    CLI.parent.mkdir(exist_ok=True)
    if CLI.exists() and CLI.stat().st_mtime > max(CLI_SRC.stat().st_mtime, LIB.stat().st_mtime):
        return
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(CLI_SRC), "-L", str(LIB.parent), "-lodis_gpu",
           "-Wl,-rpath,$ORIGIN/../lib", "-o", str(CLI)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"building odis_run failed:\n{res.stdout}\n{res.stderr}")


if __name__ == "__main__":
    build(verbose=True)
