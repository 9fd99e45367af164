"""Builds the in-tree native libraries of the STQ broad phase.

  _build/libstq_gb300.so  CUDA kernels + the C ABI (include/stq_abi.h), sm_103a
  _build/libstq_scenes.so synthetic scene generators (host C++)

Each CUDA translation unit is compiled by its own nvcc process, in parallel,
for exactly one target (-gencode arch=compute_103a,code=sm_103a), then
linked with nvcc into one shared library. No CMake.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
ROOT = PKG.parent

CUDA_SOURCES = ["boxes.cu", "batch.cu", "radix_sort.cu", "sweep.cu", "abi.cu", "server.cu", "static_sweep.cu",
                "mesh_io.cpp"]
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [
    GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
    # IEEE float semantics: the box builder subtracts the smallest denormal
    "-ftz=false", "-prec-div=true", "-prec-sqrt=true",
    "-Xptxas", "-v", "--expt-relaxed-constexpr",
    "-I" + str(ROOT / "include"),
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the STQ CUDA library cannot be built")


def _run(cmd: list[str], log: Path) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    log.write_text(" ".join(cmd) + "\n" + proc.stdout + proc.stderr)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed ({' '.join(cmd[:3])} ...):\n{proc.stderr[-4000:]}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False) -> dict[str, Path]:
    OUT.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted((ROOT / "include").glob("*.h"))
    objs, jobs = [], []
    for src in CUDA_SOURCES:
        s = CSRC / src
        o = OUT / (s.stem + ".o")
        objs.append(o)
        if _stale(o, [s, *headers]):
            jobs.append(([nvcc, *NVCC_FLAGS, "-c", str(s), "-o", str(o)], OUT / (s.stem + ".log")))
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, cmd, log) for cmd, log in jobs]:
            f.result()
    lib = OUT / "libstq_gb300.so"
    if _stale(lib, objs):
        _run([nvcc, GENCODE, "-shared", "-Xcompiler", "-fPIC", *map(str, objs), "-o", str(lib)],
             OUT / "link.log")
    scenes = OUT / "libstq_scenes.so"
    ssrc = CSRC / "scenes.cpp"
    if _stale(scenes, [ssrc, CSRC / "scenes.h"]):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", str(ssrc), "-o", str(scenes)],
             OUT / "scenes.log")
    if verbose:
        for log in sorted(OUT.glob("*.log")):
            print(log.read_text())
    return {"stq": lib, "scenes": scenes}


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
