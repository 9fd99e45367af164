"""The C++ drop-in (include/stq_gpu.hpp): compiles on CPU; on the GPU, a C++
program calls it the way the reference's app does and its boxes and pairs
must equal the oracle's."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "shim_check.cpp"


def cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return str(Path(nvcc).resolve().parent.parent / "include")


def test_shim_header_compiles():
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", f"-I{ROOT / 'include'}",
                    f"-I{cuda_include()}", str(SRC)], check=True)


def write_mesh(path, mesh):
    with open(path, "wb") as f:
        np.array([mesh.V0.shape[0], mesh.E.shape[0], mesh.F.shape[0]], np.int64).tofile(f)
        for a in (mesh.V0, mesh.V1, mesh.E, mesh.F):
            np.ascontiguousarray(a).tofile(f)


@pytest.fixture(scope="module")
def shim_binary(pkg, tmp_path_factory):
    out = tmp_path_factory.mktemp("shim") / "shim_check"
    lib_dir = ROOT / "broadphase-gpu_gb300" / "_build"
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    subprocess.run([nvcc, "-std=c++17", f"-I{ROOT / 'include'}", str(SRC), f"-L{lib_dir}", "-lstq_gb300",
                    f"-Xlinker=-rpath={lib_dir}", "-o", str(out)], check=True)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("g", [12, 120])
def test_shim_matches_oracle(stq, oracle, shim_binary, tmp_path, g):
    mesh = stq.cloth_pair(g=g, z_offset=0.004, sigma=0.004, seed=g)
    write_mesh(tmp_path / "mesh.bin", mesh)
    prefix = tmp_path / "out"
    r = subprocess.run([str(shim_binary), str(tmp_path / "mesh.bin"), str(prefix)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    boxes = np.fromfile(f"{prefix}.boxes", stq.AABB_DTYPE)
    want_boxes = oracle.construct_boxes(mesh.V0, mesh.V1, mesh.E, mesh.F, stq.AABB_DTYPE)
    assert boxes.tobytes() == want_boxes.tobytes()
    want = oracle.broadphase(want_boxes)
    for kind in ("stq", "plain"):
        raw = np.fromfile(f"{prefix}.{kind}", np.int32).reshape(-1, 2)
        got = oracle.canonical(raw)
        assert len(got) == len(raw), kind
        assert np.array_equal(got, want), kind
