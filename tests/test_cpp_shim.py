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
    for extra in ([], ["-DSTQ_GPU_MAX_OVERLAP_SIZE=1000"]):
        subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", *extra, f"-I{ROOT / 'include'}",
                        f"-I{cuda_include()}", str(SRC)], check=True)


def test_resume_cursor_covers_every_position_once(tmp_path):
    """The drop-in's tidstart / MAX_OVERLAP_CUTOFF count start boxes and map
    onto the prepared positions: any cutoff sequence, halved or not, covers
    all positions in order, once (host logic: no GPU)."""
    exe = tmp_path / "cursor_check"
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-O1", f"-I{ROOT / 'include'}", f"-I{cuda_include()}",
                    str(ROOT / "tests" / "cpp" / "cursor_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr


def write_mesh(path, mesh):
    with open(path, "wb") as f:
        np.array([mesh.V0.shape[0], mesh.E.shape[0], mesh.F.shape[0]], np.int64).tofile(f)
        for a in (mesh.V0, mesh.V1, mesh.E, mesh.F):
            np.ascontiguousarray(a).tofile(f)


LOOP_CAP = 20000  # pair-buffer cap of the resume binary (STQ_GPU_MAX_OVERLAP_SIZE)


def _compile(out, extra=()):
    lib_dir = ROOT / "broadphase-gpu_gb300" / "_build"
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    subprocess.run([nvcc, "-std=c++17", *extra, f"-I{ROOT / 'include'}", str(SRC), f"-L{lib_dir}", "-lstq_gb300",
                    f"-Xlinker=-rpath={lib_dir}", "-o", str(out)], check=True)
    return out


@pytest.fixture(scope="module")
def shim_binary(pkg, tmp_path_factory):
    return _compile(tmp_path_factory.mktemp("shim") / "shim_check")


@pytest.fixture(scope="module")
def shim_binary_capped(pkg, tmp_path_factory):
    return _compile(tmp_path_factory.mktemp("shim_capped") / "shim_check",
                    [f"-DSTQ_GPU_MAX_OVERLAP_SIZE={LOOP_CAP}"])


def run_shim(stq, oracle, binary, tmp_path, mesh, mode):
    write_mesh(tmp_path / "mesh.bin", mesh)
    prefix = tmp_path / "out"
    r = subprocess.run([str(binary), str(tmp_path / "mesh.bin"), str(prefix), mode], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    boxes = np.fromfile(f"{prefix}.boxes", stq.AABB_DTYPE)
    want_boxes = oracle.construct_boxes(mesh.V0, mesh.V1, mesh.E, mesh.F, stq.AABB_DTYPE)
    assert boxes.tobytes() == want_boxes.tobytes()
    want = oracle.broadphase(want_boxes)
    for kind in ("stq", "plain"):
        raw = np.fromfile(f"{prefix}.{kind}", np.int32).reshape(-1, 2)
        got = oracle.canonical(raw)
        assert len(got) == len(raw), kind  # every pair once
        assert np.array_equal(got, want), kind
    stats = dict(zip(r.stdout.split()[0::2], r.stdout.split()[1::2]))
    return {k: int(v) for k, v in stats.items()}, len(want)


@pytest.mark.gpu
@pytest.mark.parametrize("g", [12, 120])
def test_shim_single_call_matches_oracle(stq, oracle, shim_binary, tmp_path, g):
    """One run_sweep_sharedqueue call with a fresh MemHandler, as the reference's
    app makes it (app/main.cu:140-143), returns every pair and tidstart >= N."""
    mesh = stq.cloth_pair(g=g, z_offset=0.004, sigma=0.004, seed=g)
    stats, _ = run_shim(stq, oracle, shim_binary, tmp_path, mesh, "once")
    assert stats["calls"] == 1 and stats["tidstart"] >= stats["boxes"]


@pytest.mark.gpu
def test_shim_resume_loop_matches_oracle(stq, oracle, shim_binary_capped, tmp_path):
    """A caller looping while (tidstart < N) on a pair buffer capped far below
    the scene's pairs: the cutoff is halved on overflow, every call resumes
    where the last ended, and the union is the oracle's pair set, each once."""
    mesh = stq.cloth_pair(g=120, z_offset=0.004, sigma=0.004, seed=120)
    stats, npairs = run_shim(stq, oracle, shim_binary_capped, tmp_path, mesh, "loop")
    assert npairs > 4 * LOOP_CAP
    assert stats["calls"] > 4 and stats["cutoff"] < stats["boxes"]
