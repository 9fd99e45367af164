"""The C ABI boundary without a GPU: the library loads, exports every symbol
include/*.h declares, and the 44-byte box layout matches the reference."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
INCLUDE = ROOT / "include"


def declared_functions():
    names = set()
    for h in INCLUDE.glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(stq_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported(stq):
    lib = stq.load_library()
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(stq.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    assert names <= exported


def test_python_binding_covers_header(stq):
    assert declared_functions() <= set(stq.ABI_SIGNATURES)


def header_enums(prefix):
    """NAME -> value of the enumerators of include/stq_abi.h that start with prefix."""
    text = re.sub(r"/\*.*?\*/", "", (INCLUDE / "stq_abi.h").read_text(), flags=re.S)
    return {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(" + prefix + r"[A-Z0-9_]+)\s*=\s*(-?\d+)", text)}


def test_python_constants_match_header(stq):
    """The binding's option, axis and status numbers are the header's."""
    opts = header_enums("STQ_OPT_")
    assert len(opts) >= 12
    for name, value in opts.items():
        assert getattr(stq, OPT_ALIASES.get(name, name[len("STQ_"):])) == value, name
    for name, value in header_enums("STQ_ERR_").items():
        assert getattr(stq, name) == value, name
    for name, value in header_enums("STQ_AXIS_").items():
        assert getattr(stq, name[len("STQ_"):]) == value, name


# binding names that shorten the header's
OPT_ALIASES = {"STQ_OPT_LANES_PER_ENTRY": "OPT_LANES", "STQ_OPT_QUEUE_DEPTH": "OPT_QUEUE",
               "STQ_OPT_BLOCK_SIZE": "OPT_BLOCK", "STQ_OPT_CANDIDATES_PER_LANE": "OPT_PER_LANE"}


def test_box_layout_matches_reference(stq, tmp_path):
    dt = stq.AABB_DTYPE
    assert dt.itemsize == 44
    assert [dt.fields[f][1] for f in ("id", "min", "max", "vertex_ids", "ref_id")] == [0, 4, 16, 28, 40]
    src = tmp_path / "layout.c"
    src.write_text(
        '#include "stq_abi.h"\n#include <stddef.h>\n'
        "_Static_assert(sizeof(stq_aabb) == 44, \"size\");\n"
        "_Static_assert(offsetof(stq_aabb, min) == 4, \"min\");\n"
        "_Static_assert(offsetof(stq_aabb, max) == 16, \"max\");\n"
        "_Static_assert(offsetof(stq_aabb, vertex_ids) == 28, \"vids\");\n"
        "_Static_assert(offsetof(stq_aabb, ref_id) == 40, \"ref_id\");\n"
        "_Static_assert(sizeof(stq_pair) == 8, \"pair\");\n")
    subprocess.run(["gcc", "-std=c11", "-fsyntax-only", f"-I{INCLUDE}", str(src)], check=True)


def test_status_strings(stq):
    lib = stq.load_library()
    assert lib.stq_abi_version() == 1
    for code in (0, 1, -1, -2, -3, -4, -5, -6, -7):
        assert lib.stq_status_string(code)
    assert b"unknown" in lib.stq_status_string(99)


def test_null_arguments_rejected_without_gpu(stq):
    lib = stq.load_library()
    assert lib.stq_context_create(0, None, None) == stq.STQ_ERR_INVALID_ARG
    assert lib.stq_prepare(None, None, 0, 0) == stq.STQ_ERR_INVALID_ARG
    assert lib.stq_context_launch_count(None) == -1
    c = ctypes.c_int64()
    assert lib.stq_sweep_prepared(None, 0, 0, None, 0, ctypes.byref(c), ctypes.byref(c), None) == \
        stq.STQ_ERR_INVALID_ARG


def test_context_creation_fails_cleanly_without_device(stq):
    import torch

    if torch.cuda.is_available():
        return
    lib = stq.load_library()
    h = ctypes.c_void_p()
    assert lib.stq_context_create(0, None, ctypes.byref(h)) == stq.STQ_ERR_INVALID_ARG
    assert not h.value


def test_scene_generators(stq):
    assert stq.grid_counts(200) == (40000, 119201, 79202)
    m = stq.cloth_pair(g=200)
    assert m.num_boxes == 476806
    nv, ne, nf = stq.grid_counts(250)
    assert 16 * (nv + ne + nf) == 5968048
    nv, ne, nf = stq.grid_counts(290)
    assert 16 * (nv + ne + nf) == 8036528
    a = stq.cloth_pair(g=30, seed=9)
    b = stq.cloth_pair(g=30, seed=9)
    assert np.array_equal(a.V1, b.V1) and np.array_equal(a.F, b.F)
    assert a.E.max() < a.V0.shape[0] and a.F.max() < a.V0.shape[0]
    c = stq.crumpled_sheets(sheets=3, g=20, seed=2)
    assert c.V0.shape == (1200, 3) and c.F.max() == 1199
    r = stq.random_boxes(600, seed=1)
    assert np.all(r["min"] <= r["max"]) and np.array_equal(r["id"], np.arange(600))
    g = stq.cloth_pair_grid_for(100_000)
    nv, ne, nf = stq.grid_counts(g)
    assert abs(2 * (nv + ne + nf) - 100_000) < 0.1 * 100_000
