"""Writes tests/golden/ref_vectors.npz: outputs of the reference's own CPU code.

The reference's src/cpu/aabb.cpp and src/cpu/sweep.cpp, compiled unchanged by
`make -C oracle ref` into oracle/_ref/libstq_ref.so (needs the reference's
source tree, so this script runs where that tree is; the vectors it writes
travel with the repository). For every case the file holds the inputs and
the reference's outputs:

  mesh cases   V0, V1 (fp64), E, F, inflation radius -> the boxes of
               stq::cpu::constructBoxes (44-byte records) and the canonical
               pairs of its sort + sweep (app/main.cpp:147-151)
  box cases    44-byte boxes -> the canonical pairs of the sort + sweep

Cases: the hand-built known-answer meshes and box sets of kat.json, seeded
cloth pairs (2 x 20^2, with and without inflation), four crumpled sheets of
16^2 and 2,000 random boxes with 5% slivers (the skewed workload's shape).

Run from the repository root:  python tests/golden/make_ref_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import __graft_entry__ as entry  # noqa: E402
from conftest import decode_boxes, decode_mesh  # noqa: E402


def main() -> None:
    stq = entry.load_package().stq
    orc = entry.load_oracle()
    if not orc.build_ref():
        raise SystemExit("the reference's source tree is needed to build oracle/_ref")
    kat = json.loads((ROOT / "tests" / "golden" / "kat.json").read_text())
    out: dict[str, np.ndarray] = {}
    names: list[str] = []

    def mesh_case(name, V0, V1, E, F, r):
        boxes = orc.ref_construct_boxes(V0, V1, E, F, stq.AABB_DTYPE, r)
        out[f"{name}.V0"], out[f"{name}.V1"] = V0, V1
        out[f"{name}.E"], out[f"{name}.F"] = E.astype(np.int32), F.astype(np.int32)
        out[f"{name}.r"] = np.array(r, np.float64)
        out[f"{name}.boxes"] = boxes.view(np.uint8).reshape(-1, 44)
        out[f"{name}.pairs"] = orc.ref_broadphase(boxes)
        names.append(f"mesh:{name}")

    def box_case(name, boxes):
        out[f"{name}.boxes"] = np.ascontiguousarray(boxes).view(np.uint8).reshape(-1, 44)
        out[f"{name}.pairs"] = orc.ref_broadphase(boxes)
        names.append(f"boxes:{name}")

    for name, m in sorted(kat["meshes"].items()):
        V0, V1, E, F = decode_mesh(m)
        mesh_case(f"kat_{name}", V0, V1, E, F, m["r"])
    for name, case in sorted(kat["pairs"].items()):
        box_case(f"kat_{name}", decode_boxes(case["boxes"], stq.AABB_DTYPE))
    for r in (0.0, 1e-4):
        m = stq.cloth_pair(g=20, z_offset=0.004, sigma=0.004, seed=20)
        mesh_case(f"cloth20_r{r:g}", m.V0, m.V1, m.E, m.F, r)
    m = stq.crumpled_sheets(4, 16, 0.05, 0.005, 5)
    mesh_case("crumpled4x16", m.V0, m.V1, m.E, m.F, 0.0)
    b = stq.random_boxes(2000, sliver_frac=0.05, seed=77)
    c = 0.5 * (b["min"] + b["max"])
    b["min"], b["max"] = c - 12 * (c - b["min"]), c + 12 * (b["max"] - c)  # denser: more pairs
    box_case("skewed2000", b)
    out["cases"] = np.array(names)
    path = ROOT / "tests" / "golden" / "ref_vectors.npz"
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({path.stat().st_size} bytes, {len(names)} cases)")


if __name__ == "__main__":
    main()
