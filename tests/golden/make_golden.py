"""Generates the golden fixtures of tests/golden/.

The reference (Ahdhn/broadphase-gpu) ships no tests, golden vectors or
fixtures, so these are known-answer cases built by hand from its semantics.
Expected values come from this script's own pure-Python / numpy statement of
the rules, independent of the C++ oracle:

  box bounds  src/cpu/aabb.cpp:16-95 (float cast, min/max, nextafter outward,
              minus / plus nextafter_up(inflation_radius))
  pair set    src/cpu/sweep.cpp:17-43, 94-121 (x via the sweep, y/z inclusive,
              is_valid_pair, !covertex), written as an all-pairs check
  output form (min id, max id), sorted, unique

Run from the repository root:  python tests/golden/make_golden.py
Writes kat.json (hand cases) and cloth_g12.npz (a seeded 2 x 12^2 cloth pair
with its boxes and pairs; the npz expected arrays are computed here in numpy).
"""
from __future__ import annotations

import json
import struct
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
F32 = np.float32
MAXF = np.finfo(np.float32).max


def f32_bits(x) -> int:
    return struct.unpack("<I", struct.pack("<f", float(x)))[0]


def next_up(x):
    x = F32(x)
    return np.nextafter(x, F32(x + MAXF) if np.isfinite(x) else x, dtype=np.float32)


def next_down(x):
    x = F32(x)
    return np.nextafter(x, F32(x - MAXF) if np.isfinite(x) else x, dtype=np.float32)


def construct_boxes(V0, V1, E, F, r=0.0):
    """Reference bounds rule, element by element in numpy float32."""
    nV, nE, nF = len(V0), len(E), len(F)
    r_up = next_up(F32(r))
    boxes = []
    vb = []
    with np.errstate(over="ignore"):
        for i in range(nV):
            lo = [next_down(min(F32(V0[i][k]), F32(V1[i][k]))) - r_up for k in range(3)]
            hi = [next_up(max(F32(V0[i][k]), F32(V1[i][k]))) + r_up for k in range(3)]
            vb.append((lo, hi))
            boxes.append(dict(id=i, min=lo, max=hi, v=[i, -i - 1, -i - 1], ref=i))
        for i, (a, b) in enumerate(E):
            lo = [min(vb[a][0][k], vb[b][0][k]) for k in range(3)]
            hi = [max(vb[a][1][k], vb[b][1][k]) for k in range(3)]
            boxes.append(dict(id=nV + i, min=lo, max=hi, v=[int(a), int(b), -int(a) - 1], ref=i))
        for i, (a, b, c) in enumerate(F):
            lo = [min(vb[a][0][k], vb[b][0][k], vb[c][0][k]) for k in range(3)]
            hi = [max(vb[a][1][k], vb[b][1][k], vb[c][1][k]) for k in range(3)]
            boxes.append(dict(id=nV + nE + i, min=lo, max=hi, v=[int(a), int(b), int(c)], ref=i))
    return boxes


def box_type(v):
    return 2 if v[2] >= 0 else (1 if v[1] >= 0 else 0)


def pair_set(boxes):
    """All-pairs statement of the sweep's output set."""
    out = set()
    for i in range(len(boxes)):
        a = boxes[i]
        for j in range(i + 1, len(boxes)):
            b = boxes[j]
            ov = all(F32(a["max"][k]) >= F32(b["min"][k]) and F32(a["min"][k]) <= F32(b["max"][k])
                     for k in range(3))
            if not ov or box_type(a["v"]) + box_type(b["v"]) != 2:
                continue
            if any(x == y for x in a["v"] for y in b["v"]):
                continue
            out.add((min(a["id"], b["id"]), max(a["id"], b["id"])))
    return sorted(out)


def enc(boxes):
    return [dict(id=b["id"], min=[f32_bits(x) for x in b["min"]], max=[f32_bits(x) for x in b["max"]],
                 vertex_ids=b["v"], ref_id=b["ref"]) for b in boxes]


def raw_box(i, lo, hi, v):
    return dict(id=i, min=[F32(x) for x in lo], max=[F32(x) for x in hi], v=v, ref=i)


def vbox(i, lo, hi, vid):
    return raw_box(i, lo, hi, [vid, -vid - 1, -vid - 1])


def ebox(i, lo, hi, a, b):
    return raw_box(i, lo, hi, [a, b, -a - 1])


def fbox(i, lo, hi, a, b, c):
    return raw_box(i, lo, hi, [a, b, c])


def pair_cases():
    dn = float(np.nextafter(F32(0), F32(1)))  # smallest denormal
    cases = {}
    # touching: equality on every axis counts as overlap (inclusive tests)
    cases["touching_vf"] = [vbox(0, [0, 0, 0], [1, 1, 1], 0), fbox(1, [1, 1, 1], [2, 2, 2], 5, 6, 7)]
    # separated by one ulp on x
    cases["gap_one_ulp_x"] = [vbox(0, [0, 0, 0], [1, 1, 1], 0),
                              fbox(1, [float(next_up(1.0)), 0, 0], [2, 1, 1], 5, 6, 7)]
    # separated by one ulp on z only (the sweep axis overlaps)
    cases["gap_one_ulp_z"] = [vbox(0, [0, 0, 0], [1, 1, 1], 0),
                              fbox(1, [0, 0, float(next_up(1.0))], [1, 1, 2], 5, 6, 7)]
    # shared vertex: excluded by covertex
    cases["shared_vertex"] = [vbox(0, [0, 0, 0], [1, 1, 1], 3), fbox(1, [0, 0, 0], [1, 1, 1], 3, 6, 7),
                              fbox(2, [0, 0, 0], [1, 1, 1], 4, 6, 7)]
    # type filter: only V-F, F-V and E-E pairs survive
    cases["type_filter"] = [vbox(0, [0, 0, 0], [1, 1, 1], 0), vbox(1, [0, 0, 0], [1, 1, 1], 1),
                            ebox(2, [0, 0, 0], [1, 1, 1], 10, 11), ebox(3, [0, 0, 0], [1, 1, 1], 12, 13),
                            fbox(4, [0, 0, 0], [1, 1, 1], 20, 21, 22), fbox(5, [0, 0, 0], [1, 1, 1], 23, 24, 25)]
    # E-E sharing a vertex through either slot
    cases["edge_edge_shared"] = [ebox(0, [0, 0, 0], [1, 1, 1], 1, 2), ebox(1, [0, 0, 0], [1, 1, 1], 2, 3),
                                 ebox(2, [0, 0, 0], [1, 1, 1], 4, 1), ebox(3, [0, 0, 0], [1, 1, 1], 5, 6)]
    # equal sweep keys (ties in sort order) and identical boxes
    cases["equal_keys"] = [vbox(i, [0.5, i * 0.1, 0], [0.5, i * 0.1 + 0.15, 1], i) for i in range(4)] + \
                          [fbox(4 + i, [0.5, i * 0.1, 0], [0.5, i * 0.1 + 0.15, 1], 10 + i, 20 + i, 30 + i)
                           for i in range(4)]
    # signed zero and denormal bounds
    cases["signed_zero"] = [vbox(0, [-0.0, -0.0, -0.0], [0.0, 0.0, 0.0], 0),
                            fbox(1, [0.0, 0.0, 0.0], [1, 1, 1], 5, 6, 7),
                            fbox(2, [-1, -1, -1], [-0.0, -0.0, -0.0], 8, 9, 10)]
    cases["denormal"] = [vbox(0, [-dn, -dn, -dn], [dn, dn, dn], 0),
                         fbox(1, [2 * dn, 0, 0], [1, 1, 1], 5, 6, 7),
                         fbox(2, [dn, -dn, -dn], [dn, dn, dn], 8, 9, 10),
                         ebox(3, [-dn, 0, 0], [0, 0, 0], 11, 12), ebox(4, [0, 0, 0], [dn, 0, 0], 13, 14)]
    # one long box spanning many short ones (a long x-run), negative coordinates
    long = [vbox(0, [-5, -1, -1], [5, 1, 1], 0)]
    for i in range(40):
        x = -4.5 + i * 0.25
        long.append(fbox(1 + i, [x, 0.5 if i % 3 == 0 else -0.5, 0], [x + 0.1, 2 if i % 3 == 0 else 0.9, 0.5],
                         100 + i, 200 + i, 0 if i == 7 else 300 + i))
    cases["long_run"] = long
    cases["empty"] = []
    cases["one_box"] = [vbox(0, [0, 0, 0], [1, 1, 1], 0)]
    cases["two_boxes"] = [vbox(0, [0, 0, 0], [1, 1, 1], 0), fbox(1, [0.5, 0.5, 0.5], [2, 2, 2], 1, 2, 3)]
    # ids not equal to array positions (the output id is Aabb.id)
    perm = [vbox(70, [0, 0, 0], [1, 1, 1], 0), fbox(12, [0.2, 0.2, 0.2], [2, 2, 2], 1, 2, 3),
            ebox(33, [0, 0, 0], [1, 1, 1], 4, 5), ebox(5, [0.9, 0.9, 0.9], [3, 3, 3], 6, 7)]
    cases["ids_not_positions"] = perm
    return cases


def mesh_cases():
    dn = 1.401298464324817e-45
    cases = {}
    # two triangles sharing an edge, with coordinates that exercise rounding
    V0 = [[0.0, 0.0, 0.0], [1.0, 0.0, 0.1], [0.0, 1.0, -0.0], [1.0 / 3.0, 2.0 / 3.0, 1e-50]]
    V1 = [[0.0, 0.0, 0.0], [1.0, 1e-300, 0.1 + 1e-17], [-1e-46, 1.0, 0.0], [0.3333333333333333, 0.7, -1e-50]]
    E = [[0, 1], [1, 2], [2, 0], [1, 3], [3, 2]]
    F = [[0, 1, 2], [1, 3, 2]]
    cases["two_triangles"] = dict(V0=V0, V1=V1, E=E, F=F, r=0.0)
    cases["two_triangles_inflated"] = dict(V0=V0, V1=V1, E=E, F=F, r=1e-3)
    # values that are not representable in float (rounding direction matters)
    V0 = [[0.1, 0.2, 0.3], [16777217.0, -16777217.0, 1e30], [-3.4e38, 3.4e38, dn / 2]]
    V1 = [[0.1 + 1e-9, 0.2 - 1e-9, 0.3], [16777219.0, -16777219.0, -1e30], [-3.4e38, 3.4e38, -dn / 2]]
    cases["rounding"] = dict(V0=V0, V1=V1, E=[[0, 1], [1, 2]], F=[[0, 1, 2]], r=0.0)
    return cases


def main() -> None:
    out = {"pairs": {}, "meshes": {}}
    for name, boxes in pair_cases().items():
        out["pairs"][name] = dict(boxes=enc(boxes), expected=pair_set(boxes))
    for name, m in mesh_cases().items():
        boxes = construct_boxes(m["V0"], m["V1"], m["E"], m["F"], m["r"])
        out["meshes"][name] = dict(V0=[[float(x).hex() for x in row] for row in m["V0"]],
                                   V1=[[float(x).hex() for x in row] for row in m["V1"]],
                                   E=m["E"], F=m["F"], r=m["r"], boxes=enc(boxes),
                                   expected=pair_set(boxes))
    (HERE / "kat.json").write_text(json.dumps(out, indent=1) + "\n")

    # seeded cloth fixture: inputs as committed bytes, expectations from numpy
    rng = np.random.default_rng(12)
    g = 12
    xs = np.linspace(0.0, 1.0, g)
    X, Y = np.meshgrid(xs, xs)
    P = np.stack([X.ravel(), Y.ravel(), 0.02 * np.sin(6 * np.pi * X.ravel()) * np.cos(4 * np.pi * Y.ravel())], 1)
    th = np.deg2rad(10.0)
    Q = P.copy()
    Q[:, 0] = 0.5 + np.cos(th) * (P[:, 0] - 0.5) - np.sin(th) * (P[:, 1] - 0.5)
    Q[:, 1] = 0.5 + np.sin(th) * (P[:, 0] - 0.5) + np.cos(th) * (P[:, 1] - 0.5)
    Q[:, 2] = P[:, 2] + 0.02
    V0 = np.concatenate([P, Q])
    V1 = V0 + rng.normal(0.0, 0.02, V0.shape)
    E, F = [], []
    for s in range(2):
        b = s * g * g
        vid = lambda r, c: b + r * g + c  # noqa: E731
        for r in range(g):
            for c in range(g - 1):
                E.append([vid(r, c), vid(r, c + 1)])
        for r in range(g - 1):
            for c in range(g):
                E.append([vid(r, c), vid(r + 1, c)])
        for r in range(g - 1):
            for c in range(g - 1):
                E.append([vid(r, c), vid(r + 1, c + 1)])
        for r in range(g - 1):
            for c in range(g - 1):
                F.append([vid(r, c), vid(r, c + 1), vid(r + 1, c + 1)])
                F.append([vid(r, c), vid(r + 1, c + 1), vid(r + 1, c)])
    E = np.array(E, np.int32)
    F = np.array(F, np.int32)
    boxes = construct_boxes(V0, V1, E, F, 0.0)
    lo = np.array([b["min"] for b in boxes], np.float32)
    hi = np.array([b["max"] for b in boxes], np.float32)
    vids = np.array([b["v"] for b in boxes], np.int32)
    # vectorised all-pairs check for the expected set
    ov = np.ones((len(boxes), len(boxes)), bool)
    for k in range(3):
        ov &= (hi[:, None, k] >= lo[None, :, k]) & (lo[:, None, k] <= hi[None, :, k])
    t = np.where(vids[:, 2] >= 0, 2, np.where(vids[:, 1] >= 0, 1, 0))
    ov &= (t[:, None] + t[None, :]) == 2
    for a in range(3):
        for b in range(3):
            ov &= vids[:, None, a] != vids[None, :, b]
    ii, jj = np.nonzero(np.triu(ov, 1))
    pairs = np.stack([ii, jj], 1).astype(np.int32)
    np.savez_compressed(HERE / "cloth_g12.npz", V0=V0, V1=V1, E=E, F=F, box_min=lo, box_max=hi,
                        vertex_ids=vids, pairs=pairs)
    print(f"kat.json: {len(out['pairs'])} pair cases, {len(out['meshes'])} mesh cases; "
          f"cloth_g12.npz: {len(boxes)} boxes, {len(pairs)} pairs")


if __name__ == "__main__":
    sys.exit(main())
