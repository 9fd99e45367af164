"""Mesh input and ground-truth comparison (host code of the library; no GPU):
OBJ / PLY readers, libigl-ordered unique edges, the JSON truth compare."""
import json

import numpy as np
import pytest


def write_obj(path, V, F):
    with open(path, "w") as f:
        f.write("# test mesh\n")
        for v in V:
            f.write("v %r %r %r\n" % tuple(float(x) for x in v))
        for t in F:
            f.write("f %d/1/1 %d %d//3\n" % tuple(int(i) + 1 for i in t))


def write_ply(path, V, F, binary):
    with open(path, "wb") as f:
        fmt = "binary_little_endian" if binary else "ascii"
        f.write((f"ply\nformat {fmt} 1.0\ncomment test\nelement vertex {len(V)}\n"
                 "property double x\nproperty double y\nproperty double z\n"
                 f"element face {len(F)}\nproperty list uchar int vertex_indices\nend_header\n").encode())
        if binary:
            f.write(np.ascontiguousarray(V, "<f8").tobytes())
            rec = np.zeros(len(F), dtype=[("n", "u1"), ("i", "<i4", (3,))])
            rec["n"], rec["i"] = 3, F
            f.write(rec.tobytes())
        else:
            for v in V:
                f.write(("%r %r %r\n" % tuple(float(x) for x in v)).encode())
            for t in F:
                f.write(("3 %d %d %d\n" % tuple(int(i) for i in t)).encode())


def igl_edges(F):
    """Unique undirected edges in the column-major order of an upper-triangular
    adjacency matrix: sorted by (larger, smaller)."""
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
    e = np.sort(e, axis=1)
    e = np.unique(e, axis=0)
    return e[np.lexsort((e[:, 0], e[:, 1]))].astype(np.int32)


@pytest.mark.parametrize("fmt", ["obj", "ply_ascii", "ply_binary"])
def test_read_mesh_round_trip(stq, tmp_path, fmt):
    m = stq.cloth_pair(g=15, seed=3)
    path = tmp_path / ("m.obj" if fmt == "obj" else "m.ply")
    if fmt == "obj":
        write_obj(path, m.V0, m.F)
    else:
        write_ply(path, m.V0, m.F, fmt == "ply_binary")
    V, F = stq.read_mesh(path)
    assert np.array_equal(V, m.V0) and np.array_equal(F, m.F)


def test_mesh_edges_match_generator_and_igl_order(stq):
    m = stq.cloth_pair(g=20, seed=4)
    E = stq.mesh_edges(m.F)
    assert np.array_equal(E, igl_edges(m.F))
    gen = {tuple(sorted(e)) for e in m.E.tolist()}
    assert {tuple(e) for e in E.tolist()} == gen and len(E) == len(gen)


def test_parse_mesh_two_files(stq, tmp_path):
    m = stq.cloth_pair(g=12, seed=5)
    write_obj(tmp_path / "t0.obj", m.V0, m.F)
    write_obj(tmp_path / "t1.obj", m.V1, m.F)
    p = stq.parse_mesh(tmp_path / "t0.obj", tmp_path / "t1.obj")
    assert np.array_equal(p.V0, m.V0) and np.array_equal(p.V1, m.V1) and np.array_equal(p.F, m.F)
    assert len(p.E) == len(m.E)


def test_malformed_inputs_rejected(stq, tmp_path):
    (tmp_path / "quad.obj").write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1 2 3 4\n")
    (tmp_path / "bad.obj").write_text("v 0 0 0\nf 1 2 3\n")
    (tmp_path / "x.stl").write_text("solid\n")
    for name in ("quad.obj", "bad.obj", "x.stl", "missing.obj"):
        with pytest.raises(stq.STQError):
            stq.read_mesh(tmp_path / name)


def test_compare_truth_json(stq, oracle, tmp_path):
    m = stq.cloth_pair(g=14, seed=6)
    boxes = oracle.construct_boxes(m.V0, m.V1, m.E, m.F, stq.AABB_DTYPE)
    pairs = oracle.broadphase(boxes)
    truth = pairs[::2][:, ::-1]  # every other pair, written (larger, smaller)
    (tmp_path / "truth.json").write_text(json.dumps(truth.tolist()))
    found, total, extra = stq.compare_truth_json(tmp_path / "truth.json", pairs)
    assert (found, total, extra) == (len(truth), len(truth), len(pairs) - len(truth))
    found, total, extra = stq.compare_truth_json(tmp_path / "truth.json", pairs[1::2])
    assert found == 0 and total == len(truth)
    (tmp_path / "broken.json").write_text("[[1, 2], [3]]")
    with pytest.raises(stq.STQError):
        stq.compare_truth_json(tmp_path / "broken.json", pairs)
