"""CPU oracle checks: the restatement of the reference's src/cpu path against
the golden fixtures and against independent all-pairs checks."""
import numpy as np
import pytest

from conftest import decode_boxes, decode_mesh, expected_pairs


def test_kat_pair_cases(stq, oracle, kat):
    for name, case in kat["pairs"].items():
        boxes = decode_boxes(case["boxes"], stq.AABB_DTYPE)
        got = oracle.broadphase(boxes)
        want = expected_pairs(case["expected"])
        assert np.array_equal(got, want), name


def test_kat_mesh_cases(stq, oracle, kat):
    for name, m in kat["meshes"].items():
        V0, V1, E, F = decode_mesh(m)
        boxes = oracle.construct_boxes(V0, V1, E, F, stq.AABB_DTYPE, m["r"])
        want = decode_boxes(m["boxes"], stq.AABB_DTYPE)
        assert boxes.tobytes() == want.tobytes(), name
        assert np.array_equal(oracle.broadphase(boxes), expected_pairs(m["expected"])), name


def test_cloth_fixture(stq, oracle, cloth_fixture):
    f = cloth_fixture
    boxes = oracle.construct_boxes(f["V0"], f["V1"], f["E"], f["F"], stq.AABB_DTYPE)
    assert np.array_equal(boxes["min"], f["box_min"])
    assert np.array_equal(boxes["max"], f["box_max"])
    assert np.array_equal(boxes["vertex_ids"], f["vertex_ids"])
    assert np.array_equal(boxes["id"], np.arange(len(boxes)))
    assert np.array_equal(oracle.broadphase(boxes), f["pairs"])


def numpy_all_pairs(boxes):
    lo, hi, v = boxes["min"], boxes["max"], boxes["vertex_ids"]
    ov = np.ones((len(boxes), len(boxes)), bool)
    for k in range(3):
        ov &= (hi[:, None, k] >= lo[None, :, k]) & (lo[:, None, k] <= hi[None, :, k])
    t = np.where(v[:, 2] >= 0, 2, np.where(v[:, 1] >= 0, 1, 0))
    ov &= (t[:, None] + t[None, :]) == 2
    for a in range(3):
        for b in range(3):
            ov &= v[:, None, a] != v[None, :, b]
    i, j = np.nonzero(np.triu(ov, 1))
    ids = boxes["id"]
    p = np.stack([np.minimum(ids[i], ids[j]), np.maximum(ids[i], ids[j])], 1).astype(np.int32)
    return p[np.lexsort((p[:, 1], p[:, 0]))]


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_boxes_vs_all_pairs(stq, oracle, seed):
    boxes = stq.random_boxes(1500, sliver_frac=0.05, seed=seed)
    # widen so that pairs are plentiful
    c = 0.5 * (boxes["min"] + boxes["max"])
    boxes["min"] = c - 0.02
    boxes["max"] = c + 0.02
    assert np.array_equal(oracle.broadphase(boxes), numpy_all_pairs(boxes))


def test_pair_set_is_axis_independent(stq, oracle):
    """Sweeping along x emits exactly the 3-D inclusive overlaps: permuting the
    coordinate axes leaves the pair set unchanged (why any sweep axis is exact)."""
    m = stq.cloth_pair(g=20, seed=4)
    boxes = oracle.construct_boxes(m.V0, m.V1, m.E, m.F, stq.AABB_DTYPE)
    base = oracle.broadphase(boxes)
    for perm in ([1, 0, 2], [2, 1, 0], [1, 2, 0]):
        b = boxes.copy()
        b["min"] = boxes["min"][:, perm]
        b["max"] = boxes["max"][:, perm]
        assert np.array_equal(oracle.broadphase(b), base)


def test_raw_sweep_orientation_and_prefix(stq, oracle):
    """stq::cpu::sweep emits (earlier, later) in sort order, once per pair; a
    prefix of start boxes yields exactly the pairs whose earlier box is in it
    (the batching of sweep_cpu_single_batch, src/cpu/sweep.cpp:144-157)."""
    m = stq.cloth_pair(g=16, seed=5)
    boxes = oracle.construct_boxes(m.V0, m.V1, m.E, m.F, stq.AABB_DTYPE)
    s = boxes.copy()
    oracle.sort_along_xaxis(s)
    pos = np.empty(len(s), np.int64)
    pos[s["id"]] = np.arange(len(s))
    raw = oracle.sweep_sorted(s, len(s))
    assert np.all(pos[raw[:, 0]] < pos[raw[:, 1]])
    full = oracle.canonical(raw)
    assert len(full) == len(raw)
    assert np.array_equal(full, oracle.broadphase(boxes))
    n = len(s) // 3
    part = oracle.sweep_sorted(s, n)
    assert np.all(pos[part[:, 0]] < n)
    assert len(part) == int(np.sum(pos[raw[:, 0]] < n))


def test_compare_counts(oracle):
    a = np.array([[0, 1], [0, 2], [3, 4]], np.int32)
    b = np.array([[0, 2], [3, 4], [5, 6], [7, 8]], np.int32)
    assert oracle.compare(a, b) == (1, 2)
