"""The oracle restatement pinned to the reference's own CPU code.

tests/golden/ref_vectors.npz holds outputs of the reference's src/cpu/aabb.cpp
and src/cpu/sweep.cpp, compiled unchanged (tests/golden/make_ref_golden.py);
the oracle must reproduce them bit for bit. Where the reference's source tree
is present, oracle/_ref/libstq_ref.so is built from it and the oracle is
also checked against it live on the full-size cloth pair, a 1M-box slice of
the 16-sheet scene and a skewed random scene.
"""
import numpy as np
import pytest

from conftest import GOLDEN


@pytest.fixture(scope="module")
def ref_vectors():
    return np.load(GOLDEN / "ref_vectors.npz")


def test_oracle_matches_reference_vectors(stq, oracle, ref_vectors):
    d = ref_vectors
    assert len(d["cases"]) >= 20
    for case in d["cases"]:
        kind, name = str(case).split(":")
        want_boxes = d[f"{name}.boxes"].reshape(-1).view(stq.AABB_DTYPE)
        if kind == "mesh":
            boxes = oracle.construct_boxes(d[f"{name}.V0"], d[f"{name}.V1"], d[f"{name}.E"], d[f"{name}.F"],
                                           stq.AABB_DTYPE, float(d[f"{name}.r"]))
            assert boxes.tobytes() == want_boxes.tobytes(), name
        assert np.array_equal(oracle.broadphase(want_boxes), d[f"{name}.pairs"]), name


@pytest.fixture(scope="module")
def ref_build(oracle):
    if not oracle.build_ref():
        pytest.skip("the reference's source tree is not present: oracle/_ref cannot be built")
    return oracle


@pytest.mark.parametrize("r", [0.0, 2.5e-3])
def test_oracle_matches_reference_build_cloth200(stq, oracle, ref_build, r):
    m = stq.cloth_pair(g=200, z_offset=0.01, sigma=0.003, seed=0)
    boxes = oracle.construct_boxes(m.V0, m.V1, m.E, m.F, stq.AABB_DTYPE, r)
    ref_boxes = oracle.ref_construct_boxes(m.V0, m.V1, m.E, m.F, stq.AABB_DTYPE, r)
    assert boxes.tobytes() == ref_boxes.tobytes()
    want = oracle.ref_broadphase(ref_boxes)
    assert len(want) > 1_000_000
    assert np.array_equal(oracle.broadphase(boxes), want)


def test_oracle_matches_reference_build_crumpled_slice(stq, oracle, ref_build):
    m = stq.crumpled_sheets(16, 250, 0.05, 0.005, 1)
    boxes = oracle.construct_boxes(m.V0, m.V1, m.E, m.F, stq.AABB_DTYPE)
    ref_boxes = oracle.ref_construct_boxes(m.V0, m.V1, m.E, m.F, stq.AABB_DTYPE)
    assert boxes.tobytes() == ref_boxes.tobytes()
    part = np.ascontiguousarray(boxes[::6])  # ~1M boxes of every kind, ids kept
    assert len(part) > 990_000
    want = oracle.ref_broadphase(part)
    assert len(want) > 100_000
    assert np.array_equal(oracle.broadphase(part), want)


def test_oracle_matches_reference_build_skewed(stq, oracle, ref_build):
    b = stq.random_boxes(200_000, sliver_frac=0.05, seed=9)
    want = oracle.ref_broadphase(b)
    assert len(want) > 1000
    assert np.array_equal(oracle.broadphase(b), want)
