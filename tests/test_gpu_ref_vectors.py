"""The GPU pipeline against outputs of the reference's own CPU code
(tests/golden/ref_vectors.npz, written by tests/golden/make_ref_golden.py from
the reference's src/cpu/aabb.cpp and src/cpu/sweep.cpp compiled unchanged):
device-built boxes bit for bit, and the sorted pair lists of the sweep under
every sweep axis."""
import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("axis", [-1, 0, 1, 2])
def test_gpu_matches_reference_vectors(stq, ctx, cuda, axis):
    import torch

    d = np.load(GOLDEN / "ref_vectors.npz")
    for case in d["cases"]:
        kind, name = str(case).split(":")
        want_boxes = d[f"{name}.boxes"].reshape(-1).view(stq.AABB_DTYPE)
        n = len(want_boxes)
        boxes = torch.empty((max(n, 1), 11), dtype=torch.int32, device=cuda)
        if kind == "mesh":
            V0, V1, E, F = (torch.from_numpy(np.ascontiguousarray(d[f"{name}.{k}"])).to(cuda)
                            for k in ("V0", "V1", "E", "F"))
            ctx.build_boxes(V0, V1, E, F, boxes, float(d[f"{name}.r"]))
            assert boxes[:n].cpu().numpy().tobytes() == want_boxes.tobytes(), name
        else:
            boxes[:n] = torch.from_numpy(want_boxes.view(np.int32).reshape(-1, 11).copy()).to(cuda)
        want = d[f"{name}.pairs"]
        cap = max(4 * len(want), 64)
        pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
        r = ctx.sweep(boxes, n, pairs, cap, axis=axis)
        assert r.status == stq.STQ_OK, name
        ctx.sort_pairs(pairs, r.count)
        assert np.array_equal(pairs[: r.count].cpu().numpy(), want), name
