"""Bit-exact parity at the full benchmark configurations.

Every scene the benchmark times is checked here against the CPU oracle (the
reference's src/cpu sweep, sort along x + sweep with the is_valid_pair /
covertex filter, src/cpu/sweep.cpp:94-121): the whole sorted pair list, not a
count.
  - the large single scenes: 16 crumpled sheets of 250^2 (5,968,048 boxes) and
    of 290^2 (8,036,528 boxes), device-built boxes and their pairs;
  - the 256-scene cloth-pair batch (box counts log-uniform in [1e3, 2e5])
    through the fused graph-captured call, scene by scene against 256 plain
    per-scene runs and against the oracle;
  - the skewed batch, 64 scenes x 500,000 random boxes with 5% slivers, sweep
    axis x in half of the scenes and largest variance in the other half,
    scene by scene against the oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def sorted_device_pairs(ctx, pairs, count):
    """The first `count` pairs, sorted lexicographically on the device."""
    ctx.sort_pairs(pairs, count)
    return pairs[:count].cpu().numpy()


def split_by_scene(pairs, box_off):
    """Lexicographically sorted batch pairs (ids global to the batch) -> the
    slice of each scene (both ids of a pair lie in one scene)."""
    cut = np.searchsorted(pairs[:, 0], np.asarray(box_off, np.int64), side="left")
    return [pairs[cut[s]:cut[s + 1]] for s in range(len(box_off) - 1)]


@pytest.mark.parametrize("g, n_boxes", [(250, 5_968_048), (290, 8_036_528)])
def test_crumpled_scene_vs_oracle(stq, oracle, cuda, ctx, g, n_boxes):
    import torch

    mesh = stq.crumpled_sheets(16, g, 0.05, 0.005, 1)
    n = mesh.num_boxes
    assert n == n_boxes
    V0, V1, E, F = (torch.from_numpy(x).to(cuda) for x in (mesh.V0, mesh.V1, mesh.E, mesh.F))
    boxes = torch.empty((n, 11), dtype=torch.int32, device=cuda)
    ctx.build_boxes(V0, V1, E, F, boxes)
    want_boxes = oracle.construct_boxes(mesh.V0, mesh.V1, mesh.E, mesh.F, stq.AABB_DTYPE)
    assert boxes.cpu().numpy().tobytes() == want_boxes.tobytes()
    ctx.prepare(boxes, n, stq.AXIS_AUTO)
    cap = 24 * n
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    r = ctx.sweep_prepared(pairs, cap)
    assert r.status == stq.STQ_OK
    got = sorted_device_pairs(ctx, pairs, r.count)
    want = oracle.broadphase(want_boxes)
    assert len(want) > 10_000_000
    assert got.shape == want.shape and np.array_equal(got, want)


def test_batch_256_scenes_vs_plain_runs_and_oracle(stq, oracle, cuda, ctx):
    import torch

    meshes = stq.batch_scenes(256, 1e3, 2e5, seed=2)
    V0, V1, E, F, vo, eo, fo = stq.concat_meshes(meshes)
    d = [torch.from_numpy(x).to(cuda) for x in (V0, V1, E, F)]
    N = int(sum(m.num_boxes for m in meshes))
    box_off = np.concatenate([[0], np.cumsum([m.num_boxes for m in meshes])]).astype(np.int64)
    cap = 40 * N
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    r, per = ctx.batch_broadphase(d[0], d[1], vo, d[2], eo, d[3], fo, pairs, cap)
    assert r.status == stq.STQ_OK and int(per.sum()) == r.count
    batch = split_by_scene(sorted_device_pairs(ctx, pairs, r.count), box_off)
    plain_pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    boxes = torch.empty((max(m.num_boxes for m in meshes), 11), dtype=torch.int32, device=cuda)
    for k, m in enumerate(meshes):
        v = slice(int(vo[k]), int(vo[k + 1]))
        ctx.build_boxes(d[0][v], d[1][v], d[2][int(eo[k]):int(eo[k + 1])], d[3][int(fo[k]):int(fo[k + 1])], boxes)
        rp = ctx.sweep(boxes, m.num_boxes, plain_pairs, cap, axis=stq.AXIS_AUTO)
        assert rp.status == stq.STQ_OK
        plain = sorted_device_pairs(ctx, plain_pairs, rp.count)
        want = oracle.broadphase(oracle.construct_boxes(m.V0, m.V1, m.E, m.F, stq.AABB_DTYPE))
        assert np.array_equal(plain, want), f"plain run of scene {k}"
        assert per[k] == len(want), f"batched count of scene {k}"
        assert np.array_equal(batch[k] - box_off[k], want), f"batched scene {k}"


def test_skewed_64x500k_batch_vs_oracle(stq, oracle, cuda, ctx):
    import torch

    n_s, per = 64, 500_000
    scenes = [stq.random_boxes(per, sliver_frac=0.05, seed=1000 + k) for k in range(n_s)]
    allb = np.concatenate(scenes)
    allb["id"] = np.arange(len(allb), dtype=np.int32)
    box_off = np.arange(n_s + 1, dtype=np.int64) * per
    axes = [0 if k % 2 == 0 else stq.AXIS_AUTO for k in range(n_s)]
    boxes = torch.from_numpy(allb.view(np.int32).reshape(-1, 11).copy()).to(cuda)
    cap = 8 * len(allb)
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    ctx.batch_prepare(boxes, box_off, axes=axes)
    r = ctx.sweep_prepared(pairs, cap)
    assert r.status == stq.STQ_OK
    counts = ctx.batch_scene_pairs(n_s)
    got = split_by_scene(sorted_device_pairs(ctx, pairs, r.count), box_off)
    for k in range(n_s):
        want = oracle.broadphase(allb[box_off[k]:box_off[k + 1]])
        assert counts[k] == len(want), f"count of scene {k}"
        assert np.array_equal(got[k], want), f"scene {k}"
