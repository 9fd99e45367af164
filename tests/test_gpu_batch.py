"""Batched STQ on the GPU: many scenes through one launch sequence must give,
scene by scene, exactly the pairs of the oracle run on that scene alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(arr, cuda):
    import torch

    return torch.from_numpy(np.ascontiguousarray(arr)).to(cuda)


@pytest.fixture(scope="module")
def scenes(stq, oracle):
    """24 cloth-pair scenes, box counts log-uniform in [1e3, 6e4], plus their
    oracle pair lists."""
    meshes = stq.batch_scenes(24, 1e3, 6e4, seed=5)
    want = []
    for m in meshes:
        b = oracle.construct_boxes(m.V0, m.V1, m.E, m.F, stq.AABB_DTYPE)
        want.append(oracle.broadphase(b))
    return meshes, want


def split_by_scene(pairs, box_off):
    s = np.searchsorted(box_off, pairs[:, 0], side="right") - 1
    s2 = np.searchsorted(box_off, pairs[:, 1], side="right") - 1
    assert np.array_equal(s, s2), "a pair crosses scenes"
    return s


def check_batch(oracle, raw, box_off, want, per_scene=None):
    got = oracle.canonical(raw)
    assert len(got) == len(raw), "duplicate pairs"
    sid = split_by_scene(got, box_off)
    for k, w in enumerate(want):
        local = got[sid == k] - box_off[k]
        assert np.array_equal(local, w), f"scene {k}"
        if per_scene is not None:
            assert per_scene[k] == len(w), f"scene {k} count"


def test_batch_build_matches_single_builds(ctx, stq, oracle, cuda, scenes):
    import torch

    meshes, _ = scenes
    V0, V1, E, F, vo, eo, fo = stq.concat_meshes(meshes)
    n = sum(m.num_boxes for m in meshes)
    out = torch.empty((n, 11), dtype=torch.int32, device=cuda)
    bo = ctx.batch_build_boxes(dev(V0, cuda), dev(V1, cuda), vo, dev(E, cuda), eo, dev(F, cuda), fo, out)
    assert bo[-1] == n
    got = out.cpu().numpy().view(stq.AABB_DTYPE).reshape(-1)
    for k, m in enumerate(meshes):
        want = oracle.construct_boxes(m.V0, m.V1, m.E, m.F, stq.AABB_DTYPE)
        part = got[bo[k]:bo[k + 1]].copy()
        assert np.array_equal(part["id"], np.arange(bo[k], bo[k + 1]))
        part["id"] -= bo[k]
        assert part.tobytes() == want.tobytes(), k


@pytest.mark.parametrize("shape", [1, 2])
@pytest.mark.parametrize("mixed_axes", [False, True])
@pytest.mark.parametrize("run_cap", [0, 3])
def test_batch_prepare_and_sweep(ctx, stq, oracle, cuda, scenes, mixed_axes, run_cap, shape):
    """Scene by scene against the oracle, with the per-scene pair counts
    (queue and flat shapes)."""
    import torch

    meshes, want = scenes
    ctx.set_option(stq.OPT_RUN_CAP, run_cap)
    ctx.set_option(stq.OPT_SWEEP_SHAPE, shape)
    V0, V1, E, F, vo, eo, fo = stq.concat_meshes(meshes)
    n = sum(m.num_boxes for m in meshes)
    boxes = torch.empty((n, 11), dtype=torch.int32, device=cuda)
    bo = ctx.batch_build_boxes(dev(V0, cuda), dev(V1, cuda), vo, dev(E, cuda), eo, dev(F, cuda), fo, boxes)
    axes = [(-1, 0, 1, 2)[k % 4] for k in range(len(meshes))] if mixed_axes else None
    ctx.batch_prepare(boxes, bo, axes=axes)
    cap = sum(len(w) for w in want) + 16
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    r = ctx.sweep_prepared(pairs, cap)
    assert r.status == stq.STQ_OK and r.count == cap - 16
    per = ctx.batch_scene_pairs(len(meshes))
    check_batch(oracle, pairs[: r.count].cpu().numpy(), bo, want, per)


def test_batch_overflow_resume(ctx, stq, oracle, cuda, scenes):
    import torch

    meshes, want = scenes
    V0, V1, E, F, vo, eo, fo = stq.concat_meshes(meshes)
    n = sum(m.num_boxes for m in meshes)
    boxes = torch.empty((n, 11), dtype=torch.int32, device=cuda)
    bo = ctx.batch_build_boxes(dev(V0, cuda), dev(V1, cuda), vo, dev(E, cuda), eo, dev(F, cuda), fo, boxes)
    ctx.batch_prepare(boxes, bo)
    total = sum(len(w) for w in want)
    cap = total // 5 + 1
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    start, parts = 0, []
    while start < ctx.prepared_length:
        r = ctx.sweep_prepared(pairs, cap, start=start)
        parts.append(pairs[: r.count].cpu().numpy().copy())
        start = r.next_start
    assert len(parts) >= 5
    check_batch(oracle, np.concatenate(parts), bo, want)


@pytest.mark.parametrize("graph", [1, 2])
@pytest.mark.parametrize("shape", [1, 2])
def test_batch_broadphase_fused(ctx, stq, oracle, cuda, scenes, graph, shape):
    import torch

    meshes, want = scenes
    ctx.set_option(stq.OPT_GRAPH, graph)
    ctx.set_option(stq.OPT_SWEEP_SHAPE, shape)
    V0, V1, E, F, vo, eo, fo = stq.concat_meshes(meshes)
    n = sum(m.num_boxes for m in meshes)
    bo = np.concatenate([[0], np.cumsum([m.num_boxes for m in meshes])])
    d = [dev(x, cuda) for x in (V0, V1, E, F)]
    cap = sum(len(w) for w in want) + 100
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    for rep in range(3):  # the captured graph is replayed
        r, per = ctx.batch_broadphase(d[0], d[1], vo, d[2], eo, d[3], fo, pairs, cap)
        assert r.status == stq.STQ_OK
        check_batch(oracle, pairs[: r.count].cpu().numpy(), bo, want, per)
    # a different batch composition within the same capacities reuses the graph
    sub = meshes[::-1]
    V0b, V1b, Eb, Fb, vob, eob, fob = stq.concat_meshes(sub)
    for t, src in zip(d, (V0b, V1b, Eb, Fb)):
        t.copy_(dev(src, cuda))
    bob = np.concatenate([[0], np.cumsum([m.num_boxes for m in sub])])
    r, per = ctx.batch_broadphase(d[0], d[1], vob, d[2], eob, d[3], fob, pairs, cap)
    check_batch(oracle, pairs[: r.count].cpu().numpy(), bob, want[::-1], per)
    # too small a buffer reports overflow and the true total
    r, per = ctx.batch_broadphase(d[0], d[1], vob, d[2], eob, d[3], fob, pairs, 1000)
    assert r.status == stq.STQ_OVERFLOW and r.total == cap - 100 and r.count == 1000


def test_batch_with_empty_and_tiny_scenes(ctx, stq, oracle, cuda):
    import torch

    boxes = []
    for k, n in enumerate([0, 1, 2, 500, 0, 3000]):
        b = stq.random_boxes(n, seed=40 + k) if n else np.zeros(0, stq.AABB_DTYPE)
        if n:
            c = 0.5 * (b["min"] + b["max"])
            b["min"], b["max"] = c - 0.05, c + 0.05
        boxes.append(b)
    bo = np.concatenate([[0], np.cumsum([len(b) for b in boxes])]).astype(np.int64)
    allb = np.concatenate(boxes)
    allb["id"] = np.arange(len(allb))
    want = []
    for k, b in enumerate(boxes):
        bb = allb[bo[k]:bo[k + 1]].copy()
        want.append(oracle.broadphase(bb) - bo[k] if len(bb) else np.zeros((0, 2), np.int32))
    d = torch.from_numpy(allb.view(np.int32).reshape(-1, 11).copy()).to(cuda)
    ctx.batch_prepare(d, bo)
    cap = sum(len(w) for w in want) + 8
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    r = ctx.sweep_prepared(pairs, cap)
    check_batch(oracle, pairs[: r.count].cpu().numpy(), bo, want, ctx.batch_scene_pairs(len(boxes)))


def test_batch_skewed_boxes_mixed_axes(ctx, stq, oracle, cuda):
    """Random boxes with 5% slivers stretched 200x, several scenes in one batch,
    the sweep axis fixed to x in half of them and chosen by variance in the
    others: each scene's pairs equal the oracle's on that scene alone."""
    import torch

    sizes = [30_000, 1, 12_000, 45_000, 0, 25_000]
    boxes = [stq.random_boxes(n, sliver_frac=0.05, seed=70 + k) if n else np.zeros(0, stq.AABB_DTYPE)
             for k, n in enumerate(sizes)]
    bo = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    allb = np.concatenate(boxes)
    allb["id"] = np.arange(len(allb))
    want = []
    for k in range(len(sizes)):
        bb = allb[bo[k]:bo[k + 1]].copy()
        want.append(oracle.broadphase(bb) - bo[k] if len(bb) else np.zeros((0, 2), np.int32))
    d = torch.from_numpy(allb.view(np.int32).reshape(-1, 11).copy()).to(cuda)
    axes = [0 if k % 2 == 0 else -1 for k in range(len(sizes))]
    ctx.batch_prepare(d, bo, axes=axes)
    cap = sum(len(w) for w in want) + 8
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    r = ctx.sweep_prepared(pairs, cap)
    assert r.status == stq.STQ_OK
    check_batch(oracle, pairs[: r.count].cpu().numpy(), bo, want, ctx.batch_scene_pairs(len(sizes)))


def test_autotune_keeps_results_exact_and_caches(ctx, stq, oracle, cuda, scenes):
    import torch

    meshes, want = scenes
    V0, V1, E, F, vo, eo, fo = stq.concat_meshes(meshes)
    n = sum(m.num_boxes for m in meshes)
    boxes = torch.empty((n, 11), dtype=torch.int32, device=cuda)
    bo = ctx.batch_build_boxes(dev(V0, cuda), dev(V1, cuda), vo, dev(E, cuda), eo, dev(F, cuda), fo, boxes)
    cap = sum(len(w) for w in want) + 16
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    ms, settings = ctx.autotune(boxes, bo, pairs, cap)
    assert ms > 0
    assert settings["shape"] in (stq.SHAPE_QUEUE, stq.SHAPE_FLAT)
    assert settings["lanes"] in (1, 4, 8, 16) and settings["queue"] in (16, 32, 64)
    assert settings["per_lane"] in (2, 4, 8) or settings["lanes"] > 1
    assert settings["queue"] >= 32 or settings["lanes"] > 1
    assert settings["run_cap"] in (512, 4096)
    assert settings["block"] in (128, 256, 512) and settings["radix_bits"] in (4, 8)
    assert settings["cell_scale"] in (1, 2, 4, 8)
    r = ctx.sweep_prepared(pairs, cap)
    check_batch(oracle, pairs[: r.count].cpu().numpy(), bo, want, ctx.batch_scene_pairs(len(meshes)))
    ms2, settings2 = ctx.autotune(boxes, bo, pairs, cap)  # same shape bucket: cached
    assert ms2 == 0 and settings2 == settings
