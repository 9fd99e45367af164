"""GPU parity: the CUDA path through the C ABI against the CPU oracle and the
golden fixtures. Integer/index results and float bounds are bit-exact."""
import numpy as np
import pytest

from conftest import decode_boxes, decode_mesh, expected_pairs

pytestmark = pytest.mark.gpu


def dev(arr, cuda):
    import torch

    return torch.from_numpy(np.ascontiguousarray(arr)).to(cuda)


def boxes_dev(boxes, cuda):
    import torch

    flat = np.ascontiguousarray(boxes).view(np.int32).reshape(-1, 11)
    return torch.from_numpy(flat.copy()).to(cuda)


def build_dev(ctx, mesh_arrays, cuda, r=0.0):
    import torch

    V0, V1, E, F = mesh_arrays
    n = V0.shape[0] + E.shape[0] + F.shape[0]
    out = torch.empty((max(n, 1), 11), dtype=torch.int32, device=cuda)
    ctx.build_boxes(dev(V0, cuda), dev(V1, cuda), dev(E.reshape(-1, 2), cuda),
                    dev(F.reshape(-1, 3), cuda), out, r)
    return out, n


def to_host_boxes(t, n, stq):
    return t[:n].cpu().numpy().view(stq.AABB_DTYPE).reshape(-1)


def sweep_pairs(ctx, stq, oracle, bdev, n, cuda, axis=0, cap=None):
    import torch

    cap = cap if cap is not None else max(16, 64 * n)
    pairs = torch.empty((max(cap, 1), 2), dtype=torch.int32, device=cuda)
    r = ctx.sweep(bdev, n, pairs, cap, axis=axis)
    assert r.status == stq.STQ_OK, r
    assert r.count == r.total and r.next_start == ctx.prepared_length
    raw = pairs[: r.count].cpu().numpy()
    assert np.all(raw[:, 0] < raw[:, 1]) if len(raw) else True  # (smaller id, larger id)
    got = oracle.canonical(raw)
    assert len(got) == len(raw), "duplicate pairs"
    return got


# ---- box construction -----------------------------------------------------------

def test_build_kat_meshes(ctx, stq, kat, cuda):
    for name, m in kat["meshes"].items():
        arrays = decode_mesh(m)
        out, n = build_dev(ctx, arrays, cuda, m["r"])
        got = to_host_boxes(out, n, stq)
        want = decode_boxes(m["boxes"], stq.AABB_DTYPE)
        assert got.tobytes() == want.tobytes(), name


def test_build_cloth_fixture(ctx, stq, cloth_fixture, cuda):
    f = cloth_fixture
    out, n = build_dev(ctx, (f["V0"], f["V1"], f["E"], f["F"]), cuda)
    got = to_host_boxes(out, n, stq)
    assert np.array_equal(got["min"].view(np.uint32), f["box_min"].view(np.uint32))
    assert np.array_equal(got["max"].view(np.uint32), f["box_max"].view(np.uint32))
    assert np.array_equal(got["vertex_ids"], f["vertex_ids"])


@pytest.mark.parametrize("r", [0.0, 1e-4, 2.5e-3])
def test_build_cloth_pair_vs_oracle(ctx, stq, oracle, cuda, r):
    m = stq.cloth_pair(g=200, seed=0)
    out, n = build_dev(ctx, (m.V0, m.V1, m.E, m.F), cuda, r)
    got = to_host_boxes(out, n, stq)
    want = oracle.construct_boxes(m.V0, m.V1, m.E, m.F, stq.AABB_DTYPE, r)
    assert got.tobytes() == want.tobytes()


def test_build_rejects_bad_index(ctx, stq, cuda):
    m = stq.cloth_pair(g=8, seed=1)
    E = m.E.copy()
    E[3, 1] = m.V0.shape[0]
    with pytest.raises(stq.STQError) as e:
        build_dev(ctx, (m.V0, m.V1, E, m.F), cuda)
    assert e.value.status == stq.STQ_ERR_INVALID_INPUT


# ---- sweep ------------------------------------------------------------------------

@pytest.mark.parametrize("axis", [-1, 0, 1, 2])
def test_sweep_kat_cases(ctx, stq, oracle, kat, cuda, axis):
    for name, case in kat["pairs"].items():
        boxes = decode_boxes(case["boxes"], stq.AABB_DTYPE)
        got = sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, axis)
        assert np.array_equal(got, expected_pairs(case["expected"])), (name, axis)


def test_sweep_kat_meshes_device_built(ctx, stq, oracle, kat, cuda):
    for name, m in kat["meshes"].items():
        out, n = build_dev(ctx, decode_mesh(m), cuda, m["r"])
        got = sweep_pairs(ctx, stq, oracle, out, n, cuda, -1)
        assert np.array_equal(got, expected_pairs(m["expected"])), name


def test_sweep_cloth_fixture(ctx, stq, oracle, cloth_fixture, cuda):
    f = cloth_fixture
    out, n = build_dev(ctx, (f["V0"], f["V1"], f["E"], f["F"]), cuda)
    for axis in (-1, 0, 1, 2):
        assert np.array_equal(sweep_pairs(ctx, stq, oracle, out, n, cuda, axis), f["pairs"])


@pytest.fixture(scope="module")
def c0(stq, oracle):
    """The single-scene cloth pair: 2 sheets of 200^2 vertices, 476,806 boxes."""
    m = stq.cloth_pair(g=200, seed=0)
    boxes = oracle.construct_boxes(m.V0, m.V1, m.E, m.F, stq.AABB_DTYPE)
    return m, boxes, oracle.broadphase(boxes)


@pytest.mark.parametrize("axis", [-1, 0, 1, 2])
def test_sweep_cloth_pair_vs_oracle(ctx, stq, oracle, cuda, c0, axis):
    m, boxes, want = c0
    out, n = build_dev(ctx, (m.V0, m.V1, m.E, m.F), cuda)
    got = sweep_pairs(ctx, stq, oracle, out, n, cuda, axis)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("lanes", [1, 2, 4, 8, 16, 32])
@pytest.mark.parametrize("queue", [16, 32, 64, 128])
@pytest.mark.parametrize("block", [128, 256, 512])
def test_sweep_tuning_space(ctx, stq, oracle, cuda, c0, lanes, queue, block):
    """Queue depth 16 holds one entry per lane group for groups of 2 or more
    lanes; one start box per lane keeps a ring of at least 32."""
    m, boxes, want = c0
    ctx.set_option(stq.OPT_SWEEP_SHAPE, stq.SHAPE_QUEUE)
    ctx.set_option(stq.OPT_LANES, lanes)
    ctx.set_option(stq.OPT_QUEUE, queue)
    ctx.set_option(stq.OPT_BLOCK, block)
    got = sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, 0)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("per_lane", [1, 2, 4, 8])
@pytest.mark.parametrize("queue", [32, 128])
@pytest.mark.parametrize("block", [128, 512])
def test_sweep_one_lane_per_box(ctx, stq, oracle, cuda, c0, per_lane, queue, block):
    m, boxes, want = c0
    ctx.set_option(stq.OPT_SWEEP_SHAPE, stq.SHAPE_QUEUE)
    ctx.set_option(stq.OPT_LANES, 1)
    ctx.set_option(stq.OPT_PER_LANE, per_lane)
    ctx.set_option(stq.OPT_QUEUE, queue)
    ctx.set_option(stq.OPT_BLOCK, block)
    assert ctx.get_option(stq.OPT_PER_LANE) == per_lane
    for axis in (0, -1):
        got = sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, axis)
        assert np.array_equal(got, want), axis


@pytest.mark.parametrize("steps", [2, 4])
@pytest.mark.parametrize("block", [128, 256])
def test_sweep_flat_shape(ctx, stq, oracle, cuda, c0, steps, block):
    """The flat shape (runs of 32 start boxes laid end to end, one candidate
    per lane and step, run ends from the gather) gives the oracle's pairs and
    tests the same candidates as the queue shape."""
    m, boxes, want = c0
    ctx.set_option(stq.OPT_SWEEP_SHAPE, stq.SHAPE_QUEUE)
    sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, 0)
    cand = ctx.candidates
    ctx.set_option(stq.OPT_SWEEP_SHAPE, stq.SHAPE_FLAT)
    ctx.set_option(stq.OPT_PER_LANE, steps)
    ctx.set_option(stq.OPT_BLOCK, block)
    assert ctx.get_option(stq.OPT_SWEEP_SHAPE) == stq.SHAPE_FLAT
    for axis in (0, -1, 1, 2):
        got = sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, axis)
        assert np.array_equal(got, want), axis
        if axis == 0:
            assert ctx.candidates == cand
    for cells in (1, 7):  # one cell; a fixed grid
        ctx.set_option(stq.OPT_CELLS, cells)
        got = sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, -1)
        assert np.array_equal(got, want), cells


@pytest.mark.parametrize("run_cap", [1, 5, 64])
@pytest.mark.parametrize("shape", [(1, 4, 1), (1, 8, 1), (8, 0, 1), (2, 0, 1), (1, 2, 2), (1, 4, 2)])
def test_long_runs_go_to_the_warp_pass(ctx, stq, oracle, cuda, c0, run_cap, shape):
    """Runs longer than the cap continue in the warp pass: same pairs, same
    candidates tested as without the hand-over (queue and flat shapes)."""
    m, boxes, want = c0
    ctx.set_option(stq.OPT_LANES, shape[0])
    ctx.set_option(stq.OPT_SWEEP_SHAPE, shape[2])
    if shape[1]:
        ctx.set_option(stq.OPT_PER_LANE, shape[1])
    ctx.set_option(stq.OPT_RUN_CAP, (1 << 20))
    sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, 0)
    cand = ctx.candidates
    ctx.set_option(stq.OPT_RUN_CAP, run_cap)
    assert ctx.get_option(stq.OPT_RUN_CAP) == run_cap
    got = sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, 0)
    assert np.array_equal(got, want)
    assert ctx.candidates == cand


@pytest.fixture(scope="module")
def dense_cloth(stq, oracle):
    """Two cloth sheets 0.002 apart with large motion (sigma 0.03): coarse
    cells, long lists and runs of thousands of candidates."""
    m = stq.cloth_pair(g=90, z_offset=0.002, sigma=0.03, seed=9)
    boxes = oracle.construct_boxes(m.V0, m.V1, m.E, m.F, stq.AABB_DTYPE)
    return m, boxes, oracle.broadphase(boxes)


@pytest.mark.parametrize("shape", [1, 2])
@pytest.mark.parametrize("run_cap", [0, 16])
def test_dense_scene_vs_oracle(ctx, stq, oracle, cuda, dense_cloth, run_cap, shape):
    import torch

    m, boxes, want = dense_cloth
    assert len(want) > 40 * len(boxes)
    ctx.set_option(stq.OPT_RUN_CAP, run_cap)
    ctx.set_option(stq.OPT_SWEEP_SHAPE, shape)
    got = sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, -1, cap=len(want) + 8)
    assert np.array_equal(got, want)
    # overflow and resume: count mode adds the warp pass's counts
    cap = len(want) // 7 + 1
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    ctx.prepare(boxes_dev(boxes, cuda), len(boxes), -1)
    start, chunks = 0, []
    while start < ctx.prepared_length:
        r = ctx.sweep_prepared(pairs, cap, start=start)
        assert r.next_start > start
        chunks.append(pairs[: r.count].cpu().numpy().copy())
        start = r.next_start
    assert len(chunks) >= 7
    allp = np.concatenate(chunks)
    assert np.array_equal(oracle.canonical(allp), want) and len(allp) == len(want)


def test_sweep_radix_4bit(ctx, stq, oracle, cuda, c0):
    m, boxes, want = c0
    ctx.set_option(stq.OPT_RADIX_BITS, 4)
    assert np.array_equal(sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, 1), want)


@pytest.mark.parametrize("shape", [1, 2])
@pytest.mark.parametrize("seed", [3, 4])
def test_sweep_skewed_boxes_vs_oracle(ctx, stq, oracle, cuda, seed, shape):
    ctx.set_option(stq.OPT_SWEEP_SHAPE, shape)
    boxes = stq.random_boxes(200_000, sliver_frac=0.05, seed=seed)
    want = oracle.broadphase(boxes)
    for axis in (0, -1):
        got = sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, axis)
        assert np.array_equal(got, want), axis


def test_sweep_ids_are_box_ids_not_positions(ctx, stq, oracle, cuda, c0):
    m, boxes, want = c0
    rng = np.random.default_rng(0)
    perm = rng.permutation(len(boxes))
    shuffled = boxes[perm]
    got = sweep_pairs(ctx, stq, oracle, boxes_dev(shuffled, cuda), len(boxes), cuda, 0)
    assert np.array_equal(got, want)


# ---- overflow and resume ---------------------------------------------------------------

@pytest.mark.parametrize("shape", [1, 2])
@pytest.mark.parametrize("div", [2, 7, 50])
def test_overflow_resume_covers_everything_once(ctx, stq, oracle, cuda, c0, div, shape):
    import torch

    m, boxes, want = c0
    ctx.set_option(stq.OPT_SWEEP_SHAPE, shape)
    cap = len(want) // div + 1
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    ctx.prepare(boxes_dev(boxes, cuda), len(boxes), 0)
    length = ctx.prepared_length
    start, chunks, calls = 0, [], 0
    while start < length:
        r = ctx.sweep_prepared(pairs, cap, start=start)
        assert r.count <= cap
        assert r.next_start > start
        if r.next_start < length:
            assert r.status == stq.STQ_OVERFLOW
        chunks.append(pairs[: r.count].cpu().numpy().copy())
        start = r.next_start
        calls += 1
    assert calls >= div
    allp = np.concatenate(chunks)
    got = oracle.canonical(allp)
    assert len(got) == len(allp)
    assert np.array_equal(got, want)


def test_max_start_batches(ctx, stq, oracle, cuda, c0):
    """The reference's MAX_OVERLAP_CUTOFF batching over start boxes with the
    tidstart cursor (src/simulation.cu:239, 747)."""
    import torch

    m, boxes, want = c0
    cap = len(want)
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    for cells in (1, 0):
        ctx.set_option(stq.OPT_CELLS, cells)
        ctx.prepare(boxes_dev(boxes, cuda), len(boxes), -1)
        length = ctx.prepared_length
        if cells == 1:  # one cell: vertex, edge and face lists, two inner sentinels
            assert length == len(boxes) + 2
        start, parts = 0, []
        while start < length:
            r = ctx.sweep_prepared(pairs, cap, start=start, max_start=length // 5 + 1)
            assert r.status == stq.STQ_OK
            parts.append(pairs[: r.count].cpu().numpy().copy())
            start = r.next_start
        assert len(parts) == 5
        assert np.array_equal(oracle.canonical(np.concatenate(parts)), want)


def test_capacity_too_small_for_one_box(ctx, stq, cuda):
    import torch

    boxes = np.zeros(6, stq.AABB_DTYPE)
    for i in range(6):
        boxes[i] = (i, [0, 0, 0], [1, 1, 1], [i, -i - 1, -i - 1] if i == 0 else [10 + i, 20 + i, 30 + i], i)
    pairs = torch.empty((2, 2), dtype=torch.int32, device=cuda)
    with pytest.raises(stq.STQError) as e:
        ctx.sweep(boxes_dev(boxes, cuda), 6, pairs, 2)
    assert e.value.status == stq.STQ_ERR_CAPACITY


# ---- edge cases ---------------------------------------------------------------------------

def test_empty_and_tiny(ctx, stq, oracle, cuda):
    import torch

    pairs = torch.empty((4, 2), dtype=torch.int32, device=cuda)
    r = ctx.sweep(None, 0, pairs, 4)
    assert (r.status, r.count, r.next_start) == (stq.STQ_OK, 0, 0)
    one = np.zeros(1, stq.AABB_DTYPE)
    one[0] = (0, [0, 0, 0], [1, 1, 1], [0, -1, -1], 0)
    r = ctx.sweep(boxes_dev(one, cuda), 1, pairs, 4)
    assert (r.status, r.count, r.next_start) == (stq.STQ_OK, 0, ctx.prepared_length)
    r = ctx.sweep(boxes_dev(one, cuda), 1, pairs, 0)
    assert r.count == 0


def degenerate_scenes(stq):
    """Geometry the grid policy and the sweep must survive: point boxes
    (zero extent, median extent 0), boxes flat on one plane, every box the
    same, huge and tiny coordinates side by side, and one giant box among
    small ones."""
    rng = np.random.default_rng(9)
    out = {}
    b = stq.random_boxes(20_000, sliver_frac=0.0, seed=21)
    b["max"] = b["min"]  # points: pairs only where points coincide
    b["min"][::7] = b["min"][3]
    b["max"][::7] = b["min"][3]
    out["points"] = b
    b = stq.random_boxes(20_000, sliver_frac=0.05, seed=22)
    b["min"][:, 2] = 0.25
    b["max"][:, 2] = 0.25
    out["plane"] = b
    b = stq.random_boxes(1_500, sliver_frac=0.0, seed=23)
    b["min"][:] = (0.1, 0.2, 0.3)
    b["max"][:] = (0.4, 0.5, 0.6)
    out["identical"] = b
    b = stq.random_boxes(20_000, sliver_frac=0.0, seed=24)
    k = rng.choice(len(b), 300, replace=False)
    b["min"][k] = b["min"][k] * np.float32(3e30)
    b["max"][k] = b["min"][k] + np.float32(1e29)
    b["min"][:50] = -np.float32(1e-30)
    b["max"][:50] = np.float32(1e-30)
    out["magnitudes"] = b
    b = stq.random_boxes(20_000, sliver_frac=0.0, seed=25)
    b["min"][7] = (-1.0, -1.0, -1.0)
    b["max"][7] = (2.0, 2.0, 2.0)
    out["giant"] = b
    return out


@pytest.mark.parametrize("name", ["points", "plane", "identical", "magnitudes", "giant"])
def test_degenerate_geometry_vs_oracle(ctx, stq, oracle, cuda, name):
    boxes = degenerate_scenes(stq)[name]
    want = oracle.broadphase(boxes)
    for cells, axis in ((0, -1), (0, 0), (0, 2), (16, -1)):
        ctx.set_option(stq.OPT_CELLS, cells)
        got = sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, axis,
                          cap=len(want) + 16)
        assert np.array_equal(got, want), (name, cells, axis)


def test_nan_bound_rejected(ctx, stq, cuda):
    import torch

    boxes = stq.random_boxes(1000, seed=5)
    boxes[417]["max"][2] = np.nan
    pairs = torch.empty((100000, 2), dtype=torch.int32, device=cuda)
    with pytest.raises(stq.STQError) as e:
        ctx.sweep(boxes_dev(boxes, cuda), len(boxes), pairs, 100000)
    assert e.value.status == stq.STQ_ERR_INVALID_INPUT


def test_invalid_arguments(ctx, stq, cuda):
    import torch

    pairs = torch.empty((4, 2), dtype=torch.int32, device=cuda)
    with pytest.raises(stq.STQError):
        ctx.sweep(None, -1, pairs, 4)
    with pytest.raises(stq.STQError):
        ctx.set_option(stq.OPT_LANES, 3)
    ctx2 = stq.Context(0)
    with pytest.raises(stq.STQError) as e:
        ctx2.sweep_prepared(pairs, 4)
    assert e.value.status == stq.STQ_ERR_NOT_PREPARED
    ctx2.close()


# ---- other entry points ---------------------------------------------------------------------

def test_brute_force_agrees(ctx, stq, oracle, cuda):
    import torch

    boxes = stq.random_boxes(4000, seed=8)
    c = 0.5 * (boxes["min"] + boxes["max"])
    boxes["min"], boxes["max"] = c - 0.03, c + 0.03
    want = oracle.broadphase(boxes)
    cap = 4 * len(want) + 16
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    n = ctx.brute_force(boxes_dev(boxes, cuda), len(boxes), pairs, cap)
    assert np.array_equal(oracle.canonical(pairs[:n].cpu().numpy()), want)
    assert np.array_equal(sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, -1), want)


def test_sort_pairs_lexicographic(ctx, stq, oracle, cuda, c0):
    import torch

    m, boxes, want = c0
    cap = len(want)
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    r = ctx.sweep(boxes_dev(boxes, cuda), len(boxes), pairs, cap)
    ctx.sort_pairs(pairs, r.count)
    assert np.array_equal(pairs[: r.count].cpu().numpy(), want)


def test_sweep_host_end_to_end(stq, oracle, cuda, c0):
    m, boxes, want = c0
    with stq.Context(0) as ctx:
        out = np.empty((len(want) + 10, 2), np.int32)
        r = ctx.sweep_host(boxes, out)
        assert r.status == stq.STQ_OK and r.count == len(want)
        assert np.array_equal(oracle.canonical(out[: r.count]), want)
        small = np.empty((len(want) // 3, 2), np.int32)
        r = ctx.sweep_host(boxes, small)
        assert r.status == stq.STQ_OVERFLOW and r.total == len(want) and r.count <= len(small)
        assert ctx.launches > 0


@pytest.fixture(scope="module")
def big_cloth(stq):
    """Cloth pair of 2 x 450^2 vertices (about 2.4 M boxes): large enough for
    the host calls to sweep in windows."""
    return stq.cloth_pair(g=450, seed=3)


@pytest.mark.parametrize("overlap", [1, 2])
@pytest.mark.parametrize("pinned", [True, False])
def test_host_call_windows_match_device_sweep(stq, oracle, cuda, big_cloth, overlap, pinned):
    """Host calls sweep large scenes in windows, two at a time, each window's
    pairs copied while later ones run (OPT_HOST_OVERLAP=1), or copy once after
    the sweep (=2); both give the device sweep's pairs, into page-locked or
    pageable buffers, and the overflow prefix of the one-window path."""
    import torch

    m = big_cloth
    alloc = ((lambda shape: torch.empty(shape, dtype=torch.int32).pin_memory().numpy()) if pinned
             else (lambda shape: np.empty(shape, np.int32)))
    with stq.Context(0) as ctx:
        d = [torch.from_numpy(np.ascontiguousarray(x)).to(cuda) for x in (m.V0, m.V1, m.E, m.F)]
        boxes = torch.empty((m.num_boxes, 11), dtype=torch.int32, device=cuda)
        ctx.build_boxes(*d, boxes)
        ctx.prepare(boxes, m.num_boxes, stq.AXIS_AUTO)
        length = ctx.prepared_length
        assert length >= 2 << 19
        cap = 64 * m.num_boxes
        dp = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
        r = ctx.sweep_prepared(dp, cap)
        want = oracle.canonical(dp[: r.count].cpu().numpy())
        ctx.set_option(stq.OPT_HOST_OVERLAP, overlap)
        assert ctx.get_option(stq.OPT_HOST_OVERLAP) == overlap
        out = alloc((len(want) + 10, 2))
        for _ in range(2):  # the buffers are reused: no stale pairs
            out[:] = -7
            l0 = ctx.launches
            r = ctx.broadphase_host(m, out, stq.AXIS_AUTO)
            launches = ctx.launches - l0
            assert r.status == stq.STQ_OK and r.count == len(want)
            got = oracle.canonical(out[: r.count])
            assert len(got) == r.count and np.array_equal(got, want)
            assert (out[r.count:] == -7).all()
        # the windowed call launches one sweep per window instead of one
        ctx.set_option(stq.OPT_HOST_OVERLAP, 3 - overlap)
        l0 = ctx.launches
        ctx.broadphase_host(m, out, stq.AXIS_AUTO)
        other = ctx.launches - l0
        ctx.set_option(stq.OPT_HOST_OVERLAP, overlap)
        windows = min(ctx.get_option(stq.OPT_HOST_WINDOWS), length >> 19)
        assert windows == min(16, length >> 19)
        # per window: a sweep, its warp pass and the kernel that publishes its pair count
        assert launches - other == (3 * windows - 2 if overlap == 1 else 2 - 3 * windows)
        hb = boxes.cpu().numpy().view(stq.AABB_DTYPE).reshape(-1)
        r = ctx.sweep_host(hb, out)
        assert r.status == stq.STQ_OK and np.array_equal(oracle.canonical(out[: r.count]), want)
        # overflow: the windows' pairs do not fit; the result is the prefix rule's
        small = alloc((len(want) // 3, 2))
        rs = ctx.sweep_host(hb, small)
        ref = ctx.sweep_prepared(dp, len(want) // 3)
        assert rs.status == ref.status == stq.STQ_OVERFLOW and rs.total == len(want)
        assert rs.count == ref.count
        assert np.array_equal(oracle.canonical(small[: rs.count]), oracle.canonical(dp[: ref.count].cpu().numpy()))


@pytest.mark.parametrize("shape", [1, 2])
@pytest.mark.parametrize("windows", [2, 3, 32])
def test_host_call_window_counts(stq, oracle, cuda, big_cloth, windows, shape):
    """Any window count (odd counts end on the first slot; 32 is more than
    this scene's 2^19-position windows allow) gives the device sweep's pairs;
    a capacity that the first window alone exceeds gives the prefix rule's."""
    import torch

    m = big_cloth
    with stq.Context(0) as ctx:
        d = [torch.from_numpy(np.ascontiguousarray(x)).to(cuda) for x in (m.V0, m.V1, m.E, m.F)]
        boxes = torch.empty((m.num_boxes, 11), dtype=torch.int32, device=cuda)
        ctx.build_boxes(*d, boxes)
        ctx.prepare(boxes, m.num_boxes, stq.AXIS_AUTO)
        length = ctx.prepared_length
        cap = 64 * m.num_boxes
        dp = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
        r = ctx.sweep_prepared(dp, cap)
        want = oracle.canonical(dp[: r.count].cpu().numpy())
        ctx.set_option(stq.OPT_HOST_WINDOWS, windows)
        assert ctx.get_option(stq.OPT_HOST_WINDOWS) == windows
        ctx.set_option(stq.OPT_SWEEP_SHAPE, shape)
        out = torch.empty((len(want), 2), dtype=torch.int32).pin_memory().numpy()
        ctx.set_option(stq.OPT_HOST_OVERLAP, 2)
        l0 = ctx.launches
        ctx.broadphase_host(m, out, stq.AXIS_AUTO)
        one = ctx.launches - l0
        ctx.set_option(stq.OPT_HOST_OVERLAP, 1)
        out[:] = -7
        l0 = ctx.launches
        r = ctx.broadphase_host(m, out, stq.AXIS_AUTO)
        assert ctx.launches - l0 - one == 3 * min(windows, length >> 19) - 2
        assert r.status == stq.STQ_OK and r.count == len(want)
        assert np.array_equal(oracle.canonical(out), want)
        # runs handed to the warp pass in every window, on both slots' lists
        ctx.set_option(stq.OPT_RUN_CAP, 8)
        out[:] = -7
        r = ctx.broadphase_host(m, out, stq.AXIS_AUTO)
        assert r.status == stq.STQ_OK and r.count == len(want)
        assert np.array_equal(oracle.canonical(out), want)
        ctx.set_option(stq.OPT_RUN_CAP, 0)
        tiny = np.empty((100, 2), np.int32)
        hb = boxes.cpu().numpy().view(stq.AABB_DTYPE).reshape(-1)
        rs = ctx.sweep_host(hb, tiny)
        ref = ctx.sweep_prepared(dp, 100)
        assert rs.status == ref.status == stq.STQ_OVERFLOW and rs.total == len(want)
        assert rs.count == ref.count
        assert np.array_equal(oracle.canonical(tiny[: rs.count]), oracle.canonical(dp[: ref.count].cpu().numpy()))


def test_prepared_scene_reused_across_windows(ctx, stq, oracle, cuda, c0):
    import torch

    m, boxes, want = c0
    pairs = torch.empty((len(want), 2), dtype=torch.int32, device=cuda)
    bd = boxes_dev(boxes, cuda)
    ctx.prepare(bd, len(boxes), 2)
    del bd  # the prepared scene does not keep the input buffer
    torch.cuda.empty_cache()
    r1 = ctx.sweep_prepared(pairs, len(want), start=0, max_start=100_000)
    a = pairs[: r1.count].cpu().numpy().copy()
    r2 = ctx.sweep_prepared(pairs, len(want), start=r1.next_start)
    b = pairs[: r2.count].cpu().numpy().copy()
    assert np.array_equal(oracle.canonical(np.concatenate([a, b])), want)


# ---- cells (y/z grid segmentation with reference-point dedup) -------------------------

@pytest.mark.parametrize("cells", [1, 2, 3, 7, 12, 16, 24, 64, 512])
def test_cells_fixed_grids(ctx, stq, oracle, cuda, c0, cells):
    m, boxes, want = c0
    ctx.set_option(stq.OPT_CELLS, cells)
    for axis in (0, -1):
        got = sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, axis)
        assert np.array_equal(got, want), (cells, axis)
        if cells == 1:
            assert ctx.prepared_length == len(boxes) + 2


@pytest.mark.parametrize("cells", [3, 5, 8, 11])
@pytest.mark.parametrize("ties", [False, True])
def test_list_order_vs_oracle(ctx, stq, oracle, cuda, cells, ties):
    """Lists of a few hundred to about ten thousand replicas, with and
    without many equal minima: boxes sorted along the sweep axis, replicas
    emitted in that order, then a stable sort by list id, with 8- and 4-bit
    digits. list_stats reports the grid's lists."""
    boxes = stq.random_boxes(120_000, seed=20 + cells)
    c = 0.5 * (boxes["min"] + boxes["max"])
    boxes["min"], boxes["max"] = c - 0.004, c + 0.004
    if ties:
        boxes["min"][:, 0] = np.round(boxes["min"][:, 0] * 64) / 64
    want = oracle.broadphase(boxes)
    ctx.set_option(stq.OPT_CELLS, cells)
    for radix in (8, 4):
        ctx.set_option(stq.OPT_RADIX_BITS, radix)
        got = sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, 0)
        assert np.array_equal(got, want), radix
        stats = ctx.list_stats()
        assert stats["lists"] == 3 * cells * cells and stats["replicas"] >= len(boxes)
        assert stats["longest"] > stats["replicas"] // stats["lists"]


@pytest.mark.parametrize("scale", [1, 2, 4, 16])
def test_cells_auto_scales(ctx, stq, oracle, cuda, c0, scale):
    m, boxes, want = c0
    ctx.set_option(stq.OPT_CELL_SCALE, scale)
    for axis in (0, 1, 2):
        got = sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, axis)
        assert np.array_equal(got, want), (scale, axis)
    assert ctx.prepared_length > len(boxes)  # replicas + one slot per cell


def test_cells_skewed_slivers(ctx, stq, oracle, cuda):
    boxes = stq.random_boxes(300_000, sliver_frac=0.05, seed=11)
    want = oracle.broadphase(boxes)
    for scale in (1, 4, 32):
        ctx.set_option(stq.OPT_CELL_SCALE, scale)
        got = sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, -1)
        assert np.array_equal(got, want), scale


@pytest.mark.parametrize("shape", [1, 2])
def test_cells_coarse_levels(ctx, stq, oracle, cuda, shape):
    """Grid levels above 0. A cell of level L is a 2^L x 2^L block of level-0
    cells (the level-0 coordinate shifted right by L), with the first-cell rule
    at the block's lower bounds; when no level fits the replica budget the
    scene is one cell. Boxes of side 0.03 in the unit cube span about 5 level-0
    cells at cell scale 1 (a 44 x 44 grid), 2.7 at level 1 and 1.7 at level 2,
    so budgets 64, 4, 2 and 1 take levels 0, 1, 2 and one cell; each gives the
    oracle's pairs."""
    boxes = stq.random_boxes(150_000, sliver_frac=0.0, seed=31)
    c = 0.5 * (boxes["min"] + boxes["max"])
    boxes["min"], boxes["max"] = c - np.float32(0.015), c + np.float32(0.015)
    want = oracle.broadphase(boxes)
    ctx.set_option(stq.OPT_SWEEP_SHAPE, shape)
    ctx.set_option(stq.OPT_CELL_SCALE, 1)
    lists = {}
    for budget in (64, 4, 2, 1):
        ctx.set_option(stq.OPT_REPLICA_BUDGET, budget)
        got = sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, -1)
        assert np.array_equal(got, want), budget
        stats = ctx.list_stats()
        assert stats["replicas"] <= budget * len(boxes), budget
        lists[budget] = stats["lists"]
    assert lists[64] > lists[4] > lists[2] > lists[1] == 3, lists


def test_cells_inverted_and_infinite_boxes(ctx, stq, oracle, cuda):
    boxes = stq.random_boxes(20_000, seed=12)
    c = 0.5 * (boxes["min"] + boxes["max"])
    boxes["min"], boxes["max"] = c - 0.01, c + 0.01
    inv = boxes.copy()
    inv["min"][::97, 1], inv["max"][::97, 1] = inv["max"][::97, 1], inv["min"][::97, 1]
    inf = boxes.copy()
    inf["max"][5, 2] = np.inf
    inf["min"][9, 1] = -np.inf
    for b in (inv, inf):
        want = oracle.broadphase(b)
        for cells in (0, 16):
            ctx.set_option(stq.OPT_CELLS, cells)
            got = sweep_pairs(ctx, stq, oracle, boxes_dev(b, cuda), len(b), cuda, -1)
            assert np.array_equal(got, want)


def test_cells_overflow_resume(ctx, stq, oracle, cuda):
    import torch

    boxes = stq.random_boxes(150_000, sliver_frac=0.05, seed=13)
    want = oracle.broadphase(boxes)
    cap = len(want) // 9 + 1
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
    ctx.set_option(stq.OPT_CELLS, 32)
    ctx.prepare(boxes_dev(boxes, cuda), len(boxes), -1)
    start, chunks = 0, []
    while start < ctx.prepared_length:
        r = ctx.sweep_prepared(pairs, cap, start=start)
        chunks.append(pairs[: r.count].cpu().numpy().copy())
        start = r.next_start
    allp = np.concatenate(chunks)
    assert len(oracle.canonical(allp)) == len(allp)
    assert np.array_equal(oracle.canonical(allp), want)


def _f32_lower_bound(C, lo, inv):
    """Smallest float32 v with (v - lo) * inv >= C in float32 round-to-nearest
    steps: the lower bound of cell C, found as the device finds it."""
    def okey(f):
        u = int(np.float32(f).view(np.uint32))
        return (~u & 0xFFFFFFFF) if u & 0x80000000 else (u | 0x80000000)

    def ofloat(k):
        u = (k & 0x7FFFFFFF) if k & 0x80000000 else (~k & 0xFFFFFFFF)
        return np.uint32(u).view(np.float32)

    a, b = okey(-np.inf), okey(np.inf)
    while b - a > 1:
        m = (a + b) // 2
        if np.float32(np.float32(ofloat(m) - lo) * inv) >= np.float32(C):
            b = m
        else:
            a = m
    return ofloat(b)


@pytest.mark.parametrize("shape", [1, 2])
@pytest.mark.parametrize("lo,hi,n", [(0.0, 1.0, 8), (0.1, 0.8, 7), (-0.37, 1.91, 13), (1000.25, 1003.0, 11)])
def test_first_cell_rule_at_cell_bounds(ctx, stq, oracle, cuda, lo, hi, n, shape):
    """A pair found in several cells is emitted in the cell of its reference
    point, tested on the candidate's minima against the start box's cell lower
    bounds. Boxes whose minima sit one float below, on and one float above
    every cell bound (computed on the host in the same float32 steps as the
    device's grid: origin lo, n / (hi - lo) cells per unit) give the oracle's
    pairs exactly."""
    f32 = np.float32
    lo, hi = f32(lo), f32(hi)
    inv = f32(f32(n) / f32(hi - lo))
    down = lambda v: np.nextafter(v, f32(-np.inf), dtype=np.float32)  # noqa: E731
    up = lambda v: np.nextafter(v, f32(np.inf), dtype=np.float32)  # noqa: E731
    cell = lambda v: int(min(max(f32(f32(v - lo) * inv), f32(0)), f32(n - 1)))  # noqa: E731
    bounds = [_f32_lower_bound(C, lo, inv) for C in range(1, n)]
    for C, t in enumerate(bounds, start=1):
        assert cell(t) == C and cell(down(t)) == C - 1
    w = f32((hi - lo) / (4 * n))  # a quarter cell: boxes reach into the next cell at most
    rows = []
    # the whole scene on y and z: fixes the grid's origin and extent
    rows.append(((f32(0), lo, lo), (f32(1), hi, hi)))
    for tb in bounds:
        for tc in bounds[:: max(1, len(bounds) // 4)]:
            for mb in (down(tb), tb, up(tb)):
                for mc in (down(tc), tc, up(tc)):
                    rows.append(((f32(0.25), mb, mc), (f32(0.75), f32(mb + w), f32(mc + w))))
    boxes = np.zeros(len(rows), stq.AABB_DTYPE)
    for i, (mn, mx) in enumerate(rows):
        boxes[i]["id"] = i
        boxes[i]["min"] = mn
        boxes[i]["max"] = mx
        boxes[i]["vertex_ids"] = (2 * i, 2 * i + 1, -2 * i - 1)  # edges, no shared vertex
    want = oracle.broadphase(boxes)
    assert len(want) > len(boxes)
    ctx.set_option(stq.OPT_CELLS, n)
    ctx.set_option(stq.OPT_REPLICA_BUDGET, 64)
    ctx.set_option(stq.OPT_SWEEP_SHAPE, shape)
    got = sweep_pairs(ctx, stq, oracle, boxes_dev(boxes, cuda), len(boxes), cuda, axis=0)
    assert ctx.list_stats()["lists"] == 3 * n * n  # the grid the host computed
    assert np.array_equal(got, want)
