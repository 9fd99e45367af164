"""Serving loop on the GPU: every timestep's pair set is exact (checked
against the oracle on the positions the device used), a request's results do
not depend on what it is batched with, and admission respects the budget in
arrival order."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def oracle_step(stq, oracle, mesh, V0, V1):
    boxes = oracle.construct_boxes(V0, V1, mesh.E, mesh.F, stq.AABB_DTYPE)
    pairs = oracle.broadphase(boxes)
    return len(pairs), stq.pair_checksum(pairs)


def run_until_done(server, ids, limit=10_000):
    done = set()
    for _ in range(limit):
        done.update(server.tick())
        if set(ids) <= done:
            return
    raise AssertionError("requests did not finish")


def test_each_timestep_is_exact(stq, oracle, cuda):
    mesh = stq.cloth_pair(g=40, z_offset=0.004, sigma=0.004, seed=31)
    with stq.Server(0, None, budget_bytes=8 << 30, max_boxes=1 << 20, max_scenes=8) as sv:
        rid = sv.submit(mesh, steps=4, sigma=0.003, seed=77)
        want = []
        for step in range(4):
            sv.tick()                     # launches this step (and collects the previous)
            V0, V1 = sv.mesh(rid)         # the positions the device used for it
            want.append(oracle_step(stq, oracle, mesh, V0, V1))
        run_until_done(sv, [rid])
        counts, checks = sv.result(rid)
    assert [int(c) for c in counts] == [w[0] for w in want]
    assert [int(c) for c in checks] == [w[1] for w in want]
    assert want[0][0] > 0 and len(set(w[1] for w in want)) == 4  # the scene moved


def test_large_request_each_timestep_is_exact(stq, oracle, cuda):
    """A request of over a million boxes, batched with a small one: every
    timestep's pair count and checksum equal the oracle's on the positions the
    device used, and the request ran one step per tick."""
    mesh = stq.cloth_pair(g=292, z_offset=0.004, sigma=0.004, seed=33)
    assert mesh.num_boxes >= 1_000_000
    small = stq.cloth_pair(g=20, z_offset=0.004, sigma=0.004, seed=34)
    with stq.Server(0, None, budget_bytes=32 << 30, max_boxes=1 << 22, max_scenes=8) as sv:
        other = sv.submit(small, steps=5, sigma=0.003, seed=1)
        rid = sv.submit(mesh, steps=3, sigma=0.003, seed=78)
        want = []
        for step in range(3):
            sv.tick()
            V0, V1 = sv.mesh(rid)
            want.append(oracle_step(stq, oracle, mesh, V0, V1))
        run_until_done(sv, [rid, other])
        counts, checks = sv.result(rid)
        first, last = sv.request_ticks(rid)
    assert [int(c) for c in counts] == [w[0] for w in want]
    assert [int(c) for c in checks] == [w[1] for w in want]
    assert want[0][0] > 1_000_000
    assert first == 0 and last - first + 1 == 3


def test_dense_request_outgrows_the_pair_estimate(stq, oracle, cuda):
    """Two sheets 0.002 apart with large motion find over 40 pairs per box, more
    than the server's first pair-buffer estimate: the tick grows the buffer and
    sweeps the step again. Every step still equals the oracle."""
    mesh = stq.cloth_pair(g=60, z_offset=0.002, sigma=0.03, seed=9)
    with stq.Server(0, None, budget_bytes=8 << 30, max_boxes=1 << 20, max_scenes=8) as sv:
        rid = sv.submit(mesh, steps=2, sigma=0.003, seed=12)
        want = []
        for step in range(2):
            sv.tick()
            V0, V1 = sv.mesh(rid)
            want.append(oracle_step(stq, oracle, mesh, V0, V1))
        run_until_done(sv, [rid])
        counts, checks = sv.result(rid)
    assert want[0][0] > 25 * mesh.num_boxes
    assert [int(c) for c in counts] == [w[0] for w in want]
    assert [int(c) for c in checks] == [w[1] for w in want]


def test_many_scene_slots_checksums(stq, oracle, cuda):
    """A server with more scene slots than the checksum kernel's shared-memory
    table holds (4,096) adds its checksums straight to global memory; they equal
    the oracle's."""
    meshes = [stq.cloth_pair(g=g, z_offset=0.004, sigma=0.004, seed=70 + g) for g in (14, 22, 31)]
    with stq.Server(0, None, budget_bytes=8 << 30, max_boxes=1 << 18, max_scenes=5000) as sv:
        ids = [sv.submit(m, steps=1, sigma=0.0, seed=k) for k, m in enumerate(meshes)]
        run_until_done(sv, ids)
        for rid, m in zip(ids, meshes):
            counts, checks = sv.result(rid)
            want = oracle_step(stq, oracle, m, m.V0, m.V1)
            assert (int(counts[0]), int(checks[0])) == want


@pytest.mark.parametrize("shape", [(1, 8, 1), (4, 0, 1), (8, 0, 1), (1, 4, 2), (1, 2, 2)])
def test_server_sweep_shapes_agree(stq, cuda, shape):
    """stq_server_set_option retunes the server's sweep (the next tick captures
    again); every shape gives the same per-step counts and checksums."""
    mesh = stq.cloth_pair(g=60, z_offset=0.003, sigma=0.006, seed=8)
    results = []
    for s in ((8, 0, 1), shape):
        with stq.Server(0, None, budget_bytes=8 << 30, max_boxes=1 << 20, max_scenes=8) as sv:
            sv.set_option(stq.OPT_LANES, s[0])
            sv.set_option(stq.OPT_SWEEP_SHAPE, s[2])
            if s[1]:
                sv.set_option(stq.OPT_PER_LANE, s[1])
            sv.set_option(stq.OPT_RUN_CAP, 4)  # the warp pass too
            rid = sv.submit(mesh, steps=3, sigma=0.003, seed=5)
            run_until_done(sv, [rid])
            results.append(sv.result(rid))
    assert np.array_equal(results[0][0], results[1][0]) and np.array_equal(results[0][1], results[1][1])
    with pytest.raises(stq.STQError):
        with stq.Server(0, None, budget_bytes=8 << 30, max_boxes=1 << 20, max_scenes=8) as sv:
            sv.set_option(stq.OPT_LANES, 3)


def test_same_result_alone_and_in_a_mix(stq, cuda):
    target = stq.cloth_pair(g=30, z_offset=0.003, sigma=0.005, seed=41)
    others = [stq.cloth_pair(g=g, z_offset=0.004, sigma=0.004, seed=50 + g) for g in (12, 55, 20, 70, 33)]
    with stq.Server(0, None, budget_bytes=8 << 30, max_boxes=1 << 20, max_scenes=8) as sv:
        rid = sv.submit(target, steps=5, sigma=0.003, seed=99)
        run_until_done(sv, [rid])
        alone = sv.result(rid)
    with stq.Server(0, None, budget_bytes=8 << 30, max_boxes=1 << 20, max_scenes=8) as sv:
        ids = [sv.submit(others[0], steps=3, sigma=0.003, seed=1)]
        sv.tick()
        ids.append(sv.submit(others[1], steps=7, sigma=0.003, seed=2))
        rid = sv.submit(target, steps=5, sigma=0.003, seed=99)
        sv.tick()
        sv.tick()
        ids += [sv.submit(m, steps=2 + k, sigma=0.002, seed=3 + k) for k, m in enumerate(others[2:])]
        run_until_done(sv, ids + [rid])
        mixed = sv.result(rid)
        assert sv.stats()["ticks"] >= 7
    assert np.array_equal(alone[0], mixed[0]) and np.array_equal(alone[1], mixed[1])
    assert len(alone[0]) == 5


def test_budget_admits_in_arrival_order(stq, cuda):
    meshes = [stq.cloth_pair(g=25 + 5 * k, seed=60 + k) for k in range(4)]
    with stq.Server(0, None, budget_bytes=8 << 30, max_boxes=20_000, max_scenes=8) as sv:
        # each request has more than half the box capacity: one at a time
        assert all(m.num_boxes > 10_000 or k == 0 for k, m in enumerate(meshes))
        ids = [sv.submit(m, steps=2, sigma=0.003, seed=k) for k, m in enumerate(meshes) if m.num_boxes <= 20_000]
        order, peak = [], 0
        for _ in range(1000):
            order += sv.tick()
            st = sv.stats()
            peak = max(peak, st["active"])
            if len(order) == len(ids):
                break
        assert order == ids  # first come, first served
        for rid in ids:
            counts, _ = sv.result(rid)
            assert len(counts) == 2
    with pytest.raises(stq.STQError):
        with stq.Server(0, None, budget_bytes=8 << 30, max_boxes=1000, max_scenes=2) as sv:
            sv.submit(meshes[0], steps=1, sigma=0.0, seed=0)
