"""stq_sweep_static: the sweep for callers that cannot allocate device memory
when they need a broad phase (steps under a memory budget reserved up front,
hosts whose own pooling allocator owns the device memory, real-time loops that
cannot take cudaFree's device-wide synchronisation). It must return
exactly the pairs of the ordinary entry point stq_sweep, call after call,
while using only the library's static scratch array.

Collected last on purpose (file name), so a run that stops at the first
failure has run every other test before this one."""
import ctypes

import numpy as np
import pytest


def call_static(stq, boxes_dev, n, axis, pairs, cap, stream):
    lib = stq.load_library()
    count, total = ctypes.c_int64(), ctypes.c_int64()
    st = lib.stq_sweep_static(ctypes.c_void_p(boxes_dev.data_ptr() if boxes_dev is not None else 0), n,
                              axis, ctypes.c_void_p(pairs.data_ptr() if pairs is not None else 0), cap,
                              ctypes.byref(count), ctypes.byref(total), ctypes.c_void_p(stream))
    return st, count.value, total.value


def test_static_limit_is_rejected_without_gpu_work(stq):
    lib = stq.load_library()
    count = ctypes.c_int64(-1)
    st = lib.stq_sweep_static(None, 65537, 0, None, 0, ctypes.byref(count), None, None)
    assert st == stq.STQ_ERR_CAPACITY
    assert lib.stq_sweep_static(None, 10, 3, None, 0, ctypes.byref(count), None, None) == \
        stq.STQ_ERR_INVALID_ARG


@pytest.mark.gpu
def test_static_sweep_matches_stq_sweep_twice_in_a_row(stq, oracle, cuda):
    import torch

    stream = torch.cuda.current_stream(cuda).cuda_stream
    scenes = []
    m = stq.cloth_pair(g=60, z_offset=0.004, sigma=0.004, seed=21)   # 42k boxes
    scenes.append(oracle.construct_boxes(m.V0, m.V1, m.E, m.F, stq.AABB_DTYPE))
    b = stq.random_boxes(65536, sliver_frac=0.05, seed=22)          # the maximum size
    c = 0.5 * (b["min"] + b["max"])
    b["min"], b["max"] = c - 0.01, c + 0.01
    scenes.append(b)
    cap = 4_000_000
    with stq.Context(0, stream) as ctx:
        for axis, boxes in zip((0, 2), scenes):
            d = torch.from_numpy(boxes.view(np.int32).reshape(-1, 11).copy()).to(cuda)
            n = len(boxes)
            pa = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
            pb = torch.empty((cap, 2), dtype=torch.int32, device=cuda)
            st, count, total = call_static(stq, d, n, axis, pa, cap, stream)
            assert st == stq.STQ_OK and count == total
            r = ctx.sweep(d, n, pb, cap, axis=axis)
            assert r.status == stq.STQ_OK
            got = oracle.canonical(pa[:count].cpu().numpy())
            want = oracle.canonical(pb[: r.count].cpu().numpy())
            assert len(got) == count  # no duplicates
            assert np.array_equal(got, want)
            assert np.array_equal(want, oracle.broadphase(boxes))
        # a buffer that is too small reports the true total
        d = torch.from_numpy(scenes[0].view(np.int32).reshape(-1, 11).copy()).to(cuda)
        st, count, total = call_static(stq, d, len(scenes[0]), 0, pa, 100, stream)
        assert st == stq.STQ_OVERFLOW and count == 100 and total > 100


@pytest.mark.gpu
def test_static_sweep_edge_cases(stq, oracle, cuda):
    """Empty and one-box scenes, a zero-capacity buffer (the true total is still
    reported), and a NaN bound far from the first block: the error is reported
    and the next clean call is not affected by it."""
    import torch

    stream = torch.cuda.current_stream(cuda).cuda_stream
    pa = torch.empty((1 << 20, 2), dtype=torch.int32, device=cuda)
    b = stq.random_boxes(20000, sliver_frac=0.05, seed=23)
    c = 0.5 * (b["min"] + b["max"])
    b["min"], b["max"] = c - 0.01, c + 0.01
    d = torch.from_numpy(b.view(np.int32).reshape(-1, 11).copy()).to(cuda)
    want = oracle.broadphase(b)
    assert len(want) > 1000
    assert call_static(stq, None, 0, 0, pa, 1 << 20, stream) == (stq.STQ_OK, 0, 0)
    assert call_static(stq, d, 1, 1, pa, 1 << 20, stream) == (stq.STQ_OK, 0, 0)
    st, count, total = call_static(stq, d, len(b), 0, None, 0, stream)
    assert (st, count, total) == (stq.STQ_OVERFLOW, 0, len(want))
    bad = b.copy()
    bad["min"][15000, 1] = np.nan  # in block 58 of the key pass, not block 0
    dbad = torch.from_numpy(bad.view(np.int32).reshape(-1, 11).copy()).to(cuda)
    st, _, _ = call_static(stq, dbad, len(bad), 0, pa, 1 << 20, stream)
    assert st == stq.STQ_ERR_INVALID_INPUT
    st, count, total = call_static(stq, d, len(b), 0, pa, 1 << 20, stream)
    assert st == stq.STQ_OK and count == total == len(want)
    assert np.array_equal(oracle.canonical(pa[:count].cpu().numpy()), want)
