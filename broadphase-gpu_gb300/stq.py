"""Python host binding of the STQ broad phase C ABI (include/stq_abi.h).

A thin ctypes layer: every compute call goes through libstq_gb300.so. PyTorch
is used only to hold device memory and to name the CUDA stream. There is no
CPU fallback: loading fails loudly if the native library is missing.

Reference interfaces mirrored (Ahdhn/broadphase-gpu):
  Context.build_boxes   stq::gpu::constructBoxes          src/io.cuh:9-13
  Context.select_axis   calc_mean / calc_variance          src/sweep.cu:93-123
  Context.sweep         stq::gpu::run_sweep_sharedqueue   src/simulation.cuh:22-27
  Context.sweep_host    the same with host boxes and host pairs
                        (KEEP_CPU_OVERLAPS, src/simulation.cu:763-780)
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libstq_gb300.so"
SCENES_PATH = PKG / "_build" / "libstq_scenes.so"

# stq_aabb: 44 bytes, the reference's stq::gpu::Aabb (src/aabb.cuh:15-43)
AABB_DTYPE = np.dtype([
    ("id", "<i4"), ("min", "<f4", (3,)), ("max", "<f4", (3,)),
    ("vertex_ids", "<i4", (3,)), ("ref_id", "<i4"),
])
assert AABB_DTYPE.itemsize == 44

STQ_OK = 0
STQ_OVERFLOW = 1
STQ_ERR_INVALID_ARG = -1
STQ_ERR_INVALID_INPUT = -2
STQ_ERR_CUDA = -3
STQ_ERR_NO_MEMORY = -4
STQ_ERR_CAPACITY = -5
STQ_ERR_TIMEOUT = -6
STQ_ERR_NOT_PREPARED = -7

AXIS_AUTO, AXIS_X, AXIS_Y, AXIS_Z = -1, 0, 1, 2
OPT_LANES, OPT_QUEUE, OPT_BLOCK, OPT_CELLS, OPT_RADIX_BITS, OPT_CELL_SCALE = 1, 2, 3, 4, 5, 6
OPT_REPLICA_BUDGET, OPT_GRAPH, OPT_HOST_OVERLAP, OPT_PER_LANE, OPT_RUN_CAP = 7, 8, 9, 10, 11
OPT_HOST_WINDOWS, OPT_SWEEP_SHAPE = 12, 13
SHAPE_QUEUE, SHAPE_FLAT = 1, 2

_c_i64p = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p

# name -> (restype, argtypes): the full exported surface of include/stq_abi.h
ABI_SIGNATURES = {
    "stq_abi_version": (ctypes.c_int, []),
    "stq_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "stq_context_create": (ctypes.c_int, [ctypes.c_int, _vp, ctypes.POINTER(_vp)]),
    "stq_context_destroy": (None, [_vp]),
    "stq_context_set_stream": (ctypes.c_int, [_vp, _vp]),
    "stq_context_set_option": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int64]),
    "stq_context_get_option": (ctypes.c_int64, [_vp, ctypes.c_int]),
    "stq_context_last_error": (ctypes.c_char_p, [_vp]),
    "stq_context_launch_count": (ctypes.c_int64, [_vp]),
    "stq_context_candidates": (ctypes.c_int64, [_vp]),
    "stq_context_list_stats": (ctypes.c_int, [_vp, _vp]),
    "stq_build_boxes": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int64, _vp, ctypes.c_int64,
                                       _vp, ctypes.c_int64, ctypes.c_float, _vp]),
    "stq_select_axis": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, ctypes.POINTER(ctypes.c_int)]),
    "stq_prepare": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, ctypes.c_int]),
    "stq_prepared_length": (ctypes.c_int64, [_vp]),
    "stq_sweep_prepared": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int64, _vp, ctypes.c_int64,
                                          _c_i64p, _c_i64p, _c_i64p]),
    "stq_sweep": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, ctypes.c_int, ctypes.c_int64,
                                 ctypes.c_int64, _vp, ctypes.c_int64, _c_i64p, _c_i64p, _c_i64p]),
    "stq_sweep_host": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, ctypes.c_int, _vp, ctypes.c_int64,
                                      _c_i64p, _c_i64p]),
    "stq_broadphase_host": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int64, _vp, ctypes.c_int64, _vp,
                                           ctypes.c_int64, ctypes.c_float, ctypes.c_int, _vp,
                                           ctypes.c_int64, _c_i64p, _c_i64p]),
    "stq_context_enable_timing": (ctypes.c_int, [_vp, ctypes.c_int]),
    "stq_context_stage_times": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double), _c_i64p,
                                               ctypes.c_int]),
    "stq_stage_name": (ctypes.c_char_p, [ctypes.c_int]),
    "stq_batch_build_boxes": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int,
                                             ctypes.c_float, _vp, _vp]),
    "stq_batch_prepare": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, _vp, ctypes.c_int]),
    "stq_batch_scene_pairs": (ctypes.c_int, [_vp, _vp, ctypes.c_int]),
    "stq_batch_broadphase": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int,
                                            ctypes.c_float, ctypes.c_int, _vp, ctypes.c_int64, _c_i64p,
                                            _c_i64p, _vp]),
    "stq_autotune": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, _vp, ctypes.c_int64,
                                    ctypes.POINTER(ctypes.c_double)]),
    "stq_server_create": (ctypes.c_int, [ctypes.c_int, _vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                                         ctypes.POINTER(_vp)]),
    "stq_server_destroy": (None, [_vp]),
    "stq_server_submit": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int64, _vp, ctypes.c_int64, _vp,
                                         ctypes.c_int64, ctypes.c_int, ctypes.c_double, ctypes.c_uint64,
                                         _c_i64p]),
    "stq_server_tick": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "stq_server_result": (ctypes.c_int, [_vp, ctypes.c_int64, _vp, _vp, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_int)]),
    "stq_server_mesh": (ctypes.c_int, [_vp, ctypes.c_int64, _vp, _vp]),
    "stq_server_request_ticks": (ctypes.c_int, [_vp, ctypes.c_int64, _c_i64p, _c_i64p]),
    "stq_server_stats": (ctypes.c_int, [_vp, _c_i64p, _c_i64p, _c_i64p, _c_i64p]),
    "stq_server_set_option": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int64]),
    "stq_read_mesh": (ctypes.c_int, [ctypes.c_char_p, _vp, _c_i64p, _vp, _c_i64p]),
    "stq_mesh_edges": (ctypes.c_int, [_vp, ctypes.c_int64, _vp, _c_i64p]),
    "stq_compare_truth_json": (ctypes.c_int, [ctypes.c_char_p, _vp, ctypes.c_int64, _c_i64p, _c_i64p,
                                              _c_i64p]),
    "stq_sweep_static": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int, _vp, ctypes.c_int64, _c_i64p,
                                        _c_i64p, _vp]),
    "stq_sort_pairs": (ctypes.c_int, [_vp, _vp, ctypes.c_int64]),
    "stq_brute_force": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, ctypes.c_int64, _c_i64p]),
}

_lib = None
_scenes = None


def load_library() -> ctypes.CDLL:
    """Loads libstq_gb300.so (built in-tree); raises if it is missing."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"native STQ library missing: {LIB_PATH} (run build())")
        lib = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in ABI_SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def load_scenes() -> ctypes.CDLL:
    global _scenes
    if _scenes is None:
        if not SCENES_PATH.exists():
            raise RuntimeError(f"scene library missing: {SCENES_PATH} (run build())")
        _scenes = ctypes.CDLL(str(SCENES_PATH))
    return _scenes


class STQError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"STQ status {status}: {message}")
        self.status = status


@dataclass
class SweepResult:
    status: int
    count: int
    next_start: int
    total: int


def _ptr(t) -> int | None:
    if t is None:
        return None
    if isinstance(t, np.ndarray):
        return t.ctypes.data
    return t.data_ptr()


class Context:
    """One STQ context on one device and one stream (stq_context*)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self.lib = load_library()
        self._h = _vp()
        st = self.lib.stq_context_create(device, stream, ctypes.byref(self._h))
        if st != STQ_OK:
            raise STQError(st, "context creation failed")
        self.device = device

    def close(self) -> None:
        if self._h:
            self.lib.stq_context_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- helpers --------------------------------------------------------------
    def _check(self, st: int, allow=(STQ_OK,)) -> int:
        if st not in allow:
            msg = self.lib.stq_context_last_error(self._h)
            raise STQError(st, (msg or b"").decode())
        return st

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream: int | None) -> None:
        self._check(self.lib.stq_context_set_stream(self._h, stream))

    def set_option(self, option: int, value: int) -> None:
        self._check(self.lib.stq_context_set_option(self._h, option, value))

    def get_option(self, option: int) -> int:
        return int(self.lib.stq_context_get_option(self._h, option))

    @property
    def candidates(self) -> int:
        """Candidates the last sweep tested."""
        return int(self.lib.stq_context_candidates(self._h))

    def list_stats(self) -> dict:
        """(cell, type) lists of the prepared scene: count, replicas, longest."""
        out = np.zeros(3, np.int64)
        self._check(self.lib.stq_context_list_stats(self._h, out.ctypes.data))
        return dict(zip(("lists", "replicas", "longest"), (int(v) for v in out)))

    @property
    def launches(self) -> int:
        return int(self.lib.stq_context_launch_count(self._h))

    # -- pipeline -------------------------------------------------------------
    def build_boxes(self, V0, V1, E, F, out, inflation_radius: float = 0.0) -> None:
        """Swept boxes from device tensors V0/V1 [nV,3] f64, E [nE,2] i32, F [nF,3] i32
        into `out` (device buffer of (nV+nE+nF)*44 bytes)."""
        nV, nE, nF = V0.shape[0], E.shape[0], F.shape[0]
        self._check(self.lib.stq_build_boxes(self._h, _ptr(V0), _ptr(V1), nV, _ptr(E), nE,
                                             _ptr(F), nF, float(inflation_radius), _ptr(out)))

    def select_axis(self, boxes, n: int) -> int:
        a = ctypes.c_int(-1)
        self._check(self.lib.stq_select_axis(self._h, _ptr(boxes), n, ctypes.byref(a)))
        return a.value

    def prepare(self, boxes, n: int, axis: int = AXIS_X) -> None:
        self._check(self.lib.stq_prepare(self._h, _ptr(boxes), n, axis))

    @property
    def prepared_length(self) -> int:
        """Sweep positions of the prepared scene (the resume cursor's range)."""
        return int(self.lib.stq_prepared_length(self._h))

    def sweep_prepared(self, pairs, capacity: int, start: int = 0, max_start: int = 0) -> SweepResult:
        c, nx, tot = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        st = self.lib.stq_sweep_prepared(self._h, start, max_start, _ptr(pairs), capacity,
                                         ctypes.byref(c), ctypes.byref(nx), ctypes.byref(tot))
        self._check(st, allow=(STQ_OK, STQ_OVERFLOW))
        return SweepResult(st, c.value, nx.value, tot.value)

    def sweep(self, boxes, n: int, pairs, capacity: int, axis: int = AXIS_X,
              start: int = 0, max_start: int = 0) -> SweepResult:
        c, nx, tot = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        st = self.lib.stq_sweep(self._h, _ptr(boxes), n, axis, start, max_start, _ptr(pairs),
                                capacity, ctypes.byref(c), ctypes.byref(nx), ctypes.byref(tot))
        self._check(st, allow=(STQ_OK, STQ_OVERFLOW))
        return SweepResult(st, c.value, nx.value, tot.value)

    def sweep_host(self, boxes: np.ndarray, pairs: np.ndarray, axis: int = AXIS_X) -> SweepResult:
        """Host boxes (AABB_DTYPE) in, host pairs (int32 [cap, 2]) out."""
        assert boxes.dtype == AABB_DTYPE and boxes.flags.c_contiguous
        assert pairs.dtype == np.int32 and pairs.flags.c_contiguous
        c, tot = ctypes.c_int64(), ctypes.c_int64()
        st = self.lib.stq_sweep_host(self._h, boxes.ctypes.data, boxes.shape[0], axis,
                                     pairs.ctypes.data, pairs.shape[0], ctypes.byref(c),
                                     ctypes.byref(tot))
        self._check(st, allow=(STQ_OK, STQ_OVERFLOW))
        return SweepResult(st, c.value, boxes.shape[0], tot.value)

    def broadphase_host(self, mesh: "Mesh", pairs: np.ndarray, axis: int = AXIS_AUTO,
                        inflation_radius: float = 0.0) -> SweepResult:
        """Host mesh in (ideally pinned), host pairs (int32 [cap, 2]) out: copies,
        device box build, sort and sweep in one native call."""
        for a in (mesh.V0, mesh.V1, mesh.E, mesh.F, pairs):
            assert a.flags.c_contiguous
        c, tot = ctypes.c_int64(), ctypes.c_int64()
        st = self.lib.stq_broadphase_host(
            self._h, mesh.V0.ctypes.data, mesh.V1.ctypes.data, mesh.V0.shape[0],
            mesh.E.ctypes.data, mesh.E.shape[0], mesh.F.ctypes.data, mesh.F.shape[0],
            float(inflation_radius), axis, pairs.ctypes.data, pairs.shape[0], ctypes.byref(c),
            ctypes.byref(tot))
        self._check(st, allow=(STQ_OK, STQ_OVERFLOW))
        return SweepResult(st, c.value, mesh.num_boxes, tot.value)

    def enable_timing(self, enable: bool = True) -> None:
        self._check(self.lib.stq_context_enable_timing(self._h, int(enable)))

    def stage_times(self) -> dict:
        ms = (ctypes.c_double * 16)()
        calls = (ctypes.c_int64 * 16)()
        k = self.lib.stq_context_stage_times(self._h, ms, calls, 16)
        return {self.lib.stq_stage_name(i).decode(): (ms[i], calls[i]) for i in range(k)}

    # -- batches of scenes ----------------------------------------------------
    def batch_build_boxes(self, V0, V1, voff, E, eoff, F, foff, out,
                          inflation_radius: float = 0.0) -> np.ndarray:
        """Device meshes of several scenes (host offsets voff/eoff/foff, S+1 each)
        -> boxes in `out`; returns the S+1 box offsets."""
        S = len(voff) - 1
        vo, eo, fo = (np.ascontiguousarray(x, np.int64) for x in (voff, eoff, foff))
        bo = np.zeros(S + 1, np.int64)
        self._check(self.lib.stq_batch_build_boxes(self._h, _ptr(V0), _ptr(V1), vo.ctypes.data, _ptr(E),
                                                   eo.ctypes.data, _ptr(F), fo.ctypes.data, S,
                                                   float(inflation_radius), _ptr(out), bo.ctypes.data))
        return bo

    def batch_prepare(self, boxes, box_off, axes=None, axis: int = AXIS_AUTO) -> None:
        bo = np.ascontiguousarray(box_off, np.int64)
        ax = None if axes is None else np.ascontiguousarray(axes, np.int32)
        self._check(self.lib.stq_batch_prepare(self._h, _ptr(boxes), bo.ctypes.data, len(bo) - 1,
                                               None if ax is None else ax.ctypes.data, axis))

    def autotune(self, boxes, box_off, pairs, capacity: int) -> tuple:
        """Tunes the context's options on this batch; returns (best_ms, settings)."""
        bo = np.ascontiguousarray(box_off, np.int64)
        ms = ctypes.c_double()
        self._check(self.lib.stq_autotune(self._h, _ptr(boxes), bo.ctypes.data, len(bo) - 1, _ptr(pairs),
                                          capacity, ctypes.byref(ms)))
        names = {OPT_LANES: "lanes", OPT_QUEUE: "queue", OPT_BLOCK: "block", OPT_RADIX_BITS: "radix_bits",
                 OPT_CELL_SCALE: "cell_scale", OPT_PER_LANE: "per_lane", OPT_SWEEP_SHAPE: "shape",
                 OPT_RUN_CAP: "run_cap"}
        return ms.value, {v: self.get_option(k) for k, v in names.items()}

    def batch_scene_pairs(self, n_scenes: int) -> np.ndarray:
        out = np.zeros(n_scenes, np.int64)
        self._check(self.lib.stq_batch_scene_pairs(self._h, out.ctypes.data, n_scenes))
        return out

    def batch_broadphase(self, V0, V1, voff, E, eoff, F, foff, pairs, capacity: int,
                         axis: int = AXIS_AUTO, inflation_radius: float = 0.0):
        """Fused batched pipeline (graph-captured unless OPT_GRAPH=2).
        Returns (SweepResult, per-scene pair counts)."""
        S = len(voff) - 1
        vo, eo, fo = (np.ascontiguousarray(x, np.int64) for x in (voff, eoff, foff))
        per = np.zeros(S, np.int64)
        c, tot = ctypes.c_int64(), ctypes.c_int64()
        st = self.lib.stq_batch_broadphase(self._h, _ptr(V0), _ptr(V1), vo.ctypes.data, _ptr(E),
                                           eo.ctypes.data, _ptr(F), fo.ctypes.data, S,
                                           float(inflation_radius), axis, _ptr(pairs), capacity,
                                           ctypes.byref(c), ctypes.byref(tot), per.ctypes.data)
        self._check(st, allow=(STQ_OK, STQ_OVERFLOW))
        return SweepResult(st, c.value, self.prepared_length, tot.value), per

    def sort_pairs(self, pairs, count: int) -> None:
        self._check(self.lib.stq_sort_pairs(self._h, _ptr(pairs), count))

    def brute_force(self, boxes, n: int, pairs, capacity: int) -> int:
        c = ctypes.c_int64()
        self._check(self.lib.stq_brute_force(self._h, _ptr(boxes), n, _ptr(pairs), capacity,
                                             ctypes.byref(c)), allow=(STQ_OK, STQ_OVERFLOW))
        return c.value


class Server:
    """Continuous-batching serving loop (stq_server*): time-stepped requests,
    admission by HBM budget, one batched launch per tick."""

    def __init__(self, device: int = 0, stream: int | None = None, budget_bytes: int = 160 << 30,
                 max_boxes: int = 1 << 24, max_scenes: int = 256):
        self.lib = load_library()
        self._h = _vp()
        st = self.lib.stq_server_create(device, stream, budget_bytes, max_boxes, max_scenes,
                                        ctypes.byref(self._h))
        if st != STQ_OK:
            raise STQError(st, "server creation failed")
        self.max_scenes = max_scenes
        self._meshes = {}

    def close(self) -> None:
        if self._h:
            self.lib.stq_server_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, mesh: "Mesh", steps: int, sigma: float, seed: int) -> int:
        rid = ctypes.c_int64()
        st = self.lib.stq_server_submit(self._h, mesh.V0.ctypes.data, mesh.V1.ctypes.data, mesh.V0.shape[0],
                                        mesh.E.ctypes.data, mesh.E.shape[0], mesh.F.ctypes.data,
                                        mesh.F.shape[0], steps, float(sigma), ctypes.c_uint64(seed),
                                        ctypes.byref(rid))
        if st != STQ_OK:
            raise STQError(st, "submit failed")
        self._meshes[rid.value] = mesh.V0.shape[0]
        return rid.value

    def tick(self) -> list:
        ids = (ctypes.c_int64 * 1024)()
        n = ctypes.c_int()
        st = self.lib.stq_server_tick(self._h, ids, 1024, ctypes.byref(n))
        if st != STQ_OK:
            raise STQError(st, "tick failed")
        return [ids[i] for i in range(min(n.value, 1024))]

    def result(self, rid: int):
        counts = np.zeros(4096, np.int64)
        checks = np.zeros(4096, np.uint64)
        done = ctypes.c_int()
        st = self.lib.stq_server_result(self._h, rid, counts.ctypes.data, checks.ctypes.data, 4096,
                                        ctypes.byref(done))
        if st != STQ_OK:
            raise STQError(st, "unknown request")
        return counts[: done.value].copy(), checks[: done.value].copy()

    def request_ticks(self, rid: int) -> tuple:
        """(first, last): indices of the ticks that ran the request's first and
        last timestep (-1 until then)."""
        a, b = ctypes.c_int64(), ctypes.c_int64()
        st = self.lib.stq_server_request_ticks(self._h, rid, ctypes.byref(a), ctypes.byref(b))
        if st != STQ_OK:
            raise STQError(st, "unknown request")
        return a.value, b.value

    def mesh(self, rid: int):
        nv = self._meshes[rid]
        V0, V1 = np.empty((nv, 3)), np.empty((nv, 3))
        st = self.lib.stq_server_mesh(self._h, rid, V0.ctypes.data, V1.ctypes.data)
        if st != STQ_OK:
            raise STQError(st, "request not active")
        return V0, V1

    def set_option(self, option: int, value: int) -> None:
        st = self.lib.stq_server_set_option(self._h, option, value)
        if st != STQ_OK:
            raise STQError(st, "server option")

    def stats(self) -> dict:
        a, q, b, t = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self.lib.stq_server_stats(self._h, ctypes.byref(a), ctypes.byref(q), ctypes.byref(b), ctypes.byref(t))
        return {"active": a.value, "queued": q.value, "bytes": b.value, "ticks": t.value}


def read_mesh(path) -> tuple:
    """(V [nV,3] f64, F [nF,3] i32) of an OBJ or PLY triangle mesh (stq_read_mesh)."""
    lib = load_library()
    nv, nf = ctypes.c_int64(), ctypes.c_int64()
    st = lib.stq_read_mesh(str(path).encode(), None, ctypes.byref(nv), None, ctypes.byref(nf))
    if st != STQ_OK:
        raise STQError(st, f"cannot read mesh {path}")
    V = np.empty((nv.value, 3))
    F = np.empty((nf.value, 3), np.int32)
    st = lib.stq_read_mesh(str(path).encode(), V.ctypes.data, ctypes.byref(nv), F.ctypes.data, ctypes.byref(nf))
    if st != STQ_OK:
        raise STQError(st, f"cannot read mesh {path}")
    return V, F


def mesh_edges(F: np.ndarray) -> np.ndarray:
    """Unique undirected edges of triangles F, ordered as libigl's edges()."""
    lib = load_library()
    F = np.ascontiguousarray(F, np.int32)
    ne = ctypes.c_int64()
    st = lib.stq_mesh_edges(F.ctypes.data, F.shape[0], None, ctypes.byref(ne))
    if st != STQ_OK:
        raise STQError(st, "edges")
    E = np.empty((ne.value, 2), np.int32)
    st = lib.stq_mesh_edges(F.ctypes.data, F.shape[0], E.ctypes.data, ctypes.byref(ne))
    if st != STQ_OK:
        raise STQError(st, "edges")
    return E


def parse_mesh(file_t0, file_t1) -> "Mesh":
    """parseMesh (src/io.cu:30-51): positions at t0 and t1 from two files with the
    same faces, edges from the faces."""
    V0, F0 = read_mesh(file_t0)
    V1, F1 = read_mesh(file_t1)
    if V0.shape != V1.shape or not np.array_equal(F0, F1):
        raise STQError(STQ_ERR_INVALID_INPUT, "t0 and t1 meshes differ in topology")
    return Mesh(V0, V1, mesh_edges(F1), F1)


def compare_truth_json(path, pairs: np.ndarray) -> tuple:
    """compare_mathematica: (truth pairs found, distinct truth pairs, pairs not in the truth)."""
    lib = load_library()
    p = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    f, t, e = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    st = lib.stq_compare_truth_json(str(path).encode(), p.ctypes.data, p.shape[0], ctypes.byref(f),
                                    ctypes.byref(t), ctypes.byref(e))
    if st != STQ_OK:
        raise STQError(st, f"cannot read {path}")
    return f.value, t.value, e.value


def pair_checksum(pairs: np.ndarray) -> int:
    """XOR over pairs of splitmix64((lo << 32) | hi): the serving loop's checksum."""
    p = np.asarray(pairs, np.int64).reshape(-1, 2)
    z = (p[:, 0].astype(np.uint64) << np.uint64(32)) | p[:, 1].astype(np.uint64)
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return int(np.bitwise_xor.reduce(z)) if len(z) else 0


# ---- synthetic scenes (libstq_scenes.so) ----------------------------------------
@dataclass
class Mesh:
    V0: np.ndarray  # [nV, 3] f64
    V1: np.ndarray
    E: np.ndarray   # [nE, 2] i32
    F: np.ndarray   # [nF, 3] i32

    @property
    def num_boxes(self) -> int:
        return self.V0.shape[0] + self.E.shape[0] + self.F.shape[0]


def grid_counts(g: int) -> tuple[int, int, int]:
    lib = load_scenes()
    nv, ne, nf = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    lib.stq_grid_counts(ctypes.c_int(g), ctypes.byref(nv), ctypes.byref(ne), ctypes.byref(nf))
    return nv.value, ne.value, nf.value


def _alloc_mesh(sheets: int, g: int) -> Mesh:
    nv, ne, nf = grid_counts(g)
    return Mesh(np.empty((sheets * nv, 3)), np.empty((sheets * nv, 3)),
                np.empty((sheets * ne, 2), np.int32), np.empty((sheets * nf, 3), np.int32))


def cloth_pair(g: int = 200, z_offset: float = 0.01, angle_deg: float = 10.0,
               sigma: float = 0.003, seed: int = 0) -> Mesh:
    """Two g x g cloth sheets (the single-scene and batched cloth-pair workloads)."""
    lib = load_scenes()
    m = _alloc_mesh(2, g)
    lib.stq_scene_cloth_pair(ctypes.c_int(g), ctypes.c_double(z_offset), ctypes.c_double(angle_deg),
                             ctypes.c_double(sigma), ctypes.c_uint64(seed),
                             m.V0.ctypes.data_as(_vp), m.V1.ctypes.data_as(_vp),
                             m.E.ctypes.data_as(_vp), m.F.ctypes.data_as(_vp))
    return m


def crumpled_sheets(sheets: int = 16, g: int = 250, amp: float = 0.05, sigma: float = 0.005,
                    seed: int = 1) -> Mesh:
    """`sheets` interpenetrating crumpled g x g sheets (the large single-scene workload)."""
    lib = load_scenes()
    m = _alloc_mesh(sheets, g)
    lib.stq_scene_crumpled(ctypes.c_int(sheets), ctypes.c_int(g), ctypes.c_double(amp),
                           ctypes.c_double(sigma), ctypes.c_uint64(seed),
                           m.V0.ctypes.data_as(_vp), m.V1.ctypes.data_as(_vp),
                           m.E.ctypes.data_as(_vp), m.F.ctypes.data_as(_vp))
    return m


def random_boxes(n: int, sliver_frac: float = 0.05, seed: int = 3) -> np.ndarray:
    """n random boxes with lognormal extents and 200x slivers (the skewed workload)."""
    lib = load_scenes()
    out = np.empty(n, AABB_DTYPE)
    lib.stq_scene_random_boxes(ctypes.c_int64(n), ctypes.c_double(sliver_frac),
                               ctypes.c_uint64(seed), out.ctypes.data_as(_vp))
    return out


def cloth_pair_grid_for(boxes: int) -> int:
    lib = load_scenes()
    lib.stq_cloth_pair_grid_for.restype = ctypes.c_int
    return int(lib.stq_cloth_pair_grid_for(ctypes.c_int64(boxes)))


def scene_step(mesh: Mesh, sigma: float, seed: int) -> None:
    """One serving time step: V0 <- V1, V1 <- V1 + N(0, sigma^2)."""
    lib = load_scenes()
    lib.stq_scene_step(ctypes.c_int64(mesh.V0.shape[0]), ctypes.c_double(sigma),
                       ctypes.c_uint64(seed), mesh.V0.ctypes.data_as(_vp), mesh.V1.ctypes.data_as(_vp))


def splitmix64(x: int) -> int:
    lib = load_scenes()
    lib.stq_splitmix64.restype = ctypes.c_uint64
    return int(lib.stq_splitmix64(ctypes.c_uint64(x)))


def concat_meshes(meshes: list) -> tuple:
    """Concatenates meshes into one batch: (V0, V1, E, F, voff, eoff, foff), with
    vertex indices kept local to each scene."""
    V0 = np.concatenate([m.V0 for m in meshes]) if meshes else np.zeros((0, 3))
    V1 = np.concatenate([m.V1 for m in meshes]) if meshes else np.zeros((0, 3))
    E = np.concatenate([m.E for m in meshes]) if meshes else np.zeros((0, 2), np.int32)
    F = np.concatenate([m.F for m in meshes]) if meshes else np.zeros((0, 3), np.int32)
    off = lambda k: np.concatenate([[0], np.cumsum([k(m) for m in meshes])]).astype(np.int64)  # noqa: E731
    return (V0, V1, E, F, off(lambda m: m.V0.shape[0]), off(lambda m: m.E.shape[0]),
            off(lambda m: m.F.shape[0]))


def batch_scenes(n_scenes: int = 256, lo: float = 1e3, hi: float = 2e5, seed: int = 2) -> list:
    """Cloth-pair scenes with box counts log-uniform in [lo, hi], sheet offset
    U(0.002, 0.05) and motion sigma U(0.001, 0.01), per-scene seeds by splitmix64."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(n_scenes):
        target = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        g = cloth_pair_grid_for(int(target))
        out.append(cloth_pair(g=g, z_offset=float(rng.uniform(0.002, 0.05)), angle_deg=10.0,
                              sigma=float(rng.uniform(0.001, 0.01)), seed=splitmix64(seed * 1000003 + s)))
    return out
