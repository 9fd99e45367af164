"""ctypes binding of the CPU oracle (oracle/stq_oracle.cpp). TEST INFRASTRUCTURE.

Only the tests, the smoke check and the benchmark's CPU-baseline and reference
legs use this module, to check and time against.

Parity status: pinned to the reference's own code. Where the reference's
source tree is present, `make ref` compiles its src/cpu/aabb.cpp and
src/cpu/sweep.cpp unchanged (against the stand-in headers of ref_shim/) into
_ref/libstq_ref.so; the tests check the restatement against it (ref_* below),
and tests/golden/make_ref_golden.py writes its outputs as golden vectors that
travel with the repository. The hand-derived known-answer cases under
tests/golden/ pin the corner cases on top.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libstq_oracle.so"
REF_LIB = HERE / "_ref" / "libstq_ref.so"
REF_TREE = Path("/root/reference")  # the reference's sources, where present

_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = ctypes.CDLL(str(LIB))
        L.oracle_construct_boxes.argtypes = [_vp, _vp, _i64, _vp, _i64, _vp, _i64, ctypes.c_double, _vp]
        L.oracle_construct_boxes.restype = None
        L.oracle_sort_along_xaxis.argtypes = [_vp, _i64, ctypes.c_int]
        L.oracle_sweep.argtypes = [_vp, _i64, _i64, ctypes.c_int, ctypes.POINTER(_vp)]
        L.oracle_sweep.restype = _i64
        L.oracle_broadphase.argtypes = [_vp, _i64, ctypes.c_int, ctypes.POINTER(_vp)]
        L.oracle_broadphase.restype = _i64
        L.oracle_canonicalize.argtypes = [_vp, _i64, ctypes.c_int]
        L.oracle_canonicalize.restype = _i64
        L.oracle_compare.argtypes = [_vp, _i64, _vp, _i64, ctypes.POINTER(_i64), ctypes.POINTER(_i64)]
        L.oracle_time_sample.argtypes = [_vp, _i64, _i64, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        L.oracle_time_sample.restype = _i64
        L.oracle_default_threads.restype = ctypes.c_int
        L.oracle_free.argtypes = [_vp]
        _lib = L
    return _lib


def _take(ptr: _vp, n: int) -> np.ndarray:
    L = lib()
    if n == 0:
        L.oracle_free(ptr)
        return np.zeros((0, 2), np.int32)
    arr = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_int32)), shape=(n * 2,))
    out = arr.reshape(n, 2).copy()
    L.oracle_free(ptr)
    return out


def construct_boxes(V0, V1, E, F, aabb_dtype, inflation_radius: float = 0.0) -> np.ndarray:
    """stq::cpu::constructBoxes restated (src/cpu/aabb.cpp:7-95)."""
    V0 = np.ascontiguousarray(V0, np.float64)
    V1 = np.ascontiguousarray(V1, np.float64)
    E = np.ascontiguousarray(E, np.int32).reshape(-1, 2)
    F = np.ascontiguousarray(F, np.int32).reshape(-1, 3)
    out = np.empty(V0.shape[0] + E.shape[0] + F.shape[0], aabb_dtype)
    lib().oracle_construct_boxes(V0.ctypes.data, V1.ctypes.data, V0.shape[0], E.ctypes.data,
                                 E.shape[0], F.ctypes.data, F.shape[0], inflation_radius,
                                 out.ctypes.data)
    return out


def broadphase(boxes: np.ndarray, threads: int = 0) -> np.ndarray:
    """Sort along x + sweep (src/cpu/sweep.cpp:72-121), canonical sorted unique pairs."""
    boxes = np.ascontiguousarray(boxes)
    p = _vp()
    n = lib().oracle_broadphase(boxes.ctypes.data, boxes.shape[0], threads, ctypes.byref(p))
    return _take(p, n)


def sweep_sorted(sorted_boxes: np.ndarray, n_start: int, threads: int = 0) -> np.ndarray:
    """stq::cpu::sweep over the first n_start start boxes, raw (a.id, b.id) pairs."""
    p = _vp()
    n = lib().oracle_sweep(sorted_boxes.ctypes.data, sorted_boxes.shape[0], n_start, threads,
                           ctypes.byref(p))
    return _take(p, n)


def sort_along_xaxis(boxes: np.ndarray, threads: int = 0) -> None:
    lib().oracle_sort_along_xaxis(boxes.ctypes.data, boxes.shape[0], threads)


def canonical(pairs: np.ndarray, threads: int = 0) -> np.ndarray:
    """(min id, max id), sorted lexicographically, duplicates removed."""
    p = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2).copy()
    n = lib().oracle_canonicalize(p.ctypes.data, p.shape[0], threads)
    return p[:n]


def compare(a: np.ndarray, b: np.ndarray) -> tuple[int, int]:
    """Counts of canonical pairs only in a and only in b."""
    a = np.ascontiguousarray(a, np.int32)
    b = np.ascontiguousarray(b, np.int32)
    oa, ob = _i64(), _i64()
    lib().oracle_compare(a.ctypes.data, a.shape[0], b.ctypes.data, b.shape[0],
                         ctypes.byref(oa), ctypes.byref(ob))
    return oa.value, ob.value


def time_sample(boxes: np.ndarray, stride: int, threads: int = 0) -> tuple[float, float, int]:
    """Seconds to sort all boxes along x and to sweep every stride-th start box."""
    s1, s2 = ctypes.c_double(), ctypes.c_double()
    n = lib().oracle_time_sample(boxes.ctypes.data, boxes.shape[0], stride, threads,
                                 ctypes.byref(s1), ctypes.byref(s2))
    return s1.value, s2.value, n


def default_threads() -> int:
    return int(lib().oracle_default_threads())


# ---- the benchmark's synthetic inputs, from the generators linked into the
# oracle library (the same source as the package's), for CPU-only processes --
def _grid_counts(g: int) -> tuple[int, int, int]:
    nv, ne, nf = _i64(), _i64(), _i64()
    lib().stq_grid_counts(ctypes.c_int(g), ctypes.byref(nv), ctypes.byref(ne), ctypes.byref(nf))
    return nv.value, ne.value, nf.value


def crumpled_sheets(sheets: int, g: int, amp: float, sigma: float, seed: int):
    """V0, V1, E, F of `sheets` crumpled g x g sheets (scenes.h stq_scene_crumpled)."""
    nv, ne, nf = _grid_counts(g)
    V0, V1 = np.empty((sheets * nv, 3)), np.empty((sheets * nv, 3))
    E, F = np.empty((sheets * ne, 2), np.int32), np.empty((sheets * nf, 3), np.int32)
    lib().stq_scene_crumpled(ctypes.c_int(sheets), ctypes.c_int(g), ctypes.c_double(amp), ctypes.c_double(sigma),
                             ctypes.c_uint64(seed), V0.ctypes.data_as(_vp), V1.ctypes.data_as(_vp),
                             E.ctypes.data_as(_vp), F.ctypes.data_as(_vp))
    return V0, V1, E, F


def cloth_pair(g: int, z_offset: float, sigma: float, seed: int, angle_deg: float = 10.0):
    """V0, V1, E, F of a cloth pair (scenes.h stq_scene_cloth_pair)."""
    nv, ne, nf = _grid_counts(g)
    V0, V1 = np.empty((2 * nv, 3)), np.empty((2 * nv, 3))
    E, F = np.empty((2 * ne, 2), np.int32), np.empty((2 * nf, 3), np.int32)
    lib().stq_scene_cloth_pair(ctypes.c_int(g), ctypes.c_double(z_offset), ctypes.c_double(angle_deg),
                               ctypes.c_double(sigma), ctypes.c_uint64(seed), V0.ctypes.data_as(_vp),
                               V1.ctypes.data_as(_vp), E.ctypes.data_as(_vp), F.ctypes.data_as(_vp))
    return V0, V1, E, F


# the 44-byte box record (id, min, max, vertex ids, ref_id)
AABB_DTYPE = np.dtype([("id", "<i4"), ("min", "<f4", (3,)), ("max", "<f4", (3,)),
                       ("vertex_ids", "<i4", (3,)), ("ref_id", "<i4")])


# ---- the reference's own CPU code (oracle/_ref), where it could be built ------
_ref = None


def build_ref() -> bool:
    """Compiles oracle/_ref/libstq_ref.so from the reference's source tree, if
    that tree is present; returns whether the library exists."""
    if (REF_TREE / "src" / "cpu" / "sweep.cpp").exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={REF_TREE}"], check=True)
    return REF_LIB.exists()


def ref_available() -> bool:
    return REF_LIB.exists()


def ref_lib() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        L = ctypes.CDLL(str(REF_LIB))
        L.ref_construct_boxes.argtypes = [_vp, _vp, _i64, _vp, _i64, _vp, _i64, ctypes.c_double, ctypes.c_int, _vp]
        L.ref_construct_boxes.restype = None
        L.ref_broadphase.argtypes = [_vp, _i64, ctypes.c_int, ctypes.POINTER(_vp)]
        L.ref_broadphase.restype = _i64
        L.ref_free.argtypes = [_vp]
        _ref = L
    return _ref


def ref_construct_boxes(V0, V1, E, F, aabb_dtype, inflation_radius: float = 0.0, threads: int = 0) -> np.ndarray:
    """stq::cpu::constructBoxes of the reference itself (src/cpu/aabb.cpp:7-95)."""
    V0 = np.ascontiguousarray(V0, np.float64)
    V1 = np.ascontiguousarray(V1, np.float64)
    E = np.ascontiguousarray(E, np.int32).reshape(-1, 2)
    F = np.ascontiguousarray(F, np.int32).reshape(-1, 3)
    out = np.empty(V0.shape[0] + E.shape[0] + F.shape[0], aabb_dtype)
    ref_lib().ref_construct_boxes(V0.ctypes.data, V1.ctypes.data, V0.shape[0], E.ctypes.data, E.shape[0],
                                  F.ctypes.data, F.shape[0], inflation_radius, threads, out.ctypes.data)
    return out


def ref_broadphase(boxes: np.ndarray, threads: int = 0) -> np.ndarray:
    """The reference's own sort + sweep (src/cpu/sweep.cpp:72-157, driven as
    app/main.cpp:147-151 drives it): canonical sorted unique pairs."""
    boxes = np.ascontiguousarray(boxes)
    p = _vp()
    L = ref_lib()
    n = L.ref_broadphase(boxes.ctypes.data, boxes.shape[0], threads, ctypes.byref(p))
    if n == 0:
        L.ref_free(p)
        return np.zeros((0, 2), np.int32)
    raw = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_int32)), shape=(n * 2,)).reshape(n, 2).copy()
    L.ref_free(p)
    return canonical(raw, threads)
