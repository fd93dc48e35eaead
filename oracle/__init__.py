"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke()
(as the checker) and by bench.py's CPU-baseline leg.  The product never
imports this package.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .build_lib import ORACLE_LIB, build_oracle

_lib = None

NODE2 = np.dtype([("bmin", "<f4", 3), ("bmax", "<f4", 3), ("left", "<u4"), ("right", "<u4")])
NODE8 = np.dtype([("p", "<f4", 3), ("e", "u1", 3), ("imask", "u1"), ("child_base", "<u4"), ("prim_base", "<u4"),
                  ("meta", "u1", 8), ("qlo", "u1", (3, 8)), ("qhi", "u1", (3, 8))])
INVALID = 0xFFFFFFFF


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not ORACLE_LIB.exists():
            build_oracle()
        lib = ctypes.CDLL(str(ORACLE_LIB))
        P = ctypes.c_void_p
        U = ctypes.c_uint32
        sig = {
            "orc_set_threads": (None, [ctypes.c_int]),
            "orc_set_level_collapse": (None, [ctypes.c_int]),
            "orc_get_threads": (ctypes.c_int, []),
            "orc_set_area_form": (None, [ctypes.c_int]),
            "orc_get_area_form": (ctypes.c_int, []),
            "orc_set_u8_mode": (None, [ctypes.c_int]),
            "orc_get_u8_mode": (ctypes.c_int, []),
            "orc_set_min_zero_mode": (None, [ctypes.c_int]),
            "orc_area": (ctypes.c_float, [P]),
            "orc_fmin": (ctypes.c_float, [ctypes.c_float, ctypes.c_float]),
            "orc_fmax": (ctypes.c_float, [ctypes.c_float, ctypes.c_float]),
            "orc_f2u8": (ctypes.c_uint8, [ctypes.c_float]),
            "orc_scene_bounds": (None, [P, ctypes.c_int, U, P, P]),
            "orc_morton": (None, [P, U, P, ctypes.c_int, P, P]),
            "orc_morton_quantised": (None, [P, U, P, ctypes.c_int, P, P]),
            "orc_radix_sort": (None, [ctypes.c_int, P, P, U, U, U, P, P]),
            "orc_stable_sort": (None, [ctypes.c_int, P, U, U, U, P, P]),
            "orc_hploc": (ctypes.c_int, [ctypes.c_int, P, P, U, U, P, P]),
            "orc_bvh8": (ctypes.c_int, [P, U, U, P, U, P, P, P]),
            "orc_bvh8_ex": (ctypes.c_int, [P, U, U, P, U, P, P, P, U]),
            "orc_compare_bvh8_unordered": (ctypes.c_uint64, [P, U, P, P, U, P, U, P]),
            "orc_bvh2_cost": (ctypes.c_double, [P, U, P]),
            "orc_bvh8_cost": (ctypes.c_double, [P, U, P]),
            "orc_validate_bvh2": (ctypes.c_uint64, [P, U, U, P]),
            "orc_validate_bvh8": (ctypes.c_uint64, [P, U, P, U, P, P]),
            "orc_compare_bvh2": (ctypes.c_uint64, [P, U, P, U, U]),
            "orc_compare_bvh8": (ctypes.c_uint64, [P, U, P, P, U, P, U]),
            "orc_build": (ctypes.c_int, [P, ctypes.c_int, U, ctypes.c_int, U, P, P, U, P, P, P]),
            "orc_digest_bvh2": (ctypes.c_uint64, [P, U, U]),
            "orc_digest_bvh8": (ctypes.c_uint64, [P, U, P, U]),
            "orc_find_nn": (None, [U, P, U, P]),
            "orc_auction": (ctypes.c_int, [P, P, U, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _p(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def set_threads(t: int) -> None:
    load().orc_set_threads(t)


def threads() -> int:
    return load().orc_get_threads()


def scene_bounds(prims: np.ndarray):
    """-> (leaves NODE2[n], scene float32[6])"""
    n = prims.shape[0]
    prims = np.ascontiguousarray(prims, dtype=np.float32)
    leaves = np.zeros(n, dtype=NODE2)
    scene = np.zeros(6, dtype=np.float32)
    load().orc_scene_bounds(_p(prims), 1 if prims.shape[1] == 9 else 0, n, _p(leaves), _p(scene))
    return leaves, scene


def morton(leaves: np.ndarray, scene: np.ndarray, key_bits: int) -> np.ndarray:
    n = leaves.shape[0]
    keys = np.zeros(n, dtype=np.uint32 if key_bits == 30 else np.uint64)
    load().orc_morton(_p(leaves), n, _p(np.ascontiguousarray(scene, np.float32)), key_bits, _p(keys), None)
    return keys


def morton_quantised(leaves, scene, key_bits):
    """-> (q uint32[n,3], products float32[n,3]) with IEEE division."""
    n = leaves.shape[0]
    q = np.zeros((n, 3), dtype=np.uint32)
    prod = np.zeros((n, 3), dtype=np.float32)
    load().orc_morton_quantised(_p(leaves), n, _p(np.ascontiguousarray(scene, np.float32)), key_bits, _p(q), _p(prod))
    return q, prod


def radix_sort(keys: np.ndarray, begin_bit: int, end_bit: int, vals: np.ndarray | None = None):
    n = keys.shape[0]
    kout = np.zeros_like(keys)
    vout = np.zeros(n, dtype=np.uint32)
    vin = None if vals is None else _p(np.ascontiguousarray(vals, np.uint32))
    load().orc_radix_sort(keys.itemsize, _p(np.ascontiguousarray(keys)), vin, n, begin_bit, end_bit, _p(kout),
                          _p(vout))
    return kout, vout


def stable_sort(keys: np.ndarray, begin_bit: int, end_bit: int):
    n = keys.shape[0]
    kout = np.zeros_like(keys)
    vout = np.zeros(n, dtype=np.uint32)
    load().orc_stable_sort(keys.itemsize, _p(np.ascontiguousarray(keys)), n, begin_bit, end_bit, _p(kout), _p(vout))
    return kout, vout


def hploc(sorted_keys: np.ndarray, perm: np.ndarray, leaves: np.ndarray, radius: int = 8):
    """-> (nodes NODE2[2n-1], root, error bits)"""
    n = leaves.shape[0]
    nodes = np.zeros(2 * n - 1, dtype=NODE2)
    nodes[:n] = leaves
    root = ctypes.c_uint32(0)
    err = load().orc_hploc(sorted_keys.itemsize, _p(np.ascontiguousarray(sorted_keys)),
                           _p(np.ascontiguousarray(perm, np.uint32)), n, radius, _p(nodes), ctypes.byref(root))
    return nodes, root.value, err


def bvh8_capacity(n: int) -> int:
    return (4 * n - 1 + 6) // 7


def set_level_collapse(on: bool) -> None:
    """build(): BVH8 stage by the level-parallel collapse (the timed CPU
    baseline) instead of the work-slot-order one (the default)."""
    load().orc_set_level_collapse(1 if on else 0)


def bvh8(bvh2_nodes: np.ndarray, n: int, root: int, auction: bool = False, levels: bool = False):
    """-> (nodes NODE8[count], prim_idx uint32[n], error bits); auction selects
    the USE_AUCTION slot assignment (WideConverter.cu:50-102); levels the
    level-parallel collapse (same tree, breadth-first numbering)."""
    cap = bvh8_capacity(n)
    out = np.zeros(cap, dtype=NODE8)
    prim = np.zeros(n, dtype=np.uint32)
    nc = ctypes.c_uint32(0)
    lc = ctypes.c_uint32(0)
    err = load().orc_bvh8_ex(_p(np.ascontiguousarray(bvh2_nodes)), n, root, _p(out), cap, _p(prim),
                             ctypes.byref(nc), ctypes.byref(lc), (1 if auction else 0) | (2 if levels else 0))
    return out[: nc.value].copy(), prim, err


def bvh2_cost(nodes: np.ndarray, root_box: np.ndarray) -> float:
    return load().orc_bvh2_cost(_p(np.ascontiguousarray(nodes)), nodes.shape[0],
                                _p(np.ascontiguousarray(root_box, np.float32)))


def bvh8_cost(nodes: np.ndarray, root_box: np.ndarray) -> float:
    return load().orc_bvh8_cost(_p(np.ascontiguousarray(nodes)), nodes.shape[0],
                                _p(np.ascontiguousarray(root_box, np.float32)))


BVH2_REPORT = ("visited", "leaves", "dup_prims", "missing_prims", "bad_union", "not_contained", "bad_index",
               "max_depth")
BVH8_REPORT = ("visited", "leaves", "dup_prims", "missing_prims", "bad_index", "lo_not_conservative",
               "hi_not_conservative", "slots_used", "max_depth", "meta_errors")


def validate_bvh2(nodes: np.ndarray, n: int, root: int):
    rep = np.zeros(8, dtype=np.uint64)
    errs = load().orc_validate_bvh2(_p(np.ascontiguousarray(nodes)), n, root, _p(rep))
    return int(errs), dict(zip(BVH2_REPORT, map(int, rep)))


def validate_bvh8(nodes: np.ndarray, prim_idx: np.ndarray, n: int, leaves: np.ndarray):
    rep = np.zeros(10, dtype=np.uint64)
    errs = load().orc_validate_bvh8(_p(np.ascontiguousarray(nodes)), nodes.shape[0],
                                    _p(np.ascontiguousarray(prim_idx, np.uint32)), n, _p(np.ascontiguousarray(leaves)),
                                    _p(rep))
    return int(errs), dict(zip(BVH8_REPORT, map(int, rep)))


def compare_bvh2(a: np.ndarray, a_root: int, b: np.ndarray, b_root: int, n: int) -> int:
    return int(load().orc_compare_bvh2(_p(np.ascontiguousarray(a)), a_root, _p(np.ascontiguousarray(b)), b_root, n))


def compare_bvh8(a: np.ndarray, a_prim: np.ndarray, b: np.ndarray, b_prim: np.ndarray, n: int) -> int:
    return int(load().orc_compare_bvh8(_p(np.ascontiguousarray(a)), a.shape[0],
                                       _p(np.ascontiguousarray(a_prim, np.uint32)), _p(np.ascontiguousarray(b)),
                                       b.shape[0], _p(np.ascontiguousarray(b_prim, np.uint32)), n))


def compare_bvh8_unordered(a: np.ndarray, a_prim: np.ndarray, b: np.ndarray, b_prim: np.ndarray, n: int):
    """-> (0 if the trees are equal up to the slot order inside nodes, number
    of node pairs whose slot order differs)"""
    r = ctypes.c_uint32(0)
    res = load().orc_compare_bvh8_unordered(_p(np.ascontiguousarray(a)), a.shape[0],
                                            _p(np.ascontiguousarray(a_prim, np.uint32)), _p(np.ascontiguousarray(b)),
                                            b.shape[0], _p(np.ascontiguousarray(b_prim, np.uint32)), n, ctypes.byref(r))
    return int(res), int(r.value)


def digest_bvh2(nodes: np.ndarray, root: int, n: int) -> int:
    return int(load().orc_digest_bvh2(_p(np.ascontiguousarray(nodes)), root, n))


def digest_bvh8(nodes: np.ndarray, prim_idx: np.ndarray, n: int) -> int:
    return int(load().orc_digest_bvh8(_p(np.ascontiguousarray(nodes)), nodes.shape[0],
                                      _p(np.ascontiguousarray(prim_idx, np.uint32)), n))


def build(prims: np.ndarray, key_bits: int, radius: int = 8, wide: bool = True):
    """Whole CPU pipeline.  -> dict(bvh2, root, bvh8, prim_idx, stage_ms, err)"""
    n = prims.shape[0]
    prims = np.ascontiguousarray(prims, dtype=np.float32)
    nodes = np.zeros(2 * n - 1, dtype=NODE2)
    cap = bvh8_capacity(n)
    b8 = np.zeros(cap, dtype=NODE8) if wide else None
    prim = np.zeros(n, dtype=np.uint32)
    counts = np.zeros(3, dtype=np.uint32)
    ms = np.zeros(5, dtype=np.float64)
    err = load().orc_build(_p(prims), 1 if prims.shape[1] == 9 else 0, n, key_bits, radius, _p(nodes),
                           _p(b8) if wide else None, cap, _p(prim), _p(counts), _p(ms))
    out = dict(bvh2=nodes, root=int(counts[2]), stage_ms=ms.tolist(), err=err)
    if wide:
        out.update(bvh8=b8[: counts[0]].copy(), prim_idx=prim, bvh8_leaves=int(counts[1]))
    return out
