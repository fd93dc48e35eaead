"""Test helpers: run each stage of the CUDA pipeline through the C ABI on
torch-allocated device buffers and return numpy arrays."""
from __future__ import annotations

import numpy as np

import nexusbvh_gb300 as nxb
from nexusbvh_gb300 import BVH2_NODE_DTYPE, BVH8_NODE_DTYPE


def torch():
    import torch as t
    return t


def dev(a: np.ndarray):
    return torch().from_numpy(np.ascontiguousarray(a)).cuda()


def host(t, dtype=None) -> np.ndarray:
    a = t.cpu().numpy()
    return a.view(dtype) if dtype is not None else a


def stream() -> int:
    return int(torch().cuda.current_stream().cuda_stream)


def check(status, what):
    nxb.check(status, what)


def stage_bounds(prims: np.ndarray):
    t = torch()
    lib = nxb.load()
    n = prims.shape[0]
    d_prims = dev(prims.astype(np.float32))
    d_nodes = t.zeros((2 * n - 1) * 32, dtype=t.uint8, device="cuda")
    d_scene = t.zeros(6, dtype=t.float32, device="cuda")
    ptype = nxb.NXB_PRIM_TRIANGLE if prims.shape[1] == 9 else nxb.NXB_PRIM_AABB
    check(lib.nxb_stage_scene_bounds(d_prims.data_ptr(), ptype, n, d_nodes.data_ptr(), d_scene.data_ptr(), stream()),
          "nxb_stage_scene_bounds")
    t.cuda.synchronize()
    return d_nodes, d_scene


def stage_morton(d_nodes, d_scene, n: int, key_bits: int):
    t = torch()
    lib = nxb.load()
    d_keys = t.zeros(n, dtype=t.int32 if key_bits == 30 else t.int64, device="cuda")
    check(lib.nxb_stage_morton(d_nodes.data_ptr(), n, d_scene.data_ptr(), key_bits, d_keys.data_ptr(), None, stream()),
          "nxb_stage_morton")
    t.cuda.synchronize()
    return d_keys


def stage_sort(d_keys, n: int, key_bits: int, begin=None, end=None, d_vals=None):
    t = torch()
    lib = nxb.load()
    kb = 4 if key_bits == 30 else 8
    begin = (2 if kb == 4 else 1) if begin is None else begin
    end = kb * 8 if end is None else end
    d_kout = t.empty_like(d_keys)
    d_vout = t.empty(n, dtype=t.int32, device="cuda")
    scratch = lib.nxb_sort_scratch_bytes(n, kb, begin, end)
    d_scr = t.empty(scratch, dtype=t.uint8, device="cuda")
    d_err = t.zeros(1, dtype=t.int32, device="cuda")
    check(lib.nxb_stage_radix_sort(kb, d_keys.data_ptr(), d_kout.data_ptr(),
                                   None if d_vals is None else d_vals.data_ptr(), d_vout.data_ptr(), n, begin, end,
                                   d_scr.data_ptr(), scratch, d_err.data_ptr(), stream()), "nxb_stage_radix_sort")
    t.cuda.synchronize()
    assert int(d_err.item()) == 0, f"sort error word {int(d_err.item()):#x}"
    return d_kout, d_vout


def stage_hploc(d_sorted_keys, d_perm, d_nodes, n: int, key_bits: int, radius: int = 8):
    """Runs H-PLOC on copies (the stage overwrites cluster ids)."""
    t = torch()
    lib = nxb.load()
    kb = 4 if key_bits == 30 else 8
    nodes = d_nodes.clone()
    cluster = d_perm.clone()
    scratch = lib.nxb_hploc_scratch_bytes(n)
    d_scr = t.empty(scratch, dtype=t.uint8, device="cuda")
    d_err = t.zeros(1, dtype=t.int32, device="cuda")
    check(lib.nxb_stage_hploc(kb, d_sorted_keys.data_ptr(), cluster.data_ptr(), nodes.data_ptr(), n, radius,
                              d_scr.data_ptr(), scratch, d_err.data_ptr(), stream()), "nxb_stage_hploc")
    t.cuda.synchronize()
    assert int(d_err.item()) == 0, f"hploc error word {int(d_err.item()):#x}"
    return nodes


def stage_bvh8(d_bvh2_nodes, n: int, flags: int = 0):
    t = torch()
    lib = nxb.load()
    cap = (4 * n - 1 + 6) // 7
    d_out = t.zeros(cap * 80, dtype=t.uint8, device="cuda")
    d_prim = t.zeros(n, dtype=t.int32, device="cuda")
    d_counts = t.zeros(2, dtype=t.int32, device="cuda")
    scratch = lib.nxb_bvh8_scratch_bytes(n)
    d_scr = t.empty(scratch, dtype=t.uint8, device="cuda")
    d_err = t.zeros(1, dtype=t.int32, device="cuda")
    check(lib.nxb_stage_bvh8_ex(d_bvh2_nodes.data_ptr(), n, d_out.data_ptr(), d_prim.data_ptr(),
                                d_counts.data_ptr(), d_scr.data_ptr(), scratch, flags, d_err.data_ptr(), stream()),
          "nxb_stage_bvh8_ex")
    t.cuda.synchronize()
    assert int(d_err.item()) == 0, f"bvh8 error word {int(d_err.item()):#x}"
    counts = host(d_counts).astype(np.uint32)
    nodes = host(d_out).view(BVH8_NODE_DTYPE)[: counts[0]].copy()
    return nodes, host(d_prim).astype(np.uint32), int(counts[0]), int(counts[1])


def cost_bvh2(d_nodes, count: int, root_box: np.ndarray) -> float:
    t = torch()
    d_root = dev(root_box.astype(np.float32))
    d_cost = t.zeros(1, dtype=t.float32, device="cuda")
    check(nxb.load().nxb_eval_bvh2_cost(d_nodes.data_ptr(), count, d_root.data_ptr(), d_cost.data_ptr(), stream()),
          "nxb_eval_bvh2_cost")
    return float(d_cost.item())


def cost_bvh8(bvh8_nodes: np.ndarray, root_box: np.ndarray) -> float:
    t = torch()
    d_nodes = dev(bvh8_nodes.view(np.uint8))
    d_root = dev(root_box.astype(np.float32))
    d_cost = t.zeros(1, dtype=t.float32, device="cuda")
    check(nxb.load().nxb_eval_bvh8_cost(d_nodes.data_ptr(), bvh8_nodes.shape[0], d_root.data_ptr(),
                                        d_cost.data_ptr(), stream()), "nxb_eval_bvh8_cost")
    return float(d_cost.item())


def nodes2(d_nodes) -> np.ndarray:
    return host(d_nodes).view(BVH2_NODE_DTYPE).copy()


def build_async(prims: np.ndarray, key_bits: int, radius: int = 8, wide: bool = True):
    """Whole pipeline through nxb_build_async."""
    t = torch()
    b = nxb.Builder()
    cfg = nxb.BuildConfig(prioritize_speed=key_bits == 30, search_radius=radius)
    out = b.build(dev(prims.astype(np.float32)), cfg, wide=wide)
    t.cuda.synchronize()
    return out


def root_box(nodes: np.ndarray, root: int) -> np.ndarray:
    return np.concatenate([nodes[root]["bmin"], nodes[root]["bmax"]]).astype(np.float32)
