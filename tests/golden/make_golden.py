"""Generates the golden fixtures from the reference's own CUDA build.

Run on a machine with a GPU after oracle/build_ref.py has built
oracle/_ref/libnxbref_r*.so (the reference compiled from its sources):

    python tests/golden/make_golden.py

For each case the reference is driven through its public API (BuildBVH2,
BuildBVH8) and through its private stage kernels (scene bounds, Morton
codes, CUB radix sort), and the outputs are saved next to the inputs:

  small cases (n <= 4096): tests/golden/<case>.npz with the triangles, the
      scene box, unsorted and sorted Morton keys, the sorted permutation,
      every BVH2 node, every BVH8 node and primIdx, the SAH/BVH8 costs;
  the 65,536-triangle plain config: keys and permutation in full, BVH2 and
      BVH8 as canonical digests (the triangles regenerate from the seed;
      their SHA-256 is stored to check that).

The reference ships no tests or golden data of its own; these fixtures are
the pin for both the CPU oracle (tests/test_golden.py, no GPU) and the CUDA
kernels (GPU tests).
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent

SMALL_CASES = [
    # name, generator, args, key_bits, radius, prim kind
    ("soup4096_k30", "uniform_soup", dict(n=4096, seed=0), 30, 8, "tri"),
    ("soup4096_k63", "uniform_soup", dict(n=4096, seed=0), 63, 8, "tri"),
    ("sphere64x32_k30", "displaced_sphere", dict(nu=64, nv=32, seed=1), 30, 8, "tri"),
    ("sphere64x32_k63", "displaced_sphere", dict(nu=64, nv=32, seed=1), 63, 8, "tri"),
    ("clustered4096_k63", "clustered", dict(n=4096, seed=2), 63, 8, "tri"),
    ("clustered4096_k63_r16", "clustered", dict(n=4096, seed=2), 63, 16, "tri"),
    ("clustered4096_k63_r4", "clustered", dict(n=4096, seed=2), 63, 4, "tri"),
    ("aabb3000_k63", "clustered", dict(n=3000, seed=5), 63, 8, "aabb"),
    ("aabb3000_k30", "uniform_soup", dict(n=3000, seed=7), 30, 8, "aabb"),
    ("n1_k30", "uniform_soup", dict(n=1, seed=1), 30, 8, "tri"),
    ("n2_k63", "uniform_soup", dict(n=2, seed=2), 63, 8, "tri"),
    ("n17_k30", "uniform_soup", dict(n=17, seed=17), 30, 8, "tri"),
    ("n33_k63", "uniform_soup", dict(n=33, seed=33), 63, 8, "tri"),
    ("n100_k30", "uniform_soup", dict(n=100, seed=100), 30, 8, "tri"),
]
DIGEST_CASES = [("soup65536_k30", "uniform_soup", dict(n=65536, seed=0), 30, 8, "tri"),
                ("soup65536_k63", "uniform_soup", dict(n=65536, seed=0), 63, 8, "tri")]


def make_prims(gen, kw, kind):
    from nexusbvh_gb300 import scenes
    p = getattr(scenes, gen)(**kw)
    return scenes.to_boxes(p) if kind == "aabb" else p


def run_reference(prims, key_bits, radius):
    import torch

    from oracle import build_ref
    lib = ctypes.CDLL(str(build_ref.lib_path(radius)))
    P, U = ctypes.c_void_p, ctypes.c_uint32
    lib.ref_build_bvh8.argtypes = [P, ctypes.c_int, U, ctypes.c_int, P, P, P, P, P]
    lib.ref_build_bvh2.argtypes = [P, ctypes.c_int, U, ctypes.c_int, P, P, P]
    lib.ref_stages.argtypes = [P, ctypes.c_int, U, ctypes.c_int, P, P, P, P, P]
    n = prims.shape[0]
    pt = 1 if prims.shape[1] == 9 else 0
    ps = 1 if key_bits == 30 else 0
    kt = torch.int32 if key_bits == 30 else torch.int64
    kdt = np.uint32 if key_bits == 30 else np.uint64
    d = torch.from_numpy(np.ascontiguousarray(prims)).cuda()
    leaves = torch.zeros((2 * n - 1) * 32, dtype=torch.uint8, device="cuda")
    keys = torch.zeros(n, dtype=kt, device="cuda")
    sk = torch.zeros(n, dtype=kt, device="cuda")
    perm = torch.zeros(n, dtype=torch.int32, device="cuda")
    scene = (ctypes.c_float * 6)()
    assert lib.ref_stages(d.data_ptr(), pt, n, ps, leaves.data_ptr(), scene, keys.data_ptr(), sk.data_ptr(),
                          perm.data_ptr()) == 0
    b2 = torch.zeros((2 * n - 1) * 32, dtype=torch.uint8, device="cuda")
    m2 = (ctypes.c_float * 9)()
    assert lib.ref_build_bvh2(d.data_ptr(), pt, n, ps, b2.data_ptr(), None, m2) == 0
    cap = (4 * n - 1 + 6) // 7
    b8 = torch.zeros(cap * 80, dtype=torch.uint8, device="cuda")
    pr = torch.zeros(n, dtype=torch.int32, device="cuda")
    nc = U(0)
    m8 = (ctypes.c_float * 9)()
    assert lib.ref_build_bvh8(d.data_ptr(), pt, n, ps, b8.data_ptr(), pr.data_ptr(), ctypes.byref(nc), None, m8) == 0
    torch.cuda.synchronize()
    return dict(scene=np.array(scene[:], np.float32), keys=keys.cpu().numpy().view(kdt),
                sorted_keys=sk.cpu().numpy().view(kdt), perm=perm.cpu().numpy().view(np.uint32),
                bvh2=b2.cpu().numpy(), bvh8=b8.cpu().numpy()[: nc.value * 80], prim_idx=pr.cpu().numpy().view(np.uint32),
                bvh2_cost=np.float32(m8[6]), bvh8_cost=np.float32(m8[7]), bvh2_cost_b2=np.float32(m2[6]))


def main():
    import oracle
    manifest = {}
    for name, gen, kw, kb, r, kind in SMALL_CASES:
        prims = make_prims(gen, kw, kind)
        out = run_reference(prims, kb, r)
        np.savez_compressed(OUT / f"{name}.npz", prims=prims, key_bits=kb, radius=r, **out)
        manifest[name] = dict(generator=gen, args=kw, key_bits=kb, radius=r, kind=kind, n=int(prims.shape[0]))
        print(name, "ok", flush=True)
    for name, gen, kw, kb, r, kind in DIGEST_CASES:
        prims = make_prims(gen, kw, kind)
        n = prims.shape[0]
        out = run_reference(prims, kb, r)
        b2 = out["bvh2"].view(oracle.NODE2)
        b8 = out["bvh8"].view(oracle.NODE8)
        np.savez_compressed(OUT / f"{name}.npz", key_bits=kb, radius=r, scene=out["scene"], keys=out["keys"],
                            perm=out["perm"], sorted_keys=out["sorted_keys"],
                            bvh2_digest=np.uint64(oracle.digest_bvh2(b2, 2 * n - 2, n)),
                            bvh8_digest=np.uint64(oracle.digest_bvh8(b8, out["prim_idx"], n)),
                            bvh8_nodes=np.uint32(b8.shape[0]), bvh2_cost=out["bvh2_cost"], bvh8_cost=out["bvh8_cost"],
                            prims_sha256=np.frombuffer(hashlib.sha256(prims.tobytes()).digest(), np.uint8))
        manifest[name] = dict(generator=gen, args=kw, key_bits=kb, radius=r, kind=kind, n=int(n), digest_only=True)
        print(name, "ok", flush=True)
    (OUT / "manifest.json").write_text(json.dumps(manifest, indent=1) + "\n")


if __name__ == "__main__":
    main()
