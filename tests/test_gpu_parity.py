"""Parity of the CUDA pipeline with the CPU oracle, stage by stage, through
the C ABI.  Each stage is fed the GPU output of the previous stage, so every
comparison isolates one kernel:
  bounds/leaves   bit-exact
  Morton codes    bit-exact except where the fast-math divide and the
                  oracle's IEEE divide land on opposite sides of a
                  quantisation step (checked: +-1 in that axis only, at a
                  boundary)
  sort            keys and permutation bit-exact
  H-PLOC BVH2     canonical topology + every box bit-exact
  BVH8            canonical structure, every node byte (except base indices)
  costs           within 0.1%
"""
import numpy as np
import pytest

import nexusbvh_gb300 as nxb
from nexusbvh_gb300 import scenes
from tests import stages as S

pytestmark = pytest.mark.gpu


def deinterleave(keys: np.ndarray, key_bits: int) -> np.ndarray:
    per = 10 if key_bits == 30 else 21
    k = keys.astype(np.uint64)
    q = np.zeros((keys.shape[0], 3), dtype=np.uint64)
    for b in range(per):
        for a in range(3):
            q[:, a] |= ((k >> np.uint64(3 * b + a)) & np.uint64(1)) << np.uint64(b)
    return q.astype(np.int64)


def check_morton(keys_g, leaves, scene, key_bits, orc):
    keys_o = orc.morton(leaves, scene, key_bits)
    diff = np.nonzero(keys_g != keys_o)[0]
    if diff.size == 0:
        return 0
    qg = deinterleave(keys_g[diff], key_bits)
    q_o, prod = orc.morton_quantised(leaves[diff], scene, key_bits)
    q_o = q_o.astype(np.int64)
    d = qg - q_o
    assert np.abs(d).max() <= 1, "Morton quantisation differs by more than one step"
    # every differing axis must sit at a quantisation boundary
    p = prod.astype(np.float64)
    boundary = np.where(d > 0, q_o + 1, q_o).astype(np.float64)
    dist = np.abs(p - boundary)
    tol = np.maximum(np.abs(p), 1.0) * 2.0 ** -20
    bad = (d != 0) & (dist > tol)
    assert not bad.any(), f"{int(bad.sum())} Morton differences away from a quantisation boundary"
    return int(diff.size)


CASES = [
    ("soup65k-30", lambda: scenes.uniform_soup(65536, seed=0), 30),
    ("soup65k-63", lambda: scenes.uniform_soup(65536, seed=0), 63),
    ("sphere64k-30", lambda: scenes.displaced_sphere(256, 128, seed=1), 30),
    ("sphere64k-63", lambda: scenes.displaced_sphere(256, 128, seed=1), 63),
    ("clustered100k-63", lambda: scenes.clustered(100_000, seed=2), 63),
    ("aabb50k-63", lambda: scenes.to_boxes(scenes.clustered(50_000, seed=5)), 63),
    ("aabb50k-30", lambda: scenes.to_boxes(scenes.uniform_soup(50_000, seed=7)), 30),
]


def run_chain(prims, key_bits, orc, radius=8, whole=True):
    """The stage chain against the oracle fed each previous GPU stage; with
    `whole`, also the whole pipeline (nxb_build_async, whose collapse reads
    the child-pair records H-PLOC writes instead of the BVH2 nodes) against
    that chain."""
    n = prims.shape[0]
    d_nodes, d_scene = S.stage_bounds(prims)
    leaves_g = S.nodes2(d_nodes)[:n]
    scene_g = S.host(d_scene)
    leaves_o, scene_o = orc.scene_bounds(prims)
    assert leaves_g.tobytes() == leaves_o.tobytes(), "leaf boxes differ"
    np.testing.assert_array_equal(scene_g, scene_o)

    d_keys = S.stage_morton(d_nodes, d_scene, n, key_bits)
    keys_g = S.host(d_keys).view(np.uint32 if key_bits == 30 else np.uint64)
    morton_diffs = check_morton(keys_g, leaves_o, scene_o, key_bits, orc)

    begin, end = (2, 32) if key_bits == 30 else (1, 64)
    d_sk, d_perm = S.stage_sort(d_keys, n, key_bits)
    sk_g = S.host(d_sk).view(keys_g.dtype)
    perm_g = S.host(d_perm).view(np.uint32)
    sk_o, perm_o = orc.radix_sort(keys_g, begin, end)
    np.testing.assert_array_equal(sk_g, sk_o)
    np.testing.assert_array_equal(perm_g, perm_o)

    d_b2 = S.stage_hploc(d_sk, d_perm, d_nodes, n, key_bits, radius)
    b2_g = S.nodes2(d_b2)
    b2_o, root_o, err = orc.hploc(sk_g, perm_g, leaves_g, radius)
    assert err == 0
    assert root_o == 2 * n - 2
    assert orc.compare_bvh2(b2_g, 2 * n - 2, b2_o, root_o, n) == 0, "BVH2 differs from the oracle"
    errs, rep = orc.validate_bvh2(b2_g, n, 2 * n - 2)
    assert errs == 0, rep
    # the device validator reads the tree in place and reports the same fields
    g_errs, g_rep = nxb.validate_bvh2(d_b2, n)
    assert g_errs == 0 and g_rep["extra_parents"] == 0, g_rep
    assert list(g_rep.values())[:8] == list(rep.values()), (g_rep, rep)

    b8_g, prim_g, nc, lc = S.stage_bvh8(d_b2, n)
    b8_o, prim_o, err8 = orc.bvh8(b2_g, n, 2 * n - 2)
    assert err8 == 0
    assert nc == b8_o.shape[0] and lc == n
    assert orc.compare_bvh8(b8_g, prim_g, b8_o, prim_o, n) == 0, "BVH8 differs from the oracle"
    errs8, rep8 = orc.validate_bvh8(b8_g, prim_g, n, leaves_g)
    assert errs8 == 0, rep8
    g_errs8, g_rep8 = nxb.validate_bvh8(S.dev(b8_g.view(np.uint8)), nc, S.dev(prim_g.view(np.int32)),
                                        S.dev(prims.astype(np.float32)))
    assert g_errs8 == 0, g_rep8
    assert list(g_rep8.values())[:10] == list(rep8.values()), (g_rep8, rep8)

    rb = S.root_box(b2_g, 2 * n - 2)
    c2g, c2o = S.cost_bvh2(d_b2, 2 * n - 1, rb), orc.bvh2_cost(b2_g, rb)
    c8g, c8o = S.cost_bvh8(b8_g, rb), orc.bvh8_cost(b8_g, rb)
    assert abs(c2g - c2o) <= 1e-3 * abs(c2o)
    assert abs(c8g - c8o) <= 1e-3 * abs(c8o)
    if whole:
        out = S.build_async(prims, key_bits, radius=radius)
        w2 = S.nodes2(out.bvh2.nodes.view(-1))
        assert orc.compare_bvh2(w2, 2 * n - 2, b2_g, 2 * n - 2, n) == 0, "whole-pipeline BVH2 differs"
        w8 = S.host(out.nodes.reshape(-1)).view(nxb.BVH8_NODE_DTYPE)
        wp = S.host(out.prim_idx).view(np.uint32)
        assert out.node_count == nc
        assert orc.compare_bvh8(w8, wp, b8_g, prim_g, n) == 0, "whole-pipeline BVH8 differs"
    return dict(b2=b2_g, b8=b8_g, prim=prim_g, leaves=leaves_g, morton_diffs=morton_diffs, rep8=rep8,
                costs=(c2g, c8g))


@pytest.mark.parametrize("name,make,key_bits", CASES, ids=[c[0] for c in CASES])
def test_stage_chain_matches_oracle(gpu, orc, name, make, key_bits):
    run_chain(make(), key_bits, orc)


@pytest.mark.parametrize("radius", [4, 16])
def test_search_radius(gpu, orc, radius):
    run_chain(scenes.clustered(60_000, seed=11), 63, orc, radius=radius)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 16, 17, 31, 32, 33, 100, 257, 1000, 4097])
def test_small_sizes(gpu, orc, n):
    run_chain(scenes.uniform_soup(n, seed=n), 30, orc)
    run_chain(scenes.uniform_soup(n, seed=n + 1), 63, orc)


# Sizes on and around the tile edges of the tiled kernels: 256-primitive
# bounds/Morton tiles, 3,072-key (64-bit) and 4,096-key (32-bit) sort tiles,
# 256-leaf H-PLOC refill chunks.
TILE_EDGES = [255, 256, 257, 3071, 3072, 3073, 4095, 4096, 6145, 8191, 8192, 8193, 12289]


@pytest.mark.parametrize("n", TILE_EDGES)
def test_tile_edges_with_runs_of_equal_keys(gpu, orc, n):
    """Clustered data in which every third triangle repeats its predecessor,
    so runs of equal Morton keys cross tile edges: the sort must stay stable
    across tiles and H-PLOC must break the ties by position."""
    t = scenes.clustered(n, seed=n, components=4)
    t[2::3] = t[1::3][: t[2::3].shape[0]]
    run_chain(t, 30, orc)
    run_chain(t, 63, orc)


def test_degenerate_inputs(gpu, orc):
    # every triangle identical: all keys equal, ties broken by index
    t = np.tile(np.array([[0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9]], np.float32), (3000, 1))
    run_chain(t, 30, orc)
    run_chain(t, 63, orc)
    # zero extent on one axis (0/0 in the normalisation)
    f = scenes.uniform_soup(5000, seed=3)
    f[:, 2::3] = 0.25
    run_chain(f, 63, orc)
    # signed zeros and coordinates on the axes
    z = scenes.displaced_sphere(64, 32, seed=4)
    z[::7, 0] = -0.0
    z[::5, 3] = 0.0
    run_chain(z, 30, orc)


def test_pipeline_entry_points_agree(gpu, orc):
    """nxb_build_async, nxb_build_bvh8 / nxb_build_bvh2 and the stage chain
    produce the same trees; metrics are filled like the reference's."""
    prims = scenes.clustered(80_000, seed=9)
    n = prims.shape[0]
    chain = run_chain(prims, 63, orc)
    out = S.build_async(prims, 63)
    b2 = S.nodes2(out.bvh2.nodes.view(-1))
    assert orc.compare_bvh2(b2, 2 * n - 2, chain["b2"], 2 * n - 2, n) == 0
    b8 = S.host(out.nodes.reshape(-1)).view(nxb.BVH8_NODE_DTYPE)
    prim = S.host(out.prim_idx).view(np.uint32)
    assert orc.compare_bvh8(b8, prim, chain["b8"], chain["prim"], n) == 0

    m = nxb.BVHBuildMetrics()
    plain = nxb.build_bvh8(S.dev(prims), nxb.BuildConfig(), m)
    b8p = S.host(plain.nodes.reshape(-1)).view(nxb.BVH8_NODE_DTYPE)
    assert orc.compare_bvh8(b8p, S.host(plain.prim_idx).view(np.uint32), chain["b8"], chain["prim"], n) == 0
    assert m.total_time > 0 and m.bvh8_conversion_time > 0
    assert abs(m.bvh2_cost - chain["costs"][0]) <= 1e-3 * chain["costs"][0]
    assert abs(m.bvh8_cost - chain["costs"][1]) <= 1e-3 * chain["costs"][1]
    assert abs(m.average_child_per_node - (n + plain.node_count - 1) / plain.node_count) < 1e-5

    p2 = nxb.build_bvh2(S.dev(prims), nxb.BuildConfig())
    assert p2.node_count == 2 * n - 1
    assert orc.compare_bvh2(S.nodes2(p2.nodes.view(-1)), 2 * n - 2, chain["b2"], 2 * n - 2, n) == 0
    assert np.allclose(np.array(p2.bounds[0]), chain["b2"][2 * n - 2]["bmin"])

    # NXB_BUILD_VALIDATE: the same trees, checked on the device before the call returns
    m2 = nxb.BVHBuildMetrics()
    v8 = nxb.build_bvh8(S.dev(prims), nxb.BuildConfig(validate=True), m2)
    b8v = S.host(v8.nodes.reshape(-1)).view(nxb.BVH8_NODE_DTYPE)
    assert orc.compare_bvh8(b8v, S.host(v8.prim_idx).view(np.uint32), chain["b8"], chain["prim"], n) == 0
    assert abs(m2.bvh8_cost - chain["costs"][1]) <= 1e-3 * chain["costs"][1]
    v2 = nxb.build_bvh2(S.dev(scenes.to_boxes(prims)), nxb.BuildConfig(prioritize_speed=True, validate=True))
    assert v2.node_count == 2 * n - 1


def test_numerics_selftest(gpu, orc):
    rep = nxb.selftest_numerics()
    assert rep[0] > 0
    assert rep[3] == 0, "pinned area form differs from the plain expression under --use_fast_math"
    assert rep[27] == 0, "paired f32x2 area differs from the single-box area"
    values = [254.5, 255.0, 255.25, 256.0, 256.5, 300.0, 511.75, -1.5]
    import math
    for k, v in enumerate(values):
        assert rep[4 + k] == orc.load().orc_f2u8(math.floor(v)), f"floor cast of {v}"
        assert rep[12 + k] == orc.load().orc_f2u8(math.ceil(v)), f"ceil cast of {v}"
    f = np.array(rep[20:24], dtype=np.uint32).view(np.float32)
    lib = orc.load()
    assert np.float32(lib.orc_fmin(0.0, -0.0)).tobytes() == f[0].tobytes()
    assert np.float32(lib.orc_fmin(-0.0, 0.0)).tobytes() == f[1].tobytes()
    assert np.float32(lib.orc_fmax(0.0, -0.0)).tobytes() == f[2].tobytes()
    assert np.float32(lib.orc_fmax(-0.0, 0.0)).tobytes() == f[3].tobytes()


def test_bounded_waits_report_errors(gpu):
    import ctypes
    words = (ctypes.c_uint32 * 2)()
    lib = nxb.load()
    lib.nxb_selftest_bounded_waits.restype = ctypes.c_int
    lib.nxb_selftest_bounded_waits.argtypes = [ctypes.c_void_p]
    nxb.check(lib.nxb_selftest_bounded_waits(ctypes.cast(words, ctypes.c_void_p)), "nxb_selftest_bounded_waits")
    assert words[0] == 0x1 and words[1] == 0x2
    # the context is still usable
    run = S.build_async(scenes.uniform_soup(1000, seed=1), 30)
    assert run.node_count > 0


def test_errors_are_status_codes(gpu):
    import ctypes
    import torch
    lib = nxb.load()
    prims = S.dev(scenes.uniform_soup(1000))
    b = nxb.Builder()
    cfg = nxb.BuildConfig()
    s = b.sizes(1000, cfg)
    ws = torch.empty(s.workspace_bytes - 256, dtype=torch.uint8, device="cuda")
    nodes = torch.empty((s.bvh2_node_count, 32), dtype=torch.uint8, device="cuda")
    b8 = torch.empty((s.bvh8_node_capacity, 80), dtype=torch.uint8, device="cuda")
    prim_idx = torch.empty(1000, dtype=torch.int32, device="cuda")
    res = torch.zeros(64, dtype=torch.uint8, device="cuda")
    with pytest.raises(nxb.NxbError) as ei:
        b.enqueue(prims, 1000, cfg, ws, nodes, b8, prim_idx, res)
    assert ei.value.status == 5
    # a build that stops at the BVH2 needs no child-pair records (64 bytes per primitive)
    small = torch.empty(s.workspace_bytes - 64 * 1000, dtype=torch.uint8, device="cuda")
    b.enqueue(prims, 1000, cfg, small, nodes, None, None, res)
    torch.cuda.synchronize()
    with pytest.raises(nxb.NxbError) as ei:
        b.enqueue(prims, 1000, cfg, small[:-256], nodes, None, None, res)
    assert ei.value.status == 5
    bad = nxb.BuildConfig(search_radius=7)
    with pytest.raises(nxb.NxbError) as ei:
        nxb.build_bvh8(prims, bad)
    assert ei.value.status == 2
    out = nxb.CBVH8()
    c = cfg.to_c()
    assert lib.nxb_build_bvh8(None, 1, 10, ctypes.byref(c), None, ctypes.byref(out), None) == 1
    assert lib.nxb_build_bvh8(prims.data_ptr(), 1, 0, ctypes.byref(c), None, ctypes.byref(out), None) == 1
    assert lib.nxb_build_bvh8(prims.data_ptr(), 3, 10, ctypes.byref(c), None, ctypes.byref(out), None) == 1


@pytest.mark.parametrize("name,make,key_bits", [
    ("clustered60k-63", lambda: scenes.clustered(60_000, seed=21), 63),
    ("soup40k-30", lambda: scenes.uniform_soup(40_000, seed=22), 30),
    ("sphere32k-63", lambda: scenes.displaced_sphere(128, 128, seed=23), 63),
])
def test_auction_assignment(gpu, orc, name, make, key_bits):
    """NXB_BUILD_AUCTION (the reference's USE_AUCTION branch): the BVH8
    kernel's auction against the oracle's, over the same GPU BVH2.

    Tolerance: the auction scales its cost table by MAX_COST / maxDim and
    stops at epsilon < 1/n, two divisions that are the fast-math divide on
    the GPU (as in the reference) and IEEE in the oracle; the auction's bids
    end in near-ties, so a one-ulp difference can swap two children's slots.
    The trees must be identical up to slot order inside nodes (same nodes,
    boxes, quantisation, primitives), with at most 2 % of the nodes in
    another slot order."""
    prims = make()
    n = prims.shape[0]
    chain = run_chain(prims, key_bits, orc)
    d_b2 = S.dev(chain["b2"].view(np.uint8))
    b8_g, prim_g, nc, lc = S.stage_bvh8(d_b2, n, flags=nxb.NXB_BUILD_AUCTION)
    b8_o, prim_o, err = orc.bvh8(chain["b2"], n, 2 * n - 2, auction=True)
    assert err == 0 and lc == n and nc == b8_o.shape[0]
    res, reordered = orc.compare_bvh8_unordered(b8_g, prim_g, b8_o, prim_o, n)
    assert res == 0, "auction BVH8 differs from the oracle beyond slot order"
    assert reordered <= 0.02 * nc, f"{reordered} of {nc} nodes in another slot order than the oracle's"
    errs, rep = orc.validate_bvh8(b8_g, prim_g, n, chain["leaves"])
    assert errs == 0, rep
    # the same tree as the greedy build, children in another order
    assert orc.compare_bvh8(b8_g, prim_g, chain["b8"], chain["prim"], n) != 0
    rb = S.root_box(chain["b2"], 2 * n - 2)
    assert abs(orc.bvh8_cost(b8_g, rb) - chain["costs"][1]) <= 1e-3 * chain["costs"][1]
    # whole pipeline with the flag: the same as the stage call, slot for slot
    out = nxb.Builder().build(S.dev(prims), nxb.BuildConfig(prioritize_speed=key_bits == 30, auction=True))
    b8p = S.host(out.nodes.reshape(-1)).view(nxb.BVH8_NODE_DTYPE)
    assert orc.compare_bvh8(b8p, S.host(out.prim_idx).view(np.uint32), b8_g, prim_g, n) == 0


@pytest.mark.gpu
def test_bvh8_file_round_trip_of_a_gpu_build(gpu, orc, tmp_path):
    """A BVH8 built on the GPU, copied to the host through the C ABI
    (nxb_bvh8_to_host), written to a file and read back is byte-identical and
    still a valid tree over its primitives."""
    import ctypes
    import torch
    prims = scenes.uniform_soup(20000, seed=21)
    n = prims.shape[0]
    cfg = nxb.BuildConfig(prioritize_speed=True).to_c()
    d = torch.from_numpy(prims).cuda()
    dev, host = nxb.CBVH8(), nxb.CBVH8()
    nxb.check(gpu.nxb_build_bvh8(d.data_ptr(), nxb.NXB_PRIM_TRIANGLE, n, ctypes.byref(cfg), None, ctypes.byref(dev),
                                 None), "nxb_build_bvh8")
    try:
        nxb.check(gpu.nxb_bvh8_to_host(ctypes.byref(dev), ctypes.byref(host)), "nxb_bvh8_to_host")
        path = str(tmp_path / "gpu.nxb8").encode()
        nxb.check(gpu.nxb_write_bvh8(path, ctypes.byref(host)), "nxb_write_bvh8")
        back = nxb.CBVH8()
        nxb.check(gpu.nxb_read_bvh8(path, ctypes.byref(back)), "nxb_read_bvh8")
        try:
            assert back.node_count == host.node_count and back.prim_count == host.prim_count == n
            assert ctypes.string_at(back.nodes, 80 * back.node_count) == ctypes.string_at(host.nodes,
                                                                                         80 * host.node_count)
            assert ctypes.string_at(back.prim_idx, 4 * n) == ctypes.string_at(host.prim_idx, 4 * n)
            assert list(back.bounds.bmin) == list(host.bounds.bmin)
            nodes = np.frombuffer(ctypes.string_at(back.nodes, 80 * back.node_count), dtype=orc.NODE8).copy()
            prim = np.frombuffer(ctypes.string_at(back.prim_idx, 4 * n), dtype=np.uint32).copy()
            leaves, _ = orc.scene_bounds(prims)
            errs, rep = orc.validate_bvh8(nodes, prim, n, leaves)
            assert errs == 0, rep
        finally:
            gpu.nxb_free_host_bvh8(ctypes.byref(back))
    finally:
        gpu.nxb_free_host_bvh8(ctypes.byref(host))
        gpu.nxb_free_device_bvh8(ctypes.byref(dev))


def test_device_validators_flag_planted_mistakes(gpu, orc):
    """Each mistake is planted in a host copy of a correct oracle tree; the
    device validators read the uploaded copy (every index they follow is
    range-checked first) and flag what the oracle's validators flag."""
    prims = scenes.uniform_soup(4096, seed=1)
    n = prims.shape[0]
    r = orc.build(prims, 30)
    root = r["root"]
    d_prims = S.dev(prims.astype(np.float32))

    def both2(b2):
        g = nxb.validate_bvh2(S.dev(b2.view(np.uint8)), n, root)
        return g, orc.validate_bvh2(b2, n, root)

    def both8(b8, prim):
        g = nxb.validate_bvh8(S.dev(b8.view(np.uint8)), b8.shape[0], S.dev(prim.view(np.int32)), d_prims)
        return g, orc.validate_bvh8(b8, prim, n, r["bvh2"][:n])

    (ge, g), (oe, o) = both2(r["bvh2"])
    assert ge == 0 and oe == 0 and list(g.values())[:8] == list(o.values())
    (ge, g), (oe, o) = both8(r["bvh8"], r["prim_idx"])
    assert ge == 0 and oe == 0 and list(g.values())[:10] == list(o.values())

    inner = np.nonzero(r["bvh2"]["left"] != orc.INVALID)[0]
    # a child that escapes its parent
    b2 = r["bvh2"].copy()
    b2[b2[inner[5]]["left"]]["bmax"][0] += 1.0
    (ge, g), (oe, o) = both2(b2)
    assert ge > 0 and g["not_contained"] >= 1 and list(g.values())[:8] == list(o.values())
    # a duplicated primitive
    b2 = r["bvh2"].copy()
    leaf = np.nonzero(b2["left"] == orc.INVALID)[0]
    b2[leaf[0]]["right"] = b2[leaf[1]]["right"]
    (ge, g), (oe, o) = both2(b2)
    assert g["dup_prims"] == 1 and g["missing_prims"] == 1 and list(g.values())[:8] == list(o.values())
    # a child index past the last node: its subtrees are no longer reached
    b2 = r["bvh2"].copy()
    b2[inner[7]]["right"] = 2 * n + 5
    (ge, g), (oe, o) = both2(b2)
    assert ge > 0 and oe > 0 and g["bad_index"] == o["bad_index"] == 1 and g["reached"] == o["visited"]
    # a reference back to the root (a cycle; only the device validator, which
    # does not walk, is run on it)
    b2 = r["bvh2"].copy()
    b2[inner[9]]["left"] = root
    ge, g = nxb.validate_bvh2(S.dev(b2.view(np.uint8)), n, root)
    assert ge > 0 and g["extra_parents"] >= 1 and g["reached"] < 2 * n - 1

    # a BVH8 child box shrunk below its exact box
    b8 = r["bvh8"].copy()
    b8[0]["qhi"][0][0] = 0
    b8[0]["qlo"][0][0] = 255
    (ge, g), (oe, o) = both8(b8, r["prim_idx"])
    assert g["hi_not_conservative"] + g["lo_not_conservative"] >= 1
    assert list(g.values())[:10] == list(o.values())
    # two swapped leaf primitives
    p = r["prim_idx"].copy()
    p[[0, 1]] = p[[1, 0]]
    (ge, g), (oe, o) = both8(r["bvh8"], p)
    assert list(g.values())[:10] == list(o.values())
    # a wrong meta byte
    b8 = r["bvh8"].copy()
    occupied = np.nonzero(b8[0]["meta"])[0][0]
    b8[0]["meta"][occupied] ^= 0x40
    (ge, g), (oe, o) = both8(b8, r["prim_idx"])
    assert ge > 0 and g["meta_errors"] >= 1 and oe > 0
    # children renumbered onto the root: extra references and lost subtrees
    b8 = r["bvh8"].copy()
    k = int(np.nonzero(b8["imask"][1:])[0][0]) + 1
    b8[k]["child_base"] = 0
    (ge, g), (oe, o) = both8(b8, r["prim_idx"])
    assert ge > 0 and oe > 0 and g["bad_index"] >= 1
