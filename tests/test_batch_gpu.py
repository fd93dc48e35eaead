"""Batched builds (nxb_batch_*) against plain builds of each mesh alone and
against the oracle.  The batch must reproduce every mesh's plain build:
BVH2 arrays byte for byte (the node numbering is deterministic), BVH8
canonically (BVH8 node numbering comes from atomics in both), scene boxes
and counts exactly."""
import ctypes

import numpy as np
import pytest

import nexusbvh_gb300 as nxb
from nexusbvh_gb300 import scenes
from tests import stages as S

pytestmark = pytest.mark.gpu

# ragged sizes: empty meshes, single primitives, warp and merge-window edges
COUNTS = [1, 2, 3, 0, 16, 17, 31, 32, 33, 0, 100, 257, 1000, 4097, 5, 20000, 0, 65536, 7]


def make_batch(counts, seed=5, boxes=False):
    prims = scenes.batch_meshes(counts, seed=seed)
    if boxes:
        prims = scenes.to_boxes(prims)
    return prims


def plain(prims_m, radius=8):
    """Plain 30-bit build of one mesh through nxb_build_async."""
    out = S.build_async(prims_m, 30, radius=radius)
    n = prims_m.shape[0]
    b2 = S.nodes2(out.bvh2.nodes.view(-1))[: 2 * n - 1]
    b8 = S.host(out.nodes.reshape(-1)).view(nxb.BVH8_NODE_DTYPE)
    prim = S.host(out.prim_idx).view(np.uint32)
    return b2, b8, prim, out.bounds


def check_against_plain(batch, meshes, prims, counts, orc, radius=8, only=None):
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    for m, n in enumerate(counts):
        if only is not None and m not in only:
            continue
        info = meshes[m]
        assert info.prim_offset == off[m] and info.prim_count == n
        if n == 0:
            assert info.bvh2_node_count == 0 and info.bvh8_node_count == 0 and info.bvh8_leaf_count == 0
            continue
        pm = prims[off[m]:off[m + 1]]
        b2p, b8p, primp, bounds = plain(pm, radius)
        b2b = batch.mesh_bvh2_host(m, meshes)
        assert b2b.tobytes() == b2p.tobytes(), f"mesh {m} (n={n}): BVH2 differs from the plain build"
        assert tuple(info.scene_bounds.bmin) == bounds[0] and tuple(info.scene_bounds.bmax) == bounds[1]
        b8b, primb = batch.mesh_bvh8_host(m)
        assert info.bvh8_node_count == b8p.shape[0] and info.bvh8_leaf_count == n
        assert orc.compare_bvh8(b8b, primb, b8p, primp, n) == 0, f"mesh {m} (n={n}): BVH8 differs"


def test_batch_matches_plain_builds(gpu, orc):
    prims = make_batch(COUNTS)
    batch = nxb.Batch(COUNTS)
    meshes = batch.build(S.dev(prims))
    check_against_plain(batch, meshes, prims, COUNTS, orc)


def test_batch_matches_oracle(gpu, orc):
    """Each mesh's BVH2 against the oracle's H-PLOC over that mesh's GPU
    Morton order (the oracle's own IEEE divide can move a code by one step
    at a quantisation boundary), and its BVH8 against the oracle's collapse."""
    counts = [3000, 1, 0, 5000, 257]
    prims = make_batch(counts, seed=8)
    batch = nxb.Batch(counts)
    d_prims = S.dev(prims)
    meshes = batch.build(d_prims)
    off = np.concatenate([[0], np.cumsum(counts)])
    for m, n in enumerate(counts):
        if n >= 1:  # every tree checked on the device in place, with the oracle's report
            (e2, g2), (e8, g8) = batch.validate_mesh(m, d_prims, meshes)
            assert e2 == 0 and e8 == 0 and g2["leaves"] == n and g8["leaves"] == n, (g2, g8)
        if n < 2:
            continue
        pm = prims[off[m]:off[m + 1]]
        d_nodes, d_scene = S.stage_bounds(pm)
        leaves = S.nodes2(d_nodes)[:n]
        d_keys = S.stage_morton(d_nodes, d_scene, n, 30)
        d_sk, d_perm = S.stage_sort(d_keys, n, 30)
        sk = S.host(d_sk).view(np.uint32)
        perm = S.host(d_perm).view(np.uint32)
        b2_o, root_o, err = orc.hploc(sk, perm, leaves, 8)
        assert err == 0
        b2 = batch.mesh_bvh2_host(m, meshes)
        assert orc.compare_bvh2(b2, 2 * n - 2, b2_o, root_o, n) == 0
        errs, rep = orc.validate_bvh2(b2, n, 2 * n - 2)
        assert errs == 0, rep
        b8, prim = batch.mesh_bvh8_host(m)
        b8_o, prim_o, err8 = orc.bvh8(b2, n, 2 * n - 2)
        assert err8 == 0
        assert orc.compare_bvh8(b8, prim, b8_o, prim_o, n) == 0
        errs8, rep8 = orc.validate_bvh8(b8, prim, n, leaves)
        assert errs8 == 0, rep8
        assert list(g2.values())[:8] == list(rep.values()) and list(g8.values())[:10] == list(rep8.values())


@pytest.mark.parametrize("groups", [2, 4, 8])
def test_batch_grouped_collapse_matches_plain_builds(gpu, orc, groups):
    """BVH2/BVH8 fusion point: meshes cut into groups, the collapse of each
    group overlapping H-PLOC of the next; results equal the plain builds."""
    prims = make_batch(COUNTS, seed=12)
    batch = nxb.Batch(COUNTS)
    t = batch.tuning()
    t.fusion_groups = groups
    batch.set_tuning(t)
    d = S.dev(prims)
    for _ in range(3):  # capture, then replays
        meshes = batch.build(d)
    check_against_plain(batch, meshes, prims, COUNTS, orc)


def test_batch_groups_with_empty_tail(gpu, orc):
    """A cut that leaves a group of empty meshes only (all triangles in the
    first mesh) still builds every mesh."""
    counts = [3000, 0, 0, 1, 0]
    prims = make_batch(counts, seed=13)
    batch = nxb.Batch(counts)
    t = batch.tuning()
    t.fusion_groups = 4
    batch.set_tuning(t)
    meshes = batch.build(S.dev(prims))
    check_against_plain(batch, meshes, prims, counts, orc)


def test_batch_aabb_input(gpu, orc):
    counts = [500, 0, 1, 2000]
    prims = make_batch(counts, seed=9, boxes=True)
    batch = nxb.Batch(counts, prim_type=nxb.NXB_PRIM_AABB)
    meshes = batch.build(S.dev(prims))
    check_against_plain(batch, meshes, prims, counts, orc)


def test_batch_replay_and_tuning_keep_results(gpu, orc):
    counts = [1000, 33, 7000, 0, 1, 300]
    prims = make_batch(counts, seed=4)
    d = S.dev(prims)
    batch = nxb.Batch(counts)
    first = batch.build(d)
    ref = [(batch.mesh_bvh2_host(m, first).tobytes(), batch.mesh_bvh8_host(m)) for m in range(len(counts))
           if counts[m]]
    for digits, ctas, groups, block in ((4, 0, 2, 128), (5, 0, 1, 128), (6, 4, 2, 512), (7, 0, 4, 256),
                                        (8, 4, 1, 512)):
        t = batch.tuning()
        t.sort_digit_bits, t.hploc_ctas_per_sm, t.fusion_groups, t.block_size = digits, ctas, groups, block
        batch.set_tuning(t)
        for _ in range(2):  # capture, then replay
            again = batch.build(d)
            got = [(batch.mesh_bvh2_host(m, again).tobytes(), batch.mesh_bvh8_host(m)) for m in range(len(counts))
                   if counts[m]]
            for (a2, (a8, ap)), (b2, (b8, bp)), n in zip(ref, got, [c for c in counts if c]):
                assert a2 == b2
                assert orc.compare_bvh8(a8, ap, b8, bp, n) == 0
    # a new input buffer triggers a new capture
    d2 = S.dev(prims.copy())
    third = batch.build(d2)
    assert batch.mesh_bvh2_host(0, third).tobytes() == ref[0][0]
    chosen = batch.autotune(d, repeats=2)
    assert chosen.candidates_tried >= 4 and chosen.search_radius == 8 and chosen.build_ms > 0
    after = batch.build(d)
    assert batch.mesh_bvh2_host(2, after).tobytes() == ref[2][0]


def test_batch_radius_tuning(gpu, orc):
    counts = [4000, 3000]
    prims = make_batch(counts, seed=6)
    d = S.dev(prims)
    batch = nxb.Batch(counts)
    chosen = batch.autotune(d, flags=nxb.NXB_TUNE_RADIUS, repeats=1)
    assert chosen.search_radius in (4, 8, 16)
    meshes = batch.build(d)
    check_against_plain(batch, meshes, prims, counts, orc, radius=chosen.search_radius)


def test_batch_arguments(gpu):
    lib = nxb.load()
    h = ctypes.c_void_p()
    off = np.array([0, 10, 5], dtype=np.uint32)  # decreasing
    c = nxb.BuildConfig(prioritize_speed=True).to_c()
    assert lib.nxb_batch_create(1, off.ctypes.data, 2, ctypes.byref(c), ctypes.byref(h)) == 1
    ok = np.array([0, 10, 20], dtype=np.uint32)
    c63 = nxb.BuildConfig(prioritize_speed=False).to_c()
    assert lib.nxb_batch_create(1, ok.ctypes.data, 2, ctypes.byref(c63), ctypes.byref(h)) == 2
    assert lib.nxb_batch_create(1, ok.ctypes.data, 0, ctypes.byref(c), ctypes.byref(h)) == 1
    b = nxb.Batch([10, 10])
    t = b.tuning()
    t.sort_digit_bits = 3
    with pytest.raises(nxb.NxbError):
        b.set_tuning(t)


def test_batch_ten_pass_plan(gpu, orc):
    """1,024 meshes make 40-bit batch keys (30-bit codes, 10-bit mesh
    index): 4-bit digits sort them in 10 passes, 8-bit digits in 5; every
    mesh's trees are the same either way."""
    rng = np.random.default_rng(17)
    counts = [int(x) for x in rng.integers(0, 300, size=1024)]
    prims = make_batch(counts, seed=17)
    d = S.dev(prims)
    batch = nxb.Batch(counts)
    eight = batch.build(d)
    ref = [batch.mesh_bvh2_host(m, eight).tobytes() for m in range(len(counts)) if counts[m]]
    t = batch.tuning()
    t.sort_digit_bits = 4
    batch.set_tuning(t)
    four = batch.build(d)
    got = [batch.mesh_bvh2_host(m, four).tobytes() for m in range(len(counts)) if counts[m]]
    assert got == ref
    k = next(m for m in range(len(counts)) if counts[m] > 100)
    check_against_plain(batch, four, prims, counts, orc, only=[k])
