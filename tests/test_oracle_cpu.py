"""CPU tests of the oracle itself: known answers derived from the
definitions, self-consistency, exhaustive validity, planted mistakes.

The reference ships no tests, golden vectors or CPU path; these checks
pin the restatement to the reference's definitions, and the committed
golden fixtures (tests/golden/) pin it to the reference's own CUDA build.
"""
import ctypes

import numpy as np
import pytest

from nexusbvh_gb300 import scenes


def leaves_of(boxes):
    import oracle
    n = len(boxes)
    lv = np.zeros(n, dtype=oracle.NODE2)
    for i, (mn, mx) in enumerate(boxes):
        lv[i]["bmin"], lv[i]["bmax"] = mn, mx
        lv[i]["left"], lv[i]["right"] = oracle.INVALID, i
    return lv


def test_morton_known_answers(orc):
    # scene [0,1]^3 fixed by the first two boxes; point boxes at the corners
    pts = [(0, 0, 0), (1, 1, 1), (1, 0, 0), (0, 1, 0), (0, 0, 1), (0.5, 0.5, 0.5)]
    lv = leaves_of([(p, p) for p in pts])
    scene = np.array([0, 0, 0, 1, 1, 1], np.float32)
    k30 = orc.morton(lv, scene, 30)
    k63 = orc.morton(lv, scene, 63)
    assert k30[0] == 0 and k30[1] == 0x3FFFFFFF
    assert k30[2] == 0x09249249 and k30[3] == 0x12492492 and k30[4] == 0x24924924
    assert k63[2] == 0x1249249249249249 and k63[3] == 0x1249249249249249 << 1
    assert k63[4] == 0x1249249249249249 << 2 and k63[1] == (1 << 63) - 1
    # 0.5 * 1023 = 511.5 truncates to 511 = 0b0111111111
    q, _ = orc.morton_quantised(lv, scene, 30)
    assert q[5].tolist() == [511, 511, 511]


def test_morton_zero_extent_axis_is_zero(orc):
    lv = leaves_of([((0, 0, 2), (0, 0, 2)), ((1, 1, 2), (1, 1, 2))])
    scene = np.array([0, 0, 2, 1, 1, 2], np.float32)
    q, _ = orc.morton_quantised(lv, scene, 63)
    assert q[:, 2].tolist() == [0, 0]  # 0/0 -> NaN -> 0


@pytest.mark.parametrize("key_bytes,begin,end", [(4, 2, 32), (8, 1, 64), (4, 0, 32), (8, 8, 40)])
def test_radix_sort_is_the_stable_sort(orc, key_bytes, begin, end):
    rng = np.random.default_rng(42)
    dt = np.uint32 if key_bytes == 4 else np.uint64
    keys = rng.integers(0, 1 << 20, size=200_003).astype(dt)
    keys <<= dt(begin)  # collisions in the sorted range, varied low bits
    keys |= rng.integers(0, 4, size=keys.shape[0]).astype(dt)
    k1, v1 = orc.radix_sort(keys, begin, end)
    k2, v2 = orc.stable_sort(keys, begin, end)
    np.testing.assert_array_equal(k1, k2)
    np.testing.assert_array_equal(v1, v2)


def nn_rule(num, boxes, radius, area):
    """The order the literal warp algorithm scans candidates in: i+1, i-1,
    i+2, i-2, ..., first strict minimum of the union area bit pattern."""
    out = []
    for i in range(32):
        best, bi = 0xFFFFFFFF, 0xFFFFFFFF
        if i < num:
            for r in range(1, radius + 1):
                for j in (i + r, i - r):
                    if 0 <= j < num:
                        u = np.concatenate([np.minimum(boxes[j, :3], boxes[i, :3]),
                                            np.maximum(boxes[j, 3:], boxes[i, 3:])]).astype(np.float32)
                        a = np.float32(area(u)).view(np.uint32)
                        if a < best:
                            best, bi = int(a), j
        out.append(bi)
    return out


@pytest.mark.parametrize("radius", [4, 8, 16])
def test_nearest_neighbour_rule_matches_warp_emulation(orc, radius):
    """The GPU kernel implements FindNearestNeighbor by the rule above; the
    oracle emulates the reference's shuffles lane by lane.  They agree."""
    lib = orc.load()
    lib.orc_find_nn.restype = None
    lib.orc_find_nn.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]
    rng = np.random.default_rng(radius)

    def area(u):
        return lib.orc_area(u.ctypes.data)

    for trial in range(300):
        num = int(rng.integers(2, 33))
        c = rng.random((32, 3)).astype(np.float32)
        h = (rng.random((32, 3)) * 0.1).astype(np.float32)
        if trial % 3 == 0:  # many exact ties
            c = np.round(c * 4) / 4
            h = np.full_like(h, 0.125)
        boxes = np.ascontiguousarray(np.concatenate([c - h, c + h], axis=1).astype(np.float32))
        nn = np.zeros(32, np.uint32)
        lib.orc_find_nn(num, boxes.ctypes.data, radius, nn.ctypes.data)
        expect = nn_rule(num, boxes, radius, area)
        assert nn[:num].tolist() == expect[:num]


@pytest.mark.parametrize("n", [1, 2, 3, 16, 17, 33, 64, 1000, 65536])
@pytest.mark.parametrize("key_bits", [30, 63])
def test_oracle_trees_are_valid(orc, n, key_bits):
    prims = scenes.uniform_soup(n, seed=n)
    r = orc.build(prims, key_bits)
    assert r["err"] == 0
    assert r["root"] == 2 * n - 2
    errs, rep = orc.validate_bvh2(r["bvh2"], n, r["root"])
    assert errs == 0, rep
    errs8, rep8 = orc.validate_bvh8(r["bvh8"], r["prim_idx"], n, r["bvh2"][:n])
    assert errs8 == 0, rep8
    assert rep8["leaves"] == n and rep8["visited"] == r["bvh8"].shape[0]
    assert r["bvh8_leaves"] == n


def test_degenerate_and_aabb_inputs(orc):
    same = np.tile(np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32), (500, 1))
    flat = scenes.uniform_soup(2000, seed=5)
    flat[:, 1::3] = 3.0
    boxes = scenes.to_boxes(scenes.clustered(20000, seed=3))
    for prims in (same, flat, boxes):
        for kb in (30, 63):
            n = prims.shape[0]
            r = orc.build(prims, kb)
            assert r["err"] == 0
            assert orc.validate_bvh2(r["bvh2"], n, r["root"])[0] == 0
            assert orc.validate_bvh8(r["bvh8"], r["prim_idx"], n, r["bvh2"][:n])[0] == 0


def test_build_is_deterministic_up_to_numbering(orc):
    prims = scenes.clustered(50000, seed=8)
    n = prims.shape[0]
    a = orc.build(prims, 63)
    orc.set_threads(1)
    try:
        b = orc.build(prims, 63)
    finally:
        orc.set_threads(0)
    assert orc.compare_bvh2(a["bvh2"], a["root"], b["bvh2"], b["root"], n) == 0
    assert orc.compare_bvh8(a["bvh8"], a["prim_idx"], b["bvh8"], b["prim_idx"], n) == 0


def test_validators_catch_planted_mistakes(orc):
    prims = scenes.uniform_soup(4096, seed=1)
    n = prims.shape[0]
    r = orc.build(prims, 30)
    b2 = r["bvh2"].copy()
    root = r["root"]
    # a child that escapes its parent
    inner = np.nonzero(b2["left"] != orc.INVALID)[0][5]
    b2[b2[inner]["left"]]["bmax"][0] += 1.0
    assert orc.validate_bvh2(b2, n, root)[0] > 0
    assert orc.compare_bvh2(b2, root, r["bvh2"], root, n) != 0
    # a duplicated primitive
    b2 = r["bvh2"].copy()
    leaf = np.nonzero(b2["left"] == orc.INVALID)[0]
    b2[leaf[0]]["right"] = b2[leaf[1]]["right"]
    errs, rep = orc.validate_bvh2(b2, n, root)
    assert rep["dup_prims"] == 1 and rep["missing_prims"] == 1
    # a cycle back to the root: every walk stops (validate, compare, digest)
    b2 = r["bvh2"].copy()
    b2[inner]["left"] = root
    errs, rep = orc.validate_bvh2(b2, n, root)
    assert errs > 0 and rep["visited"] == 2 * n
    assert orc.compare_bvh2(b2, root, b2, root, n) != 0
    assert orc.digest_bvh2(b2, root, n) == 0
    b8 = r["bvh8"].copy()
    k = int(np.nonzero(b8["imask"][1:])[0][0]) + 1
    b8[k]["child_base"] = 0
    assert orc.compare_bvh8(b8, r["prim_idx"], b8, r["prim_idx"], n) != 0
    assert orc.compare_bvh8_unordered(b8, r["prim_idx"], b8, r["prim_idx"], n)[0] != 0
    assert orc.digest_bvh8(b8, r["prim_idx"], n) == 0
    # a BVH8 child box shrunk below its exact box
    b8 = r["bvh8"].copy()
    b8[0]["qhi"][0][0] = 0
    b8[0]["qlo"][0][0] = 255
    _, rep8 = orc.validate_bvh8(b8, r["prim_idx"], n, r["bvh2"][:n])
    assert rep8["hi_not_conservative"] + rep8["lo_not_conservative"] >= 1
    assert orc.compare_bvh8(b8, r["prim_idx"], r["bvh8"], r["prim_idx"], n) != 0
    # a swapped BVH8 leaf primitive
    p = r["prim_idx"].copy()
    p[[0, 1]] = p[[1, 0]]
    assert orc.compare_bvh8(r["bvh8"], p, r["bvh8"], r["prim_idx"], n) != 0


def test_costs_follow_the_reference_weights(orc):
    # two unit boxes side by side: root area (half) of [0,2]x[0,1]x[0,1] = 2+1+2 = 5
    lv = leaves_of([((0, 0, 0), (1, 1, 1)), ((1, 0, 0), (2, 1, 1))])
    keys = np.array([0, 1], np.uint32)
    nodes, root, err = orc.hploc(keys, np.array([0, 1], np.uint32), lv)
    assert err == 0 and root == 2
    rb = np.array([0, 0, 0, 2, 1, 1], np.float32)
    # internal 3 * 5/5 + two leaves 2 * 3/5
    assert orc.bvh2_cost(nodes, rb) == pytest.approx(3.0 + 2 * 2 * 3 / 5)
    b8, prim, err8 = orc.bvh8(nodes, 2, root)
    assert err8 == 0 and b8.shape[0] == 1
    # BVH8 cost: children only, leaf weight 3
    assert orc.bvh8_cost(b8, rb) == pytest.approx(2 * 3 * 3 / 5, rel=1e-6)


def test_fast_math_helpers(orc):
    lib = orc.load()
    # subnormals are flushed like -ftz=true
    tiny = np.float32(1e-40)
    assert lib.orc_fmin(tiny, np.float32(1.0)) == 0.0
    assert lib.orc_f2u8(300.0) in (44, 255)
    assert lib.orc_f2u8(-3.0) == 0


def test_auction_oracle_keeps_the_tree(orc):
    """The auction assignment only permutes children inside BVH8 nodes: same
    node count, same cost, valid conservative quantisation."""
    from nexusbvh_gb300 import scenes
    p = scenes.clustered(8000, seed=31)
    o = orc.build(p, 63)
    g8, gp, ge = orc.bvh8(o["bvh2"], 8000, o["root"])
    a8, ap, ae = orc.bvh8(o["bvh2"], 8000, o["root"], auction=True)
    assert ge == 0 and ae == 0 and g8.shape == a8.shape
    rb = np.concatenate([o["bvh2"][o["root"]]["bmin"], o["bvh2"][o["root"]]["bmax"]]).astype(np.float32)
    assert abs(orc.bvh8_cost(a8, rb) - orc.bvh8_cost(g8, rb)) <= 1e-6 * orc.bvh8_cost(g8, rb)
    errs, rep = orc.validate_bvh8(a8, ap, 8000, o["bvh2"][:8000])
    assert errs == 0, rep
    assert orc.compare_bvh8(a8, ap, g8, gp, 8000) != 0
    res, reordered = orc.compare_bvh8_unordered(a8, ap, g8, gp, 8000)
    assert res == 0 and 0 < reordered <= a8.shape[0]
    bad = a8.copy()
    occupied = np.nonzero(bad[0]["meta"])[0][0]
    bad[0]["qhi"][1][occupied] ^= 1
    assert orc.compare_bvh8_unordered(bad, ap, g8, gp, 8000)[0] != 0


@pytest.mark.parametrize("n,key_bits,boxes,auction", [(2, 30, False, False), (3, 63, False, False),
                                                      (17, 30, True, False), (1000, 63, False, True),
                                                      (65536, 30, False, False), (65536, 63, True, False)])
def test_level_parallel_collapse_equals_the_work_slot_one(orc, n, key_bits, boxes, auction):
    """The collapse timed as the CPU baseline builds the same BVH8 as the
    parity oracle's (canonically: only node and primitive-slot numbering
    differ), with the same node count and a valid, equally costly tree."""
    prims = scenes.clustered(n, seed=n)
    if boxes:
        prims = scenes.to_boxes(prims)
    r = orc.build(prims, key_bits)
    a8, ap, ae = orc.bvh8(r["bvh2"], n, r["root"], auction=auction)
    b8, bp, be = orc.bvh8(r["bvh2"], n, r["root"], auction=auction, levels=True)
    assert ae == 0 and be == 0 and a8.shape == b8.shape
    assert orc.compare_bvh8(b8, bp, a8, ap, n) == 0
    assert orc.validate_bvh8(b8, bp, n, r["bvh2"][:n])[0] == 0
    rb = np.concatenate([r["bvh2"][r["root"]]["bmin"], r["bvh2"][r["root"]]["bmax"]]).astype(np.float32)
    assert abs(orc.bvh8_cost(b8, rb) - orc.bvh8_cost(a8, rb)) <= 1e-6 * orc.bvh8_cost(a8, rb)
    # and through build(), where the CPU baseline uses it
    orc.set_level_collapse(True)
    try:
        r2 = orc.build(prims, key_bits)
    finally:
        orc.set_level_collapse(False)
    assert r2["err"] == 0 and orc.compare_bvh8(r2["bvh8"], r2["prim_idx"], r["bvh8"], r["prim_idx"], n) == 0
