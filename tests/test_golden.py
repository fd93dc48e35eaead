"""Golden fixtures produced by the reference's own CUDA build
(tests/golden/make_golden.py).  The CPU tests pin the oracle to them; the
GPU tests pin the CUDA kernels to them bit for bit."""
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
MANIFEST = GOLDEN / "manifest.json"
CASES = json.loads(MANIFEST.read_text()) if MANIFEST.exists() else {}
SMALL = sorted(k for k, v in CASES.items() if not v.get("digest_only"))
DIGEST = sorted(k for k, v in CASES.items() if v.get("digest_only"))

if not CASES:
    pytest.skip("golden fixtures not generated yet", allow_module_level=True)


def load(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def regenerate(name):
    from nexusbvh_gb300 import scenes
    c = CASES[name]
    p = getattr(scenes, c["generator"])(**c["args"])
    return scenes.to_boxes(p) if c["kind"] == "aabb" else p


def morton_within_boundary(keys_o, keys_ref, leaves, scene, key_bits, orc):
    """Oracle (IEEE divide) vs reference (fast-math divide): equal, or +-1 in
    one quantisation step exactly at a boundary."""
    from tests.test_gpu_parity import deinterleave
    diff = np.nonzero(keys_o != keys_ref)[0]
    if diff.size == 0:
        return 0
    qr = deinterleave(keys_ref[diff], key_bits)
    q_o, prod = orc.morton_quantised(leaves[diff], scene, key_bits)
    d = qr - q_o.astype(np.int64)
    assert np.abs(d).max() <= 1
    p = prod.astype(np.float64)
    boundary = np.where(d > 0, q_o.astype(np.int64) + 1, q_o.astype(np.int64)).astype(np.float64)
    assert not ((d != 0) & (np.abs(p - boundary) > np.maximum(np.abs(p), 1.0) * 2.0 ** -20)).any()
    return int(diff.size)


@pytest.mark.parametrize("name", SMALL)
def test_oracle_matches_reference_fixture(orc, name):
    g = load(name)
    prims = g["prims"]
    n = prims.shape[0]
    kb = int(g["key_bits"])
    r = int(g["radius"])
    b2_ref = g["bvh2"].view(orc.NODE2)
    leaves, scene = orc.scene_bounds(prims)
    assert leaves.tobytes() == b2_ref[:n].tobytes(), "leaf boxes"
    np.testing.assert_array_equal(scene, g["scene"])
    keys_o = orc.morton(leaves, scene, kb)
    morton_within_boundary(keys_o, g["keys"], leaves, scene, kb, orc)
    begin, end = (2, 32) if kb == 30 else (1, 64)
    sk, perm = orc.radix_sort(g["keys"], begin, end)
    np.testing.assert_array_equal(sk, g["sorted_keys"])
    np.testing.assert_array_equal(perm, g["perm"])
    b2, root, err = orc.hploc(g["sorted_keys"], g["perm"], leaves, r)
    assert err == 0 and root == 2 * n - 2
    assert orc.compare_bvh2(b2, root, b2_ref, 2 * n - 2, n) == 0, "BVH2 vs reference"
    b8_ref = g["bvh8"].view(orc.NODE8)
    b8, prim, err8 = orc.bvh8(b2_ref, n, 2 * n - 2)
    assert err8 == 0
    assert b8.shape[0] == b8_ref.shape[0]
    assert orc.compare_bvh8(b8, prim, b8_ref, g["prim_idx"], n) == 0, "BVH8 vs reference"
    rb = np.concatenate([b2_ref[2 * n - 2]["bmin"], b2_ref[2 * n - 2]["bmax"]]).astype(np.float32)
    assert orc.bvh2_cost(b2_ref, rb) == pytest.approx(float(g["bvh2_cost"]), rel=1e-3)
    assert orc.bvh8_cost(b8_ref, rb) == pytest.approx(float(g["bvh8_cost"]), rel=1e-3)
    # the reference's trees are valid (conservativeness is reported, not assumed)
    assert orc.validate_bvh2(b2_ref, n, 2 * n - 2)[0] == 0
    assert orc.validate_bvh8(b8_ref, g["prim_idx"], n, b2_ref[:n])[0] == 0


@pytest.mark.parametrize("name", DIGEST)
def test_oracle_matches_reference_digests(orc, name):
    import hashlib
    g = load(name)
    prims = regenerate(name)
    assert hashlib.sha256(prims.tobytes()).digest() == g["prims_sha256"].tobytes()
    n = prims.shape[0]
    kb = int(g["key_bits"])
    leaves, scene = orc.scene_bounds(prims)
    np.testing.assert_array_equal(scene, g["scene"])
    morton_within_boundary(orc.morton(leaves, scene, kb), g["keys"], leaves, scene, kb, orc)
    begin, end = (2, 32) if kb == 30 else (1, 64)
    sk, perm = orc.radix_sort(g["keys"], begin, end)
    np.testing.assert_array_equal(perm, g["perm"])
    b2, root, err = orc.hploc(g["sorted_keys"], g["perm"], leaves, int(g["radius"]))
    assert err == 0
    assert orc.digest_bvh2(b2, root, n) == int(g["bvh2_digest"])
    b8, prim, err8 = orc.bvh8(b2, n, root)
    assert err8 == 0 and b8.shape[0] == int(g["bvh8_nodes"])
    assert orc.digest_bvh8(b8, prim, n) == int(g["bvh8_digest"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", SMALL + DIGEST)
def test_cuda_matches_reference_fixture(gpu, orc, name):
    """Morton codes and the sorted permutation bit-exact, BVH2 and BVH8
    canonically identical to the reference's own build."""
    from tests import stages as S
    import nexusbvh_gb300 as nxb
    g = load(name)
    prims = g["prims"] if "prims" in g else regenerate(name)
    n = prims.shape[0]
    kb = int(g["key_bits"])
    r = int(g["radius"])
    d_nodes, d_scene = S.stage_bounds(prims)
    np.testing.assert_array_equal(S.host(d_scene), g["scene"])
    d_keys = S.stage_morton(d_nodes, d_scene, n, kb)
    keys = S.host(d_keys).view(np.uint32 if kb == 30 else np.uint64)
    np.testing.assert_array_equal(keys, g["keys"])
    d_sk, d_perm = S.stage_sort(d_keys, n, kb)
    np.testing.assert_array_equal(S.host(d_perm).view(np.uint32), g["perm"])
    out = S.build_async(prims, kb, r)
    b2 = S.nodes2(out.bvh2.nodes.view(-1))
    b8 = S.host(out.nodes.reshape(-1)).view(nxb.BVH8_NODE_DTYPE)
    prim = S.host(out.prim_idx).view(np.uint32)
    if "bvh2" in g:
        b2_ref = g["bvh2"].view(orc.NODE2)
        assert orc.compare_bvh2(b2, 2 * n - 2, b2_ref, 2 * n - 2, n) == 0
        assert b2[:n].tobytes() == b2_ref[:n].tobytes()
        assert orc.compare_bvh8(b8, prim, g["bvh8"].view(orc.NODE8), g["prim_idx"], n) == 0
    else:
        assert orc.digest_bvh2(b2, 2 * n - 2, n) == int(g["bvh2_digest"])
        assert b8.shape[0] == int(g["bvh8_nodes"])
        assert orc.digest_bvh8(b8, prim, n) == int(g["bvh8_digest"])
