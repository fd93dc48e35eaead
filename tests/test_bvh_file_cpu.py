"""BVH files (nxb_write_bvh2/8, nxb_read_bvh2/8): round trips of host trees
and the checks a reader makes on a file.  Host code only: no GPU needed."""
import numpy as np
import pytest

import nexusbvh_gb300 as nxb
from nexusbvh_gb300 import scenes


@pytest.fixture(scope="module")
def tree(orc):
    from nexusbvh_gb300 import _build
    _build.build_cuda()
    prims = scenes.uniform_soup(3000, seed=3)
    r = orc.build(prims, 30, 8)
    assert r["err"] == 0
    n = prims.shape[0]
    b2 = r["bvh2"].view(nxb.BVH2_NODE_DTYPE)
    root = b2[2 * n - 2]
    bounds = np.stack([root["bmin"], root["bmax"]])
    return b2, r["bvh8"].view(nxb.BVH8_NODE_DTYPE), r["prim_idx"], bounds


def test_bvh2_round_trip(tree, tmp_path):
    b2, _, _, bounds = tree
    path = tmp_path / "mesh.nxb2"
    nxb.save_bvh2(path, b2, bounds)
    assert path.stat().st_size == 64 + 32 * len(b2)
    nodes, got_bounds = nxb.load_bvh2(path)
    assert nodes.tobytes() == b2.tobytes()
    assert np.array_equal(got_bounds, bounds)


def test_bvh8_round_trip(tree, tmp_path):
    _, b8, prim, bounds = tree
    path = tmp_path / "mesh.nxb8"
    nxb.save_bvh8(path, b8, prim, bounds)
    assert path.stat().st_size == 64 + 80 * len(b8) + 4 * len(prim)
    nodes, got_prim, got_bounds = nxb.load_bvh8(path)
    assert nodes.tobytes() == b8.tobytes()
    assert np.array_equal(got_prim, prim)
    assert np.array_equal(got_bounds, bounds)


def test_reader_rejects_wrong_kind_truncation_and_bad_header(tree, tmp_path):
    b2, b8, prim, bounds = tree
    p2, p8 = tmp_path / "a.nxb2", tmp_path / "a.nxb8"
    nxb.save_bvh2(p2, b2, bounds)
    nxb.save_bvh8(p8, b8, prim, bounds)
    # a BVH2 file is not a BVH8 file and the other way round
    with pytest.raises(nxb.NxbError, match="NXB_ERR_IO"):
        nxb.load_bvh8(p2)
    with pytest.raises(nxb.NxbError, match="NXB_ERR_IO"):
        nxb.load_bvh2(p8)
    data = p8.read_bytes()
    cases = {
        "short": data[:-1],          # one byte missing
        "long": data + b"\0",        # one byte too many
    }
    bad = bytearray(data)
    bad[8] = 2                       # another format version
    cases["version"] = bytes(bad)
    bad = bytearray(data)
    bad[12:16] = (0xFFFFFFF).to_bytes(4, "little")  # more nodes than the primitives allow
    cases["count"] = bytes(bad)
    for name, blob in cases.items():
        (tmp_path / f"{name}.nxb8").write_bytes(blob)
        with pytest.raises(nxb.NxbError, match="NXB_ERR_IO"):
            nxb.load_bvh8(tmp_path / f"{name}.nxb8")
    with pytest.raises(nxb.NxbError, match="NXB_ERR_IO"):
        nxb.load_bvh2(tmp_path / "missing.nxb2")


def test_writer_checks_its_arguments(tree, tmp_path):
    b2, b8, prim, bounds = tree
    # a BVH8 with more nodes than its primitives allow
    with pytest.raises(nxb.NxbError, match="NXB_ERR_INVALID_ARGUMENT"):
        nxb.save_bvh8(tmp_path / "x.nxb8", np.concatenate([b8] * 4), prim[:10], bounds)
    with pytest.raises(nxb.NxbError, match="NXB_ERR_IO"):
        nxb.save_bvh2(tmp_path / "no_such_dir" / "x.nxb2", b2, bounds)
