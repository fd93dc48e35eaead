"""Parity at every full size the benchmark configurations name, stage by
stage against the oracle fed each previous GPU stage (bit-exact leaves,
Morton codes up to the fast-math boundary rule, sort, BVH2 and BVH8
canonically identical, exhaustive validity, costs within 0.1%), and the
whole pipeline against that chain:
  * the 4,194,304-triangle displaced sphere with 30-bit and 63-bit codes;
  * the 12,582,912-triangle clustered mesh, 63-bit, search radius 8 and 16
    (BinaryBuilder.cu:9 fixes 8; 16 is the configuration's second radius);
  * the 28,311,552-triangle clustered build injected into the served stream
    (63-bit, radius 8)."""
import numpy as np
import pytest

import nexusbvh_gb300 as nxb
from nexusbvh_gb300 import scenes
from tests import stages as S
from tests.test_gpu_parity import run_chain

pytestmark = pytest.mark.gpu


FULL = [("clustered12m", 63, 8), ("clustered12m", 63, 16), ("sphere4m", 30, 8), ("sphere4m", 63, 8),
        ("clustered28m", 63, 8)]


@pytest.mark.parametrize("name,key_bits,radius", FULL, ids=[f"{a}-{b}-r{c}" for a, b, c in FULL])
def test_full_size_chain(gpu, orc, name, key_bits, radius):
    prims = scenes.by_name(name)
    n = prims.shape[0]
    chain = run_chain(prims, key_bits, orc, radius=radius, whole=False)
    out = S.build_async(prims, key_bits, radius=radius)
    b8 = S.host(out.nodes.reshape(-1)).view(nxb.BVH8_NODE_DTYPE)
    prim = S.host(out.prim_idx).view(np.uint32)
    assert orc.compare_bvh8(b8, prim, chain["b8"], chain["prim"], n) == 0
    b2 = S.nodes2(out.bvh2.nodes.view(-1))
    assert orc.compare_bvh2(b2, 2 * n - 2, chain["b2"], 2 * n - 2, n) == 0
