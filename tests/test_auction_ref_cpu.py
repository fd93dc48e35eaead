"""The oracle's auction slot assignment against the reference's own code.

The reference's BVH8 kernel built with USE_AUCTION assigns child slots with
AuctionAssignment over a cost table (NexusBVH/src/Cuda/WideConverter.cu:
50-102, 337-361).  oracle/build_ref.py compiles exactly those lines, copied
from the reference's source, as host code (oracle/_ref/libref_auction.so);
this test feeds both that code and the oracle's restatement (orc_auction)
the same parent and child boxes and requires the same assignment, bit for
bit.  Both divide in IEEE arithmetic here.  Cases where the oracle stops
bidding and falls back to the greedy assignment (its bid limit, a deviation
from the reference's unbounded loop) are excluded, and counted.
"""
import ctypes

import numpy as np
import pytest

import oracle
from oracle import build_ref


@pytest.fixture(scope="module")
def ref():
    try:
        path = build_ref.build_auction()
    except RuntimeError as exc:  # no compiler
        pytest.skip(f"reference auction harness not built: {exc}")
    if path is None:
        pytest.skip("the reference's sources are not available")
    lib = ctypes.CDLL(str(path))
    lib.ref_auction.restype = ctypes.c_uint32
    lib.ref_auction.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32]
    return lib


def child_sets(rng, count):
    """Parent boxes and 2..8 children inside them, as a BVH8 node sees them:
    random boxes, children with equal centroids (ties), flat axes, and
    children spanning the whole parent."""
    for k in range(count):
        n = int(rng.integers(2, 9))
        lo = rng.uniform(-100, 100, size=3).astype(np.float32)
        ext = np.exp(rng.uniform(np.log(1e-3), np.log(50), size=3)).astype(np.float32)
        mode = k % 5
        a = rng.random((n, 3)).astype(np.float32)
        b = rng.random((n, 3)).astype(np.float32)
        if mode == 1:  # equal centroids for half the children
            a[: n // 2] = a[0]
            b[: n // 2] = b[0]
        if mode == 2:  # one flat axis
            a[:, 1] = b[:, 1] = 0.5
        cmin = lo + np.minimum(a, b) * ext
        cmax = lo + np.maximum(a, b) * ext
        if mode == 3:  # a child that fills the parent
            cmin[0], cmax[0] = lo, lo + ext
        if mode == 4:  # tiny children
            cmax = cmin + (cmax - cmin) * np.float32(1e-4)
        pmin, pmax = cmin.min(axis=0), cmax.max(axis=0)
        yield (np.concatenate([pmin, pmax]).astype(np.float32),
               np.concatenate([cmin, cmax], axis=1).astype(np.float32).copy(), n)


def test_oracle_auction_matches_reference_code(ref):
    lib = oracle.load()
    rng = np.random.default_rng(2024)
    compared = fallback = 0
    out = np.zeros(1, dtype=np.uint32)
    for parent, children, n in child_sets(rng, 20_000):
        ok = lib.orc_auction(parent.ctypes.data, children.ctypes.data, n, out.ctypes.data)
        if not ok:
            fallback += 1
            continue
        want = ref.ref_auction(parent.ctypes.data, children.ctypes.data, n)
        assert int(out[0]) == want, (parent, children, hex(int(out[0])), hex(want))
        compared += 1
    assert compared >= 19_000, (compared, fallback)
