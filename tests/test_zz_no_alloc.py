"""The allocation-free radix sort (nxb_stage_radix_sort_noalloc).

Callers that cannot allocate device memory (a renderer's frame loop, where
cudaMalloc/cudaFree would synchronise the device, or an engine whose memory
belongs to its own sub-allocator) sort through an entry point whose scratch
is a fixed array inside the library.  This test calls it through the C ABI
twice in a row and checks each result against the regular entry point,
nxb_stage_radix_sort, which takes caller scratch.  The sort is integer work,
so the comparison is exact.  The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NOALLOC_MAX = 262144  # NXB_NOALLOC_SORT_MAX_COUNT


def noalloc(lib):
    fn = lib.nxb_stage_radix_sort_noalloc
    P, U = ctypes.c_void_p, ctypes.c_uint32
    fn.restype = ctypes.c_int
    fn.argtypes = [U, P, P, P, P, U, U, U, P, P]
    return fn


def sort_both(lib, keys_np, begin, end, vals_np=None):
    import torch

    from tests import stages as S
    n = keys_np.shape[0]
    kb = keys_np.itemsize
    d_keys = S.dev(keys_np.view(np.int32 if kb == 4 else np.int64))
    d_vals = None if vals_np is None else S.dev(vals_np.view(np.int32))
    # regular entry point (caller scratch)
    ref_k, ref_v = S.stage_sort(d_keys, n, 30 if kb == 4 else 63, begin, end, d_vals)
    # allocation-free entry point
    out_k = torch.empty_like(d_keys)
    out_v = torch.empty(n, dtype=torch.int32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    status = noalloc(lib)(kb, d_keys.data_ptr(), out_k.data_ptr(), None if d_vals is None else d_vals.data_ptr(),
                          out_v.data_ptr(), n, begin, end, err.data_ptr(), S.stream())
    torch.cuda.synchronize()
    assert status == 0, status
    assert int(err.item()) == 0
    return S.host(ref_k), S.host(ref_v), S.host(out_k), S.host(out_v)


@pytest.mark.parametrize("key_bytes,begin,end", [(4, 2, 32), (8, 1, 64)])
def test_noalloc_sort_matches_regular_sort_twice(gpu, key_bytes, begin, end):
    rng = np.random.default_rng(key_bytes)
    dt = np.uint32 if key_bytes == 4 else np.uint64
    for call, n in enumerate((NOALLOC_MAX, 100_003)):  # two calls in a row, the second smaller
        keys = rng.integers(0, np.iinfo(dt).max, size=n, dtype=dt)
        keys[::7] = keys[0]  # ties: the sort must stay stable
        vals = rng.integers(0, 1 << 31, size=n, dtype=np.uint32) if call else None
        rk, rv, ok, ov = sort_both(gpu, keys, begin, end, vals)
        np.testing.assert_array_equal(ok, rk)
        np.testing.assert_array_equal(ov, rv)


def test_noalloc_sort_rejects_oversize(gpu):
    import torch
    n = NOALLOC_MAX + 1
    d = torch.zeros(n, dtype=torch.int32, device="cuda")
    o = torch.zeros(n, dtype=torch.int32, device="cuda")
    assert noalloc(gpu)(4, d.data_ptr(), o.data_ptr(), None, o.data_ptr(), n, 0, 32, None, None) == 2


def test_noalloc_sort_allocates_nothing_once_warm(gpu):
    """After a first (warm-up) call on the device, a call leaves the
    device's free memory exactly as it was: no allocation happens."""
    import torch

    from tests import stages as S
    n = 50_000
    keys = np.random.default_rng(5).integers(0, 1 << 62, size=n, dtype=np.uint64)
    d_keys = S.dev(keys.view(np.int64))
    out_k = torch.empty_like(d_keys)
    out_v = torch.empty(n, dtype=torch.int32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    fn = noalloc(gpu)

    def call():
        status = fn(8, d_keys.data_ptr(), out_k.data_ptr(), None, out_v.data_ptr(), n, 1, 64, err.data_ptr(),
                    S.stream())
        torch.cuda.synchronize()
        assert status == 0 and int(err.item()) == 0

    call()  # warm-up: loads the kernels on this device, looks up the array
    free_before = torch.cuda.mem_get_info()[0]
    call()
    call()
    assert torch.cuda.mem_get_info()[0] == free_before
    want = np.argsort(keys >> np.uint64(1), kind="stable").astype(np.uint32)
    np.testing.assert_array_equal(S.host(out_v).view(np.uint32), want)

