"""The 64-bit sort on the reference's bit range [1,64) (Setup.cu:74-78:
cub::DeviceRadixSort::SortPairs with begin_bit 1), which this library runs
as four 9-bit passes over bits [28,64), an in-place sort of every bucket of
equal key >> 28 in shared memory, and a whole-array fallback for buckets too
large for shared memory.  Each case builds keys whose buckets sit where the
bucket kernel changes behaviour -- at its 2,048-position windows, at its
1,024-key bucket limit, at the end of the array -- and checks the keys and
the permutation bit for bit against numpy's stable argsort of key >> 1 (the
values are the input positions, so the permutation is the argsort itself).
"""
import numpy as np
import pytest

from tests import stages as S

pytestmark = pytest.mark.gpu

WINDOW = 2048  # bucket_sort_kernel's window
CAP = 1024     # its largest bucket


def keys_from_buckets(sizes, rng, low_bits=27, dup=0.3):
    """Keys whose value >> 28 changes exactly at the bucket edges given by
    `sizes`; the low bits [1,28) are random with a share `dup` of repeats
    (ties the sort must keep in input order), bit 0 random."""
    n = int(np.sum(sizes))
    tops = np.sort(rng.choice(np.uint64(1) << np.uint64(36), size=len(sizes), replace=False).astype(np.uint64))
    top = np.repeat(tops, sizes)
    low = rng.integers(0, 1 << low_bits, size=n, dtype=np.uint64)
    rep = rng.random(n) < dup
    idx = np.nonzero(rep)[0]
    low[idx[idx > 0]] = low[idx[idx > 0] - 1]
    bit0 = rng.integers(0, 2, size=n, dtype=np.uint64)
    keys = (top << np.uint64(28)) | (low << np.uint64(1)) | bit0
    # shuffle the input order: the sort must bring each bucket together
    return keys[rng.permutation(n)]


def check_sort(keys: np.ndarray):
    n = keys.shape[0]
    d_sk, d_perm = S.stage_sort(S.dev(keys.view(np.int64)), n, 63)
    sk = S.host(d_sk).view(np.uint64)
    perm = S.host(d_perm).view(np.uint32)
    want = np.argsort(keys >> np.uint64(1), kind="stable").astype(np.uint32)
    np.testing.assert_array_equal(perm, want)
    np.testing.assert_array_equal(sk, keys[want])


def test_small_buckets_across_windows():
    rng = np.random.default_rng(1)
    sizes = rng.integers(1, 40, size=6000)
    check_sort(keys_from_buckets(sizes, rng))


@pytest.mark.parametrize("big", [CAP - 1, CAP, CAP + 1, WINDOW, 3000])
def test_bucket_at_the_limit(big):
    """One bucket of `big` keys among small ones, starting at several
    offsets around a window edge (a bucket above the limit takes the
    fallback)."""
    rng = np.random.default_rng(big)
    for start in (0, WINDOW - 1, WINDOW - 37, 3 * WINDOW + 5):
        pre = []
        while sum(pre) < start:
            pre.append(int(min(start - sum(pre), rng.integers(1, 30))))
        post = list(rng.integers(1, 30, size=400))
        check_sort(keys_from_buckets(pre + [big] + post, rng))


def test_bucket_filling_window_and_halo():
    """Buckets that run from late in a window through all of its overflow
    slots (and one key past them)."""
    rng = np.random.default_rng(7)
    for tail in (CAP, CAP + 1):
        sizes = [WINDOW - 1, 1 + tail - 1, 5, 7]
        check_sort(keys_from_buckets(sizes, rng))


def test_all_keys_equal_and_full_width():
    rng = np.random.default_rng(3)
    check_sort(np.full(10_000, 0x7123456789ABCDEF, dtype=np.uint64))
    # random 64-bit keys, bit 63 included (the top digit is bits [55,64))
    check_sort(rng.integers(0, np.iinfo(np.uint64).max, size=200_000, dtype=np.uint64, endpoint=True))


@pytest.mark.parametrize("n", [1, 2, 33, 2047, 2048, 2049, 3072, 3073, 6145])
def test_sizes(n):
    rng = np.random.default_rng(n)
    check_sort(rng.integers(0, 1 << 40, size=n, dtype=np.uint64) << np.uint64(rng.integers(0, 24)))


def test_large_mixed():
    """3M keys: mostly small buckets, a few large ones (fallback), ties."""
    rng = np.random.default_rng(11)
    sizes = rng.integers(1, 8, size=900_000)
    sizes[::50_000] = 1500
    check_sort(keys_from_buckets(sizes, rng))
    sizes[::50_000] = 600
    check_sort(keys_from_buckets(sizes, rng))
