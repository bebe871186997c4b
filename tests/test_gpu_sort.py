"""ORDER BY on the device (sdb_sort_rows): the row order must equal a stable
lexicographic sort of the keys -- int32 keys signed, uint64 keys unsigned,
each ascending or descending -- on inputs with many ties."""
import ctypes

import numpy as np
import pytest

from sycldb_gb300 import capi
from tests.gpu_util import dev, host, stream, zeros

pytestmark = pytest.mark.gpu


def sortable(a, desc):
    """The key as an unsigned integer whose ascending order is the wanted order."""
    if a.dtype == np.int32:
        u = (a.view(np.uint32) ^ np.uint32(0x80000000)).astype(np.uint64)
        return (np.uint64(0xFFFFFFFF) - u) if desc else u
    u = a.astype(np.uint64)
    return (np.uint64(0xFFFFFFFFFFFFFFFF) - u) if desc else u


def gpu_sort(keys, desc):
    L = capi.lib()
    n = len(keys[0])
    ptrs = (ctypes.c_void_p * len(keys))(*[dev(k)[1] for k in keys])
    types = (ctypes.c_int * len(keys))(*[1 if k.dtype == np.uint64 else 0 for k in keys])
    dsc = (ctypes.c_int * len(keys))(*[1 if d else 0 for d in desc])
    pb, perm = zeros(max(n, 1), np.uint32)
    sb = L.sdb_sort_scratch_bytes(n)
    _, scratch = zeros(max(sb, 1), np.uint8)
    capi.check(L.sdb_sort_rows(ptrs, types, dsc, len(keys), n, perm, scratch, sb, stream()))
    return host(pb, perm, n, np.uint32)


@pytest.mark.parametrize("n", [1, 2, 255, 256, 257, 1000, 4095, 4096, 4097, 3 * 4096 + 1, 65_537, 1_000_003])
def test_sort_matches_a_stable_lexicographic_sort(n):
    rng = np.random.default_rng(n)
    k0 = rng.integers(-3, 4, n).astype(np.int32)                                  # few values: many ties
    k1 = rng.integers(0, 2**40, n).astype(np.uint64) * np.uint64(2**20)          # wide, high words matter
    k1[rng.random(n) < 0.3] = np.uint64(2**63 + 5)                                 # above 2^63: unsigned order
    k2 = rng.integers(-2**31, 2**31 - 1, n, dtype=np.int64).astype(np.int32)
    k2[::7] = np.int32(-2**31)
    for desc in ([False, False, False], [True, False, True], [False, True, False], [True, True, True]):
        got = gpu_sort([k0, k1, k2], desc)
        want = np.lexsort((sortable(k2, desc[2]), sortable(k1, desc[1]), sortable(k0, desc[0])))
        assert np.array_equal(got, want.astype(np.uint32)), desc
    # one key with all rows equal: the identity (stability)
    assert np.array_equal(gpu_sort([np.zeros(n, np.int32)], [True]), np.arange(n, dtype=np.uint32))


def test_sort_argument_checks():
    L = capi.lib()
    ptrs = (ctypes.c_void_p * 1)(0x1000)
    types = (ctypes.c_int * 1)(2)
    dsc = (ctypes.c_int * 1)(0)
    assert L.sdb_sort_rows(ptrs, types, dsc, 1, 10, 0x2000, 0x3000, 1 << 20, None) == capi.SDB_ERR_INVALID
    types[0] = 0
    assert L.sdb_sort_rows(ptrs, types, dsc, 1, 10, 0x2000, 0x3000, 16, None) == capi.SDB_ERR_INVALID  # scratch
    assert L.sdb_sort_rows(ptrs, types, dsc, 0, 10, 0x2000, 0x3000, 1 << 20, None) == capi.SDB_ERR_INVALID
    assert L.sdb_sort_rows(ptrs, types, dsc, 1, 0, 0x2000, 0x3000, 1 << 20, None) == capi.SDB_OK  # nothing to do
