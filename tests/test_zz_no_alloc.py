"""The compaction entry point that allocates nothing (sdb_compact_row_ids_noalloc).

Callers that may not allocate device memory -- an executor that owns every
byte of its device memory in its own pool, or a serving loop that must not
call cudaMalloc/cudaFree because they can synchronise the device -- use this
entry instead of sdb_compact_row_ids: it keeps its scratch in a fixed array
inside the library.  This file checks, through the C ABI, that two calls in a
row give the same row ids and count as the entry that takes caller scratch,
and that sizes beyond the fixed scratch are refused.  It is named so that
pytest collects it last."""
import ctypes

import numpy as np
import pytest

from sycldb_gb300 import capi
from tests import kernel_cases as kc
from tests.gpu_util import dev, host, stream, zeros

pytestmark = pytest.mark.gpu


def compact_with_scratch(flags_ptr, n):
    """The existing entry: caller-provided scratch."""
    L = capi.lib()
    ib, ids = zeros(max(n, 1), np.int32)
    cb, cnt = zeros(1, np.uint32)
    sbytes = L.sdb_compact_scratch_bytes(n)
    _, scratch = zeros(max(sbytes, 1), np.uint8)
    capi.check(L.sdb_compact_row_ids(flags_ptr, n, ids, cnt, scratch, sbytes, stream()))
    c = int(host(cb, cnt, 1, np.uint32)[0])
    return c, host(ib, ids, c, np.int32)


def compact_no_alloc(flags_ptr, n):
    L = capi.lib()
    ib, ids = zeros(max(n, 1), np.int32)
    cb, cnt = zeros(1, np.uint32)
    capi.check(L.sdb_compact_row_ids_noalloc(flags_ptr, n, ids, cnt, stream()))
    c = int(host(cb, cnt, 1, np.uint32)[0])
    return c, host(ib, ids, c, np.int32)


def test_no_alloc_compaction_matches_the_scratch_entry_twice_in_a_row():
    n = 3_000_017
    for call, p in enumerate((0.3, 0.02)):  # the second call reuses the shared scratch
        rng = np.random.default_rng(77 + call)
        fl = kc.flags(rng, n, p, canonical=False)
        _, f = dev(fl)
        want_c, want_ids = compact_with_scratch(f, n)
        got_c, got_ids = compact_no_alloc(f, n)
        assert got_c == want_c
        assert np.array_equal(got_ids, want_ids)
        assert got_c == int(np.count_nonzero(fl))


def test_no_alloc_compaction_refuses_sizes_beyond_its_scratch():
    L = capi.lib()
    # refused on the host before any device work: the pointers are never used
    st = L.sdb_compact_row_ids_noalloc(0x1000, (1 << 28) + 1, 0x2000, 0x3000, None)
    assert st == capi.SDB_ERR_INVALID
    assert "exceed" in capi.last_error()
    cb, cnt = dev(np.array([123], np.uint32))
    capi.check(L.sdb_compact_row_ids_noalloc(None, 0, None, cnt, stream()))
    assert int(host(cb, cnt, 1, np.uint32)[0]) == 0
