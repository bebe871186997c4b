"""The autotuner's table format and its loading into the library (no GPU)."""
import ctypes
import json

from sycldb_gb300 import autotune, capi


def test_rows_bucket_matches_the_library():
    for n in (1, 2, 3, 1023, 1024, 1 << 20, 120_000_000, 300_000_000):
        assert 2 ** autotune.rows_bucket(n) <= n < 2 ** (autotune.rows_bucket(n) + 1)


def test_load_sets_the_tuning_table(tmp_path):
    L = capi.lib()
    table = {"entries": [{"terminal": "groupby", "nregs": 2, "rows_bucket": 26, "variant": 4},
                         {"terminal": "sum", "nregs": 1, "rows_bucket": 20, "variant": 3}]}
    p = tmp_path / "t.json"
    p.write_text(json.dumps(table))
    try:
        assert autotune.load_default(str(p)) == table
        assert L.sdb_chain_tune_get(2, 2, 1 << 26) == 4
        assert L.sdb_chain_tune_get(2, 2, (1 << 27) - 1) == 4
        assert L.sdb_chain_tune_get(1, 1, 1 << 20) == 3
        assert L.sdb_chain_tune_get(1, 1, 1 << 21) in range(6)
    finally:
        capi.force_chain_variant(-1)
        autotune.load_default()


def test_missing_table_is_not_an_error(tmp_path):
    assert autotune.load_default(str(tmp_path / "absent.json")) is None


def test_first_op_keys_are_separate():
    L = capi.lib()
    table = {"entries": [{"terminal": "groupby", "nregs": 2, "first_op": 3, "rows_bucket": 26, "variant": 5},
                         {"terminal": "groupby", "nregs": 2, "first_op": 1, "rows_bucket": 26, "variant": 6}]}
    try:
        capi.force_chain_variant(-1)
        autotune.load(table)
        assert L.sdb_chain_tune_get_op(2, 2, 3, 1 << 26) == 5
        assert L.sdb_chain_tune_get_op(2, 2, 1, 1 << 26) == 6
        assert L.sdb_chain_tune_get_op(2, 2, 0, 1 << 26) == 5  # unset entries use the default
        assert L.sdb_chain_tune_set_op(2, 2, 9, 1, 5) == capi.SDB_ERR_INVALID
        assert L.sdb_chain_tune_set_op(2, 2, 1, 1, 9) == capi.SDB_ERR_INVALID
    finally:
        capi.force_chain_variant(-1)
        autotune.load_default()


def test_measured_buckets_cover_the_sizes_above_them(tmp_path):
    """A measured bucket's variant holds up to the next measured bucket of
    the same key, and the largest one's for every size above it."""
    L = capi.lib()
    table = {"entries": [{"terminal": "groupby", "nregs": 2, "first_op": 3, "rows_bucket": 22, "variant": 5},
                         {"terminal": "groupby", "nregs": 2, "first_op": 3, "rows_bucket": 24, "variant": 7},
                         {"terminal": "groupby", "nregs": 2, "first_op": 1, "rows_bucket": 26, "variant": 6}]}
    p = tmp_path / "t.json"
    p.write_text(json.dumps(table))
    try:
        capi.force_chain_variant(-1)
        autotune.load_default(str(p))
        assert L.sdb_chain_tune_get_op(2, 2, 3, 1 << 22) == 5
        assert L.sdb_chain_tune_get_op(2, 2, 3, 1 << 23) == 5   # between 22 and 24
        assert L.sdb_chain_tune_get_op(2, 2, 3, 1 << 24) == 7
        assert L.sdb_chain_tune_get_op(2, 2, 3, 1 << 28) == 7   # beyond the largest measured size
        assert L.sdb_chain_tune_get_op(2, 2, 1, 1 << 30) == 6   # another first op keeps its own
    finally:
        capi.force_chain_variant(-1)
        autotune.load_default()


def _clear_op_shapes():
    for kk in range(len(capi.OP_KERNELS)):
        for bk in range(40):
            capi.check(capi.lib().sdb_op_tune_set(kk, 1 << bk, 0, 0))


def test_operator_launch_shapes_set_get_and_load():
    L = capi.lib()
    b, p = ctypes.c_int(), ctypes.c_int()
    k = capi.OP_KERNELS.index("probe_full")
    _clear_op_shapes()  # the defaults (an engine may have loaded the committed table)
    capi.check(L.sdb_op_tune_get(k, 1 << 24, ctypes.byref(b), ctypes.byref(p)))
    assert (b.value, p.value) == (256, 8)
    assert L.sdb_op_tune_set(k, 1 << 24, 384, 2) == capi.SDB_ERR_INVALID
    assert L.sdb_op_tune_set(k, 1 << 24, 512, 8) == capi.SDB_ERR_INVALID  # over 2048 threads per SM
    assert L.sdb_op_tune_set(len(capi.OP_KERNELS), 1, 256, 4) == capi.SDB_ERR_INVALID
    try:
        table = {"entries": [], "op_entries": [
            {"kernel": "probe_full", "rows_bucket": 20, "block": 512, "blocks_per_sm": 2},
            {"kernel": "probe_full", "rows_bucket": 24, "block": 128, "blocks_per_sm": 16}]}
        assert autotune.load_ops(table) == 2
        for rows, want in ((1 << 19, (256, 8)), (1 << 21, (512, 2)), (1 << 24, (128, 16)), (1 << 30, (128, 16))):
            capi.check(L.sdb_op_tune_get(k, rows, ctypes.byref(b), ctypes.byref(p)))
            assert (b.value, p.value) == want, rows
        s = capi.OP_KERNELS.index("sum")
        capi.check(L.sdb_op_tune_get(s, 1 << 24, ctypes.byref(b), ctypes.byref(p)))
        assert (b.value, p.value) == (256, 4)
    finally:
        _clear_op_shapes()
        autotune.load_default()
