"""Seeded star-schema datasets shared by the tests."""
import functools

import numpy as np

from sycldb_gb300 import ssb

ALL_FACT = tuple(range(17))


@functools.lru_cache(maxsize=8)
def dataset(sf: float, seed: int = ssb.SEED, fact_cols=ALL_FACT):
    n = ssb.fact_rows(sf)
    ds = {"lineorder": ssb.gen_lineorder_host(n, fact_cols, sf, seed)}
    ds.update(ssb.gen_dims(sf, seed))
    return ds


def oracle_tables(ds, seg=None):
    from oracle import oracle as O

    seg = seg or O.SEGMENT_SIZE
    return {name: O.make_table(name.split("@")[0] if "@" not in name else name, cols, seg)
            for name, cols in ds.items()}


def oracle_run(ds, plan, seg=None):
    from oracle import oracle as O

    ex = O.OracleExecutor(oracle_tables(ds, seg), segment_size=seg or O.SEGMENT_SIZE)
    return O.canonical_rows(ex.execute(plan))


def checksum(a: np.ndarray) -> int:
    """Order-sensitive 64-bit checksum of an int32 column."""
    x = a.astype(np.uint64)
    w = (np.arange(a.size, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)) | np.uint64(1)
    return int(np.bitwise_xor.reduce(x * w) if a.size else 0) ^ int(a.size)
