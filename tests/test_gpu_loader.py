"""Tables from the reference's columnar files (one raw int32 file per
column, <NAME><i>): loaded in the foreground or in the background, plans give
the rows they give on tables registered from memory; missing or short files
leave their column unloaded, as the reference's loader does."""
import os

import numpy as np
import pytest

from sycldb_gb300 import capi, plans, ssb
from sycldb_gb300.engine import Engine
from tests import datasets

pytestmark = pytest.mark.gpu

SF = 0.05
PLANS = [plans.plan_filter_sum(1994), plans.plan_date_join(1995), plans.plan_star(2, 11),
         plans.plan_star(1, 3, 1993, 1996, 12)]


@pytest.fixture(scope="module")
def ds():
    return datasets.dataset(SF)


@pytest.fixture(scope="module")
def want(ds):
    with Engine(arena_bytes=1 << 30) as eng:
        for name, cols in ds.items():
            eng.load_table(name, cols)
        return [eng.execute(p).canonical() for p in PLANS]


@pytest.fixture()
def coldir(ds, tmp_path):
    ssb.write_columnar(str(tmp_path), ds)
    return str(tmp_path)


@pytest.mark.parametrize("background", [False, True])
def test_loaded_from_files_gives_the_same_rows(coldir, want, background):
    with Engine(arena_bytes=1 << 30, segment_rows=1 << 16) as eng:
        for name in ("lineorder", "supplier", "part", "ddate"):
            eng.load_dir(coldir, name, background=background)
        for p, w in zip(PLANS, want):
            assert eng.execute(p).canonical() == w
        eng.sync_tables()  # nothing left to wait for
    with Engine(arena_bytes=1 << 30) as eng:  # background loads left unread are finished by destroy
        eng.load_dir(coldir, "lineorder", background=True)


def test_missing_and_short_files_leave_columns_unloaded(coldir, want, ds):
    os.remove(os.path.join(coldir, "LINEORDER12"))                      # revenue: star joins need it
    np.asarray(ds["lineorder"][9][:-1], np.int32).tofile(os.path.join(coldir, "LINEORDER9"))  # one row short
    with Engine(arena_bytes=1 << 30) as eng:
        for name in ("lineorder", "supplier", "part", "ddate"):
            eng.load_dir(coldir, name)
        for p in PLANS:  # every plan reads revenue or extendedprice
            with pytest.raises(capi.SdbError) as e:
                eng.execute(p)
            assert "not loaded" in str(e.value)
        # a plan on the columns that loaded still runs
        b = plans.PlanBuilder()
        b.scan("lineorder")
        b.filter(plans.search(11, 1, 3))
        b.project([plans.col(8)])
        b.aggregate([], 0)
        assert eng.execute(b.plan()).canonical() == datasets.oracle_run(ds, b.plan())


def test_column_mask_and_errors(coldir, ds, tmp_path):
    with Engine(arena_bytes=1 << 30) as eng:
        eng.load_dir(coldir, "lineorder", columns=[7, 8])  # 7 is outside the reference loader's set
        b = plans.PlanBuilder()
        b.scan("lineorder")
        b.filter(plans.expr("<", plans.col(8), plans.lit(10)))
        b.project([plans.col(7)])
        b.aggregate([], 0)
        assert eng.execute(b.plan()).canonical() == datasets.oracle_run(ds, b.plan())
        with pytest.raises(capi.SdbError) as e:
            eng.load_dir(str(tmp_path / "nothing"), "lineorder")
        assert "no column file" in str(e.value)
        eng.load_dir(str(tmp_path / "nothing"), "supplier", background=True)
        with pytest.raises(capi.SdbError) as e:  # a failed background load reports at first use
            eng.execute(plans.plan_star(2, 11))
        assert "no column file" in str(e.value)
        with pytest.raises(capi.SdbError):
            eng.load_dir(coldir, "nosuchtable")
