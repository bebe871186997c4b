"""CPU-only checks of the benchmark's CPU leg and of the test evaluators:

* the oracle's seeded generator gives, bit for bit, the columns of the
  native library's generator (so the CPU leg runs on the GPU arm's inputs
  without loading the library);
* the CPU leg (``bench.py --impl reference``) loads no product library and
  reports the oracle's results;
* the vectorised naive evaluators (used at full size on the GPU) give the
  loop evaluators' rows."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import oracle as O
from sycldb_gb300 import ssb
from tests import datasets, naive

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("sf,salt,row0", [(0.01, 0, 0), (0.5, 7, 0), (0.05, 3, 123_457)])
def test_oracle_generator_is_the_library_generator(sf, salt, row0):
    n = ssb.fact_rows(sf)
    gen = O.OracleGen()
    a = ssb.gen_lineorder_host(n, range(17), sf, row0=row0, salt=salt)
    b = ssb.gen_lineorder_host(n, range(17), sf, row0=row0, salt=salt, gen=gen)
    for c in a:
        assert np.array_equal(a[c], b[c]), c
    da, db = ssb.gen_dims(sf), ssb.gen_dims(sf, gen=gen)
    for t in da:
        for c in da[t]:
            assert np.array_equal(da[t][c], db[t][c]), (t, c)


def test_cpu_leg_loads_no_product_library():
    code = (
        "import runpy, sys\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '1', '--sf', '0.05']\n"
        "try:\n"
        "    runpy.run_path('bench.py', run_name='__main__')\n"
        "except SystemExit:\n"
        "    pass\n"
        "print('MAPS', sorted({l.split()[-1] for l in open('/proc/self/maps') if '.so' in l}))\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(next(l for l in r.stdout.splitlines() if l.startswith("{")))
    maps = next(l for l in r.stdout.splitlines() if l.startswith("MAPS"))
    assert "libsycldb_gb300" not in maps
    assert "libsdb_oracle" in maps
    assert line["impl"] == "reference" and line["value"] > 0
    assert set(line["configs"]) == {"filter_project_sum_sf1", "date_join_groupby_sf1"}
    # the digests are those of the oracle's own results on the library's inputs
    from importlib import util

    spec = util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    ds = datasets.dataset(0.05)
    star = datasets.oracle_run(ds, bench._plan_star())
    assert line["result_digests"]["star"] == bench.rows_digest(star)
    assert line["config"]["groups"] == len(star)


@pytest.mark.parametrize("sf", [0.05, 0.2])
def test_vectorised_naive_equals_loops(sf):
    ds = datasets.dataset(sf)
    f = ds["lineorder"]
    for y in (1992, 1995, 1998):
        assert naive.filter_sum_vec(f, y) == naive.filter_sum(f, y)
        assert naive.filter_sum_vec(f, y, 0, 10, 51) == naive.filter_sum(f, y, 0, 10, 51)
        assert naive.date_join_vec(f, ds["ddate"], y) == naive.date_join(f, ds["ddate"], y)
    for args in [(2, 11), (1, 3, 1993, 1996, 12), (0, 0, 1992, 1992, 1), (4, 24, 1992, 1998, 40)]:
        want = naive.star(f, ds["supplier"], ds["part"], ds["ddate"], *args)
        assert naive.star_vec(f, ds["supplier"], ds["part"], ds["ddate"], *args) == want
