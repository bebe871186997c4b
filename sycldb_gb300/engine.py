"""Python front end of the host executor (``sdb_engine_*`` in the C ABI).

``Engine`` owns one native engine: base tables are registered with
``load_table`` (numpy arrays = host memory, copied to the device; torch CUDA
tensors = device memory, used in place) and plans in the Thrift PlanResult
JSON shape run with ``execute``, which returns the result rows as numpy
columns (int32 keys, uint64 sums), in row order.
"""
from __future__ import annotations

import ctypes
import json
from typing import Dict, List, Mapping, Optional

import numpy as np

from . import capi

TABLE_COLUMN_NUMBERS = {"lineorder": 17, "part": 9, "supplier": 7, "customer": 8, "ddate": 17}


def _ptr_and_loc(a):
    """(pointer, on_device, nrows) of a numpy array or torch tensor."""
    if isinstance(a, np.ndarray):
        if a.dtype != np.int32 or not a.flags["C_CONTIGUOUS"]:
            raise TypeError("host columns must be contiguous int32 numpy arrays")
        return a.ctypes.data, 0, a.size
    try:
        import torch
    except ImportError:  # pragma: no cover
        torch = None
    if torch is not None and isinstance(a, torch.Tensor):
        if a.dtype != torch.int32 or not a.is_contiguous():
            raise TypeError("columns must be contiguous int32 tensors")
        return a.data_ptr(), 1 if a.is_cuda else 0, a.numel()
    raise TypeError("unsupported column type %r" % type(a))


class Result:
    """Result rows: ``columns`` is a list of numpy arrays (int32 or uint64)."""

    def __init__(self, columns: List[np.ndarray]):
        self.columns = columns

    @property
    def nrows(self) -> int:
        return int(self.columns[0].size) if self.columns else 0

    def rows(self):
        return list(zip(*[c.tolist() for c in self.columns])) if self.columns else []

    def canonical(self):
        r = self.rows()
        r.sort()
        return r


_TUNING_LOADED = False


def _load_tuning_once():
    """The first engine of a process loads the committed autotuner table
    (``SYCLDB_TUNING`` names another file; an empty value skips it)."""
    global _TUNING_LOADED
    if not _TUNING_LOADED:
        _TUNING_LOADED = True
        from . import autotune

        autotune.load_default()


def _take_result(r) -> Result:
    """Copies a native sdb_result into numpy columns and frees it."""
    L = capi.lib()
    try:
        ncols, nrows = ctypes.c_int(), ctypes.c_uint64()
        L.sdb_result_shape(r, ctypes.byref(ncols), ctypes.byref(nrows))
        cols = []
        for c in range(ncols.value):
            t, d = ctypes.c_int(), ctypes.c_void_p()
            capi.check(L.sdb_result_column(r, c, ctypes.byref(t), ctypes.byref(d)))
            dt = np.uint64 if t.value == 1 else np.int32
            n = nrows.value
            if n == 0:
                cols.append(np.empty(0, dtype=dt))
            else:
                buf = (ctypes.c_char * (n * np.dtype(dt).itemsize)).from_address(d.value)
                cols.append(np.frombuffer(buf, dtype=dt).copy())
        return Result(cols)
    finally:
        L.sdb_result_free(r)


class Engine:
    def __init__(self, arena_bytes: int = 0, segment_rows: int = 0, fuse: bool = True, profile: bool = False,
                 stream: Optional[int] = None, plan_cache: int = 0, order_by: bool = False, join_tables: int = 0,
                 shared_scans: bool = True):
        L = capi.lib()
        _load_tuning_once()
        cfg = capi.EngineConfig(arena_bytes, segment_rows, 1 if fuse else 0, 1 if profile else 0, stream or None,
                                plan_cache, 1 if order_by else 0, join_tables, 0 if shared_scans else 1)
        h = ctypes.c_void_p()
        capi.check(L.sdb_engine_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._keep: Dict[str, list] = {}

    def close(self):
        if getattr(self, "_h", None):
            capi.lib().sdb_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def load_table(self, name: str, columns: Mapping[int, object]):
        """Registers base table ``name``; ``columns`` maps column index to an
        int32 array (all host or all device)."""
        ncols = TABLE_COLUMN_NUMBERS[name.split("@", 1)[0]]
        ptrs = (ctypes.c_void_p * ncols)()
        loc = None
        nrows = None
        keep = []
        for c, a in columns.items():
            if not 0 <= c < ncols:
                raise ValueError("column %d out of range for %s" % (c, name))
            p, on_dev, n = _ptr_and_loc(a)
            if loc is None:
                loc, nrows = on_dev, n
            if on_dev != loc:
                raise ValueError("all columns of a table must be on the same side (host or device)")
            if n != nrows:
                raise ValueError("column length mismatch in %s%d" % (name, c))
            ptrs[c] = p
            keep.append(a)
        capi.check(capi.lib().sdb_engine_load_table(self._h, name.encode(), ncols, ptrs, nrows or 0, loc or 0))
        if loc:
            self._keep[name] = keep  # device columns are used in place
        else:
            self._keep.pop(name, None)

    def load_dir(self, directory: str, name: str, columns=None, background: bool = False):
        """Registers table ``name`` from the reference's columnar files
        (``directory/<NAME><i>``, raw int32); ``columns`` = column indices to
        read (default: the reference loader's set).  With ``background`` the
        call returns at once and the first plan that scans the table waits
        for it."""
        mask = 0
        for c in columns or ():
            mask |= 1 << c
        capi.check(capi.lib().sdb_engine_load_dir(self._h, directory.encode(), name.encode(), mask,
                                                  1 if background else 0))
        self._keep.pop(name, None)

    def sync_tables(self):
        capi.check(capi.lib().sdb_engine_sync_tables(self._h))

    def execute(self, plan) -> Result:
        text = plan if isinstance(plan, str) else json.dumps(plan)
        L = capi.lib()
        r = ctypes.c_void_p()
        capi.check(L.sdb_engine_execute(self._h, text.encode(), ctypes.byref(r)))
        return _take_result(r)

    def batch(self, plans, eager: bool = False, chain_batch: bool = True) -> "Batch":
        """Prepares ``plans`` as one batch (see ``Batch``)."""
        return Batch(self, plans, eager=eager, chain_batch=chain_batch)

    def execute_to_res(self, plan, path: str):
        """Runs ``plan`` and writes the rows as the reference's ``.res`` file."""
        text = plan if isinstance(plan, str) else json.dumps(plan)
        L = capi.lib()
        r = ctypes.c_void_p()
        capi.check(L.sdb_engine_execute(self._h, text.encode(), ctypes.byref(r)))
        try:
            capi.check(L.sdb_result_write_res(r, path.encode()))
        finally:
            L.sdb_result_free(r)

    def last_plan_ms(self) -> float:
        v = ctypes.c_double()
        capi.check(capi.lib().sdb_engine_last_plan_ms(self._h, ctypes.byref(v)))
        return v.value

    def kernel_stats(self) -> Dict[str, tuple]:
        L = capi.lib()
        n = L.sdb_engine_kernel_stats(self._h, -1, None, None, None)
        out = {}
        for k in range(n):
            name, cnt, ms = ctypes.c_char_p(), ctypes.c_uint64(), ctypes.c_double()
            L.sdb_engine_kernel_stats(self._h, k, ctypes.byref(name), ctypes.byref(cnt), ctypes.byref(ms))
            out[name.value.decode()] = (cnt.value, ms.value)
        return out


class Batch:
    """Many plans prepared once and run together (``sdb_engine_batch_*``).

    Each run replays every plan's recorded device work -- as one CUDA graph
    unless ``eager`` -- with every plan's hash-table builds in one launch and
    the plans' aggregating fused chains in one persistent launch per chain
    shape (``chain_batch``: True; "builds": only the builds batched; False:
    every chain on its own), and returns one ``Result`` per plan, each equal
    to what ``Engine.execute`` gives for that plan alone."""

    def __init__(self, engine: Engine, plans, eager: bool = False, chain_batch=True):
        L = capi.lib()
        texts = [p if isinstance(p, str) else json.dumps(p) for p in plans]
        arr = (ctypes.c_char_p * len(texts))(*[t.encode() for t in texts])
        if chain_batch not in (True, False, "builds"):
            raise ValueError("chain_batch must be True, False or 'builds'")
        mode = {True: 0, False: capi.SDB_BATCH_NO_CHAIN_BATCH, "builds": capi.SDB_BATCH_BUILDS_ONLY}[chain_batch]
        flags = (capi.SDB_BATCH_EAGER if eager else 0) | mode
        h = ctypes.c_void_p()
        capi.check(L.sdb_engine_batch_prepare(engine._h, arr, len(texts), flags, ctypes.byref(h)))
        self._h = h
        self._engine = engine  # the batch reads the engine's tables
        self.n_plans = len(texts)
        # where each plan's rows land in the pinned result mirror
        size = ctypes.c_size_t()
        ptr = L.sdb_batch_host(h, ctypes.byref(size))
        self._mirror = (np.frombuffer((ctypes.c_char * size.value).from_address(ptr), dtype=np.uint8)
                        if size.value else np.empty(0, np.uint8))
        self._layout = []
        for p in range(self.n_plans):
            nc, ns = ctypes.c_int(), ctypes.c_int()
            types = (ctypes.c_int * 64)()
            capi.check(L.sdb_batch_layout(h, p, ctypes.byref(nc), types, 64, ctypes.byref(ns)))
            dts = [np.uint64 if types[c] == 1 else np.int32 for c in range(nc.value)]
            segs = []
            for sg in range(ns.value):
                co, cap = ctypes.c_uint64(), ctypes.c_uint64()
                offs = (ctypes.c_uint64 * max(nc.value, 1))()
                capi.check(L.sdb_batch_segment(h, p, sg, ctypes.byref(co), offs, nc.value, ctypes.byref(cap)))
                segs.append((co.value, [offs[c] for c in range(nc.value)]))
            self._layout.append((dts, segs))

    def run(self, unpack: bool = True) -> Optional[List[Result]]:
        """Runs the batch once; returns one Result per plan (numpy copies of
        the rows in the pinned result mirror) unless ``unpack`` is False."""
        L = capi.lib()
        capi.check(L.sdb_batch_run(self._h, None))
        if not unpack:
            return None
        m = self._mirror
        out = []
        for dts, segs in self._layout:
            parts = [[] for _ in dts]
            for co, offs in segs:
                cnt = int(m[co:co + 4].view(np.uint32)[0])
                for c, dt in enumerate(dts):
                    w = np.dtype(dt).itemsize
                    parts[c].append(m[offs[c]:offs[c] + cnt * w].view(dt))
            out.append(Result([np.concatenate(pc) if len(pc) > 1 else (pc[0].copy() if pc else np.empty(0, dt))
                               for pc, dt in zip(parts, dts)]))
        return out

    def run_native(self) -> List[int]:
        """Runs the batch with the results unpacked into native result
        objects, as a C caller receives them, and returns each plan's row
        count (the objects are freed; no numpy conversion)."""
        L = capi.lib()
        out = (ctypes.c_void_p * self.n_plans)()
        capi.check(L.sdb_batch_run(self._h, out))
        rows = []
        for i in range(self.n_plans):
            nc, nr = ctypes.c_int(), ctypes.c_uint64()
            L.sdb_result_shape(out[i], ctypes.byref(nc), ctypes.byref(nr))
            rows.append(nr.value)
            L.sdb_result_free(out[i])
        return rows

    def stats(self) -> dict:
        st = capi.BatchStats()
        capi.check(capi.lib().sdb_batch_info(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in capi.BatchStats._fields_ if f != "pad"}

    def close(self):
        if getattr(self, "_h", None):
            capi.lib().sdb_batch_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Server:
    """Continuous batching of arriving plans (``sdb_server_*``): a native
    dispatcher thread admits waiting plans against a device budget into up to
    ``slots`` batches in flight.  While a server exists its engine must not be
    used otherwise."""

    def __init__(self, engine: Engine, budget_bytes: int = 0, pinned_bytes: int = 0, slots: int = 0,
                 max_batch: int = 0, streams_per_slot: int = 0, direct: bool = True):
        L = capi.lib()
        cfg = capi.ServerConfig(budget_bytes, pinned_bytes, slots, max_batch, streams_per_slot, 0 if direct else 1)
        h = ctypes.c_void_p()
        capi.check(L.sdb_server_create(engine._h, ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._engine = engine

    def submit(self, plan) -> int:
        text = plan if isinstance(plan, str) else json.dumps(plan)
        rid = ctypes.c_int64()
        capi.check(capi.lib().sdb_server_submit(self._h, text.encode(), ctypes.byref(rid)))
        return rid.value

    def next(self, timeout_ms: int = -1):
        """(id, status, Result or None, latency_ms, error message) of the next
        finished request; raises SdbError(SDB_ERR_TIMEOUT) if none finished in
        time."""
        L = capi.lib()
        rid, st, r, ms = ctypes.c_int64(), ctypes.c_int(), ctypes.c_void_p(), ctypes.c_double()
        capi.check(L.sdb_server_next(self._h, timeout_ms, ctypes.byref(rid), ctypes.byref(st), ctypes.byref(r),
                                     ctypes.byref(ms)))
        err = "" if st.value == capi.SDB_OK else capi.last_error()
        res = _take_result(r) if r.value else None
        return rid.value, st.value, res, ms.value, err

    def stats(self) -> dict:
        st = capi.ServerStats()
        capi.check(capi.lib().sdb_server_stats_get(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in capi.ServerStats._fields_}

    def replay(self, plans, arrivals_s, keep_results: bool = True):
        """Open-loop replay of an arrival trace; returns (statuses, latencies_ms,
        results or None, wall_s)."""
        return _replay(capi.lib().sdb_server_replay, self._h, plans, arrivals_s, keep_results)

    def close(self):
        if getattr(self, "_h", None):
            capi.lib().sdb_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def replay_plain(engine: Engine, plans, arrivals_s, keep_results: bool = True):
    """The plain path over the same trace: one plan at a time in arrival order."""
    return _replay(capi.lib().sdb_engine_replay_plain, engine._h, plans, arrivals_s, keep_results)


def _replay(fn, handle, plans, arrivals_s, keep_results):
    n = len(plans)
    texts = [(p if isinstance(p, str) else json.dumps(p)).encode() for p in plans]
    arr = (ctypes.c_char_p * n)(*texts)
    at = (ctypes.c_double * n)(*[float(x) for x in arrivals_s])
    st = (ctypes.c_int * n)()
    lat = (ctypes.c_double * n)()
    res = (ctypes.c_void_p * n)() if keep_results else None
    wall = ctypes.c_double()
    capi.check(fn(handle, arr, at, n, st, res, lat, ctypes.byref(wall)))
    results = None
    if keep_results:
        results = [_take_result(ctypes.c_void_p(res[i])) if res[i] else None for i in range(n)]
    return list(st), list(lat), results, wall.value
