"""Batched multi-scene casting over the C ABI (phe_batch_*): many ray batches of uneven size over
several resident scenes, closest and any hit mixed, in one persistent launch replayed from a CUDA
graph, with launch parameters chosen by the autotuner."""
from __future__ import annotations

import ctypes as C
import json

from . import native as _n
from .native import check, lib, ptr

CLOSEST, ANY = 0, 1
ORDER_GIVEN, ORDER_LARGEST_FIRST = 0, 1


def _stream(stream):
    if stream is None:
        return None
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


class Batch:
    def __init__(self, scenes, items, block_size=128, blocks_per_sm=0, order=ORDER_GIVEN, use_graph=True, layout=0,
                 stack_shared=0, sort_window=0):
        """scenes: list of Scene; items: list of (scene index, kind, count, device rays, device out)."""
        self.scenes = list(scenes)
        arr = (C.c_void_p * len(scenes))(*[s.handle.value for s in scenes])
        self._items = self._table(items)
        p = _n.BatchParams(block_size, blocks_per_sm, order, 1 if use_graph else 0, layout, stack_shared, sort_window, 0)
        h = C.c_void_p()
        check(lib().phe_batch_create(arr, len(scenes), self._items, len(items), C.byref(p), C.byref(h)), "phe_batch_create")
        self.handle = h

    @staticmethod
    def _table(items):
        t = (_n.BatchItem * max(1, len(items)))()
        for i, (scene, kind, count, rays, out) in enumerate(items):
            t[i] = _n.BatchItem(scene, kind, count, 0, ptr(rays), ptr(out))
        return t

    def update(self, items) -> None:
        self._items = self._table(items)
        check(lib().phe_batch_update(self.handle, self._items, len(items)), "phe_batch_update")

    def set_params(self, block_size=128, blocks_per_sm=0, order=ORDER_GIVEN, use_graph=True, layout=0, stack_shared=0,
                   sort_window=0) -> None:
        """stack_shared: traversal-stack entries in shared memory (0 or 16); sort_window: 0, or rays traced
        grouped by direction octant within windows of that many rays (a multiple of 256 up to 4096)."""
        p = _n.BatchParams(block_size, blocks_per_sm, order, 1 if use_graph else 0, layout, stack_shared, sort_window, 0)
        check(lib().phe_batch_set_params(self.handle, C.byref(p)), "phe_batch_set_params")

    def launch(self, stream=None) -> None:
        check(lib().phe_batch_launch(self.handle, _stream(stream)), "phe_batch_launch")

    def info(self):
        t, p = C.c_uint64(), C.c_uint32()
        check(lib().phe_batch_info(self.handle, C.byref(t), C.byref(p)), "phe_batch_info")
        return int(t.value), int(p.value)

    def autotune(self, repeats=3, stream=None):
        """Returns (best params dict, best ms, all candidate rows)."""
        best = _n.BatchParams()
        ms = C.c_float()
        cap = 512
        rows = (_n.BatchTuningRow * cap)()
        n = C.c_uint32()
        check(lib().phe_batch_autotune(self.handle, repeats, _stream(stream), C.byref(best), C.byref(ms), rows, cap,
                                       C.byref(n)), "phe_batch_autotune")
        as_dict = lambda p: {"blockSize": p.blockSize, "blocksPerSM": p.blocksPerSM, "order": p.order,
                             "useGraph": p.useGraph, "layout": p.layout, "stackShared": p.stackShared,
                             "sortWindow": p.sortWindow}
        table = [dict(as_dict(rows[i].params), ms=rows[i].ms) for i in range(min(n.value, cap))]
        return as_dict(best), float(ms.value), table

    def close(self) -> None:
        if getattr(self, "handle", None):
            check(lib().phe_batch_destroy(self.handle), "phe_batch_destroy")
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def save_tuning(path, best, ms, table, command="") -> None:
    """A short record of an autotune: the winner, the best time for each value of each parameter, the ten
    fastest candidates and the slowest."""
    rows = sorted(table, key=lambda r: r["ms"])
    per = {}
    for key in ("blockSize", "order", "layout", "stackShared", "sortWindow"):
        best_of = {}
        for r in rows:
            best_of[str(r[key])] = min(best_of.get(str(r[key]), 1e30), r["ms"])
        per[key] = {k: round(v, 4) for k, v in best_of.items()}
    out = {"command": command, "candidates": len(rows), "best": best, "best_ms": round(ms, 4),
           "best_ms_per_value": per, "top10": [dict(r, ms=round(r["ms"], 4)) for r in rows[:10]],
           "slowest": dict(rows[-1], ms=round(rows[-1]["ms"], 4)) if rows else None}
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
