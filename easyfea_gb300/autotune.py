"""Autotuner of the kernel schedules (libgb300fea.so ``gfea_tune_*``).

Two schedules are chosen by measurement on the device and recorded per
problem class inside the library:

* SpMV row-block schedule -- lanes per node (4, 8, 16, 32) of the node-row
  products used by PCG, keyed by DOF per node, value type and log2 buckets of
  the row length and node count;
* element tile schedule -- blocks of 128 threads per SM (4 .. 64) of the
  element kernel, keyed by element type, value type, C mode and the log2
  bucket of the element count.

``set_mode(2)`` makes the first solve / assembly of each class tune itself;
``save``/``load`` keep decisions across processes (JSON).
"""

from __future__ import annotations

import ctypes
import json
from typing import Dict

import torch

from . import _lib

OFF, USE, TUNE = 0, 1, 2
_mode = USE  # the library's default


def set_mode(mode: int) -> None:
    global _mode
    _lib.check(_lib.load().gfea_tune_mode(int(mode)), "tune mode")
    _mode = int(mode)


def get_mode() -> int:
    return _mode


def clear() -> None:
    _lib.check(_lib.load().gfea_tune_clear(), "tune clear")


def decisions() -> Dict[int, int]:
    L = _lib.load()
    n = ctypes.c_int()
    _lib.check(L.gfea_tune_export(None, None, 0, ctypes.byref(n)), "tune export")
    keys = (ctypes.c_int64 * max(n.value, 1))()
    vals = (ctypes.c_int32 * max(n.value, 1))()
    _lib.check(L.gfea_tune_export(keys, vals, n.value, ctypes.byref(n)), "tune export")
    return {int(keys[i]): int(vals[i]) for i in range(n.value)}


def load_decisions(d: Dict[int, int]) -> None:
    if not d:
        return
    n = len(d)
    keys = (ctypes.c_int64 * n)(*[int(k) for k in d])
    vals = (ctypes.c_int32 * n)(*[int(v) for v in d.values()])
    _lib.check(_lib.load().gfea_tune_import(keys, vals, n), "tune import")


def save(path: str) -> None:
    with open(path, "w") as f:
        json.dump({str(k): v for k, v in decisions().items()}, f)


def load(path: str) -> None:
    with open(path) as f:
        load_decisions({int(k): int(v) for k, v in json.load(f).items()})


def tune_spmv(op, value_type: int = _lib.F32):
    """Tune (and record) the row-block schedule of an operator; returns
    (lanes, ms per product)."""
    L = _lib.load()
    if value_type == _lib.F32:
        op.ensure_f32()
    dt = torch.float32 if value_type == _lib.F32 else torch.float64
    x = torch.ones(op.N, dtype=dt, device=op.vals64.device)
    y = torch.empty_like(x)
    lanes, ms = ctypes.c_int32(), ctypes.c_float()
    sys = op.system(None)
    _lib.check(L.gfea_tune_spmv(ctypes.byref(sys), value_type, _lib.ptr(x), _lib.ptr(y), ctypes.byref(lanes),
                                ctypes.byref(ms), _lib.stream()), "tune spmv")
    return int(lanes.value), float(ms.value)
