"""Autotuner decision table: host-side entry points (no GPU needed)."""

import ctypes

from easyfea_gb300 import _lib, autotune


def test_mode_range():
    L = _lib.load()
    assert L.gfea_tune_mode(3) == 1 and L.gfea_tune_mode(-1) == 1
    for m in (0, 2, 1):
        assert L.gfea_tune_mode(m) == 0


def test_import_export_roundtrip(tmp_path):
    autotune.clear()
    d = {(1 << 32) | (3 << 24) | (1 << 16) | (8 << 8) | 19: 16, (2 << 32) | (4 << 24) | (0 << 16) | (0 << 8) | 19: 8}
    autotune.load_decisions(d)
    assert autotune.decisions() == d
    path = tmp_path / "tune.json"
    autotune.save(str(path))
    autotune.clear()
    assert autotune.decisions() == {}
    autotune.load(str(path))
    assert autotune.decisions() == d
    # export with a short buffer reports the total
    n = ctypes.c_int()
    keys = (ctypes.c_int64 * 1)()
    vals = (ctypes.c_int32 * 1)()
    assert _lib.load().gfea_tune_export(keys, vals, 1, ctypes.byref(n)) == 0 and n.value == 2
    autotune.clear()
