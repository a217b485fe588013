"""The C-ABI library builds, loads and exports every entry point declared in
include/gfea.h (no compute calls: runs without a GPU)."""

import os
import re

from easyfea_gb300 import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names.update(re.findall(r"\b(gfea_\w+)\s*\(", src))
    return sorted(names)


def test_library_exports_all_declared_symbols():
    path = _build.build()
    lib = _lib.load(path)
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # every declared symbol has a ctypes signature and vice versa
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_host_only_entry_points():
    import ctypes

    lib = _lib.load()
    assert lib.gfea_version().startswith(b"gfea")
    assert lib.gfea_status_string(0) == b"ok"
    ws = ctypes.c_size_t()
    assert lib.gfea_graph_workspace_size(100, 50, 4, ctypes.byref(ws)) == 0 and ws.value > 0
    assert lib.gfea_graph_workspace_size(100, 50, 0, ctypes.byref(ws)) == 1  # invalid nPe
    sysd = _lib.System(_lib.ABI_VERSION, 2, 10, 30, 0, 0, 0, 0, 0, 0, 0)
    opts = _lib.PcgOpts(_lib.ABI_VERSION, _lib.F64, 100, 10, 1e-10, 1e-4, 10, 0)
    assert lib.gfea_pcg_workspace_size(ctypes.byref(sysd), ctypes.byref(opts), ctypes.byref(ws)) == 0
    assert ws.value > 20 * 8
    # argument checks fail loudly before touching the device
    res = _lib.PcgResult()
    assert lib.gfea_pcg_solve(ctypes.byref(sysd), 0, 0, ctypes.byref(opts), 0, 0, ctypes.byref(res), 0) == 1
    assert lib.gfea_reduce_workspace_size() > 0


def test_pcg_workspace_holds_packed_tiles(monkeypatch):
    """The PCG workspace query includes the packed node tiles of the staged
    SpMV (each tile: node offsets, neighbour indices and CSR values, 15 %
    headroom) when the operator exceeds half of the L2 and a ring of eight
    tiles fits in shared memory, and leaves them out otherwise (the unstaged
    kernel then runs)."""
    import ctypes

    lib = _lib.load()
    ws = ctypes.c_size_t()

    def size(D, Nn, deg, prec):
        sysd = _lib.System(_lib.ABI_VERSION, D, Nn, Nn * deg, 0, 0, 0, 0, 0, 0, 0)
        opts = _lib.PcgOpts(_lib.ABI_VERSION, prec, 100, 0, 1e-10, 0.0, 10, 0, 0, 0)
        assert lib.gfea_pcg_workspace_size(ctypes.byref(sysd), ctypes.byref(opts), ctypes.byref(ws)) == 0
        return ws.value

    monkeypatch.delenv("GFEA_STAGE_MIN_BYTES", raising=False)
    Nn = 4_000_000
    for D, deg in ((3, 27), (2, 9), (1, 7)):
        for prec, s in ((_lib.F32, 4), (_lib.F64, 8)):
            operator = D * D * Nn * deg * s + 4 * Nn * deg
            assert size(D, Nn, deg, prec) >= 1.15 * operator
    # an L2-sized operator stays unstaged (no tiles reserved) ...
    small = 9 * 10_000 * 27 * 4
    assert size(3, 10_000, 27, _lib.F32) < small
    # ... unless the threshold is lowered
    monkeypatch.setenv("GFEA_STAGE_MIN_BYTES", "0")
    assert size(3, 10_000, 27, _lib.F32) >= 1.15 * (small + 4 * 10_000 * 27)
    # rows of 40 neighbours in FP64: eight 10-node tiles exceed shared memory
    assert size(3, 10_000, 40, _lib.F64) < 9 * 10_000 * 40 * 8
