"""Failure detection without a GPU fault: a bounded device wait that nothing
completes runs out, the kernel reports GFEA_ERR_TIMEOUT to the host, and the
context stays usable (the same wait bounds every stage of the staged SpMV)."""

import ctypes
import time

import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_context_survives():
    import torch

    from easyfea_gb300 import _lib

    L = _lib.load()
    st = ctypes.c_int32(99)
    # an arrival completes the phase: the wait succeeds at once
    _lib.check(L.gfea_selftest_wait(200000, 1, ctypes.byref(st), _lib.stream()), "selftest")
    assert st.value == _lib.OK
    # no arrival: the wait gives up after its limit (20 ms) with the timeout status
    t0 = time.perf_counter()
    _lib.check(L.gfea_selftest_wait(20000, 0, ctypes.byref(st), _lib.stream()), "selftest")
    dt = time.perf_counter() - t0
    assert st.value == _lib.ERR_TIMEOUT
    assert 0.015 <= dt < 5.0
    # the context still runs work
    x = torch.arange(1000, dtype=torch.float64, device="cuda")
    assert float((x * 2).sum().item()) == 999000.0
    _lib.check(L.gfea_selftest_wait(200000, 1, ctypes.byref(st), _lib.stream()), "selftest")
    assert st.value == _lib.OK
