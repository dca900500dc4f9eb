"""Failure paths on the GPU, produced without faulting it.

The reference ends the process on any error (the exit(100) macros of
exachem/cc/ccsd_t/ccsd_t_common.hpp:26-41); the library returns a status instead and must stay
usable.  Two failures are made on purpose, both by the library's own test switches:
- an allocation that fails (a countdown in the library's allocator makes the n-th device
  allocation report out-of-memory, as cudaMalloc does): the call returns CCSDT_E_OOM, the handle
  is destroyed and gives back all its device memory;
- a bounded device-side wait that runs out: the persistent split-precision kernel announces each
  stage's bytes but issues no TMA load, so its stage waits give up after a short poll limit; the
  call returns CCSDT_E_TIMEOUT, the kernel having released its tensor memory, and the next call on
  the same handle gives the same energies as before.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OOM, TIMEOUT = 3, 5


def _lib():
    from exachem_gb300 import ccsd_t as ct
    lib = ct.load_library()
    lib.ccsdt_debug_fail_alloc.argtypes = [ctypes.c_long, ctypes.POINTER(ctypes.c_long)]
    lib.ccsdt_debug_fail_alloc.restype = ctypes.c_int
    lib.ccsdt_debug_set_wait_test.argtypes = [ctypes.c_void_p, ctypes.c_uint, ctypes.c_int]
    lib.ccsdt_debug_set_wait_test.restype = ctypes.c_int
    return lib


def _attempts(lib, nth=0):
    n = ctypes.c_long()
    assert lib.ccsdt_debug_fail_alloc(nth, ctypes.byref(n)) == 0
    return n.value


def _sequence(d):
    """create, upload, FP64 energy, split-precision energy: the allocations of a typical call."""
    from exachem_gb300.ccsd_t import FusedTriples
    ft = FusedTriples(d["o"], d["v"], ts=40)
    try:
        ft.upload_dict(d)
        r64 = ft.energy("fp64")
        r3 = ft.energy("ozaki", slices=3)
        return r64, r3
    finally:
        ft.close()


def test_allocation_failure_returns_oom_and_destroy_frees(built):
    import torch
    from exachem_gb300.ccsd_t import CCSDTError
    from exachem_gb300.generator import generate
    lib = _lib()
    d = generate(5, 40, 3)
    _attempts(lib)                                        # reset the attempt counter
    want64, want3 = _sequence(d)
    n_alloc = _attempts(lib)
    assert n_alloc >= 10, n_alloc
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for nth in range(1, n_alloc + 1):
        _attempts(lib, nth)                               # the nth allocation from now on fails
        with pytest.raises(CCSDTError) as e:
            _sequence(d)
        assert e.value.status == OOM, (nth, e.value)
        _attempts(lib, 0)
        torch.cuda.synchronize()
        free = torch.cuda.mem_get_info()[0]
        assert free >= free0 - (4 << 20), (nth, free0 - free)   # destroy gave everything back
    # the library is still usable: a fresh handle computes the same energies bit for bit
    got64, got3 = _sequence(d)
    assert got64["e_paren_T"] == want64["e_paren_T"] and got3["e_paren_T"] == want3["e_paren_T"]


def test_bounded_wait_timeout_returns_timeout_and_handle_survives(built):
    from exachem_gb300.ccsd_t import CCSDTError, FusedTriples
    from exachem_gb300.generator import generate
    lib = _lib()
    d = generate(6, 70, 5)
    ft = FusedTriples(6, 70, ts=40)
    ft.upload_dict(d)
    want = ft.energy("ozaki", slices=3)
    assert lib.ccsdt_debug_set_wait_test(ft.h, 4096, 1) == 0    # no loads: every stage wait runs out
    with pytest.raises(CCSDTError) as e:
        ft.energy("ozaki", slices=3)
    assert e.value.status == TIMEOUT
    assert lib.ccsdt_debug_set_wait_test(ft.h, 0, 0) == 0
    got = ft.energy("ozaki", slices=3)
    assert got["e_paren_T"] == want["e_paren_T"] and got["e_bracket_T"] == want["e_bracket_T"]
    r64 = ft.energy("fp64")
    assert abs(got["e_paren_T"] - r64["e_paren_T"]) <= 5e-8 * abs(r64["e_paren_T"])
    assert lib.ccsdt_debug_set_wait_test(ft.h, 0, 3) != 0
    ft.close()
    assert np.isfinite(want["e_paren_T"])
    # the TMA energy kernel's box waits (v = 72: a row pitch TMA takes): FP32 boxes with two stages
    # and float-float ones with one; no load is in flight when they run out
    ft = FusedTriples(6, 72, ts=40)
    ft.upload_dict(generate(6, 72, 6))
    for S, store in ((2, "f32"), (4, "ff")):
        want = ft.energy("ozaki", slices=S, p_storage=store)
        assert lib.ccsdt_debug_set_wait_test(ft.h, 4096, 2) == 0
        with pytest.raises(CCSDTError) as e:
            ft.energy("ozaki", slices=S, p_storage=store)
        assert e.value.status == TIMEOUT
        assert lib.ccsdt_debug_set_wait_test(ft.h, 0, 0) == 0
        got = ft.energy("ozaki", slices=S, p_storage=store)
        assert got["e_paren_T"] == want["e_paren_T"] and got["e_bracket_T"] == want["e_bracket_T"]
    ft.close()
