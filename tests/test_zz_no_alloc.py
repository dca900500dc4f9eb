"""The allocation-free entry point (ccsdt_energy_noalloc) against the handle-based one.

It serves callers that cannot call cudaMalloc (a device owned by a pooled allocator, a fixed
device-memory budget): all its intermediates live in one fixed device array inside the library.
The test calls it through the C ABI twice in a row and compares with ccsdt_energy and with the
oracle at the FP64 parity tolerance used by the other GPU tests.  This file is collected last on
purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _noalloc(lib, d, out, stream):
    vp = ctypes.c_void_p
    f = lib.ccsdt_energy_noalloc
    f.argtypes = [ctypes.c_int, ctypes.c_int] + [vp] * 9   # 7 inputs, energies, stream
    f.restype = ctypes.c_int
    args = [vp(d[k].data_ptr()) for k in ("eps_occ", "eps_vir", "t1", "t2", "oovv", "ooov", "ovvv")]
    return f(int(d["o"]), int(d["v"]), *args, vp(out.data_ptr()), vp(stream))


@pytest.mark.parametrize("o,v,seed", [(6, 20, 4), (12, 48, 5)])
def test_noalloc_matches_handle_api_twice(built, o, v, seed):
    import torch
    import oracle
    from exachem_gb300 import ccsd_t as ct
    from exachem_gb300.generator import generate

    d = generate(o, v, seed)
    o4, o5 = oracle.energy(d)
    ref = ct.FusedTriples(o, v, ts=40)
    ref.upload_dict(d)
    want = ref.energy("fp64")
    ref.close()

    lib = ct.load_library()
    dev = {k: (torch.from_numpy(d[k]).cuda() if isinstance(d[k], np.ndarray) else d[k]) for k in d}
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
        assert _noalloc(lib, dev, out, stream) == 0
        torch.cuda.synchronize()
        e4, e5 = out.tolist()
        assert abs(e4 - want["e_bracket_T"]) <= RTOL * abs(want["e_bracket_T"])
        assert abs(e5 - want["e_paren_T"]) <= RTOL * abs(want["e_paren_T"])
        assert abs(e4 - o4) <= RTOL * abs(o4) and abs(e5 - o5) <= RTOL * abs(o5)


def test_noalloc_rejects_sizes_beyond_its_scratch(built):
    import torch
    from exachem_gb300 import ccsd_t as ct
    from exachem_gb300.generator import generate

    lib = ct.load_library()
    d = generate(3, 49, 1)
    dev = {k: (torch.from_numpy(d[k]).cuda() if isinstance(d[k], np.ndarray) else d[k]) for k in d}
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    assert _noalloc(lib, dev, out, torch.cuda.current_stream().cuda_stream) == 1   # CCSDT_E_INVALID
    d["o"] = 13
    assert _noalloc(lib, dev, out, torch.cuda.current_stream().cuda_stream) == 1
