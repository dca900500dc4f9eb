"""The open-shell (UHF) (T) on the GPU (ccsdt_energy_spin_orbital) against the spin-orbital
oracle, which the reference's own CPU kernels run unrestricted pin (test_spin_orbital_oracle.py).
Relative tolerance 1e-12 on E[T] and E(T): FP64 contractions, compensated sums."""
import numpy as np
import pytest

import oracle
from conftest import rel_close
from exachem_gb300 import ccsd_t
from exachem_gb300.generator import generate
from oracle.spin_orbital_oracle import (energy_spin_orbital, open_shell_system, spin_orbital_inputs,
                                        spin_orbital_inputs_vec)

pytestmark = pytest.mark.gpu

CASES = [(3, 2, 5, 6, 5), (4, 3, 6, 7, 6), (5, 1, 3, 7, 8), (1, 3, 4, 3, 9), (2, 2, 4, 4, 7),
         (6, 4, 10, 12, 10), (3, 0, 4, 0, 1), (0, 4, 0, 5, 2)]


def _call(oa, ob, va, vb, arrs, **kw):
    r = ccsd_t.energy_spin_orbital(oa, ob, va, vb, *arrs, **kw)
    return r["e_bracket_T"], r["e_paren_T"]


@pytest.mark.parametrize("oa,ob,va,vb,seed", CASES)
def test_open_shell_matches_spin_orbital_oracle(built, oa, ob, va, vb, seed):
    arrs = open_shell_system(oa, ob, va, vb, 7, seed)
    e4, e5 = energy_spin_orbital(*arrs)
    g4, g5 = _call(oa, ob, va, vb, arrs)
    assert rel_close(g4, e4, 1e-12) and rel_close(g5, e5, 1e-12), (g4, e4, g5, e5)


def test_fewer_than_three_occupied_gives_zero(built):
    arrs = open_shell_system(1, 1, 3, 3, 4, 3)
    assert _call(1, 1, 3, 3, arrs) == (0.0, 0.0)


def test_spin_forbidden_blocks_are_not_read(built):
    """NaN in every spin-forbidden element leaves the energies bit for bit unchanged."""
    oa, ob, va, vb = 4, 3, 6, 7
    arrs = list(open_shell_system(oa, ob, va, vb, 6, 12))
    so, sv = np.array([0] * oa + [1] * ob), np.array([0] * va + [1] * vb)

    def allowed(*sp):
        g = np.meshgrid(*sp, indexing="ij")
        return g[0] == g[1] if len(g) == 2 else g[0] + g[1] == g[2] + g[3]
    masks = [allowed(sv, so), allowed(sv, sv, so, so), allowed(so, so, sv, sv), allowed(so, so, so, sv),
             allowed(so, sv, sv, sv)]
    poisoned = arrs[:2] + [np.ascontiguousarray(np.where(m, a, np.nan)) for m, a in zip(masks, arrs[2:])]
    assert _call(oa, ob, va, vb, poisoned) == _call(oa, ob, va, vb, arrs)


def test_device_inputs_match_host_inputs(built):
    import torch
    oa, ob, va, vb = 4, 2, 7, 8
    arrs = open_shell_system(oa, ob, va, vb, 6, 13)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]
    assert _call(oa, ob, va, vb, dev) == _call(oa, ob, va, vb, arrs)


def test_shards_sum_to_the_whole(built):
    oa, ob, va, vb = 5, 4, 8, 9
    arrs = open_shell_system(oa, ob, va, vb, 6, 14)
    w4, w5 = _call(oa, ob, va, vb, arrs)
    parts = [_call(oa, ob, va, vb, arrs, shard_index=s, shard_count=3) for s in range(3)]
    assert rel_close(sum(p[0] for p in parts), w4, 1e-13) and rel_close(sum(p[1] for p in parts), w5, 1e-13)


@pytest.mark.parametrize("o,v,seed", [(3, 6, 1), (4, 9, 2)])
def test_closed_shell_inputs_give_the_closed_shell_energies(built, o, v, seed):
    d = generate(o, v, seed)
    e4, e5 = oracle.energy(d)
    g4, g5 = _call(o, o, v, v, spin_orbital_inputs(d))
    assert rel_close(g4, e4, 1e-12) and rel_close(g5, e5, 1e-12)


def test_closed_shell_inputs_match_the_closed_shell_gpu_path(built):
    """A larger restricted case, where the oracle is slow: the spin-orbital path over all four
    spin cases equals the closed-shell FP64 GPU path on the same system."""
    o, v = 8, 40
    d = generate(o, v, 3)
    g4, g5 = _call(o, o, v, v, spin_orbital_inputs_vec(d))
    ft = ccsd_t.FusedTriples(o, v, ts=16)
    try:
        ft.upload_dict(d)
        r = ft.energy("fp64")
    finally:
        ft.close()
    assert rel_close(g4, r["e_bracket_T"], 1e-11) and rel_close(g5, r["e_paren_T"], 1e-11)


def test_open_shell_matches_reference_golden(built):
    """Against ExaChem's own CPU (T) run unrestricted (tests/golden/open_shell_energies.json, made by
    tests/golden/make_open_shell_golden.py from oracle/_ref) on systems the dense oracle cannot
    hold, up to 14 occupied and 84 virtual spin orbitals with ragged alpha / beta tiles."""
    import json
    from conftest import ROOT
    from oracle.spin_orbital_oracle import golden_checksums as checksums
    cases = json.loads((ROOT / "tests" / "golden" / "open_shell_energies.json").read_text())["cases"]
    for c in cases:
        arrs = open_shell_system(c["oa"], c["ob"], c["va"], c["vb"], c["nq"], c["seed"], exact=True)
        assert checksums(arrs) == c["checksums"], c["name"]
        g4, g5 = _call(c["oa"], c["ob"], c["va"], c["vb"], arrs)
        assert rel_close(g4, c["e_bracket_T"], 1e-12) and rel_close(g5, c["e_paren_T"], 1e-12), \
            (c["name"], g4, c["e_bracket_T"], g5, c["e_paren_T"])


def test_open_shell_bench_line(built):
    """bench.py --open-shell prints one JSON line with the contract's keys (small system)."""
    import json
    import subprocess
    import sys
    from conftest import ROOT
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--open-shell", "4,3,12,14", "--steps", "1",
                          "--warmup", "3"], check=True, capture_output=True, text=True, timeout=600, cwd=ROOT)
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "dtype",
              "config", "roofline", "cpu_baseline", "e2e", "gpu_launches", "clocks"):
        assert k in line, k
    assert line["value"] > 0 and line["e2e"]["value"] > 0 and line["gpu_launches"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["energies"]["host_equals_device"]


@pytest.mark.parametrize("oa,ob,va,vb,seed", [(4, 3, 6, 7, 6), (6, 4, 10, 12, 10), (3, 0, 4, 0, 1), (0, 4, 0, 5, 2)])
def test_split_open_shell_close_to_fp64(built, oa, ob, va, vb, seed):
    """Split-precision spin-block contractions (BF16 digit planes per spin of the contraction
    index): the error against the FP64 path shrinks with the slice count, alpha-only and beta-only
    systems included."""
    arrs = open_shell_system(oa, ob, va, vb, 7, seed)
    f4, f5 = _call(oa, ob, va, vb, arrs)
    errs = {}
    # one triplet of four virtuals (the alpha-only case) has no sum to average the digit truncation
    # over: the bounds are those of a single element's few products
    for S, tol in ((2, 1e-4), (3, 1e-6), (4, 5e-8), (6, 1e-10)):
        g4, g5 = _call(oa, ob, va, vb, arrs, slices=S)
        errs[S] = abs(g5 - f5) / abs(f5)
        assert errs[S] <= tol and abs(g4 - f4) <= tol * abs(f4), (S, errs)
    assert errs[6] < errs[3] < errs[2]


def test_split_open_shell_larger_system(built):
    """A ragged spin split at the size where the contraction dominates: S = 4 within 1e-9 of the
    FP64 path, and the shards of the split path sum to its whole."""
    import torch
    oa, ob, va, vb = 7, 5, 60, 48
    arrs = open_shell_system(oa, ob, va, vb, 30, 21)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]
    f4, f5 = _call(oa, ob, va, vb, dev)
    g4, g5 = _call(oa, ob, va, vb, dev, slices=4)
    assert rel_close(g5, f5, 1e-9) and rel_close(g4, f4, 1e-9), (g5, f5)
    parts = [_call(oa, ob, va, vb, dev, shard_index=s, shard_count=2, slices=4) for s in range(2)]
    assert rel_close(parts[0][1] + parts[1][1], g5, 1e-13)
    with pytest.raises(ccsd_t.CCSDTError):
        _call(oa, ob, va, vb, dev, slices=7)
