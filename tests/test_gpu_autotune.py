"""Tile configurations of the persistent contraction and the autotuner (ccsdt_tile_configs /
ccsdt_autotune / ccsdt_set_tile_config / opts.autotune): every compiled configuration must give
bit-identical energies, so the autotuner's choice never changes a result."""
import numpy as np
import pytest

OCC, VIR = [6, 5], [32, 24, 21]       # v = 77: the N tiles of 64 and 32 pad differently


def test_tile_configs_fit_the_kernels(built):
    from exachem_gb300.ccsd_t import FusedTriples
    for S in range(1, 9):
        cfg = FusedTriples.tile_configs(S)
        assert cfg, S
        for nt, st, kc in cfg:
            smem = st * (S * 128 * kc * 2 + S * nt * kc * 2) + 1536
            assert S * nt <= 256 and 2 * S * nt <= 512 and nt % 16 == 0 and kc in (32, 64) and smem <= 227 * 1024
    assert FusedTriples.tile_configs(9) == []


@pytest.mark.gpu
def test_every_configuration_gives_identical_energies(built):
    from exachem_gb300 import ccsd_t as ct
    from exachem_gb300.generator import generate
    o, v = sum(OCC), sum(VIR)
    ft = ct.FusedTriples(o, v, OCC, VIR)
    ft.upload_dict(generate(o, v, 31))
    tri = ct.all_triplets(o)[::7]
    for S in (2, 3, 4, 5):
        ref = None
        for q in range(len(ct.FusedTriples.tile_configs(S))):
            ft.set_tile_config(S, q)
            e4, e5 = ft.triplet_energies(tri, "ozaki", slices=S)
            if ref is None:
                ref = (e4, e5)
            else:
                assert np.array_equal(e4, ref[0]) and np.array_equal(e5, ref[1]), (S, q)


@pytest.mark.gpu
def test_autotune_keeps_a_configuration_and_the_energy(built):
    from exachem_gb300 import ccsd_t as ct
    from exachem_gb300.generator import generate
    o, v = sum(OCC), sum(VIR)
    d = generate(o, v, 32)
    base = ct.FusedTriples(o, v, OCC, VIR)
    base.upload_dict(d)
    r0 = base.energy("ozaki", slices=3)
    ft = ct.FusedTriples(o, v, OCC, VIR)
    ft.upload_dict(d)
    ms, chosen = ft.autotune(3)
    assert len(ms) == len(ct.FusedTriples.tile_configs(3)) and all(t > 0 for t in ms)
    assert 0 <= chosen < len(ms) and ms[chosen] == min(ms)
    r1 = ft.energy("ozaki", slices=3)
    assert r1["e_paren_T"] == r0["e_paren_T"] and r1["e_bracket_T"] == r0["e_bracket_T"]
    auto = ct.FusedTriples(o, v, OCC, VIR)   # the same through opts.autotune on first use
    auto.upload_dict(d)
    r2 = auto.energy("ozaki", slices=3, autotune=1)
    assert r2["e_paren_T"] == r0["e_paren_T"] and r2["e_bracket_T"] == r0["e_bracket_T"]
