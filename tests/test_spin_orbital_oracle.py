"""The spin-orbital (T) oracle (oracle/spin_orbital_oracle.py), the groundwork for an open-shell
path.  Pinned two ways:
- on closed-shell systems it equals the closed-shell oracle, which the reference's golden
  vectors pin (tests/test_oracle_golden.py);
- against ExaChem's own CPU (T) kernels (oracle/_ref, ref_ccsd_t_energy_so) given the same
  spin-orbital tensors: restricted and unrestricted on RHF-derived inputs, unrestricted on
  open-shell inputs (alpha and beta orbital sets of different sizes).
CPU only; the comparisons with oracle/_ref skip where the reference tree is not built."""
import numpy as np
import pytest

import oracle
from exachem_gb300.generator import generate
from oracle.spin_orbital_oracle import energy_spin_orbital, open_shell_system, spin_orbital_inputs

needs_ref = pytest.mark.skipif(not oracle.REF_LIB.exists(), reason="reference tree not built here")


def _tiles(n, t):
    """Tile extents of n orbitals in tiles of at most t (the last one ragged)."""
    return [t] * (n // t) + ([n % t] if n % t else [])


@pytest.mark.parametrize("o,v,seed", [(3, 6, 1), (4, 7, 2), (2, 5, 3)])
def test_spin_orbital_oracle_equals_closed_shell_oracle(o, v, seed):
    d = generate(o, v, seed)
    c4, c5 = oracle.energy(d)
    s4, s5 = energy_spin_orbital(*spin_orbital_inputs(d))
    assert s4 == pytest.approx(c4, rel=1e-12, abs=0)
    assert s5 == pytest.approx(c5, rel=1e-12, abs=0)


def test_open_shell_system_has_the_reference_symmetries():
    eps_o, eps_v, t1, t2, v2ijab, v2ijka, v2iabc = open_shell_system(3, 2, 5, 4, 6, 9)
    np.testing.assert_array_equal(t2, -t2.transpose(1, 0, 2, 3))
    np.testing.assert_array_equal(t2, -t2.transpose(0, 1, 3, 2))
    np.testing.assert_allclose(v2ijab, -v2ijab.transpose(0, 1, 3, 2), rtol=0, atol=1e-15)
    np.testing.assert_allclose(v2ijab, -v2ijab.transpose(1, 0, 2, 3), rtol=0, atol=1e-15)
    np.testing.assert_allclose(v2iabc, -v2iabc.transpose(0, 1, 3, 2), rtol=0, atol=1e-15)
    # spin conservation: alpha occupied 0..2, beta 3..4; alpha virtual 0..4, beta 5..8
    assert not t1[:5, 3:].any() and not t1[5:, :3].any()
    assert not t2[:5, :5, 3:, 3:].any() and not v2ijab[:3, :3, 5:, 5:].any()


@needs_ref
@pytest.mark.parametrize("restricted", [True, False])
@pytest.mark.parametrize("o,v,ot,vt,seed", [(4, 7, 2, 4, 2), (3, 6, 2, 4, 1), (5, 5, 3, 2, 4)])
def test_reference_spin_orbital_kernels_on_closed_shell_inputs(o, v, ot, vt, seed, restricted):
    d = generate(o, v, seed)
    eps_o, eps_v, *rest = spin_orbital_inputs(d)
    c4, c5 = oracle.energy(d)
    tiles = (_tiles(o, ot), _tiles(o, ot), _tiles(v, vt), _tiles(v, vt))
    r4, r5, ntask = oracle.ref_energy_spin_orbital(tiles, np.concatenate([eps_o, eps_v]), *rest,
                                                   is_restricted=restricted)
    assert ntask > 0
    assert r4 == pytest.approx(c4, rel=1e-12, abs=0)
    assert r5 == pytest.approx(c5, rel=1e-12, abs=0)


@needs_ref
@pytest.mark.parametrize("oa,ob,va,vb,ot,vt,seed", [
    (3, 2, 5, 6, 2, 3, 5),
    (4, 3, 6, 7, 2, 4, 6),
    (2, 2, 4, 4, 1, 3, 7),
    (5, 1, 3, 7, 3, 2, 8),
])
def test_open_shell_oracle_equals_reference_unrestricted(oa, ob, va, vb, ot, vt, seed):
    sys_ = open_shell_system(oa, ob, va, vb, 7, seed)
    e4, e5 = energy_spin_orbital(*sys_)
    tiles = (_tiles(oa, ot), _tiles(ob, ot), _tiles(va, vt), _tiles(vb, vt))
    r4, r5, ntask = oracle.ref_energy_spin_orbital(tiles, np.concatenate(sys_[:2]), *sys_[2:],
                                                   is_restricted=False)
    assert ntask > 0
    assert e4 == pytest.approx(r4, rel=1e-12, abs=0)
    assert e5 == pytest.approx(r5, rel=1e-12, abs=0)


@pytest.mark.parametrize("o,v,seed", [(3, 6, 1), (2, 5, 3)])
def test_vectorised_spin_orbital_inputs_equal_the_loops(o, v, seed):
    from oracle.spin_orbital_oracle import spin_orbital_inputs_vec
    d = generate(o, v, seed)
    for a, b in zip(spin_orbital_inputs(d), spin_orbital_inputs_vec(d)):
        assert np.array_equal(a, b)


def _open_shell_golden():
    import json
    from conftest import ROOT
    return json.loads((ROOT / "tests" / "golden" / "open_shell_energies.json").read_text())["cases"]


def test_open_shell_golden_inputs_regenerate_bit_for_bit():
    """The fixtures' systems come back with the recorded exact checksums (the GPU tests rebuild
    them on another machine and compare with the reference's energies)."""
    from oracle.spin_orbital_oracle import golden_checksums as checksums
    for c in _open_shell_golden():
        arrs = open_shell_system(c["oa"], c["ob"], c["va"], c["vb"], c["nq"], c["seed"], exact=True)
        assert checksums(arrs) == c["checksums"], c["name"]


def test_open_shell_golden_matches_the_oracle():
    for c in _open_shell_golden()[:2]:
        arrs = open_shell_system(c["oa"], c["ob"], c["va"], c["vb"], c["nq"], c["seed"], exact=True)
        e4, e5 = energy_spin_orbital(*arrs)
        assert e4 == pytest.approx(c["e_bracket_T"], rel=1e-12, abs=0)
        assert e5 == pytest.approx(c["e_paren_T"], rel=1e-12, abs=0)


@needs_ref
def test_reference_reruns_its_open_shell_golden():
    c = _open_shell_golden()[2]
    arrs = open_shell_system(c["oa"], c["ob"], c["va"], c["vb"], c["nq"], c["seed"], exact=True)
    r4, r5, n = oracle.ref_energy_spin_orbital(c["tiles"], np.concatenate(arrs[:2]), *arrs[2:], is_restricted=False)
    assert (r4, r5, n) == (c["e_bracket_T"], c["e_paren_T"], c["ref_tasks"])


@pytest.mark.parametrize("oa,ob,va,vb,seed", [(3, 2, 5, 6, 5), (4, 3, 6, 7, 6), (3, 0, 4, 0, 1), (1, 3, 4, 3, 9)])
def test_c_restatement_equals_the_numpy_oracle(oa, ob, va, vb, seed):
    arrs = open_shell_system(oa, ob, va, vb, 6, seed)
    e4, e5 = energy_spin_orbital(*arrs)
    c4, c5 = oracle.energy_spin_orbital_c(oa, ob, va, vb, arrs)
    assert c4 == pytest.approx(e4, rel=1e-12, abs=1e-300) and c5 == pytest.approx(e5, rel=1e-12, abs=1e-300)


def test_c_restatement_matches_the_reference_golden():
    for c in _open_shell_golden()[:4]:
        arrs = open_shell_system(c["oa"], c["ob"], c["va"], c["vb"], c["nq"], c["seed"], exact=True)
        g4, g5 = oracle.energy_spin_orbital_c(c["oa"], c["ob"], c["va"], c["vb"], arrs)
        assert g4 == pytest.approx(c["e_bracket_T"], rel=1e-12) and g5 == pytest.approx(c["e_paren_T"], rel=1e-12), \
            c["name"]


def test_c_restatement_triplet_subsets_sum_to_the_whole():
    import itertools
    oa, ob, va, vb = 4, 3, 6, 7
    arrs = open_shell_system(oa, ob, va, vb, 6, 21)
    w4, w5 = oracle.energy_spin_orbital_c(oa, ob, va, vb, arrs)
    tri = list(itertools.combinations(range(oa + ob), 3))
    parts = [oracle.energy_spin_orbital_c(oa, ob, va, vb, arrs, tri[s::3]) for s in range(3)]
    assert sum(p[0] for p in parts) == pytest.approx(w4, rel=1e-13)
    assert sum(p[1] for p in parts) == pytest.approx(w5, rel=1e-13)
    with pytest.raises(RuntimeError):
        oracle.energy_spin_orbital_c(oa, ob, va, vb, arrs, [(1, 0, 2)])


def _open_shell_ci_ops():
    import json
    from conftest import ROOT
    return json.loads((ROOT / "tests" / "golden" / "open_shell_energies.json").read_text())["ci_ops"]


def test_unrestricted_op_count_matches_the_reference_ci(built):
    """ccsdt_reference_op_count_so with is_restricted = 0 reproduces the total_num_ops of the
    reference's CI run of an unrestricted (T) (CH4 triplet, def2-TZVP: 6 / 4 occupied, 49 / 51
    virtual, tiles of 28) - the unrestricted task list and spin filters of ccsd_t_fused_driver.hpp."""
    from exachem_gb300.ccsd_t import reference_op_count_so
    from exachem_gb300.generator import tiles_uniform
    for c in _open_shell_ci_ops():
        ops, _ = reference_op_count_so(*(tiles_uniform(n, c["ts"]) for n in (c["oa"], c["ob"], c["va"], c["vb"])))
        assert ops == c["total_num_ops"], c["file"]


def test_unrestricted_task_count_matches_the_reference_runs(built):
    from exachem_gb300.ccsd_t import reference_op_count_so
    for c in _open_shell_golden():
        assert reference_op_count_so(*c["tiles"])[1] == c["ref_tasks"], c["name"]


def test_restricted_op_count_over_spin_tiles_equals_the_closed_shell_count(built):
    from exachem_gb300.ccsd_t import reference_op_count, reference_op_count_so
    ot, vt = [3, 5], [7, 13, 20]
    assert reference_op_count_so(ot, ot, vt, vt, is_restricted=True) == reference_op_count(8, 40, ot, vt)
    # unrestricted counts every spin case: more work than the restricted half
    assert reference_op_count_so(ot, ot, vt, vt)[0] > reference_op_count(8, 40, ot, vt)[0]
