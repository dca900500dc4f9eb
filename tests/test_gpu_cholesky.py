"""Integral blocks built on the device from spatial Cholesky vectors (ccsdt_upload_cholesky):
oovv = (ia|jb), ooov = (ij|ka), ovvv = (ia|bc) = sum_Q L L (the closed-shell blocks of
exachem/cholesky/v2tensors.cpp:66-88) must give the energies of the same blocks built on the host
and uploaded with ccsdt_upload, and of the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OCC, VIR = [4, 3], [16, 14]


def _cholesky_system(o, v, nq, seed):
    """The generator's amplitudes and orbital energies with integrals from random spatial Cholesky
    vectors L[p][q][Q] (symmetric in p, q), and the host-built blocks."""
    from exachem_gb300.generator import generate
    d = generate(o, v, seed)
    rng = np.random.default_rng(seed + 1000)
    n = o + v
    L = rng.normal(0.0, 0.05, size=(n, n, nq))
    L = 0.5 * (L + L.transpose(1, 0, 2))
    Loo, Lov, Lvv = (np.ascontiguousarray(x) for x in (L[:o, :o], L[:o, o:], L[o:, o:]))
    d["oovv"] = np.einsum("iaQ,jbQ->ijab", Lov, Lov)
    d["ooov"] = np.einsum("ijQ,kaQ->ijka", Loo, Lov)
    d["ovvv"] = np.einsum("iaQ,bcQ->iabc", Lov, Lvv)
    return d, (Loo, Lov, Lvv)


def test_cholesky_blocks_match_host_blocks_and_oracle(built):
    import oracle
    from exachem_gb300.ccsd_t import FusedTriples
    o, v = sum(OCC), sum(VIR)
    d, (Loo, Lov, Lvv) = _cholesky_system(o, v, 40, 11)
    ref = FusedTriples(o, v, OCC, VIR)
    ref.upload_dict(d)
    r = ref.energy("fp64")
    ft = FusedTriples(o, v, OCC, VIR)
    ft.upload_cholesky(d["eps_occ"], d["eps_vir"], d["t1"], d["t2"], Loo, Lov, Lvv)
    g = ft.energy("fp64")
    e4, e5 = oracle.energy(d)
    for got, want, orc in ((g["e_bracket_T"], r["e_bracket_T"], e4), (g["e_paren_T"], r["e_paren_T"], e5)):
        assert abs(got - want) <= 1e-12 * abs(want)
        assert abs(got - orc) <= 1e-12 * abs(orc)
    s3 = ft.energy("ozaki", slices=3)   # the split path on the device-built blocks
    assert abs(s3["e_paren_T"] - e5) <= 1e-7 * abs(e5)


def test_cholesky_from_device_vectors(built):
    import torch
    from exachem_gb300.ccsd_t import FusedTriples
    o, v = sum(OCC), sum(VIR)
    d, L = _cholesky_system(o, v, 17, 12)   # an n_chol that is not a multiple of the GEMM's k chunk
    host = FusedTriples(o, v, OCC, VIR)
    host.upload_cholesky(d["eps_occ"], d["eps_vir"], d["t1"], d["t2"], *L)
    dev = FusedTriples(o, v, OCC, VIR)
    on = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (d["eps_occ"], d["eps_vir"], d["t1"], d["t2"], *L)]
    dev.upload_cholesky(*on)
    a, b = host.energy("fp64"), dev.energy("fp64")
    assert a["e_paren_T"] == b["e_paren_T"] and a["e_bracket_T"] == b["e_bracket_T"]


def test_cholesky_rejects_bad_input(built):
    from exachem_gb300.ccsd_t import CCSDTError, FusedTriples
    o, v = sum(OCC), sum(VIR)
    d, (Loo, Lov, Lvv) = _cholesky_system(o, v, 8, 13)
    ft = FusedTriples(o, v, OCC, VIR)
    bad = Lvv.copy()
    bad[3, 5, 2] = np.nan
    with pytest.raises(CCSDTError):                     # a non-finite vector reaches ovvv
        ft.upload_cholesky(d["eps_occ"], d["eps_vir"], d["t1"], d["t2"], Loo, Lov, bad)
    with pytest.raises(CCSDTError):                     # energy before a successful upload
        ft.energy("fp64")


def _direct_pair(o, v, nq, seed, slabs, occ=None, vir=None):
    """The same Cholesky system uploaded whole and in the Cholesky-direct mode."""
    from exachem_gb300.ccsd_t import FusedTriples
    d, L = _cholesky_system(o, v, nq, seed)
    whole = FusedTriples(o, v, occ, vir, ts=24)
    whole.upload_cholesky(d["eps_occ"], d["eps_vir"], d["t1"], d["t2"], *L)
    direct = FusedTriples(o, v, occ, vir, ts=24)
    direct.upload_cholesky(d["eps_occ"], d["eps_vir"], d["t1"], d["t2"], *L, max_ovvv_slabs=slabs)
    return d, whole, direct


@pytest.mark.parametrize("slabs", [3, 5, 9])
def test_cholesky_direct_fp64_equals_whole(built, slabs):
    """(ia|bc) formed slab by slab into a cache of 3, 5 or o slabs gives the energies of the whole
    block bit for bit (the same GEMM per element), whatever the visiting order; small caches form
    slabs more than once."""
    from exachem_gb300.ccsd_t import all_triplets
    o, v = 9, 40
    d, whole, direct = _direct_pair(o, v, 23, 21, slabs)
    tri = all_triplets(o)
    w4, w5 = whole.triplet_energies(tri, "fp64")
    g4, g5 = direct.triplet_energies(tri, "fp64")
    assert np.array_equal(w5, g5) and np.array_equal(w4, g4)
    builds = direct.ovvv_slab_builds()
    assert builds == o if slabs >= o else builds > o
    a, b = whole.energy("fp64"), direct.energy("fp64")
    assert a["e_paren_T"] == b["e_paren_T"] and a["e_bracket_T"] == b["e_bracket_T"]


@pytest.mark.parametrize("slabs", [6, 12])
def test_cholesky_direct_split_equals_whole(built, slabs):
    """The persistent split path reading its (ia|bc) digit planes from the slab cache (slices formed
    per slab, TMA coordinates through the index -> slot table, batches of slabs / 3 triplets): with
    slabs formed in FP64 the whole block's energies bit for bit, at FP32 and float-float partial
    arrays; with slabs formed from digit planes of the vectors (the default) within 1e-9 per triplet
    (measured up to 1.4e-10, against the S = 2 truncation's ~1e-7); an FP64
    call on the same handle afterwards re-forms the slabs it reads in FP64 and is bit for bit the
    whole block's."""
    import ctypes
    from exachem_gb300.ccsd_t import all_triplets
    o, v = 10, 48
    d, whole, direct = _direct_pair(o, v, 30, 22, slabs)
    lib = direct.lib
    lib.ccsdt_debug_set_slab_build.argtypes = [ctypes.c_void_p, ctypes.c_int]
    tri = all_triplets(o)
    assert lib.ccsdt_debug_set_slab_build(direct.h, 0) == 0
    for S in (2, 3):
        w4, w5 = whole.triplet_energies(tri, "ozaki", slices=S)
        g4, g5 = direct.triplet_energies(tri, "ozaki", slices=S)
        assert np.array_equal(w5, g5) and np.array_equal(w4, g4), S
    assert direct.ovvv_slab_builds() > o if slabs < o else direct.ovvv_slab_builds() == o
    assert lib.ccsdt_debug_set_slab_build(direct.h, 1) == 0
    direct.upload_cholesky(d["eps_occ"], d["eps_vir"], d["t1"], d["t2"], *_cholesky_system(o, v, 30, 22)[1],
                           max_ovvv_slabs=slabs)
    for S in (2, 3):
        w4, w5 = whole.triplet_energies(tri, "ozaki", slices=S)
        g4, g5 = direct.triplet_energies(tri, "ozaki", slices=S)
        np.testing.assert_allclose(g5, w5, rtol=1e-9, atol=1e-12 * np.abs(w5).max())
        np.testing.assert_allclose(g4, w4, rtol=1e-9, atol=1e-12 * np.abs(w4).max())
    f4, f5 = whole.triplet_energies(tri, "fp64")
    h4, h5 = direct.triplet_energies(tri, "fp64")
    assert np.array_equal(f5, h5) and np.array_equal(f4, h4)
    # a repeated call reuses the slabs already formed (digit planes current)
    before = direct.ovvv_slab_builds()
    direct.triplet_energies(tri[:1], "ozaki", slices=3)
    assert direct.ovvv_slab_builds() - before <= 3


def test_cholesky_direct_limits(built):
    from exachem_gb300.ccsd_t import CCSDTError, FusedTriples
    o, v = sum(OCC), sum(VIR)
    d, L = _cholesky_system(o, v, 8, 23)
    ft = FusedTriples(o, v, OCC, VIR)
    with pytest.raises(CCSDTError):                  # fewer slots than one triplet's slabs
        ft.upload_cholesky(d["eps_occ"], d["eps_vir"], d["t1"], d["t2"], *L, max_ovvv_slabs=2)
    ft.upload_cholesky(d["eps_occ"], d["eps_vir"], d["t1"], d["t2"], *L, max_ovvv_slabs=4)
    with pytest.raises(CCSDTError):                  # the learned features read every slab
        ft.energy("learned", slices=5)
    with pytest.raises(CCSDTError):                  # the per-triplet split kernels read ovvv whole
        ft.energy("ozaki", slices=3, legacy_mma=1)
    r = ft.energy("ozaki", slices=3)          # slabs formed from digit planes of the vectors
    ft.upload_cholesky(d["eps_occ"], d["eps_vir"], d["t1"], d["t2"], *L)   # back to the whole block
    assert abs(ft.energy("ozaki", slices=3)["e_paren_T"] - r["e_paren_T"]) <= 1e-10 * abs(r["e_paren_T"])
