"""Split-precision (Ozaki) path on the GPU: the tcgen05 kernel against the mma.sync slice
kernel (same exact level sums), INT8 against BF16 digits, and the error against the FP64
path as the slice count grows.

Tolerances are relative to |E(T)| (the synthetic energies are 1e-1 .. 1e11 Eh, so absolute
Eh bounds do not transfer): digits carry 7 bits each, so S slices bound the contraction
error near 2^(-7 S) of the operand scale; the observed |dE/E| is stated per S below.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# |dE(T)/E(T)| bounds vs FP64 per slice count, with headroom over what GB300 measured
# (o=12, v=70: S=2 9.6e-7, S=3 9.2e-9, S=4 5.5e-11, S=5 3.5e-12)
BOUND = {2: 5e-6, 3: 5e-8, 4: 5e-10, 5: 5e-11}


def _ft(o, v, seed, **kw):
    from exachem_gb300.ccsd_t import FusedTriples
    from exachem_gb300.generator import generate
    d = generate(o, v, seed, **kw)
    ft = FusedTriples(o, v, ts=40)
    ft.upload_dict(d)
    return ft


@pytest.mark.parametrize("o,v,seed", [(4, 16, 1), (6, 40, 0), (5, 130, 2)])
def test_tcgen05_equals_mma_sync_levels(built, o, v, seed):
    ft = _ft(o, v, seed)
    for S in (1, 2, 3, 4, 5):
        tc = ft.energy("ozaki", slices=S, p_storage="ff")   # the other kernels keep float-float partial arrays
        leg = ft.energy("ozaki", slices=S, legacy_mma=1)
        assert tc["e_paren_T"] == pytest.approx(leg["e_paren_T"], rel=1e-13, abs=0)
        assert tc["e_bracket_T"] == pytest.approx(leg["e_bracket_T"], rel=1e-13, abs=0)


def test_int8_digits_equal_bf16_digits(built):
    ft = _ft(6, 40, 3)
    for S in (2, 4):
        a = ft.energy("ozaki", slices=S, legacy_mma=1)["e_paren_T"]
        b = ft.energy("ozaki", slices=S, slice_kind="int8")["e_paren_T"]
        assert a == pytest.approx(b, rel=1e-13, abs=0)


def test_split_error_shrinks_with_slices(built):
    ft = _ft(12, 70, 21)
    ref = ft.energy("fp64")["e_paren_T"]
    errs = {}
    for S in (2, 3, 4, 5):
        errs[S] = abs(ft.energy("ozaki", slices=S)["e_paren_T"] - ref) / abs(ref)
        assert errs[S] <= BOUND[S], (S, errs)
    assert errs[3] < errs[2] and errs[4] < errs[3]


@pytest.mark.parametrize("kernel", [0, 2])   # 0 persistent queue, 2 one CTA per tile
def test_split_triplet_w_close_to_fp64(built, kernel):
    ft = _ft(6, 40, 0)
    for (i, j, k) in [(0, 1, 2), (1, 3, 3), (0, 0, 5)]:
        wf = ft.triplet_w(i, j, k, "fp64")
        ws = ft.triplet_w(i, j, k, "ozaki", slices=5, legacy_mma=kernel)
        assert np.abs(ws - wf).max() <= 1e-9 * np.abs(wf).max()


def test_split_per_triplet_sum_equals_total(built):
    from exachem_gb300.ccsd_t import all_triplets
    ft = _ft(7, 33, 4)
    tot = ft.energy("ozaki", slices=3)
    e4, e5 = ft.triplet_energies(all_triplets(7), "ozaki", slices=3)
    assert e5.sum() == pytest.approx(tot["e_paren_T"], rel=1e-13)


@pytest.mark.parametrize("o,v,seed", [(6, 40, 0), (5, 130, 2), (9, 70, 5)])
def test_persistent_queue_equals_per_triplet_tcgen05(built, o, v, seed):
    ft = _ft(o, v, seed)
    for S in (2, 3, 4):
        per = ft.energy("ozaki", slices=S, legacy_mma=2)
        pers = ft.energy("ozaki", slices=S, p_storage="ff")
        graph = ft.energy("ozaki", slices=S, use_graph=1, p_storage="ff")
        assert pers["e_paren_T"] == pytest.approx(per["e_paren_T"], rel=1e-13, abs=0)
        assert graph["e_paren_T"] == pers["e_paren_T"]
        # the default storage (FP32 partial arrays at S <= 3) through the graph as well
        assert ft.energy("ozaki", slices=S, use_graph=1)["e_paren_T"] == ft.energy("ozaki", slices=S)["e_paren_T"]


def test_persistent_batches_cover_every_triplet(built):
    """more triplets than one batch, a ragged last batch, results in input order"""
    from exachem_gb300.ccsd_t import all_triplets
    ft = _ft(8, 33, 6)
    tri = all_triplets(8)
    e4, e5 = ft.triplet_energies(tri, "ozaki", slices=3, p_storage="ff")   # as the per-triplet kernel
    r4, r5 = ft.triplet_energies(tri, "ozaki", slices=3, legacy_mma=2)
    np.testing.assert_allclose(e5, r5, rtol=1e-12, atol=1e-12 * np.abs(r5).max())


@pytest.mark.parametrize("o,v,seed", [(3, 9, 31), (2, 17, 32), (4, 65, 33), (1, 30, 34), (5, 129, 35)])
def test_split_edge_shapes(built, o, v, seed):
    """Shapes at the edges of the tiling: v below one 8-wide energy block, below one N tile and
    one 128-row tile, one past a multiple of 64 and of 128, and o = 1 (the only triplet is
    i = j = k, which contributes exactly zero).  Split precision (S = 3 and 5) against the plain
    FP64 path, both through the C ABI.  S = 5 is held to 1e-9: the singles part of V is formed
    from FP32 copies of (ia|jb) and t1, a relative floor of ~6e-8 x the singles' share of E(T),
    which averages out over large systems but not over the two triplets of o = 3."""
    ft = _ft(o, v, seed)
    ref = ft.energy("fp64")
    for S, tol in ((3, 1e-7), (5, 1e-9)):
        r = ft.energy("ozaki", slices=S)
        for key in ("e_bracket_T", "e_paren_T"):
            if ref[key] == 0.0:
                assert r[key] == 0.0
            else:
                assert abs(r[key] - ref[key]) <= tol * abs(ref[key]), (S, key, r[key], ref[key])


@pytest.mark.parametrize("o,v,seed,tri", [(4, 320, 41, [(0, 1, 3), (1, 1, 2)]), (3, 512, 42, [(0, 1, 2), (0, 2, 2)])])
def test_split_large_v_against_oracle(built, o, v, seed, tri):
    """Virtual extents of the headline range, up to the 512-wide contraction window the exact
    level sums rely on (K = v for the d-sum terms): the persistent tcgen05 path at S = 3 and 4
    and the FP64 path against the oracle's C restatement on the same triplets.  Inputs are built
    on the GPU (bit-identical to the host generator); the oracle reads host copies of the slabs
    the triplets need."""
    import torch
    import oracle
    from exachem_gb300.ccsd_t import FusedTriples
    from exachem_gb300.generator import generate_device
    dev = generate_device(o, v, seed, device="cuda")
    tri = np.array(tri, dtype=np.int32)
    need = sorted(set(int(x) for x in tri.ravel()))
    host = {k: dev[k].cpu().numpy() for k in ("eps_occ", "eps_vir", "t1", "t2", "oovv", "ooov")}
    host.update(o=o, v=v, ovvv_slabs={i: dev["ovvv"][i].cpu().numpy() for i in need})
    w4, w5 = oracle.triplets_slabs(host, tri)
    ft = FusedTriples(o, v, ts=40)
    ft.upload_dict(dev)
    del dev
    torch.cuda.empty_cache()
    f4, f5 = ft.triplet_energies(tri, "fp64")
    np.testing.assert_allclose(f5, w5, rtol=1e-11)
    np.testing.assert_allclose(f4, w4, rtol=1e-11)
    for S, tol in ((2, 2e-5), (3, 1e-6), (4, 1e-8)):
        s4, s5 = ft.triplet_energies(tri, "ozaki", slices=S)
        np.testing.assert_allclose(s5, w5, rtol=tol)
        np.testing.assert_allclose(s4, w4, rtol=tol)
    ft.close()


@pytest.mark.parametrize("o,v,seed", [(12, 70, 8), (4, 320, 9)])
def test_float_float_energy_stage_error(built, o, v, seed):
    """The split path's energy stage on its own: the FP64 contractions' P arrays, rounded to
    float-float, through the tiled float-float energy (whose singles use FP32 copies of (ia|jb) and
    t1), against the FP64 energy of the same arrays.  This isolates the error of the energy stage
    (float-float W sums, 1/D and accumulation, FP32 singles) from the digit truncation."""
    ft = _ft(o, v, seed)
    ref = ft.energy("fp64")
    got = ft.energy("ozaki", slices=1, legacy_mma=3)
    for key in ("e_bracket_T", "e_paren_T"):
        assert abs(got[key] - ref[key]) <= 2e-12 * abs(ref[key]), (key, got[key], ref[key])


@pytest.mark.parametrize("o,v,seed", [(12, 70, 8), (4, 320, 9)])
def test_fp32_energy_stage_error(built, o, v, seed):
    """The FP32 form of the energy stage on its own: the FP64 contractions' P arrays rounded to
    FP32 through the FP32 energy, against the FP64 energy of the same arrays.  Its error must sit
    far below the two-plane contraction error it is used with (~1e-7 per triplet)."""
    ft = _ft(o, v, seed)
    ref = ft.energy("fp64")
    got = ft.energy("ozaki", slices=1, legacy_mma=3, p_storage="f32")
    for key in ("e_bracket_T", "e_paren_T"):
        assert abs(got[key] - ref[key]) <= 1e-8 * abs(ref[key]), (key, got[key], ref[key])


@pytest.mark.parametrize("o,v,seed", [(6, 40, 0), (5, 130, 2), (4, 320, 9)])
def test_fp32_partial_arrays(built, o, v, seed):
    """Partial arrays stored in FP32 (the default at one to three digit planes) against
    float-float storage of the same contraction: the difference is the FP32 rounding, far below
    the two-plane error; at S = 2 both stay within the split path's bound against FP64; the
    debugging aid reads the FP32 arrays back."""
    ft = _ft(o, v, seed)
    ref = ft.energy("fp64")["e_paren_T"]
    for S in (1, 2, 3):
        a = ft.energy("ozaki", slices=S, p_storage="f32")
        b = ft.energy("ozaki", slices=S, p_storage="ff")
        for key in ("e_bracket_T", "e_paren_T"):
            assert abs(a[key] - b[key]) <= 1e-8 * abs(b[key]), (S, key, a[key], b[key])
    auto = ft.energy("ozaki", slices=2)["e_paren_T"]
    assert auto == ft.energy("ozaki", slices=2, p_storage="f32")["e_paren_T"]
    assert abs(auto - ref) <= BOUND[2] * abs(ref)
    if v <= 130:
        wf = ft.triplet_w(0, 1, 2, "ozaki", slices=2, p_storage="ff")
        ws = ft.triplet_w(0, 1, 2, "ozaki", slices=2)
        assert np.abs(ws - wf).max() <= 1e-6 * np.abs(wf).max()
        assert np.abs(ws - wf).max() > 0      # the default really stored FP32


@pytest.mark.parametrize("o,v,seed", [(6, 40, 0), (5, 132, 2), (4, 320, 9), (3, 130, 4)])
def test_tma_energy_equals_pass_by_pass(built, o, v, seed):
    """The energy kernel that stages the partial arrays by TMA against the pass-by-pass kernel, on
    the same contraction: FP32 and float-float partial arrays, a ragged last block (v % 8 != 0)
    and, at v = 130, a row pitch that FP32 TMA cannot take (float-float can).  The W values are
    summed in the same order, so only the per-thread accumulation order differs."""
    import ctypes
    ft = _ft(o, v, seed)
    lib = ft.lib
    lib.ccsdt_debug_set_energy_kernel.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.ccsdt_debug_set_energy_kernel.restype = ctypes.c_int
    tri = np.array([(0, 1, 2), (0, 0, 2), (1, 2, 2), (0, 1, o - 1)], dtype=np.int32)
    for S, store in ((2, "f32"), (3, "ff"), (2, "ff")):
        a4, a5 = ft.triplet_energies(tri, "ozaki", slices=S, p_storage=store)
        for kind in (1, 2):          # pass-by-pass; TMA with one box stage
            assert lib.ccsdt_debug_set_energy_kernel(ft.h, kind) == 0
            b4, b5 = ft.triplet_energies(tri, "ozaki", slices=S, p_storage=store)
            assert lib.ccsdt_debug_set_energy_kernel(ft.h, 0) == 0
            np.testing.assert_allclose(a5, b5, rtol=1e-12, atol=1e-13 * np.abs(b5).max())
            np.testing.assert_allclose(a4, b4, rtol=1e-12, atol=1e-13 * np.abs(b4).max())
    assert lib.ccsdt_debug_set_energy_kernel(ft.h, 3) != 0


@pytest.mark.parametrize("o,v,seed", [(3, 10, 31), (6, 40, 0), (4, 320, 9)])
def test_fp64_partial_arrays(built, o, v, seed):
    """p_storage = f64: the exactly folded levels widened to FP64 partial arrays and the energy in
    FP64 (W sums, FP64 singles, division, compensated sums).  At six planes the result sits at the
    FP64 path's to 1e-12 even on a tiny system, where the float-float energy's FP32 singles leave a
    floor; at S = 3 it agrees with the float-float storage to the latter's own precision."""
    from exachem_gb300.ccsd_t import CCSDTError
    ft = _ft(o, v, seed)
    ref = ft.energy("fp64")
    r6 = ft.energy("ozaki", slices=6, p_storage="f64")
    for key in ("e_bracket_T", "e_paren_T"):
        assert abs(r6[key] - ref[key]) <= 1e-12 * abs(ref[key]), (key, r6[key], ref[key])
    a = ft.energy("ozaki", slices=3, p_storage="f64")
    b = ft.energy("ozaki", slices=3, p_storage="ff")
    assert abs(a["e_paren_T"] - b["e_paren_T"]) <= 1e-10 * abs(b["e_paren_T"])
    if v <= 40:
        wf = ft.triplet_w(0, 1, 2, "fp64")
        ws = ft.triplet_w(0, 1, 2, "ozaki", slices=6, p_storage="f64")
        assert np.abs(ws - wf).max() <= 1e-12 * np.abs(wf).max()
    odd = _ft(3, 9, 1)
    with pytest.raises(CCSDTError):                 # the energy reads FP64 boxes through TMA
        odd.energy("ozaki", slices=3, p_storage="f64")


def _set_window(ft, k):
    import ctypes
    lib = ft.lib
    lib.ccsdt_debug_set_window.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.ccsdt_debug_set_window.restype = ctypes.c_int
    assert lib.ccsdt_debug_set_window(ft.h, k) == 0


@pytest.mark.parametrize("o,v,seed", [(6, 40, 13), (5, 130, 14)])
def test_six_to_eight_slices_on_tcgen05(built, o, v, seed):
    """S = 6, 7, 8 run on the persistent tcgen05 kernel (32-column tiles, K chunks of 32) and agree
    with the mma.sync slice kernel; the float-float fold is no longer exact above S = 4, so the
    comparison is at 1e-12 relative, and both sit at the FP64 result to float-float precision."""
    ft = _ft(o, v, seed)
    ref = ft.energy("fp64")
    for S in (6, 7, 8):
        tc = ft.energy("ozaki", slices=S)
        leg = ft.energy("ozaki", slices=S, legacy_mma=1)
        assert tc["e_paren_T"] == pytest.approx(leg["e_paren_T"], rel=1e-12, abs=0), S
        assert abs(tc["e_paren_T"] - ref["e_paren_T"]) <= 1e-11 * abs(ref["e_paren_T"]), (S, tc, ref)


@pytest.mark.parametrize("o,v,seed", [(7, 96, 15), (5, 200, 16)])
def test_contraction_windows(built, o, v, seed):
    """Contractions accumulated window by window (here forced to windows of 64 and 32 along K, so
    the d-sum terms take several and the l-sum terms one or two) give the single-window energies:
    each window's level sums are exact, only the float-float folds of the partial sums differ."""
    ft = _ft(o, v, seed)
    # float-float partial arrays: only the folds of the partial sums differ (1e-12); FP32 ones
    # (the S = 3 default) round each window's fold to FP32 (1e-9)
    for S, store, rel in ((3, "ff", 1e-12), (5, "auto", 1e-12), (3, "auto", 1e-9)):
        one = ft.energy("ozaki", slices=S, p_storage=store)
        for k in (64, 32):
            _set_window(ft, k)
            win = ft.energy("ozaki", slices=S, p_storage=store)
            _set_window(ft, 0)
            for key in ("e_bracket_T", "e_paren_T"):
                assert win[key] == pytest.approx(one[key], rel=rel, abs=0), (S, store, k, key)


def test_long_contraction_beyond_the_exact_window(built):
    """v = 800: the d-sum contractions (K = 800) exceed the exact window of S = 3 (768) and of
    S = 5 (576), so the persistent kernel folds two windows per term; one triplet against the FP64
    path (v = 800 lies beyond the per-triplet tcgen05 kernel's 512)."""
    import torch
    from exachem_gb300.ccsd_t import FusedTriples
    from exachem_gb300.generator import generate_device
    o, v = 2, 800
    dev = generate_device(o, v, 17, device="cuda")
    ft = FusedTriples(o, v, ts=40)
    ft.upload_dict(dev)
    del dev
    torch.cuda.empty_cache()
    tri = np.array([(0, 0, 1), (0, 1, 1)], dtype=np.int32)
    f4, f5 = ft.triplet_energies(tri, "fp64")
    for S, tol in ((3, 1e-6), (5, 1e-9)):
        s4, s5 = ft.triplet_energies(tri, "ozaki", slices=S)
        np.testing.assert_allclose(s5, f5, rtol=tol)
        np.testing.assert_allclose(s4, f4, rtol=tol)
    ft.close()
