"""The open-shell path's host logic on the CPU: the library's own contraction plan
(ccsdt_debug_spin_orbital_plan - the spin blocks, their ranges and operand offsets that the GPU
launcher turns into GEMM jobs) is evaluated here with numpy, every operand row checked to lie
inside its array, and the energy summed over a < b < c the way so_energy_kernel sums it.  The
result must equal the spin-orbital oracle (1e-12), so the planning is proven without a GPU."""
import itertools

import numpy as np
import pytest

from exachem_gb300 import ccsd_t
from oracle.spin_orbital_oracle import energy_spin_orbital, open_shell_system, spin_orbital_inputs
from exachem_gb300.generator import generate


def _gemm(A, a0, a_stride, B, b0, b_hi, b_lo, nz, K, M, N):
    """- sum_kappa A[a0 + m a_stride + kappa] B[b0 + (n // nz) b_hi + (n % nz) b_lo + kappa]."""
    ra = a0 + np.arange(M) * a_stride
    n = np.arange(N)
    rb = b0 + (n // nz) * b_hi + (n % nz) * b_lo
    if K:
        assert ra.min() >= 0 and ra.max() + K <= A.size
        assert rb.min() >= 0 and rb.max() + K <= B.size
    k = np.arange(K)
    return -(A[ra[:, None] + k[None, :]] @ B[rb[:, None] + k[None, :]].T)


def _plan_energy(oa, ob, va, vb, eps_o, eps_v, t1, t2, v2ijab, v2ijka, v2iabc):
    O, V = oa + ob, va + vb
    tt = np.ascontiguousarray(t2.transpose(2, 3, 0, 1)).ravel()      # tt[j][k][a][e]
    vv = np.ascontiguousarray(v2iabc.transpose(0, 2, 3, 1)).ravel()  # vv[i][b][c][e]
    uu = np.ascontiguousarray(v2ijka.transpose(0, 1, 3, 2)).ravel()  # uu[j][k][a][m]
    t2f = t2.ravel()
    so = lambda p: int(p >= oa)
    sv = np.array([0] * va + [1] * vb)
    rng = lambda s: (va, V) if s else (0, va)
    e4 = e5 = 0.0
    for i, j, k in itertools.combinations(range(O), 3):
        si, sj, sk = so(i), so(j), so(k)
        (a0, a1), (b0, b1), (c0, c1) = rng(si), rng(sj), rng(sk)
        if (a1 - a0) * (b1 - b0) * (c1 - c0) == 0:
            continue
        of, blocks = ccsd_t.spin_orbital_plan(oa, ob, va, vb, i, j, k)
        X = []
        for B in blocks:
            M, N = B["nx"], B["ny"] * B["nz"]
            x = np.zeros((M, N))
            if B["has_d"]:
                x += _gemm(tt, B["d_a"], V, vv, B["d_b"], V * V, V, B["nz"], B["d_k"], M, N)
            if B["has_s"]:
                x += _gemm(uu, B["s_a"], O, t2f, B["s_b"], V * O * O, O * O, B["nz"], B["s_k"], M, N)
            X.append((x.reshape(M, B["ny"], B["nz"]), B))
        a, b, c = np.meshgrid(np.arange(a0, a1), np.arange(b0, b1), np.arange(c0, c1), indexing="ij")

        def read(bi, x, y, z):
            if bi < 0:
                return np.zeros(x.shape)
            arr, B = X[bi]
            assert B["x0"] <= x.min() and x.max() < B["x0"] + B["nx"]
            assert B["y0"] <= y.min() and y.max() < B["y0"] + B["ny"]
            assert B["z0"] <= z.min() and z.max() < B["z0"] + B["nz"]
            return arr[x - B["x0"], y - B["y0"], z - B["z0"]]
        w = np.zeros(a.shape)
        for p in range(3):
            x = read(of[p][0], a, b, c) - read(of[p][1], b, a, c) - read(of[p][2], c, b, a)
            w += -x if p else x
        vt = np.zeros(a.shape)
        for p, (ip, jp, kp) in enumerate([(i, j, k), (j, i, k), (k, j, i)]):
            for q, (x, y, z) in enumerate([(a, b, c), (b, a, c), (c, b, a)]):
                ok = (sv[x] == so(ip)) & (sv[y] + sv[z] == so(jp) + so(kp))
                g = np.where(ok, t1[x, ip] * v2ijab[jp, kp, y, z], 0.0)
                vt += g if (p == 0) == (q == 0) else -g
        keep = np.ones(a.shape, dtype=bool)
        if si == sj:
            keep &= a < b
        if sj == sk:
            keep &= b < c
        d = eps_o[i] + eps_o[j] + eps_o[k] - eps_v[a] - eps_v[b] - eps_v[c]
        e4 += np.sum(np.where(keep, w * w / d, 0.0))
        e5 += np.sum(np.where(keep, (w + vt) * w / d, 0.0))
    return e4, e5


@pytest.mark.parametrize("oa,ob,va,vb,seed", [(3, 2, 5, 6, 5), (4, 3, 6, 7, 6), (5, 1, 3, 7, 8), (1, 3, 4, 3, 9),
                                              (3, 0, 4, 0, 1), (0, 3, 0, 4, 2), (3, 2, 0, 5, 3)])
def test_open_shell_plan_reproduces_the_oracle(built, oa, ob, va, vb, seed):
    arrs = open_shell_system(oa, ob, va, vb, 6, seed)
    e4, e5 = energy_spin_orbital(*arrs)
    g4, g5 = _plan_energy(oa, ob, va, vb, *arrs)
    assert g4 == pytest.approx(e4, rel=1e-12, abs=1e-300) and g5 == pytest.approx(e5, rel=1e-12, abs=1e-300)


def test_closed_shell_plan_reproduces_the_closed_shell_oracle(built):
    import oracle
    d = generate(3, 5, 2)
    e4, e5 = oracle.energy(d)
    g4, g5 = _plan_energy(3, 3, 5, 5, *spin_orbital_inputs(d))
    assert g4 == pytest.approx(e4, rel=1e-12) and g5 == pytest.approx(e5, rel=1e-12)


def test_plan_block_counts_follow_the_spin_cases(built):
    """Distinct nonzero blocks: aaa / bbb one per permutation; aab two per permutation less one
    (permutation kji at (c; b a): x is beta while j' and k' are alpha, and i' is beta while y and z
    are alpha, so neither term survives); abb three per permutation less one."""
    counts = {case: len(ccsd_t.spin_orbital_plan(3, 3, 4, 4, *tri)[1])
              for case, tri in {"aaa": (0, 1, 2), "aab": (0, 1, 3), "abb": (0, 3, 4), "bbb": (3, 4, 5)}.items()}
    assert counts == {"aaa": 3, "aab": 5, "abb": 8, "bbb": 3}


def test_plan_rejects_bad_triplets(built):
    for tri in [(1, 0, 2), (0, 0, 1), (0, 1, 6)]:
        with pytest.raises(ccsd_t.CCSDTError):
            ccsd_t.spin_orbital_plan(3, 3, 4, 4, *tri)


@pytest.mark.parametrize("oa,ob,va,vb", [(3, 2, 5, 6), (4, 4, 7, 7), (5, 1, 3, 7), (3, 0, 4, 0)])
def test_bench_flop_count_is_the_planned_work(built, oa, ob, va, vb):
    """The open-shell roofline numerator (bench.spin_orbital_flops) equals 2 x the multiply-adds
    of the GEMM blocks the library plans, summed over every triplet."""
    import bench
    total = 0
    O = oa + ob
    for tri in itertools.combinations(range(O), 3):
        s = [int(p >= oa) for p in tri]
        if min((vb if x else va) for x in s) == 0:
            continue
        for B in ccsd_t.spin_orbital_plan(oa, ob, va, vb, *tri)[1]:
            total += 2 * B["nx"] * B["ny"] * B["nz"] * (B["has_d"] * B["d_k"] + B["has_s"] * B["s_k"])
    assert bench.spin_orbital_flops(oa, ob, va, vb) == total


def test_plan_reproduces_the_reference_open_shell_golden(built):
    """The library's plan, evaluated here, against ExaChem's own CPU (T) run unrestricted on the
    golden systems (tests/golden/open_shell_energies.json, up to 14 occupied and 84 virtual spin
    orbitals): the planning the GPU launches is pinned to the reference beyond the dense oracle."""
    import json
    from conftest import ROOT
    cases = json.loads((ROOT / "tests" / "golden" / "open_shell_energies.json").read_text())["cases"]
    for c in cases:
        arrs = open_shell_system(c["oa"], c["ob"], c["va"], c["vb"], c["nq"], c["seed"], exact=True)
        g4, g5 = _plan_energy(c["oa"], c["ob"], c["va"], c["vb"], *arrs)
        assert g4 == pytest.approx(c["e_bracket_T"], rel=1e-12) and g5 == pytest.approx(c["e_paren_T"], rel=1e-12), \
            c["name"]


def test_bench_launch_count(built):
    """3 permutes + per triplet ceil(blocks / 3) GEMM launches + 1 energy launch: at oa=ob=3,
    va=vb=4 one aaa and one bbb triplet (3 blocks: 2 launches), nine aab (5 blocks: 3) and nine abb
    (8 blocks: 4)."""
    import bench
    assert bench.spin_orbital_launches(3, 3, 4, 4) == 3 + 2 * 2 + 9 * 3 + 9 * 4


def test_open_shell_entry_rejects_bad_arguments_without_gpu(built):
    """ccsdt_energy_spin_orbital checks its arguments before any CUDA call: negative or oversized
    orbital counts, a null output, a shard outside [0, count) and null arrays are CCSDT_E_INVALID;
    fewer than three occupied or virtual spin orbitals give zero energies."""
    import ctypes
    lib = ccsd_t.load_library()
    e = (ctypes.c_double * 2)(1.0, 1.0)
    ep = ctypes.cast(e, ctypes.POINTER(ctypes.c_double))
    x = np.zeros(1 << 16)
    p = [x.ctypes.data] * 7
    call = lambda oa, ob, va, vb, arrs, si, sc, out: lib.ccsdt_energy_spin_orbital(oa, ob, va, vb, *arrs, 0, si, sc,
                                                                                    out, None)
    assert call(-1, 2, 3, 3, p, 0, 1, ep) == 1
    assert call(5000, 2, 3, 3, p, 0, 1, ep) == 1
    assert call(2, 2, 3, 3, p, 0, 1, None) == 1
    assert call(2, 2, 3, 3, p, 3, 3, ep) == 1
    assert call(2, 2, 3, 3, p, -1, 2, ep) == 1
    assert call(2, 2, 3, 3, [None] * 7, 0, 1, ep) == 1
    e[0] = e[1] = 1.0
    assert call(1, 1, 3, 3, [None] * 7, 0, 1, ep) == 0 and (e[0], e[1]) == (0.0, 0.0)
    e[0] = e[1] = 1.0
    assert call(2, 2, 1, 1, [None] * 7, 0, 1, ep) == 0 and (e[0], e[1]) == (0.0, 0.0)
