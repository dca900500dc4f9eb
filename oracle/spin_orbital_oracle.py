"""Spin-orbital (T) oracle - TEST INFRASTRUCTURE ONLY (no product code calls it).

The general form of the perturbative triples over spin orbitals, the quantities ExaChem's (T)
driver sums tile by tile for both the restricted and the open-shell case
(exachem/cc/ccsd_t/ccsd_t_all_fused_cpu.hpp: the 27 contraction families of the triples block and
its energy loop; ccsd_t_fused_driver.hpp: is_restricted selects the spin filter and factor only):

    W_ijk^abc = P(i/jk) P(a/bc) [ - sum_e t_jk^ae <ie||bc> - sum_m t_im^bc <jk||ma> ]
    V_ijk^abc = P(i/jk) P(a/bc) t_i^a <jk||bc>
    E[T] = 1/36 sum W W / D,   E(T) = 1/36 sum (W + V) W / D,   D = e_i + e_j + e_k - e_a - e_b - e_c

with P(i/jk) f(ijk) = f(ijk) - f(jik) - f(kji).  Inputs in the layouts of ExaChem's spin-orbital
tensors: t1[a][i], t2[a][b][i][j] (= t_ij^ab), v2ijab[i][j][a][b] = <ij||ab>,
v2ijka[i][j][k][a] = <ij||ka>, v2iabc[i][a][b][c] = <ia||bc> (cholesky/v2tensors.cpp:67-86).
Dense numpy over all (i, j, k, a, b, c): small systems only.

spin_orbital_inputs() restates, for a closed-shell system, the spin blocks ExaChem builds
(T2: cd_ccsd_cs_ann.cpp:26-31 and :949-973; V2: v2tensors.cpp:67-86 from spin {1,1} Cholesky
vectors) - the same conventions as oracle/spin_orbital.hpp.  With them the spin-orbital energies
equal the closed-shell ones, which pins this oracle to the reference's goldens through the
closed-shell oracle.  An open-shell system is given directly in the spin-orbital layouts.
"""
from __future__ import annotations

import numpy as np


def _p3(x: np.ndarray, a0: int) -> np.ndarray:
    """P(p/qr) over axes (a0, a0 + 1, a0 + 2): x - x[p<->q] - x[p<->r]."""
    return x - np.swapaxes(x, a0, a0 + 1) - np.swapaxes(x, a0, a0 + 2)


def energy_spin_orbital(eps_o, eps_v, t1, t2, v2ijab, v2ijka, v2iabc) -> tuple[float, float]:
    """(E[T], E(T)) over spin orbitals.  eps_o[O], eps_v[V] orbital energies; t1[V][O];
    t2[V][V][O][O]; v2ijab[O][O][V][V]; v2ijka[O][O][O][V]; v2iabc[O][V][V][V]."""
    # connected part before the permutations, X[i,j,k,a,b,c]
    x = -np.einsum("aejk,iebc->ijkabc", t2, v2iabc, optimize=True)
    x -= np.einsum("bcim,jkma->ijkabc", t2, v2ijka, optimize=True)
    w = _p3(_p3(x, 0), 3)
    y = np.einsum("ai,jkbc->ijkabc", t1, v2ijab, optimize=True)
    vv = _p3(_p3(y, 0), 3)
    eo, ev = np.asarray(eps_o), np.asarray(eps_v)
    d = (eo[:, None, None, None, None, None] + eo[None, :, None, None, None, None] + eo[None, None, :, None, None, None]
         - ev[None, None, None, :, None, None] - ev[None, None, None, None, :, None] - ev[None, None, None, None, None, :])
    e4 = float(np.sum(w * w / d) / 36.0)
    e5 = float(np.sum((w + vv) * w / d) / 36.0)
    return e4, e5


def spin_orbital_inputs(d: dict):
    """Spin-orbital tensors of a closed-shell system given by the spatial arrays of ccsdt.h.
    Spin orbital p < n is alpha (spatial p), p >= n beta (spatial p - n)."""
    o, v = int(d["o"]), int(d["v"])
    O, V = 2 * o, 2 * v
    so = lambda p, n: (p % n, p // n)   # (spatial, spin)
    t1s, t2s = d["t1"], d["t2"]          # t1[i][a], t2[i][j][a][b]
    ovov = lambda i, a, j, b: d["oovv"][i, j, a, b]   # (ia|jb)
    oo_ov = lambda i, j, k, a: d["ooov"][i, j, k, a]  # (ij|ka)
    ov_vv = lambda i, a, b, c: d["ovvv"][i, a, b, c]  # (ia|bc)
    t1 = np.zeros((V, O))
    t2 = np.zeros((V, V, O, O))
    v2ijab = np.zeros((O, O, V, V))
    v2ijka = np.zeros((O, O, O, V))
    v2iabc = np.zeros((O, V, V, V))
    for a in range(V):
        A, sa = so(a, v)
        for i in range(O):
            I, si = so(i, o)
            if sa == si:
                t1[a, i] = t1s[I, A]
    for a in range(V):
        A, sa = so(a, v)
        for b in range(V):
            B, sb = so(b, v)
            for i in range(O):
                I, si = so(i, o)
                for j in range(O):
                    J, sj = so(j, o)
                    if sa == sb == si == sj:
                        t2[a, b, i, j] = t2s[I, J, A, B] - t2s[I, J, B, A]
                    elif sa == si and sb == sj and sa != sb:
                        t2[a, b, i, j] = t2s[I, J, A, B]
                    elif sa == sj and sb == si and sa != sb:
                        t2[a, b, i, j] = -t2s[J, I, A, B]
    for i in range(O):
        I, si = so(i, o)
        for j in range(O):
            J, sj = so(j, o)
            for a in range(V):
                A, sa = so(a, v)
                for b in range(V):
                    B, sb = so(b, v)
                    val = 0.0
                    if si == sa and sj == sb:
                        val += ovov(I, A, J, B)
                    if si == sb and sj == sa:
                        val -= ovov(I, B, J, A)
                    v2ijab[i, j, a, b] = val
            for k in range(O):
                K, sk = so(k, o)
                for a in range(V):
                    A, sa = so(a, v)
                    val = 0.0
                    if si == sk and sj == sa:
                        val += oo_ov(I, K, J, A)
                    if sj == sk and si == sa:
                        val -= oo_ov(J, K, I, A)
                    v2ijka[i, j, k, a] = val
    for i in range(O):
        I, si = so(i, o)
        for a in range(V):
            A, sa = so(a, v)
            for b in range(V):
                B, sb = so(b, v)
                for c in range(V):
                    C, sc = so(c, v)
                    val = 0.0
                    if si == sb and sa == sc:
                        val += ov_vv(I, B, A, C)
                    if si == sc and sa == sb:
                        val -= ov_vv(I, C, A, B)
                    v2iabc[i, a, b, c] = val
    eps_o = np.concatenate([d["eps_occ"], d["eps_occ"]])
    eps_v = np.concatenate([d["eps_vir"], d["eps_vir"]])
    return eps_o, eps_v, t1, t2, v2ijab, v2ijka, v2iabc


def open_shell_system(oa: int, ob: int, va: int, vb: int, nq: int, seed: int, exact: bool = False):
    """A synthetic open-shell (UHF-like) system over spin orbitals: separate alpha and beta orbital
    sets (oa / ob occupied, va / vb virtual), integrals from spin-blocked Cholesky vectors
    (L_alpha over the oa + va alpha orbitals, L_beta over the ob + vb beta ones, zero between spins),
    antisymmetrised as v2tensors.cpp:67-86 does, spin-conserving antisymmetric T2 and T1.
    Spin-orbital order: occupied alpha then beta, virtual alpha then beta (ExaChem's MO order).
    exact: the vectors are rounded to multiples of 2^-12 and t1 / t2 to multiples of 2^-20, so that
    every integral and amplitude is exact in FP64 and the arrays are the same bits on any machine.
    Returns (eps_o, eps_v, t1, t2, v2ijab, v2ijka, v2iabc)."""
    rng = np.random.default_rng(seed)
    O, V = oa + ob, va + vb
    spin_o = np.array([0] * oa + [1] * ob)
    spin_v = np.array([0] * va + [1] * vb)
    grid = (lambda x, b: np.round(x * 2.0 ** b) / 2.0 ** b) if exact else (lambda x, b: x)
    La = rng.normal(0.0, 0.05, size=(oa + va, oa + va, nq))
    Lb = rng.normal(0.0, 0.05, size=(ob + vb, ob + vb, nq))
    La = grid(0.5 * (La + La.transpose(1, 0, 2)), 12)
    Lb = grid(0.5 * (Lb + Lb.transpose(1, 0, 2)), 12)
    # spin-orbital vectors over occupied then virtual spin orbitals: index -> (spin, orbital of that spin)
    n = O + V
    orb = [(0, p) for p in range(oa)] + [(1, p) for p in range(ob)] + \
          [(0, oa + a) for a in range(va)] + [(1, ob + a) for a in range(vb)]
    L = np.zeros((n, n, nq))
    for p, (sp, ip) in enumerate(orb):
        for q, (sq, iq) in enumerate(orb):
            if sp == sq:
                L[p, q] = (La if sp == 0 else Lb)[ip, iq]
    g = np.einsum("prQ,qsQ->pqrs", L, L, optimize=True)          # <pq|rs> = (pr|qs)
    asym = g - g.transpose(0, 1, 3, 2)                            # <pq||rs>
    o_, v_ = slice(0, O), slice(O, n)
    v2ijab = np.ascontiguousarray(asym[o_, o_, v_, v_])
    v2ijka = np.ascontiguousarray(asym[o_, o_, o_, v_])
    v2iabc = np.ascontiguousarray(asym[o_, v_, v_, v_])
    same = spin_v[:, None] == spin_o[None, :]
    t1 = grid(np.where(same, rng.normal(0.0, 0.02, size=(V, O)), 0.0), 20)
    r = grid(rng.normal(0.0, 0.05, size=(V, V, O, O)), 20)
    sa, sb = spin_v[:, None, None, None], spin_v[None, :, None, None]
    si, sj = spin_o[None, None, :, None], spin_o[None, None, None, :]
    mask = ((sa == si) & (sb == sj)) | ((sa == sj) & (sb == si))
    r = np.where(mask, r, 0.0)
    u = r - r.transpose(1, 0, 2, 3)              # two steps: each difference negates exactly
    t2 = u - u.transpose(0, 1, 3, 2)
    eps_o = -1.0 - rng.random(O)
    eps_v = 0.3 + rng.random(V)
    return eps_o, eps_v, t1, t2, v2ijab, v2ijka, v2iabc


def golden_checksums(arrs) -> dict:
    """Exact sums of the t2 and v2iabc of an open_shell_system(exact=True) (every term and partial
    sum is representable in FP64, so any summation order gives the same bits)."""
    return {"t2": float(np.sum(arrs[3])), "v2iabc": float(np.sum(arrs[6]))}


def spin_orbital_inputs_vec(d: dict):
    """spin_orbital_inputs() with array operations (same result, element for element), for sizes
    where the loops are too slow."""
    o, v = int(d["o"]), int(d["v"])
    so, sv = np.arange(2 * o) // o, np.arange(2 * v) // v     # spins
    po, pv = np.arange(2 * o) % o, np.arange(2 * v) % v       # spatial indices
    t1s, t2s, ovov, ooov, ovvv = d["t1"], d["t2"], d["oovv"], d["ooov"], d["ovvv"]
    t1 = np.where(sv[:, None] == so[None, :], t1s.T[pv[:, None], po[None, :]], 0.0)
    A, B, I, J = np.ix_(pv, pv, po, po)
    sa, sb, si, sj = np.ix_(sv, sv, so, so)
    same = (sa == sb) & (sb == si) & (si == sj)
    t2 = np.where(same, t2s[I, J, A, B] - t2s[I, J, B, A], 0.0)
    t2 = np.where((sa == si) & (sb == sj) & (sa != sb), t2s[I, J, A, B], t2)
    t2 = np.where((sa == sj) & (sb == si) & (sa != sb), -t2s[J, I, A, B], t2)
    I, J, A, B = np.ix_(po, po, pv, pv)
    si, sj, sa, sb = np.ix_(so, so, sv, sv)
    v2ijab = (np.where((si == sa) & (sj == sb), ovov[I, J, A, B], 0.0)
              - np.where((si == sb) & (sj == sa), ovov[I, J, B, A], 0.0))
    I, J, K, A = np.ix_(po, po, po, pv)
    si, sj, sk, sa = np.ix_(so, so, so, sv)
    v2ijka = (np.where((si == sk) & (sj == sa), ooov[I, K, J, A], 0.0)
              - np.where((sj == sk) & (si == sa), ooov[J, K, I, A], 0.0))
    I, A, B, C = np.ix_(po, pv, pv, pv)
    si, sa, sb, sc = np.ix_(so, sv, sv, sv)
    v2iabc = (np.where((si == sb) & (sa == sc), ovvv[I, B, A, C], 0.0)
              - np.where((si == sc) & (sa == sb), ovvv[I, C, A, B], 0.0))
    eps_o = np.concatenate([d["eps_occ"], d["eps_occ"]])
    eps_v = np.concatenate([d["eps_vir"], d["eps_vir"]])
    return eps_o, eps_v, t1, t2, v2ijab, v2ijka, v2iabc
