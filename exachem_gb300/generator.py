"""Seeded synthetic closed-shell inputs for the (T) energy.

Draw order (numpy PCG64, ``default_rng(seed)``), fixed:
  1. eps_occ  ~ U[-1.4, -0.4]  (o values, sorted ascending)
  2. eps_vir  ~ U[ 0.2,  2.5]  (v values, sorted ascending)
  3. B[Q,p,q] ~ N(0, 0.05^2)   (Q x n x n, n = o + v, Q = 4 n unless given),
     symmetrised by copying the upper triangle onto the lower one, so every
     element keeps the N(0, 0.05^2) marginal, then rounded to a multiple of 2^-12.
  4. t1[i][a] ~ N(0, (2e-3)^2)

Integrals are (pq|rs) = sum_Q B[Q,p,q] B[Q,r,s].  Because B is a multiple of
2^-12 with |B| < 2^-1, every product is an exact multiple of 2^-24 and every
partial sum stays below 2^53 ulps, so the integrals are EXACT in FP64 whatever
the summation order.  The GPU generator (``generate_device``) therefore yields
bit-identical integrals to the numpy one while running the contractions on
TF32 tensor cores through integer splits (see ``_exact_gemm_tf32``).

T2 is the MP2 guess t_ij^ab = (ia|jb) / (((e_i + e_j) - e_a) - e_b), evaluated with
that association order on both host and device.

Layouts (row-major, chemist notation), identical to the C-ABI's:
  eps_occ[o], eps_vir[v], t1[o][v],
  t2[o][o][v][v] = t_ij^ab,  oovv[o][o][v][v] = (ia|jb),
  ooov[o][o][o][v] = (ij|ka),  ovvv[o][v][v][v] = (ia|bc)

Reference conventions these feed: closed-shell T2 ``t2_abab(a,b,i,j) = t_ij^ab``
(exachem/cc/ccsd/cd_ccsd_cs_ann.cpp:949-973) and V2 blocks built from Cholesky
vectors (exachem/cholesky/v2tensors.cpp:67-86).
"""
from __future__ import annotations

import numpy as np

QUANT = 2.0 ** -12


def tiles_uniform(n: int, ts: int) -> list[int]:
    """Tile extents of one index range: full tiles of ``ts`` then the remainder
    (exachem/cholesky/cholesky_2e.cpp:230-285, balance_tiles = false)."""
    t = [ts] * (n // ts)
    if n % ts:
        t.append(n % ts)
    return t


def tiles_ragged(n: int, rng: np.random.Generator, choices=(16, 24, 32, 40, 48)) -> list[int]:
    """Tile extents drawn uniformly from ``choices``; the last tile is truncated."""
    t, r = [], n
    while r > 0:
        x = int(rng.choice(choices))
        x = min(x, r)
        t.append(x)
        r -= x
    return t


def draw_host(o: int, v: int, seed: int, Q: int | None = None):
    """The random draws (steps 1-4 above), on the host."""
    rng = np.random.default_rng(seed)
    n = o + v
    Q = 4 * n if Q is None else Q
    eps_occ = np.sort(rng.uniform(-1.4, -0.4, o))
    eps_vir = np.sort(rng.uniform(0.2, 2.5, v))
    B = rng.normal(0.0, 0.05, (Q, n, n))
    iu = np.triu_indices(n, 1)
    B[:, iu[1], iu[0]] = B[:, iu[0], iu[1]]
    B = np.rint(B / QUANT) * QUANT
    t1 = rng.normal(0.0, 2e-3, (o, v))
    return eps_occ, eps_vir, B, t1


def mp2_t2(oovv: np.ndarray, eps_occ: np.ndarray, eps_vir: np.ndarray) -> np.ndarray:
    eo, ev = eps_occ, eps_vir
    d = ((eo[:, None, None, None] + eo[None, :, None, None]) - ev[None, None, :, None]) - ev[None, None, None, :]
    return oovv / d


def generate(o: int, v: int, seed: int, Q: int | None = None, t2_scale: float = 1.0) -> dict:
    """Host (numpy) generator for sizes where O(o v^3 Q) host work is affordable."""
    eps_occ, eps_vir, B, t1 = draw_host(o, v, seed, Q)
    Bo = B[:, :o, o:]
    Boo = B[:, :o, :o]
    Bvv = B[:, o:, o:]
    Qn = B.shape[0]
    ov = Bo.reshape(Qn, o * v)
    oovv = (ov.T @ ov).reshape(o, v, o, v).transpose(0, 2, 1, 3).copy()          # (ia|jb) at [i][j][a][b]
    ooov = (Boo.reshape(Qn, o * o).T @ ov).reshape(o, o, o, v)                    # (ij|ka)
    ovvv = (ov.T @ Bvv.reshape(Qn, v * v)).reshape(o, v, v, v)                    # (ia|bc)
    t2 = mp2_t2(oovv, eps_occ, eps_vir)
    if t2_scale != 1.0:
        t2 = t2 * t2_scale
    return dict(o=o, v=v, seed=seed, eps_occ=eps_occ, eps_vir=eps_vir, t1=np.ascontiguousarray(t1),
                t2=np.ascontiguousarray(t2), oovv=np.ascontiguousarray(oovv),
                ooov=np.ascontiguousarray(ooov), ovvv=np.ascontiguousarray(ovvv))


# ----------------------------------------------------------------------------------------------
# device generator (torch is used for device memory and cuBLAS TF32 GEMMs of integer splits)

def _split_int(x):
    """x: float tensor holding integers with |x| < 2^11.  Returns (hi, lo) with
    x = 64 hi + lo, |hi| <= 32, lo in [-32, 31]; both exact in TF32."""
    import torch
    hi = torch.floor((x + 32.0) / 64.0)
    lo = x - 64.0 * hi
    return hi, lo


def _exact_gemm_tf32(a_int, b_int):
    """Exact sum_Q a[Q,m] b[Q,n] for integer-valued float32 a, b with |.| < 2^11 and
    Q <= 4096: each TF32 product of 6-bit splits is exact and each FP32 partial sum
    stays below 2^24.  Returns float64 [m, n] (integer valued)."""
    import torch
    ah, al = _split_int(a_int)
    bh, bl = _split_int(b_int)
    hh = (ah.T @ bh).double()
    mid = (torch.cat([ah, al], 0).T @ torch.cat([bl, bh], 0)).double()
    ll = (al.T @ bl).double()
    return (hh * 4096.0 + mid * 64.0) + ll


def generate_device(o: int, v: int, seed: int, Q: int | None = None, device="cuda", t2_scale: float = 1.0,
                    vv_chunk: int = 8192) -> dict:
    """Same values as ``generate`` (bit-identical integrals), built on the GPU.
    Returns torch tensors on ``device`` in the C-ABI layouts."""
    import torch
    eps_occ, eps_vir, B, t1 = draw_host(o, v, seed, Q)
    Qn, n = B.shape[0], o + v
    if Qn > 4096:
        raise ValueError("exact TF32 generator needs Q <= 4096")
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        Bi = torch.from_numpy(np.rint(B / QUANT).astype(np.float32)).to(device)   # integers
        del B
        ov = Bi[:, :o, o:].reshape(Qn, o * v).contiguous()
        oo = Bi[:, :o, :o].reshape(Qn, o * o).contiguous()
        scale = QUANT * QUANT
        oovv = (_exact_gemm_tf32(ov, ov) * scale).reshape(o, v, o, v).permute(0, 2, 1, 3).contiguous()
        ooov = (_exact_gemm_tf32(oo, ov) * scale).reshape(o, o, o, v).contiguous()
        # (ia|bc) = (ia|cb): compute the b <= c half by row blocks of b, mirror the rest
        ovvv = torch.empty((o * v, v, v), dtype=torch.float64, device=device)
        vvm = Bi[:, o:, o:]
        nb = max(1, min(v, vv_chunk // max(1, v)))
        for b0 in range(0, v, nb):
            b1 = min(v, b0 + nb)
            blk = vvm[:, b0:b1, b0:].reshape(Qn, -1).contiguous()
            r = (_exact_gemm_tf32(ov, blk) * scale).reshape(o * v, b1 - b0, v - b0)
            ovvv[:, b0:b1, b0:] = r
            ovvv[:, b0:, b0:b1] = r.transpose(1, 2)
            del r, blk
        ovvv = ovvv.reshape(o, v, v, v)
        del Bi, ov, oo, vvm
        eo = torch.from_numpy(eps_occ).to(device)
        ev = torch.from_numpy(eps_vir).to(device)
        d = ((eo[:, None, None, None] + eo[None, :, None, None]) - ev[None, None, :, None]) - ev[None, None, None, :]
        t2 = oovv / d
        if t2_scale != 1.0:
            t2 = t2 * t2_scale
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old
    return dict(o=o, v=v, seed=seed, eps_occ=eo, eps_vir=ev, t1=torch.from_numpy(t1).to(device),
                t2=t2.contiguous(), oovv=oovv, ooov=ooov, ovvv=ovvv)


def generate_host_slabs(o: int, v: int, seed: int, slabs, Q: int | None = None) -> dict:
    """Host inputs for a sample of triplets: everything except ovvv in full, and the
    (ia|bc) slabs only for the occupied indices in ``slabs`` (key ``ovvv_slabs``:
    {i: array[v][v][v]}).  Same values as ``generate``."""
    eps_occ, eps_vir, B, t1 = draw_host(o, v, seed, Q)
    Qn = B.shape[0]
    Bo = B[:, :o, o:]
    ov = np.ascontiguousarray(Bo.reshape(Qn, o * v))
    oovv = (ov.T @ ov).reshape(o, v, o, v).transpose(0, 2, 1, 3).copy()
    ooov = (np.ascontiguousarray(B[:, :o, :o].reshape(Qn, o * o)).T @ ov).reshape(o, o, o, v)
    vv = np.ascontiguousarray(B[:, o:, o:].reshape(Qn, v * v))
    sl = {int(i): np.ascontiguousarray((np.ascontiguousarray(Bo[:, i, :]).T @ vv).reshape(v, v, v))
          for i in sorted(set(int(x) for x in slabs))}
    t2 = mp2_t2(oovv, eps_occ, eps_vir)
    return dict(o=o, v=v, seed=seed, eps_occ=eps_occ, eps_vir=eps_vir, t1=np.ascontiguousarray(t1),
                t2=np.ascontiguousarray(t2), oovv=np.ascontiguousarray(oovv),
                ooov=np.ascontiguousarray(ooov), ovvv_slabs=sl)
