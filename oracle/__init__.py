"""CPU oracle for the (T) energy - TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use this
package, and only as the checker: the product library never calls it.

  port : oracle/ccsdt_oracle.c  - closed-shell restatement (built by ``make -C oracle port``)
  ref  : oracle/_ref            - ExaChem's own CPU (T) headers compiled unmodified against
                                  oracle/ref_shim (``make -C oracle ref``; needs the reference
                                  tree, so only where it is present)
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "_build" / "libccsdt_oracle.so"
REF_LIB = HERE / "_ref" / "libccsdt_ref.so"

_port = None
_ref = None
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
KEYS = ["eps_occ", "eps_vir", "t1", "t2", "oovv", "ooov", "ovvv"]


def build_port():
    subprocess.run(["make", "-C", str(HERE), "port"], check=True, capture_output=True)


def port():
    global _port
    if _port is None:
        if not PORT_LIB.exists():
            build_port()
        _port = ctypes.CDLL(str(PORT_LIB))
        _port.oracle_triplets.argtypes = [ctypes.c_int, ctypes.c_int] + [_D] * 7 + [ctypes.c_long, _I, _D, _D]
        _port.oracle_energy.argtypes = [ctypes.c_int, ctypes.c_int] + [_D] * 7 + [_D, _D]
        _port.oracle_triplets_slabs.argtypes = [ctypes.c_int, ctypes.c_int] + [_D] * 6 + \
            [ctypes.POINTER(ctypes.c_void_p), ctypes.c_long, _I, _D, _D]
        _port.oracle_num_threads.restype = ctypes.c_int
        _port.oracle_w_rows_sample.argtypes = [ctypes.c_int, ctypes.c_int] + [_D] * 6 + \
            [ctypes.POINTER(ctypes.c_void_p)] + [ctypes.c_int] * 5
        _port.so_oracle_energy.argtypes = [ctypes.c_int] * 4 + [_D] * 7 + [ctypes.c_long, _I, _D, _D]
    return _port


def energy_spin_orbital_c(oa, ob, va, vb, arrs, tri=None) -> tuple[float, float]:
    """oracle/spin_orbital_oracle.c: (E[T], E(T)) of an open-shell system (arrs = eps_o, eps_v,
    t1, t2, v2ijab, v2ijka, v2iabc in the layouts of oracle/spin_orbital_oracle.py) over the
    triplets tri ([n][3], i < j < k; None = all of them)."""
    lib = port()
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in arrs]
    t = None if tri is None else np.ascontiguousarray(np.asarray(tri, dtype=np.int32).reshape(-1, 3))
    e4, e5 = ctypes.c_double(), ctypes.c_double()
    rc = lib.so_oracle_energy(oa, ob, va, vb, *[x.ctypes.data_as(_D) for x in a], 0 if t is None else len(t),
                              None if t is None else t.ctypes.data_as(_I), ctypes.byref(e4), ctypes.byref(e5))
    if rc:
        raise RuntimeError("so_oracle_energy failed")
    return e4.value, e5.value


def ref_available() -> bool:
    return REF_LIB.exists()


def ref():
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            raise FileNotFoundError("oracle/_ref is not built (needs the reference tree)")
        _ref = ctypes.CDLL(str(REF_LIB))
        _ref.ref_ccsd_t_energy.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _I, ctypes.c_int, _I] + \
            [_D] * 7 + [_D, _D, _D, ctypes.POINTER(ctypes.c_long)]
        if hasattr(_ref, "ref_ccsd_t_energy_so"):
            _ref.ref_ccsd_t_energy_so.argtypes = [ctypes.c_int, _I] * 4 + [_D] * 6 + \
                [ctypes.c_int, _D, _D, ctypes.POINTER(ctypes.c_long)]
    return _ref


def ref_energy_spin_orbital(tiles, eps, t1, t2, v2ijab, v2ijka, v2iabc, is_restricted=False):
    """ExaChem's own CPU (T) on inputs given over spin orbitals (ref_ccsd_t_energy_so):
    tiles = (occ_a, occ_b, virt_a, virt_b) tile extents; eps in MO order occ_a | occ_b | virt_a |
    virt_b; dense arrays in the layouts of ExaChem's tensors.  Returns (E[T], E(T), tasks)."""
    lib = ref()
    ts = [np.ascontiguousarray(np.asarray(t, dtype=np.int32)) for t in tiles]
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (eps, t1, t2, v2ijab, v2ijka, v2iabc)]
    args = []
    for t in ts:
        args += [len(t), t.ctypes.data_as(_I)]
    e4, e5, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_long()
    rc = lib.ref_ccsd_t_energy_so(*args, *[a.ctypes.data_as(_D) for a in arrs], int(bool(is_restricted)),
                                  ctypes.byref(e4), ctypes.byref(e5), ctypes.byref(n))
    if rc:
        raise RuntimeError(f"ref_ccsd_t_energy_so failed ({rc})")
    return e4.value, e5.value, n.value


def _arrs(d):
    out = []
    for k in KEYS:
        a = d[k]
        if not isinstance(a, np.ndarray):
            a = a.detach().cpu().numpy()
        out.append(np.ascontiguousarray(a, dtype=np.float64))
    return out


def energy(d) -> tuple[float, float]:
    """Full (T) from the C restatement: (E[T], E(T))."""
    a = _arrs(d)
    e4, e5 = ctypes.c_double(), ctypes.c_double()
    rc = port().oracle_energy(int(d["o"]), int(d["v"]), *[x.ctypes.data_as(_D) for x in a],
                              ctypes.byref(e4), ctypes.byref(e5))
    if rc:
        raise RuntimeError(f"oracle_energy failed ({rc})")
    return e4.value, e5.value


def triplets(d, tri) -> tuple[np.ndarray, np.ndarray]:
    """Per-triplet (E[T], E(T)) contributions for triplets i <= j <= k."""
    a = _arrs(d)
    t = np.ascontiguousarray(np.asarray(tri, dtype=np.int32).reshape(-1, 3))
    n = t.shape[0]
    e4, e5 = np.zeros(n), np.zeros(n)
    rc = port().oracle_triplets(int(d["o"]), int(d["v"]), *[x.ctypes.data_as(_D) for x in a], n,
                                t.ctypes.data_as(_I), e4.ctypes.data_as(_D), e5.ctypes.data_as(_D))
    if rc:
        raise RuntimeError(f"oracle_triplets failed ({rc})")
    return e4, e5


def triplets_slabs(d, tri) -> tuple[np.ndarray, np.ndarray]:
    """As ``triplets`` for inputs carrying only some (ia|bc) slabs (``d["ovvv_slabs"]``)."""
    o, v = int(d["o"]), int(d["v"])
    a = [np.ascontiguousarray(d[k], dtype=np.float64) for k in KEYS[:6]]
    slabs = (ctypes.c_void_p * o)()
    keep = []
    for i, s in d["ovvv_slabs"].items():
        s = np.ascontiguousarray(s, dtype=np.float64)
        keep.append(s)
        slabs[i] = s.ctypes.data
    t = np.ascontiguousarray(np.asarray(tri, dtype=np.int32).reshape(-1, 3))
    n = t.shape[0]
    e4, e5 = np.zeros(n), np.zeros(n)
    rc = port().oracle_triplets_slabs(o, v, *[x.ctypes.data_as(_D) for x in a], slabs, n,
                                      t.ctypes.data_as(_I), e4.ctypes.data_as(_D), e5.ctypes.data_as(_D))
    if rc:
        raise RuntimeError(f"oracle_triplets_slabs failed ({rc})")
    return e4, e5


def w_rows_sample(d, tri, a0, a1) -> None:
    """Timing sample: the contraction multiply-adds of triplet ``tri`` for first-virtual rows
    [a0, a1) (``d`` as for ``triplets_slabs``); the result is discarded."""
    o, v = int(d["o"]), int(d["v"])
    a = [np.ascontiguousarray(d[k], dtype=np.float64) for k in KEYS[:6]]
    slabs = (ctypes.c_void_p * o)()
    keep = []
    for i, s in d["ovvv_slabs"].items():
        s = np.ascontiguousarray(s, dtype=np.float64)
        keep.append(s)
        slabs[i] = s.ctypes.data
    i, j, k = (int(x) for x in tri)
    rc = port().oracle_w_rows_sample(o, v, *[x.ctypes.data_as(_D) for x in a], slabs, i, j, k, int(a0), int(a1))
    if rc:
        raise RuntimeError(f"oracle_w_rows_sample failed ({rc})")


def reference_energy(d, occ_tiles, vir_tiles) -> dict:
    """ExaChem's own CPU (T) on the spin-orbital tiling built from the tile lists."""
    a = _arrs(d)
    ot = np.ascontiguousarray(occ_tiles, dtype=np.int32)
    vt = np.ascontiguousarray(vir_tiles, dtype=np.int32)
    e4, e5, ops, nt = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_long()
    rc = ref().ref_ccsd_t_energy(int(d["o"]), int(d["v"]), len(ot), ot.ctypes.data_as(_I), len(vt),
                                 vt.ctypes.data_as(_I), *[x.ctypes.data_as(_D) for x in a],
                                 ctypes.byref(e4), ctypes.byref(e5), ctypes.byref(ops), ctypes.byref(nt))
    if rc:
        raise RuntimeError(f"reference (T) failed ({rc})")
    return {"e_bracket_T": e4.value, "e_paren_T": e5.value, "ops": ops.value, "tasks": nt.value}


def num_threads() -> int:
    return int(port().oracle_num_threads())
