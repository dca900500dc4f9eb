"""Python binding of the C ABI in include/ccsdt.h (ctypes; no torch types cross it).

Mirrors the call ExaChem makes, ``CCSD_T_Fused_Driver<T>::execute``
(exachem/cc/ccsd_t/ccsd_t_fused_driver.hpp:91-546), which returns
(E[T], E(T), work seconds, total seconds): ``FusedTriples.execute`` returns the same
tuple.  The CUDA library must be built (``exachem_gb300.build.build_library``); if it is
missing, loading fails loudly - there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

from .build import LIB

_lib = None

MODES = {"fp64": 0, "ozaki": 1, "learned": 2}


class CCSDTError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"ccsdt status {status}: {msg}")
        self.status = status


class Layout(ctypes.Structure):
    _fields_ = [("o", ctypes.c_int), ("v", ctypes.c_int), ("n_occ_tiles", ctypes.c_int),
                ("occ_tiles", ctypes.POINTER(ctypes.c_int)), ("n_vir_tiles", ctypes.c_int),
                ("vir_tiles", ctypes.POINTER(ctypes.c_int))]


class Opts(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("slices", ctypes.c_int), ("slice_kind", ctypes.c_int),
                ("use_graph", ctypes.c_int), ("shard_index", ctypes.c_int), ("shard_count", ctypes.c_int),
                ("energy_budget", ctypes.c_double), ("budget_triplets", ctypes.c_int),
                ("test_kernel", ctypes.c_int), ("autotune", ctypes.c_int), ("p_storage", ctypes.c_int),
                ("reserved", ctypes.c_int * 2)]


class Result(ctypes.Structure):
    _fields_ = [("e_bracket_T", ctypes.c_double), ("e_paren_T", ctypes.c_double),
                ("abs_err_bound", ctypes.c_double), ("seconds", ctypes.c_double),
                ("flops_executed", ctypes.c_double), ("flops_ref_equiv", ctypes.c_double),
                ("n_triplets", ctypes.c_long), ("n_tasks_ref", ctypes.c_long)]


EXPORTED = ["ccsdt_create", "ccsdt_upload", "ccsdt_energy", "ccsdt_triplet_energies",
            "ccsdt_last_launch_count", "ccsdt_reference_op_count", "ccsdt_destroy",
            "ccsdt_last_error", "ccsdt_status_string", "ccsdt_set_stream", "ccsdt_profile_triplet",
            "ccsdt_debug_triplet_w", "ccsdt_energy_noalloc", "ccsdt_shard_triplets",
            "ccsdt_set_phase_timing", "ccsdt_phase_times", "ccsdt_triplet_error_estimates",
            "ccsdt_upload_begin", "ccsdt_upload_blocks", "ccsdt_upload_end", "ccsdt_upload_cholesky",
            "ccsdt_tile_configs", "ccsdt_autotune", "ccsdt_set_tile_config", "ccsdt_energy_spin_orbital",
            "ccsdt_debug_spin_orbital_plan", "ccsdt_reference_op_count_so", "ccsdt_upload_cholesky_direct",
            "ccsdt_ovvv_slab_builds", "ccsdt_debug_slab_schedule", "ccsdt_energy_spin_orbital_split",
            "ccsdt_debug_set_slab_build"]
BLOCK_KINDS = {"t2": 0, "oovv": 1, "ooov": 2, "ovvv": 3}


def load_library(path: str | os.PathLike | None = None):
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: build it with exachem_gb300.build.build_library()")
    lib = ctypes.CDLL(str(p))
    vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
    lib.ccsdt_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(Layout), ctypes.c_int]
    lib.ccsdt_upload.argtypes = [vp] + [vp] * 7 + [ctypes.c_int]
    lib.ccsdt_energy.argtypes = [vp, ctypes.POINTER(Opts), ctypes.POINTER(Result)]
    lib.ccsdt_triplet_energies.argtypes = [vp, ctypes.POINTER(Opts), ctypes.c_long, ip, dp, dp]
    lib.ccsdt_last_launch_count.argtypes = [vp]
    lib.ccsdt_last_launch_count.restype = ctypes.c_long
    lib.ccsdt_reference_op_count.argtypes = [ctypes.POINTER(Layout), dp, ctypes.POINTER(ctypes.c_long)]
    lib.ccsdt_set_stream.argtypes = [vp, vp]
    lib.ccsdt_set_phase_timing.argtypes = [vp, ctypes.c_int]
    lib.ccsdt_upload_begin.argtypes = [vp, vp, vp, vp, ctypes.c_int]
    lib.ccsdt_upload_blocks.argtypes = [vp, ctypes.c_int, ctypes.c_long, ip, ctypes.POINTER(ctypes.c_longlong), vp,
                                        ctypes.c_longlong, ctypes.c_int]
    lib.ccsdt_upload_end.argtypes = [vp]
    lib.ccsdt_upload_cholesky.argtypes = [vp, vp, vp, vp, vp, ctypes.c_int, vp, vp, vp, ctypes.c_int]
    lib.ccsdt_upload_cholesky_direct.argtypes = [vp, vp, vp, vp, vp, ctypes.c_int, vp, vp, vp, ctypes.c_int,
                                                 ctypes.c_int]
    lib.ccsdt_ovvv_slab_builds.argtypes = [vp]
    lib.ccsdt_ovvv_slab_builds.restype = ctypes.c_long
    lib.ccsdt_debug_slab_schedule.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_long, ip,
                                              ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_long)]
    lib.ccsdt_tile_configs.argtypes = [ctypes.c_int, ip, ip]
    lib.ccsdt_autotune.argtypes = [vp, ctypes.c_int, dp, ip, ip]
    lib.ccsdt_set_tile_config.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    lib.ccsdt_energy_spin_orbital.argtypes = [ctypes.c_int] * 4 + [vp] * 7 + [ctypes.c_int] * 3 + [dp, dp]
    lib.ccsdt_energy_spin_orbital_split.argtypes = [ctypes.c_int] * 4 + [vp] * 7 + [ctypes.c_int] * 4 + [dp, dp]
    lib.ccsdt_debug_spin_orbital_plan.argtypes = [ctypes.c_int] * 7 + [ip, ctypes.POINTER(ctypes.c_longlong), ip]
    lib.ccsdt_reference_op_count_so.argtypes = [ctypes.c_int, ip] * 4 + [ctypes.c_int, dp,
                                                                         ctypes.POINTER(ctypes.c_long)]
    lib.ccsdt_triplet_error_estimates.argtypes = [vp, ctypes.POINTER(Opts), ctypes.c_long, ip, dp, dp, dp]
    lib.ccsdt_phase_times.argtypes = [vp, dp, ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_long)]
    lib.ccsdt_shard_triplets.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_long), ip]
    lib.ccsdt_profile_triplet.argtypes = [vp, ctypes.POINTER(Opts), ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
    lib.ccsdt_debug_triplet_w.argtypes = [vp, ctypes.POINTER(Opts), ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
    lib.ccsdt_debug_triplet_w.restype = ctypes.c_int
    lib.ccsdt_destroy.argtypes = [vp]
    lib.ccsdt_destroy.restype = None
    lib.ccsdt_last_error.argtypes = [vp]
    lib.ccsdt_last_error.restype = ctypes.c_char_p
    lib.ccsdt_status_string.argtypes = [ctypes.c_int]
    lib.ccsdt_status_string.restype = ctypes.c_char_p
    for name in ("ccsdt_create", "ccsdt_upload", "ccsdt_energy", "ccsdt_triplet_energies",
                 "ccsdt_reference_op_count", "ccsdt_set_stream", "ccsdt_profile_triplet",
                 "ccsdt_shard_triplets", "ccsdt_set_phase_timing", "ccsdt_phase_times",
                 "ccsdt_triplet_error_estimates", "ccsdt_upload_begin", "ccsdt_upload_blocks", "ccsdt_upload_end",
                 "ccsdt_upload_cholesky", "ccsdt_tile_configs", "ccsdt_autotune", "ccsdt_set_tile_config",
                 "ccsdt_energy_spin_orbital", "ccsdt_debug_spin_orbital_plan", "ccsdt_reference_op_count_so",
                 "ccsdt_upload_cholesky_direct", "ccsdt_debug_slab_schedule", "ccsdt_energy_spin_orbital_split"):
        getattr(lib, name).restype = ctypes.c_int
    if path is None:
        _lib = lib
    return lib


def _tiles(n: int, tiles) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(tiles, dtype=np.int32))


def make_layout(o: int, v: int, occ_tiles, vir_tiles):
    ot, vt = _tiles(o, occ_tiles), _tiles(v, vir_tiles)
    L = Layout(o, v, len(ot), ot.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(vt),
               vt.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return L, (ot, vt)


def reference_op_count(o: int, v: int, occ_tiles, vir_tiles) -> tuple[float, int]:
    """The reference's spin-orbital op count and task count for a tile layout."""
    lib = load_library()
    L, keep = make_layout(o, v, occ_tiles, vir_tiles)
    ops, nt = ctypes.c_double(), ctypes.c_long()
    st = lib.ccsdt_reference_op_count(ctypes.byref(L), ctypes.byref(ops), ctypes.byref(nt))
    if st:
        raise CCSDTError(st, lib.ccsdt_status_string(st).decode())
    return ops.value, nt.value


def reference_op_count_so(occ_a, occ_b, vir_a, vir_b, is_restricted: bool = False) -> tuple[float, int]:
    """The reference's op count and task count over alpha / beta tile lists of their own."""
    lib = load_library()
    ts = [_tiles(0, t) for t in (occ_a, occ_b, vir_a, vir_b)]
    args = []
    for t in ts:
        args += [len(t), t.ctypes.data_as(ctypes.POINTER(ctypes.c_int))]
    ops, nt = ctypes.c_double(), ctypes.c_long()
    st = lib.ccsdt_reference_op_count_so(*args, int(bool(is_restricted)), ctypes.byref(ops), ctypes.byref(nt))
    if st:
        raise CCSDTError(st, lib.ccsdt_status_string(st).decode())
    return ops.value, nt.value


def _ptr(x) -> int:
    """Host numpy array (C-contiguous float64) or a CUDA tensor -> raw address."""
    if isinstance(x, np.ndarray):
        if x.dtype != np.float64 or not x.flags.c_contiguous:
            raise TypeError("host inputs must be C-contiguous float64 arrays")
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        if not x.is_contiguous() or str(x.dtype) != "torch.float64":
            raise TypeError("device inputs must be contiguous float64 tensors")
        return x.data_ptr()
    raise TypeError(f"unsupported input type {type(x)}")


class FusedTriples:
    """One (T) problem resident on one GPU."""

    def __init__(self, o: int, v: int, occ_tiles=None, vir_tiles=None, ts: int = 40, device: int = 0):
        from .generator import tiles_uniform
        self.lib = load_library()
        self.o, self.v = o, v
        self.occ_tiles = list(occ_tiles) if occ_tiles is not None else tiles_uniform(o, ts)
        self.vir_tiles = list(vir_tiles) if vir_tiles is not None else tiles_uniform(v, ts)
        L, keep = make_layout(o, v, self.occ_tiles, self.vir_tiles)
        h = ctypes.c_void_p()
        st = self.lib.ccsdt_create(ctypes.byref(h), ctypes.byref(L), device)
        if st:
            raise CCSDTError(st, self.lib.ccsdt_status_string(st).decode())
        self.h = h

    def _check(self, st: int):
        if st:
            raise CCSDTError(st, self.lib.ccsdt_last_error(self.h).decode())

    def upload(self, eps_occ, eps_vir, t1, t2, oovv, ooov, ovvv):
        arrs = [eps_occ, eps_vir, t1, t2, oovv, ooov, ovvv]
        on_dev = 0 if isinstance(arrs[0], np.ndarray) else 1
        if any((isinstance(a, np.ndarray)) != (on_dev == 0) for a in arrs):
            raise TypeError("pass all inputs on the host or all on the device")
        self._keep = arrs
        self._check(self.lib.ccsdt_upload(self.h, *[ctypes.c_void_p(_ptr(a)) for a in arrs], on_dev))

    def upload_cholesky(self, eps_occ, eps_vir, t1, t2, chol_oo, chol_ov, chol_vv, max_ovvv_slabs=None):
        """Inputs with oovv / ooov / ovvv built on the device from spatial Cholesky vectors
        chol_oo[o][o][Q], chol_ov[o][v][Q], chol_vv[v][v][Q] (all on the host or all on the device).
        max_ovvv_slabs: the Cholesky-direct mode, (ia|bc) formed slab by slab into a cache of that
        many v^3 slabs (ccsdt_upload_cholesky_direct)."""
        arrs = [eps_occ, eps_vir, t1, t2, chol_oo, chol_ov, chol_vv]
        on_dev = 0 if isinstance(arrs[0], np.ndarray) else 1
        if any((isinstance(a, np.ndarray)) != (on_dev == 0) for a in arrs):
            raise TypeError("pass all inputs on the host or all on the device")
        if on_dev == 0:
            arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in arrs]
        n_chol = int(arrs[4].shape[-1])
        self._keep = arrs
        if max_ovvv_slabs is None:
            self._check(self.lib.ccsdt_upload_cholesky(self.h, *[ctypes.c_void_p(_ptr(a)) for a in arrs[:4]], n_chol,
                                                       *[ctypes.c_void_p(_ptr(a)) for a in arrs[4:]], on_dev))
        else:
            self._check(self.lib.ccsdt_upload_cholesky_direct(
                self.h, *[ctypes.c_void_p(_ptr(a)) for a in arrs[:4]], n_chol,
                *[ctypes.c_void_p(_ptr(a)) for a in arrs[4:]], on_dev, int(max_ovvv_slabs)))

    def ovvv_slab_builds(self) -> int:
        """(ia|bc) slabs formed since the last upload (Cholesky-direct mode)."""
        return int(self.lib.ccsdt_ovvv_slab_builds(self.h))

    @staticmethod
    def tile_configs(slices: int) -> list[tuple[int, int, int]]:
        """(N tile, pipeline stages, K chunk) of the compiled contraction configurations for
        `slices` digit planes; index 0 is the default."""
        lib = load_library()
        n = ctypes.c_int()
        if lib.ccsdt_tile_configs(slices, ctypes.byref(n), None):
            return []
        buf = (ctypes.c_int * (3 * n.value))()
        lib.ccsdt_tile_configs(slices, ctypes.byref(n), buf)
        return [tuple(buf[3 * q:3 * q + 3]) for q in range(n.value)]

    def autotune(self, slices: int):
        """Times every configuration on one triplet, keeps the fastest: (ms per configuration,
        index kept)."""
        ms = (ctypes.c_double * 16)()
        n, chosen = ctypes.c_int(), ctypes.c_int()
        self._check(self.lib.ccsdt_autotune(self.h, slices, ms, ctypes.byref(n), ctypes.byref(chosen)))
        return list(ms[:n.value]), chosen.value

    def set_tile_config(self, slices: int, index: int):
        self._check(self.lib.ccsdt_set_tile_config(self.h, slices, index))

    def upload_dict(self, d: dict):
        self.upload(d["eps_occ"], d["eps_vir"], d["t1"], d["t2"], d["oovv"], d["ooov"], d["ovvv"])

    @staticmethod
    def opts(mode="fp64", slices=4, slice_kind="bf16", energy_budget=1e-9, use_graph=0,
             shard_index=0, shard_count=1, legacy_mma=0, budget_triplets=0, autotune=0, p_storage=0) -> Opts:
        o = Opts()
        o.mode = MODES[mode] if isinstance(mode, str) else int(mode)
        o.slices = slices
        o.slice_kind = {"bf16": 0, "int8": 1}[slice_kind] if isinstance(slice_kind, str) else int(slice_kind)
        o.energy_budget = energy_budget
        o.use_graph = use_graph
        o.shard_index, o.shard_count = shard_index, shard_count
        o.budget_triplets = budget_triplets
        o.test_kernel = legacy_mma       # 1: mma.sync slice kernel, 2: per-triplet tcgen05 kernel (testing)
        o.autotune = autotune            # 1: tune the contraction's tile configuration on first use
        o.p_storage = ({"auto": 0, "ff": 1, "f32": 2, "f64": 3}[p_storage] if isinstance(p_storage, str)
                       else int(p_storage))
        return o

    def energy(self, mode="fp64", **kw) -> dict:
        op = self.opts(mode, **kw)
        r = Result()
        self._check(self.lib.ccsdt_energy(self.h, ctypes.byref(op), ctypes.byref(r)))
        return {k: getattr(r, k) for k, _ in Result._fields_} | {"launches": self.launch_count()}

    def triplet_energies(self, triplets, mode="fp64", **kw):
        tri = np.ascontiguousarray(np.asarray(triplets, dtype=np.int32).reshape(-1, 3))
        n = tri.shape[0]
        e4, e5 = np.zeros(n), np.zeros(n)
        op = self.opts(mode, **kw)
        dp = ctypes.POINTER(ctypes.c_double)
        self._check(self.lib.ccsdt_triplet_energies(self.h, ctypes.byref(op), n,
                                                    tri.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                                    e4.ctypes.data_as(dp), e5.ctypes.data_as(dp)))
        return e4, e5

    def set_stream(self, stream_handle: int | None):
        """Run on an external cudaStream_t (e.g. torch.cuda.current_stream().cuda_stream)."""
        self._check(self.lib.ccsdt_set_stream(self.h, ctypes.c_void_p(stream_handle or 0)))

    def profile_triplet(self, i: int, j: int, k: int, mode="fp64", **kw) -> list[float]:
        """Device ms of [l-sum GEMMs, d-sum GEMMs, energy, reduction] for one triplet."""
        out = (ctypes.c_double * 4)()
        op = self.opts(mode, **kw)
        self._check(self.lib.ccsdt_profile_triplet(self.h, ctypes.byref(op), i, j, k, out))
        return list(out)

    def triplet_w(self, i: int, j: int, k: int, mode="fp64", **kw) -> np.ndarray:
        """W_abc of one triplet (verification aid), shape (v, v, v)."""
        w = np.empty((self.v, self.v, self.v))
        op = self.opts(mode, **kw)
        self._check(self.lib.ccsdt_debug_triplet_w(self.h, ctypes.byref(op), i, j, k,
                                                   w.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return w

    # ---- device-side retile of spin-orbital tile blocks (ccsdt_upload_begin / blocks / end)
    def upload_begin(self, eps_occ, eps_vir, t1):
        self._keep = [np.ascontiguousarray(x, dtype=np.float64) for x in (eps_occ, eps_vir, t1)]
        self._check(self.lib.ccsdt_upload_begin(self.h, *[x.ctypes.data for x in self._keep], 0))

    def upload_blocks(self, kind: str, tiles, offsets, data):
        """tiles: (n, 4) tile positions; offsets: (n,) element offsets into data (numpy float64 on the
        host, or a torch CUDA float64 tensor on the handle's device)."""
        t = np.ascontiguousarray(np.asarray(tiles, dtype=np.int32).reshape(-1, 4))
        off = np.ascontiguousarray(np.asarray(offsets, dtype=np.int64))
        if hasattr(data, "data_ptr"):
            ptr, n, dev = data.data_ptr(), data.numel(), 1
        else:
            arr = np.ascontiguousarray(data, dtype=np.float64)
            ptr, n, dev = arr.ctypes.data, arr.size, 0
        self._check(self.lib.ccsdt_upload_blocks(self.h, BLOCK_KINDS[kind], len(t), t.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                                 off.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), ptr, n, dev))

    def upload_end(self):
        self._check(self.lib.ccsdt_upload_end(self.h))

    def triplet_error_estimates(self, tri, slices: int):
        """(E[T]_t, E(T)_t, estimated |E(T)_t - E(T)_t,fp64|) at `slices` BF16 digit planes."""
        t = np.ascontiguousarray(np.asarray(tri, dtype=np.int32).reshape(-1, 3))
        n = len(t)
        e4, e5, est = np.zeros(n), np.zeros(n), np.zeros(n)
        op = self.opts("ozaki", slices=slices)
        dpp = ctypes.POINTER(ctypes.c_double)
        self._check(self.lib.ccsdt_triplet_error_estimates(
            self.h, ctypes.byref(op), n, t.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
            e4.ctypes.data_as(dpp), e5.ctypes.data_as(dpp), est.ctypes.data_as(dpp)))
        return e4, e5, est

    def set_phase_timing(self, on: bool = True):
        """Start (and zero) or stop live per-phase timing of the batched split-precision path."""
        self._check(self.lib.ccsdt_set_phase_timing(self.h, int(on)))

    def phase_times(self) -> dict:
        """Accumulated device ms of the contraction and energy launches since set_phase_timing."""
        ms = (ctypes.c_double * 3)()
        b, t = ctypes.c_long(), ctypes.c_long()
        self._check(self.lib.ccsdt_phase_times(self.h, ms, ctypes.byref(b), ctypes.byref(t)))
        return {"contraction_ms": ms[0], "energy_ms": ms[1], "batches": b.value, "triplets": t.value}

    def launch_count(self) -> int:
        return int(self.lib.ccsdt_last_launch_count(self.h))

    def execute(self, mode="fp64", **kw):
        """(E[T], E(T), work seconds, total seconds), as the reference driver returns."""
        import time
        t0 = time.perf_counter()
        r = self.energy(mode, **kw)
        return r["e_bracket_T"], r["e_paren_T"], r["seconds"], time.perf_counter() - t0

    def close(self):
        if getattr(self, "h", None):
            self.lib.ccsdt_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def slab_schedule(o: int, max_ovvv_slabs: int, batch: int, triplets) -> tuple[np.ndarray, int]:
    """The Cholesky-direct mode's triplet order and slab count for a cache of max_ovvv_slabs slabs
    and batches of `batch` triplets (host only, ccsdt_debug_slab_schedule)."""
    lib = load_library()
    tri = np.ascontiguousarray(np.asarray(triplets, dtype=np.int32).reshape(-1, 3))
    order = np.zeros(len(tri), dtype=np.int64)
    builds = ctypes.c_long()
    st = lib.ccsdt_debug_slab_schedule(o, max_ovvv_slabs, batch, len(tri),
                                       tri.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                       order.ctypes.data_as(ctypes.POINTER(ctypes.c_long)), ctypes.byref(builds))
    if st:
        raise CCSDTError(st, "ccsdt_debug_slab_schedule")
    return order, builds.value


def energy_spin_orbital(oa: int, ob: int, va: int, vb: int, eps_occ, eps_vir, t1, t2, v2ijab, v2ijka,
                        v2iabc, shard_index: int = 0, shard_count: int = 1, slices: int = 0) -> dict:
    """Open-shell (T) over spin orbitals (ccsdt_energy_spin_orbital): ExaChem's MO order
    (occupied alpha | beta, virtual alpha | beta), arrays t1[V][O], t2[V][V][O][O],
    v2ijab[O][O][V][V], v2ijka[O][O][O][V], v2iabc[O][V][V][V] as host numpy arrays or CUDA
    tensors (all of one kind).  shard_index / shard_count select every shard_count-th occupied
    triplet i < j < k.  slices > 0: split-precision contractions with that many BF16 digit planes
    (ccsdt_energy_spin_orbital_split)."""
    lib = load_library()
    arrs = [eps_occ, eps_vir, t1, t2, v2ijab, v2ijka, v2iabc]
    kinds = {isinstance(a, np.ndarray) for a in arrs}
    if len(kinds) != 1:
        raise TypeError("inputs must be all host arrays or all device tensors")
    O, V = oa + ob, va + vb
    shapes = [(O,), (V,), (V, O), (V, V, O, O), (O, O, V, V), (O, O, O, V), (O, V, V, V)]
    for a, sh in zip(arrs, shapes):
        if tuple(a.shape) != sh:
            raise ValueError(f"expected shape {sh}, got {tuple(a.shape)}")
    on_device = 0 if kinds == {True} else 1
    e = (ctypes.c_double * 2)()
    sec = ctypes.c_double()
    out = ctypes.cast(e, ctypes.POINTER(ctypes.c_double))
    if slices > 0:
        st = lib.ccsdt_energy_spin_orbital_split(oa, ob, va, vb, *[_ptr(a) for a in arrs], on_device, shard_index,
                                                 shard_count, slices, out, ctypes.byref(sec))
    else:
        st = lib.ccsdt_energy_spin_orbital(oa, ob, va, vb, *[_ptr(a) for a in arrs], on_device, shard_index,
                                           shard_count, out, ctypes.byref(sec))
    if st:
        raise CCSDTError(st, lib.ccsdt_status_string(st).decode())
    return {"e_bracket_T": e[0], "e_paren_T": e[1], "seconds": sec.value}


PLAN_FIELDS = ["x0", "y0", "z0", "nx", "ny", "nz", "has_d", "d_k", "d_a", "d_b", "has_s", "s_k", "s_a", "s_b"]


def spin_orbital_plan(oa: int, ob: int, va: int, vb: int, i: int, j: int, k: int):
    """The open-shell path's contraction plan for triplet i < j < k (host logic, no GPU):
    (of[3][3] block index per permutation and position, list of block dicts)."""
    lib = load_library()
    of = (ctypes.c_int * 9)()
    blocks = (ctypes.c_longlong * (9 * 14))()
    n = ctypes.c_int()
    st = lib.ccsdt_debug_spin_orbital_plan(oa, ob, va, vb, i, j, k, of, blocks, ctypes.byref(n))
    if st:
        raise CCSDTError(st, lib.ccsdt_status_string(st).decode())
    return (np.array(list(of)).reshape(3, 3),
            [dict(zip(PLAN_FIELDS, blocks[14 * b:14 * b + 14])) for b in range(n.value)])


def all_triplets(o: int) -> np.ndarray:
    return np.array([(i, j, k) for i in range(o) for j in range(i, o) for k in range(j, o)], dtype=np.int32)
