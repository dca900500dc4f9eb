#!/usr/bin/env python
"""(T) wall-seconds at o=60, v=500 on GB300: split precision vs plain FP64.

Workload (the shape the headline metric is quoted on): closed-shell (T), o=60 occupied,
v=500 virtual orbitals, seed 3, tile extents drawn per index range from {16,24,32,40,48},
synthetic inputs from exachem_gb300.generator (built on the GPU, ovvv 60 GB in HBM).

A step is one batch of occupied triplets (i <= j <= k) of that workload, run through the
C ABI on inputs already resident in HBM.  With --mode ozaki / learned the K timed steps
partition every triplet of the call (timed_fraction 1): ``value`` is the measured device
time of the whole (T) call, the first step including the slicing of the operands into
digit planes.  ``e2e`` is the same call from pinned host buffers: ccsdt_upload (75 GB
host -> device) plus every step, host wall clock.  With --mode fp64 (hours at this size)
the timed steps cover an evenly spread sample of triplets and the whole-call time is
projected from it (timed_fraction < 1, stated).

--impl reference times the reference's CPU (T) on the host cores (the C restatement of
the oracle; the reference's own build needs its source tree), each step a bounded sample
of one triplet's contractions, projected to the whole call.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "(T) wall-s at o=60,v=500: split-prec vs plain FP64 on GB300, |dE|<=1e-6 Eh"
UNIT = "s"


def workload_tiles(o, v, seed):
    from exachem_gb300.generator import tiles_ragged
    rng = np.random.default_rng([seed, 7])
    return tiles_ragged(o, rng), tiles_ragged(v, rng)


def triplet_list(o):
    return np.array([(i, j, k) for i in range(o) for j in range(i, o) for k in range(j, o) if i != k],
                    dtype=np.int32)


def spread_sample(tri, n, offset=0):
    """n triplets evenly spread over the list (deterministic)."""
    idx = (np.arange(n) * len(tri)) // n + offset
    return tri[np.clip(idx, 0, len(tri) - 1)]


class ClockSampler:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    return json.loads(p.read_text()) if p.exists() else {}


def dgemm_peak_tflops(torch):
    """cuBLAS DGEMM 8192^3 (best of 3) - the FP64 denominator, measured in this run."""
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    del a, b
    return 2.0 * n ** 3 / best / 1e12


def profile_traffic(kernel):
    """dram bytes per launch of `kernel` from a committed ncu summary, if present."""
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text()).get(kernel)
        except json.JSONDecodeError:
            return None
    return None


def cpu_baseline_port(d_host_slabs, tri, reps=1):
    """Times the oracle's C restatement on the host cores for one sample triplet."""
    import oracle
    best = 1e30
    out = None
    for _ in range(reps):
        t0 = time.perf_counter()
        out = oracle.triplets_slabs(d_host_slabs, tri)
        best = min(best, time.perf_counter() - t0)
    return best, out, oracle.num_threads()


def host_slabs_from_device(dev, tri):
    """Host copies of what the sample triplets read (for the CPU baseline / checks)."""
    need = sorted(set(int(x) for x in np.asarray(tri).ravel()))
    h = {k: dev[k].cpu().numpy() for k in ("eps_occ", "eps_vir", "t1", "t2", "oovv", "ooov")}
    h.update(o=dev["o"], v=dev["v"], seed=dev["seed"], ovvv_slabs={i: dev["ovvv"][i].cpu().numpy() for i in need})
    return h


def run_reference(args):
    """CPU (T) of the reference path on the host cores: the oracle's C restatement, each step a
    bounded sample (the contraction rows [a0, a0 + v / q) of one triplet), projected to the whole
    call by the sampled share of the work."""
    import oracle
    from exachem_gb300.generator import generate_host_slabs
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    o, v, seed = args.o, args.v, args.seed
    tri_all = triplet_list(o)
    tri = spread_sample(tri_all, 1, offset=len(tri_all) // 2)[0]
    t0 = time.perf_counter()
    d = generate_host_slabs(o, v, seed, np.asarray(tri).ravel())
    t_gen = time.perf_counter() - t0
    # ExaChem's own CPU kernel materialises two ts^6 t3 blocks per task (ccsd_t_all_fused_cpu.hpp:
    # 103-108), far beyond host memory at these tile sizes, and its build needs the reference tree,
    # which is not on this host; the timed CPU (T) is therefore the oracle's C restatement ("port").
    kind = "port"
    q = max(1, args.ref_row_parts)
    rows = -(-v // q)
    for s in range(args.warmup):
        a0 = (s * rows) % v
        oracle.w_rows_sample(d, tri, a0, min(v, a0 + rows))
    times = []
    for s in range(args.steps):
        a0 = (s * rows) % v
        a1 = min(v, a0 + rows)
        t1 = time.perf_counter()
        oracle.w_rows_sample(d, tri, a0, a1)
        times.append((time.perf_counter() - t1) * v / (a1 - a0))   # one triplet's contractions
    per_trip = statistics.mean(times)
    value = per_trip * len(tri_all)
    cores = oracle.num_threads()
    sample = (f"per step: the contraction rows [a0, a0 + {rows}) of {v} (1/{q}) of triplet "
              f"{tuple(int(x) for x in tri)} of {len(tri_all)} (C restatement, OpenMP {cores} threads), "
              f"scaled by {v}/(rows) and by the triplet count; the O(v^3) energy of a triplet is not timed")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times) / q,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator; no dataset)",
        "config": workload_config(o, v, seed) | {"timed_fraction": args.steps / q / len(tri_all),
                                                 "projection": "sampled rows of one triplet x triplets",
                                                 "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "host_generation_s": t_gen,
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(o, v, seed):
    """The workload both arms name (identical strings, so the driver can match them)."""
    occ_tiles, vir_tiles = workload_tiles(o, v, seed)
    return {"workload": f"closed-shell (T) o={o} v={v} seed={seed} ragged tiles", "o": o, "v": v, "seed": seed,
            "occ_tiles": occ_tiles, "vir_tiles": vir_tiles}


def spin_orbital_flops(oa, ob, va, vb):
    """FP64 flops (2 x multiply-adds) of the open-shell path's contractions: per occupied triplet
    i < j < k and permutation p of it, the distinct spin blocks X_p[x][y z] its energy reads, each
    a d-term over the e of one spin and an s-term over the m of one spin where the spins allow."""
    from math import comb
    no, nv = (oa, ob), (va, vb)
    cases = {(0, 0, 0): comb(oa, 3), (0, 0, 1): comb(oa, 2) * ob, (0, 1, 1): oa * comb(ob, 2),
             (1, 1, 1): comb(ob, 3)}
    total = 0
    for (si, sj, sk), count in cases.items():
        if count == 0 or nv[si] * nv[sj] * nv[sk] == 0:
            continue
        pos = [(si, sj, sk), (sj, si, sk), (sk, sj, si)]
        per = 0
        for (s_i, s_j, s_k) in pos:                       # the permutations share the position spins
            for (sx, sy, sz) in set(pos):
                n = nv[sx] * nv[sy] * nv[sz]
                if sx in (s_j, s_k) and s_i + (s_j + s_k - sx) == sy + sz:
                    per += 2 * n * nv[s_j + s_k - sx]
                if s_i in (sy, sz) and s_j + s_k == (sy + sz - s_i) + sx:
                    per += 2 * n * no[sy + sz - s_i]
        total += per * count
    return float(total)


def spin_orbital_launches(oa, ob, va, vb):
    """Kernel launches of one open-shell call: three permutes, then per triplet its GEMM launches
    (up to three blocks each, from the library's own plan) and one energy launch."""
    from itertools import combinations
    from exachem_gb300 import ccsd_t as ct
    nv, n = (va, vb), 3
    for tri in combinations(range(oa + ob), 3):
        if min(nv[int(p >= oa)] for p in tri) == 0:
            continue
        nblk = len(ct.spin_orbital_plan(oa, ob, va, vb, *tri)[1])
        n += -(-nblk // 3) + 1
    return n


def cpu_baseline_open_shell(oa, ob, va, vb, host, budget_s=15.0):
    """The oracle's dense C restatement of the open-shell (T) (oracle/spin_orbital_oracle.c) on
    the host cores, on an evenly spread sample of triplets sized to ~budget_s of CPU time, projected
    by the triplet count (every triplet costs the same 3 V^3 (V + O) multiply-adds there)."""
    import itertools
    import oracle
    tri = list(itertools.combinations(range(oa + ob), 3))
    t0 = time.perf_counter()
    oracle.energy_spin_orbital_c(oa, ob, va, vb, host, tri[:1])
    one = time.perf_counter() - t0
    n = max(1, min(len(tri), int(budget_s / max(one, 1e-6))))
    stride = max(1, len(tri) // n)
    sample = tri[::stride][:n]
    t0 = time.perf_counter()
    oracle.energy_spin_orbital_c(oa, ob, va, vb, host, sample)
    per = (time.perf_counter() - t0) / len(sample)
    return {"value": per * len(tri), "unit": "s", "cores": oracle.num_threads(), "kind": "port",
            "sample": f"{len(sample)} of {len(tri)} triplets (every {stride}-th), dense spin-orbital "
                      f"restatement, projected by triplet count"}


def run_open_shell(args):
    """The open-shell (UHF) (T) through ccsdt_energy_spin_orbital on synthetic spin-orbital inputs:
    value = device time per call with the inputs resident in HBM, e2e = the same call from host
    buffers (copies inside the timed region)."""
    import torch
    from exachem_gb300 import ccsd_t as ct
    oa, ob, va, vb = args.open_shell
    O, V = oa + ob, va + vb
    torch.cuda.set_device(0)
    g = torch.Generator(device="cuda").manual_seed(args.seed)
    rnd = lambda *sh, s: (torch.randn(*sh, generator=g, device="cuda", dtype=torch.float64) * s).contiguous()
    eps_o = -1.0 - torch.rand(O, generator=g, device="cuda", dtype=torch.float64)
    eps_v = 0.3 + torch.rand(V, generator=g, device="cuda", dtype=torch.float64)
    dev = [eps_o, eps_v, rnd(V, O, s=0.02), rnd(V, V, O, O, s=0.02), rnd(O, O, V, V, s=0.05),
           rnd(O, O, O, V, s=0.05), rnd(O, V, V, V, s=0.05)]
    host = [t.cpu().numpy() for t in dev]
    fp64_peak = dgemm_peak_tflops(torch)
    for _ in range(args.warmup):
        ct.energy_spin_orbital(oa, ob, va, vb, *dev)
    torch.cuda.synchronize()
    secs, res = [], None
    clocks = ClockSampler(0)
    clocks.start()
    for _ in range(args.steps):
        res = ct.energy_spin_orbital(oa, ob, va, vb, *dev)
        secs.append(res["seconds"])
    clk = clocks.stop()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r2 = ct.energy_spin_orbital(oa, ob, va, vb, *host)
    e2e = (time.perf_counter() - t0) / args.steps
    value = sum(secs) / len(secs)
    flops = spin_orbital_flops(oa, ob, va, vb)
    from exachem_gb300.generator import tiles_uniform
    ref_ops, _ = ct.reference_op_count_so(*(tiles_uniform(n, 40) for n in (oa, ob, va, vb)))
    ntri = O * (O - 1) * (O - 2) // 6
    # split-precision spin-block contractions (ccsdt_energy_spin_orbital_split) on the same inputs
    split = []
    for S_ in [int(x) for x in args.os_slices.split(",") if x]:
        ct.energy_spin_orbital(oa, ob, va, vb, *dev, slices=S_)
        ts, rs = [], None
        for _ in range(args.steps):
            rs = ct.energy_spin_orbital(oa, ob, va, vb, *dev, slices=S_)
            ts.append(rs["seconds"])
        t_ = sum(ts) / len(ts)
        split.append({"slices": S_, "s_per_call": t_, "speedup_vs_fp64": value / t_,
                      "rel_error_E(T)": abs(rs["e_paren_T"] - res["e_paren_T"]) / abs(res["e_paren_T"]),
                      "rel_error_E[T]": abs(rs["e_bracket_T"] - res["e_bracket_T"]) / abs(res["e_bracket_T"]),
                      "kernel": "oz_gemm_kernel<bf16> (mma.sync) + so_energy_kernel"})
    line = {"metric": f"(T) wall-s open-shell (UHF) FP64 at oa={oa},ob={ob},va={va},vb={vb}", "value": value,
            "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded random spin-orbital tensors on the GPU)",
            "config": {"workload": f"open-shell (T) over spin orbitals oa={oa} ob={ob} va={va} vb={vb}",
                       "triplets": ntri, "l2": f"inputs ({sum(t.numel() for t in dev) * 8 / 1e9:.1f} GB) exceed L2"},
            "roofline": {"bound": "fp64-tensor", "achieved": flops / value / 1e12, "peak": fp64_peak,
                         "unit": "TFLOP/s", "frac": flops / value / 1e12 / fp64_peak, "traffic": None,
                         "kernel": "dmma_gemm_kernel + so_energy_kernel", "flops_per_call": flops,
                         "ref_equiv_tflops": ref_ops / value / 1e12,
                         "ref_ops_per_call": ref_ops, "ref_ops_layout": "unrestricted, tiles of 40",
                         "peak_source": "cuBLAS DGEMM 8192^3 measured in this run, of measured"},
            "cpu_baseline": cpu_baseline_open_shell(oa, ob, va, vb, host) if args.cpu_sample > 0 else None,
            "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": sum(a.nbytes for a in host),
                    "d2h_bytes_per_step": 16},
            "gpu_launches": spin_orbital_launches(oa, ob, va, vb) * args.steps, "clocks": clk,
            "energies": {"e_bracket_T": res["e_bracket_T"], "e_paren_T": res["e_paren_T"],
                         "host_equals_device": r2["e_paren_T"] == res["e_paren_T"]},
            "split_precision": split}
    print(json.dumps(line))
    return 0


def run_cholesky_direct(args):
    """The Cholesky-direct mode against the whole-block Cholesky upload on one system: random spatial
    Cholesky vectors L[p][q][Q] (symmetric in p, q; n_chol = --n-chol, default 4 (o + v)) built on
    the device, the whole (T) call in split precision (--slices) and, on --limit-triplets of them,
    in FP64, first with (ia|bc) whole, then with caches of each --cholesky-direct size.  Reports the
    call times, the slabs formed and the time forming them, and whether the energies are identical."""
    import torch
    from exachem_gb300 import ccsd_t as ct
    from exachem_gb300.generator import generate_device
    torch.cuda.set_device(0)
    o, v, seed = args.o, args.v, args.seed
    nq = args.n_chol or 4 * (o + v)
    wl = workload_config(o, v, seed)
    dev = generate_device(o, v, seed, device="cuda")
    amp = {k: dev[k] for k in ("eps_occ", "eps_vir", "t1", "t2")}
    del dev
    torch.cuda.empty_cache()
    g = torch.Generator(device="cuda").manual_seed(seed + 1000)
    n = o + v
    L = torch.empty((n, n, nq), dtype=torch.float64, device="cuda").normal_(0.0, 0.05, generator=g)
    L = 0.5 * (L + L.transpose(0, 1))
    Loo, Lov, Lvv = (L[:o, :o].contiguous(), L[:o, o:].contiguous(), L[o:, o:].contiguous())
    del L
    torch.cuda.empty_cache()
    stream = torch.cuda.current_stream()
    tri = triplet_list(o)
    fp64_tri = spread_sample(tri, min(len(tri), args.limit_triplets or 8))
    kw = {"slices": args.slices, "p_storage": args.p_storage}

    def run(ft, tr, mode, **k):
        ft.triplet_energies(tr[:1], mode, **k)           # warm: slicing, tensor maps, first slabs
        torch.cuda.synchronize()
        b0 = ft.ovvv_slab_builds()
        t0 = time.perf_counter()
        e4, e5 = ft.triplet_energies(tr, mode, **k)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, e4, e5, ft.ovvv_slab_builds() - b0

    ft = ct.FusedTriples(o, v, wl["occ_tiles"], wl["vir_tiles"], device=0)
    ft.set_stream(stream.cuda_stream)
    ft.upload_cholesky(amp["eps_occ"], amp["eps_vir"], amp["t1"], amp["t2"], Loo, Lov, Lvv)
    t_split, w4, w5, _ = run(ft, tri, "ozaki", **kw)
    t_fp64, f4, f5, _ = run(ft, fp64_tri, "fp64")
    ft.close()
    torch.cuda.empty_cache()
    # the time of one slab: one v x v^2 x n_chol GEMM
    slab_flops = 2.0 * v * v * v * nq
    rows = []
    for C in [int(x) for x in args.cholesky_direct.split(",") if x]:
        ft = ct.FusedTriples(o, v, wl["occ_tiles"], wl["vir_tiles"], device=0)
        ft.set_stream(stream.cuda_stream)
        ft.upload_cholesky(amp["eps_occ"], amp["eps_vir"], amp["t1"], amp["t2"], Loo, Lov, Lvv, max_ovvv_slabs=C)
        ts, s4, s5, bs = run(ft, tri, "ozaki", **kw)
        tf, g4, g5, bf = run(ft, fp64_tri, "fp64")
        rows.append({"max_ovvv_slabs": min(C, o), "split_call_s": ts, "split_slabs_formed": bs,
                     "split_vs_whole": ts / t_split,
                     "split_max_rel_diff": float(np.max(np.abs(s5 - w5) / np.maximum(np.abs(w5), 1e-300))),
                     "split_rel_diff_of_sum": float(abs(s5.sum() - w5.sum()) / abs(w5.sum())),
                     "fp64_sample_s": tf, "fp64_slabs_formed": bf, "fp64_vs_whole": tf / t_fp64,
                     "fp64_identical": bool(np.array_equal(g5, f5) and np.array_equal(g4, f4)),
                     "cache_gb": min(C, o) * v ** 3 * 8 / 1e9})
        print(json.dumps(rows[-1]), file=sys.stderr, flush=True)
        ft.close()
        torch.cuda.empty_cache()
    line = {"metric": f"(T) with (ia|bc) formed slab by slab from Cholesky vectors at o={o},v={v},n_chol={nq}: "
                      "call time vs the whole block",
            "unit": "s", "higher_is_better": False, "n_gpus": 1, "dtype": "f64 / bf16 digit planes",
            "data": "synthetic (seeded amplitudes, random symmetric Cholesky vectors, built on GPU)",
            "config": wl | {"n_chol": nq, "slices": args.slices, "triplets": int(len(tri)),
                            "fp64_sample_triplets": int(len(fp64_tri)), "whole_ovvv_gb": o * v ** 3 * 8 / 1e9,
                            "slab_gemm_flops": slab_flops,
                            "timing": "host wall clock around one call after a warm-up triplet"},
            "whole": {"split_call_s": t_split, "fp64_sample_s": t_fp64},
            "direct": rows}
    print(json.dumps(line), flush=True)
    return 0


def run_slice_sweep(args):
    """Split precision swept over the slice count for BF16 digits (persistent tcgen05 kernel, FP32
    level sums) and INT8 digits (mma.sync IMMA, INT32 level sums), on an evenly spread sample of
    triplets: per (kind, S) the device time per triplet, the projected whole call, the speedup over
    the FP64 path on the same sample and |dE(T)| of the sample against it."""
    import torch
    from exachem_gb300 import ccsd_t as ct
    from exachem_gb300.generator import generate_device
    torch.cuda.set_device(0)
    o, v, seed = args.o, args.v, args.seed
    wl = workload_config(o, v, seed)
    dev = generate_device(o, v, seed, device="cuda")
    ft = ct.FusedTriples(o, v, wl["occ_tiles"], wl["vir_tiles"], device=0)
    ft.upload_dict(dev)
    del dev
    torch.cuda.empty_cache()
    stream = torch.cuda.current_stream()
    ft.set_stream(stream.cuda_stream)
    tri_all = triplet_list(o)
    samp = spread_sample(tri_all, args.sample, offset=len(tri_all) // (2 * args.sample))

    def timed(mode, **kw):
        ft.triplet_energies(samp[:2], mode, **kw)          # warm: slicing, tensor maps, tables
        best, out = None, None
        for _ in range(max(1, args.steps)):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            out = ft.triplet_energies(samp, mode, **kw)
            e1.record(stream)
            torch.cuda.synchronize()
            t = e0.elapsed_time(e1) * 1e-3
            best = t if best is None else min(best, t)
        return best, out

    t64, (f4, f5) = timed("fp64")
    rows = []
    for kind in args.sweep_kinds.split(","):
        for S in [int(x) for x in args.sweep.split(",")]:
            if kind == "bf16" and not args.no_autotune:
                ft.autotune(S)
            t, (s4, s5) = timed("ozaki", slices=S, slice_kind=kind)
            rel = np.abs(s5 - f5) / np.abs(f5)
            rows.append({"kind": kind, "slices": S, "s_per_triplet": t / len(samp),
                         "whole_call_s": t / len(samp) * len(tri_all), "speedup_vs_fp64": t64 / t,
                         "rel_error_of_sum": float(abs(s5.sum() - f5.sum()) / abs(f5.sum())),
                         "max_rel_triplet": float(rel.max()),
                         "kernel": "persistent tcgen05 (BF16 digits)" if kind == "bf16" else "mma.sync IMMA (INT8 digits)"})
            print(json.dumps(rows[-1]), file=sys.stderr, flush=True)
    line = {"metric": f"(T) split-precision slice sweep at o={o},v={v}: |dE(T)| and speedup vs FP64 per slice count",
            "unit": "s", "higher_is_better": False, "n_gpus": 1, "steps": args.steps, "dtype": "f64 / bf16 / int8",
            "data": "synthetic (seeded generator, built on GPU)",
            "config": wl | {"sample_triplets": int(len(samp)), "triplets_total": int(len(tri_all)),
                            "timing": "best of the timed repetitions, CUDA events around one call on the sample"},
            "fp64": {"s_per_triplet": t64 / len(samp), "whole_call_s": t64 / len(samp) * len(tri_all),
                     "sum_E(T)_sample": float(f5.sum())},
            "sweep": rows}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10,
                    help="timed steps; in split mode they partition every triplet of the call")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="auto", choices=["auto", "fp64", "ozaki", "learned"])
    ap.add_argument("--slices", type=int, default=2,
                    help="digit planes of the timed call (2: the fewest whose whole-call |dE(T)|/|E(T)| "
                         "stays below 1e-6 at this shape, measured 3.5e-8)")
    ap.add_argument("--o", type=int, default=60)
    ap.add_argument("--v", type=int, default=500)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--fp64-batch", type=int, default=2, help="triplets per step in fp64 mode")
    ap.add_argument("--warm-batch", type=int, default=16, help="triplets per warm-up step")
    ap.add_argument("--sample", type=int, default=48,
                    help="evenly spread triplets of the parity sample against the FP64 path (0: skip)")
    ap.add_argument("--sample-slices", default="2,3,4", help="slice counts checked on the parity sample")
    ap.add_argument("--cpu-sample", type=int, default=1, help="triplets timed on the CPU baseline (0: skip)")
    ap.add_argument("--ref-row-parts", type=int, default=4,
                    help="--impl reference: each step times 1/q of one triplet's contraction rows")
    ap.add_argument("--limit-triplets", type=int, default=0,
                    help="profiling aid: run only this many evenly spread triplets of the call (projected)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--p-storage", default="auto", choices=["auto", "ff", "f32", "f64"],
                    help="split path: partial arrays in FP32 (auto: at 1-3 digit planes) or float-float")
    ap.add_argument("--budget", type=float, default=1e-8,
                    help="learned mode: 3 sum_t sigma_t <= budget x sum_t |E(T)_t| (1e-8: two planes miss it at "
                         "o=60 v=500, three meet it)")
    ap.add_argument("--no-learned", action="store_true", help="no learned-mode entry in the parity sample")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default tile configurations (no ccsdt_autotune before the timed region)")
    ap.add_argument("--open-shell", type=lambda x: tuple(int(y) for y in x.split(",")), default=None,
                    metavar="OA,OB,VA,VB", help="time the open-shell (UHF) path on this spin-orbital system instead")
    ap.add_argument("--sweep", default=None, metavar="S1,S2,...",
                    help="slice-count sweep on a triplet sample instead of the whole call (e.g. 4,5,6,7,8)")
    ap.add_argument("--sweep-kinds", default="bf16,int8", help="digit kinds of the sweep")
    ap.add_argument("--cholesky-direct", default=None, metavar="C1,C2,...",
                    help="Cholesky-direct mode: whole call with (ia|bc) slab caches of these sizes vs the whole block")
    ap.add_argument("--n-chol", type=int, default=0, help="Cholesky vectors for --cholesky-direct (0: 4 (o + v))")
    ap.add_argument("--os-slices", default="3,4", help="--open-shell: slice counts of the split-precision calls")
    ap.add_argument("--graph-sample", type=int, default=768,
                    help="triplets of the eager vs CUDA-graph comparison (split mode; 0: skip)")
    args = ap.parse_args()
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        return run_reference(args)
    if args.open_shell:
        return run_open_shell(args)
    if args.cholesky_direct:
        return run_cholesky_direct(args)
    if args.sweep:
        return run_slice_sweep(args)

    import torch
    from exachem_gb300 import ccsd_t as ct
    from exachem_gb300.generator import generate_device

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    mode = "ozaki" if args.mode == "auto" else args.mode
    split = mode != "fp64"
    o, v, seed = args.o, args.v, args.seed
    wl = workload_config(o, v, seed)
    occ_tiles, vir_tiles = wl["occ_tiles"], wl["vir_tiles"]
    S = args.slices

    t0 = time.perf_counter()
    dev = generate_device(o, v, seed, device="cuda")
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0
    fp64_peak = dgemm_peak_tflops(torch)

    tri_all = triplet_list(o)
    mine = tri_all[rank::world]                       # independent triplets, no data-path collective
    n_share = len(mine)
    if args.limit_triplets > 0:                          # profiling runs: a spread subset, projected
        mine = spread_sample(mine, min(len(mine), args.limit_triplets))
    cpu_samp = spread_sample(tri_all, max(1, args.cpu_sample), offset=len(tri_all) // 2)
    host_slabs = host_slabs_from_device(dev, cpu_samp) if (rank == 0 and args.cpu_sample > 0) else None
    keys = ["eps_occ", "eps_vir", "t1", "t2", "oovv", "ooov", "ovvv"]
    host = None
    if not args.no_e2e:                                 # pinned host copies: the e2e call's inputs
        try:
            host = {k: torch.empty(dev[k].shape, dtype=torch.float64, pin_memory=True) for k in keys}
        except RuntimeError:
            host = {k: torch.empty(dev[k].shape, dtype=torch.float64) for k in keys}
        for k in keys:
            host[k].copy_(dev[k])

    ft = ct.FusedTriples(o, v, occ_tiles, vir_tiles, device=local)
    ft.upload_dict(dev)
    del dev
    torch.cuda.empty_cache()
    stream = torch.cuda.current_stream()
    ft.set_stream(stream.cuda_stream)
    kw = {"slices": S, "p_storage": args.p_storage} if split else {}
    model = None
    if mode == "learned" or (mode == "ozaki" and not args.no_learned and args.sample > 0):
        from exachem_gb300 import learned
        model, _ = learned.load_model()                  # the shipped slice-count model
        learned.set_model(ft, model)
    lkw = {"slices": 5, "energy_budget": args.budget, "budget_triplets": int(len(tri_all)),
           "p_storage": args.p_storage}
    if mode == "learned":
        # each timed call is held to the same relative budget as the whole (T) (linear acceptance)
        kw = dict(lkw)

    # the contraction's tile configuration for each slice count this run uses, tuned on this system
    # before anything is timed (every configuration gives bit-identical energies)
    sample_slices = [int(x) for x in args.sample_slices.split(",") if x] if args.sample > 0 else []
    tile = None
    if split and not args.no_autotune:
        tile = {}
        used = {S} | set(sample_slices) | (set(range(1, 6)) if model is not None else set())
        for s_ in sorted(x for x in used if 1 <= x <= 5):
            ms_c, chosen = ft.autotune(s_)
            tile[str(s_)] = {"nt_st_kc": list(ct.FusedTriples.tile_configs(s_)[chosen]),
                             "ms_per_config": [round(x, 3) for x in ms_c]}

    # steps: split mode partitions every triplet of this rank's share into K batches (the whole
    # call, nothing projected); FP64 mode (hours at this size) times an evenly spread sample
    if split:
        order = np.array_split(np.arange(len(mine)), args.steps)
        batches = [mine[ix] for ix in order if len(ix)]
    else:
        batches = [spread_sample(mine, args.fp64_batch, offset=s) for s in range(args.steps)]
    warm = [spread_sample(mine, max(1, args.warm_batch), offset=len(mine) // 3 + s) for s in range(args.warmup)]
    for b in warm:
        ft.triplet_energies(b, mode, **kw)
    torch.cuda.synchronize()

    # one whole (T) call through the C ABI: upload from pinned host buffers (timed for e2e), then
    # the K steps on the resident inputs (the value; the first step also slices the operands into
    # digit planes, as every call after an upload does), each step's energies read back to the host
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    harr = {k: host[k].numpy() for k in keys} if host is not None else None
    t_up0 = time.perf_counter()
    if harr is not None:
        ft.upload(*[harr[k] for k in keys])          # host -> device, repacks, finiteness check
    torch.cuda.synchronize()
    t_up1 = time.perf_counter()
    if dist:
        dist.barrier()
    if split:
        ft.set_phase_timing(True)                        # CUDA events around each phase, live
    clocks.start()
    launches = 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t_v0 = time.perf_counter()
    e0.record(stream)
    esum4, esum5 = 0.0, 0.0
    for b in batches:
        g4, g5 = ft.triplet_energies(b, mode, **kw)      # returns host arrays (device -> host read)
        esum4 += float(g4.sum())
        esum5 += float(g5.sum())
        launches += ft.launch_count()
    e1.record(stream)
    torch.cuda.synchronize()
    t_v1 = time.perf_counter()
    clk = clocks.stop()
    elapsed = e0.elapsed_time(e1) * 1e-3
    e2e_wall = (t_up1 - t_up0) + (t_v1 - t_v0)
    timed_trip = sum(len(b) for b in batches)
    if dist:
        t = torch.tensor([elapsed, e2e_wall], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed, e2e_wall = (float(x) for x in t.tolist())
    frac = timed_trip / n_share
    value = elapsed / frac                               # == elapsed in split mode (frac 1)
    pt = None
    if split:
        pt = ft.phase_times()
        ft.set_phase_timing(False)

    # roofline of the dominant kernel.  FP64 path: the d-sum contraction launch (12 v^4 flops per
    # triplet: 3 arrays x 2 terms x v^4 multiply-adds).  Split path: the contraction launch with
    # the l-sum and d-sum terms of a batch (12 v^3 (v + o) FP64-equivalent flops per triplet)
    fp64_eq = 12.0 * float(v) ** 4
    peaks = measured_peaks()
    if not split:
        # the fused kernel: all twelve contractions of a triplet and its energy in one launch
        i, j, k = (int(x) for x in mine[len(mine) // 2])
        prof = [ft.profile_triplet(i, j, k, mode, **kw) for _ in range(3)]
        gemm_ms = statistics.median(p[1] for p in prof)
        per_launch = 12.0 * float(v) ** 3 * (v + o)
        peak, peak_src = fp64_peak, "measured (cuBLAS DGEMM 8192^3 in this run; FP64 is not in MEASURED_PEAKS.json)"
        kernel = "t3_fused_fp64_kernel"
        phase = dict(zip(["l_sum", "fused_contraction_and_energy", "energy", "reduce"], prof[1]))
        timing = "profile_triplet: CUDA events around one triplet's launches, after the timed region"
    else:
        nb, ntr = max(1, pt["batches"]), max(1, pt["triplets"])
        gemm_ms = pt["contraction_ms"] / nb                 # average contraction launch (one batch)
        fp64_eq = 12.0 * float(v) ** 3 * (v + o)           # l-sum and d-sum terms run in the same launch
        prods = S * (S + 1) / 2 if mode == "ozaki" else None
        per_launch = fp64_eq * (prods or 1.0) * ntr / nb   # BF16 digit-plane products of one launch
        peak = peaks.get("bf16_tflops_sustained") or peaks.get("bf16_tflops", 1900.0)
        peak_src = ("MEASURED_PEAKS.json bf16_tflops_sustained (the launches run back to back for minutes), "
                    "of measured")
        kernel = "oz_persist_kernel"                       # the persistent tcgen05 contraction
        phase = {"contraction_per_triplet": pt["contraction_ms"] / ntr, "energy_per_triplet": pt["energy_ms"] / ntr,
                 "batches": pt["batches"], "triplets_per_batch": ntr / nb}
        timing = "live CUDA events on the launching stream around each batch's contraction launch in the timed region"
    achieved = per_launch / (gemm_ms * 1e-3) / 1e12
    roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": profile_traffic(kernel), "kernel": kernel,
            "per_launch_flops": per_launch, "launch_ms": gemm_ms, "peak_source": peak_src,
            "fp64_equivalent_tflops": (fp64_eq * ntr / nb if split else per_launch) / (gemm_ms * 1e-3) / 1e12,
            "phase_ms": phase, "timing": timing}
    if split and mode != "ozaki":
        roof["note"] = "learned mode: per-launch flops counted at one digit-plane product (lower bound)"
    # whole-call throughput in the reference's own op count (ccsd_t.cpp:332 reports this as gflops)
    # and in the closed-shell algorithmic count 2 o^3 v^3 (o + v)
    ref_ops, ref_tasks = ct.reference_op_count(o, v, occ_tiles, vir_tiles)
    throughput = {"ref_equiv_tflops": ref_ops / value / 1e12, "ref_ops_per_call": ref_ops, "ref_tasks": ref_tasks,
                  "closed_shell_tflops": 2.0 * o ** 3 * v ** 3 * (o + v) / value / 1e12,
                  "note": "whole-call seconds; the reference's count is its spin-orbital op count for this layout"}

    # parity sample: evenly spread triplets, the FP64 path against each slice count (and the learned
    # mode), per-triplet relative errors and the error of their sum; the FP64 time of the sample
    # also gives the plain-FP64 whole-call projection (~9 hours at this size)
    # the per-batch launch sequence replayed from a CUDA graph (opts.use_graph) against the eager
    # launches the timed region uses (eager there: per-launch events feed the roofline), on a sample
    cuda_graph = None
    if rank == 0 and mode == "ozaki" and args.graph_sample > 0:
        gs = spread_sample(mine, min(len(mine), args.graph_sample))
        res = {}
        for name, g_ in (("eager", 0), ("graph", 1)):
            ft.triplet_energies(gs[:8], mode, use_graph=g_, **kw)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r4, r5 = ft.triplet_energies(gs, mode, use_graph=g_, **kw)
            torch.cuda.synchronize()
            res[name] = (time.perf_counter() - t0, r4, r5)
        cuda_graph = {"triplets": int(len(gs)), "eager_s": res["eager"][0], "graph_s": res["graph"][0],
                      "identical": bool(np.array_equal(res["eager"][2], res["graph"][2]) and
                                        np.array_equal(res["eager"][1], res["graph"][1])),
                      "graph_replays": "one capture of a batch's contraction, energy, reduction and base advance, "
                                       "replayed for every full batch"}

    energy_sample, fp64_proj = None, None
    if rank == 0 and split and args.sample > 0:
        samp = spread_sample(tri_all, args.sample, offset=len(tri_all) // (2 * args.sample))
        ft.triplet_energies(samp[:1], "fp64")
        torch.cuda.synchronize()
        ta = time.perf_counter()
        f4, f5 = ft.triplet_energies(samp, "fp64")
        fp64_s = time.perf_counter() - ta
        fp64_proj = fp64_s / len(samp) * len(tri_all) / world
        nz = np.abs(f5) > 0
        entries = {}
        runs = [(f"S={s_}", "ozaki", {"slices": s_, "p_storage": args.p_storage}) for s_ in sample_slices]
        for s_ in (2, 3):   # what the FP32 partial arrays cost in accuracy
            if args.p_storage == "auto" and s_ in sample_slices:
                runs.append((f"S={s_} float-float partial arrays", "ozaki", {"slices": s_, "p_storage": "ff"}))
        if model is not None:
            runs.append(("learned", "learned", lkw))
        for name, m_, k_ in runs:
            s4, s5 = ft.triplet_energies(samp, m_, **k_)
            rel = np.abs(s5[nz] - f5[nz]) / np.abs(f5[nz])
            entries[name] = {"max_rel_triplet": float(rel.max()), "median_rel_triplet": float(np.median(rel)),
                             "rel_error_of_sum": float(abs(s5.sum() - f5.sum()) / abs(f5.sum())),
                             "abs_error_of_sum_Eh": float(abs(s5.sum() - f5.sum())),
                             "rel_error_of_sum_E[T]": float(abs(s4.sum() - f4.sum()) / abs(f4.sum()))}
        # the learned mode's a-posteriori estimate sigma_t of each triplet's truncation error, against
        # the measured error: how often the 3-sigma band misses (a statistical estimate, not a bound)
        sigma = {}
        for s_ in (2, 3):
            _, e5s, est = ft.triplet_error_estimates(samp, s_)
            err = np.abs(e5s[nz] - f5[nz])
            sigma[f"S={s_}"] = {"miss_rate_3sigma": float(np.mean(err > 3 * est[nz])),
                                "median_sigma_over_error": float(np.median(est[nz] / np.maximum(err, 1e-300)))}
        energy_sample = {"triplets": int(len(samp)), "spread": "evenly over the lexicographic list",
                         "error_estimate": sigma,
                         "fp64_sum_E(T)_Eh": float(f5.sum()), "fp64_seconds": fp64_s, "vs_fp64": entries,
                         "tolerance": "|dE|/|E(T)| <= 1e-6 (the metric's 1e-6 Eh for any |E(T)| <= 1 Eh; the "
                                      "synthetic E(T) here is ~1e11 Eh, so absolute Eh bounds are below one ulp)"}

    # CPU baseline: the oracle's C restatement on this host, on the sample triplet(s)
    cpu = None
    if host_slabs is not None:
        t_cpu, (c4, c5), cores = cpu_baseline_port(host_slabs, cpu_samp)
        g4, g5 = ft.triplet_energies(cpu_samp, "fp64")
        cpu = {"value": t_cpu / len(cpu_samp) * len(tri_all), "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{len(cpu_samp)} triplet(s) {cpu_samp.tolist()} of {len(tri_all)} at o={o} v={v} "
                         f"(oracle C restatement, {cores} OpenMP threads, {t_cpu:.1f} s), projected to the whole call",
               "fp64_gpu_vs_cpu_max_rel": float(np.max(np.abs(g5 - c5) / np.abs(c5)))}

    e2e = None
    if harr is not None:
        h2d = sum(a.nbytes for a in harr.values())
        e2e = {"value": e2e_wall / frac, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": 16 * int(round(timed_trip / max(1, len(batches)))),
               "upload_s": t_up1 - t_up0, "energy_calls_s": t_v1 - t_v0,
               "what": "one whole (T) call through the C ABI: ccsdt_upload from pinned host buffers (the "
                       "h2d bytes, once per call) and every batch of ccsdt_triplet_energies (energies read "
                       "back each step), host wall clock" + ("" if frac >= 1 else "; projected by the timed fraction")}
        del host, harr

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / max(1, len(batches)),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if not split else "bf16 digit planes (exact FP32 levels), float-float recombination",
            "data": "synthetic (seeded generator, built on GPU)",
            "config": wl | {"mode": mode, "slices": S if mode == "ozaki" else None, "tile_config": tile,
                            "partial_arrays": None if not split else (
                                "FP64 (FP64 recombination and energy)" if args.p_storage == "f64" else
                                "FP32" if args.p_storage == "f32" or (args.p_storage == "auto" and mode == "ozaki"
                                                                      and S <= 3)
                                else "float-float" if mode == "ozaki" or args.p_storage == "ff"
                                else "FP32 at 1-3 digit planes, float-float above"),
                            "triplets_total": int(len(tri_all)), "triplets_timed": int(timed_trip),
                            "timed_fraction": frac,
                            "projection": None if frac >= 1 else "value = timed seconds / timed_fraction",
                            "warmup_steps": f"{args.warmup} x {max(1, args.warm_batch)} triplets",
                            "l2": "inputs (75 GB) and per-batch scratch (12 GB) exceed L2; no flush"},
            "roofline": roof, "throughput": throughput, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": launches, "clocks": clk, "energy_sample": energy_sample, "cuda_graph": cuda_graph,
            "partial_energy_timed": {"e_bracket_T": esum4, "e_paren_T": esum5},
            "fp64_projected_s": fp64_proj, "speedup_vs_fp64": (fp64_proj / value) if fp64_proj else None,
            "setup": {"generate_s": t_gen, "fp64_dgemm_tflops": fp64_peak},
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
