#!/usr/bin/env python
"""(T) wall-seconds at o=60, v=500 on GB300: split precision vs plain FP64.

Workload (the shape the headline metric is quoted on): closed-shell (T), o=60 occupied,
v=500 virtual orbitals, seed 3, tile extents drawn per index range from {16,24,32,40,48},
synthetic inputs from exachem_gb300.generator (built on the GPU, ovvv 60 GB in HBM).

A step is one batch of occupied triplets (i <= j <= k) of that workload, run through the
C ABI on inputs already resident in HBM.  ``value`` is the wall time of the whole (T)
call: with --mode ozaki the K timed steps cover every triplet once (timed_fraction 1);
with --mode fp64 (hours at this size) the timed steps cover a fixed, evenly spread sample
of triplets and the whole-call time is projected from it (timed_fraction < 1, stated).

--impl reference times the reference's CPU (T) on the host cores (the C restatement of
the oracle where the reference's own build is not present) on a bounded sample of the
same workload and projects the whole-call time the same way.
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
    """CPU (T) of the reference on the host cores (bounded sample, projected)."""
    import oracle
    from exachem_gb300.generator import generate_host_slabs
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    o, v, seed = args.o, args.v, args.seed
    tri_all = triplet_list(o)
    sample = spread_sample(tri_all, 1, offset=len(tri_all) // 2)
    t0 = time.perf_counter()
    d = generate_host_slabs(o, v, seed, sample.ravel())
    t_gen = time.perf_counter() - t0
    # ExaChem's own CPU kernel materialises two ts^6 t3 blocks per task (ccsd_t_all_fused_cpu.hpp:
    # 103-108), far beyond host memory at these tile sizes, and its build needs the reference
    # tree; the timed CPU (T) is therefore the oracle's C restatement ("port").
    kind = "port"
    for _ in range(args.warmup):
        oracle.triplets_slabs(d, sample)
    times = []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        oracle.triplets_slabs(d, sample)
        times.append(time.perf_counter() - t1)
    per_trip = statistics.mean(times) / len(sample)
    value = per_trip * len(tri_all)
    cores = oracle.num_threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator; no dataset)",
        "config": {"workload": f"closed-shell (T) o={o} v={v} seed={seed}", "o": o, "v": v,
                   "timed_fraction": len(sample) / len(tri_all), "projection": "per-triplet CPU time x triplets",
                   "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"triplet {tuple(int(x) for x in sample[0])} of {len(tri_all)} "
                                   f"(C restatement, OpenMP {cores} threads), projected to the whole call"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "host_generation_s": t_gen,
    }
    print(json.dumps(line), flush=True)
    return 0


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
                         "host_equals_device": r2["e_paren_T"] == res["e_paren_T"]}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="auto", choices=["auto", "fp64", "ozaki", "learned"])
    ap.add_argument("--slices", type=int, default=3)
    ap.add_argument("--o", type=int, default=60)
    ap.add_argument("--v", type=int, default=500)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--fp64-batch", type=int, default=2, help="triplets per step in fp64 mode")
    ap.add_argument("--batch", type=int, default=48, help="triplets per step in split mode")
    ap.add_argument("--cpu-sample", type=int, default=1, help="triplets timed on the CPU baseline (0: skip)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--budget", type=float, default=1e-8,
                    help="learned mode: 3 sqrt(sum sigma_t^2) <= budget x sum |E(T)_t|")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-mode side measurement")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default tile configurations (no ccsdt_autotune before the timed region)")
    ap.add_argument("--open-shell", type=lambda x: tuple(int(y) for y in x.split(",")), default=None,
                    metavar="OA,OB,VA,VB", help="time the open-shell (UHF) path on this spin-orbital system instead")
    args = ap.parse_args()
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        return run_reference(args)
    if args.open_shell:
        return run_open_shell(args)

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

    mode = args.mode
    if mode == "auto":
        mode = "ozaki"
    o, v, seed = args.o, args.v, args.seed
    occ_tiles, vir_tiles = workload_tiles(o, v, seed)
    S = args.slices

    t0 = time.perf_counter()
    dev = generate_device(o, v, seed, device="cuda")
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0
    fp64_peak = dgemm_peak_tflops(torch)

    tri_all = triplet_list(o)
    mine = tri_all[rank::world]                       # independent triplets, no data-path collective
    cpu_samp = spread_sample(tri_all, max(1, args.cpu_sample), offset=len(tri_all) // 2)
    host_slabs = host_slabs_from_device(dev, cpu_samp) if (rank == 0 and args.cpu_sample > 0) else None
    keys = ["eps_occ", "eps_vir", "t1", "t2", "oovv", "ooov", "ovvv"]
    host = None
    if not args.no_e2e and rank == 0:
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
    kw = {"slices": S} if mode != "fp64" else {}
    model = None
    if mode == "learned" or (mode == "ozaki" and not args.no_learned):
        from exachem_gb300 import learned
        model, _ = learned.load_model()                  # the shipped slice-count model
        learned.set_model(ft, model)
    if mode == "learned":
        # each timed call is a part of the whole (T) over all triplets: its acceptance share
        kw = {"slices": 5, "energy_budget": args.budget, "budget_triplets": int(len(tri_all))}

    # the contraction's tile configuration for each slice count this run uses, tuned on this system
    # before anything is timed (every configuration gives bit-identical energies)
    tile = None
    if mode != "fp64" and not args.no_autotune:
        tile = {}
        for s_ in sorted({S} | (set(range(1, 6)) if model is not None else set())):
            ms_c, chosen = ft.autotune(s_)
            tile[str(s_)] = {"nt_st_kc": list(ct.FusedTriples.tile_configs(s_)[chosen]),
                             "ms_per_config": [round(x, 3) for x in ms_c]}

    per_step = args.fp64_batch if mode == "fp64" else args.batch
    batches = [spread_sample(mine, per_step, offset=s) for s in range(args.steps)]
    warm = [spread_sample(mine, max(1, per_step // 4), offset=len(mine) // 3 + s) for s in range(args.warmup)]
    for b in warm:
        ft.triplet_energies(b, mode, **kw)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()

    split = mode != "fp64"
    if split:
        ft.set_phase_timing(True)                        # CUDA events around each phase, live
    clocks = ClockSampler(local)
    clocks.start()
    launches = 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    esum4, esum5 = 0.0, 0.0
    for b in batches:
        g4, g5 = ft.triplet_energies(b, mode, **kw)
        esum4 += float(g4.sum())
        esum5 += float(g5.sum())
        launches += ft.launch_count()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    elapsed = e0.elapsed_time(e1) * 1e-3
    timed_trip = sum(len(b) for b in batches)
    if dist:
        t = torch.tensor([elapsed], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    frac = timed_trip / len(mine)
    value = elapsed / frac                               # whole call (all triplets) on N GPUs
    pt = None
    if split:
        pt = ft.phase_times()
        ft.set_phase_timing(False)

    # roofline of the dominant kernel.  FP64 path: the d-sum contraction launch (12 v^4 flops per
    # triplet: 3 arrays x 2 terms x v^4 multiply-adds).  Split path: the contraction launch with
    # the l-sum and d-sum terms of a batch (12 v^3 (v + o) FP64-equivalent flops per triplet)
    fp64_eq = 12.0 * float(v) ** 4
    peaks = measured_peaks()
    if mode == "fp64":
        # per-phase device times of one representative triplet (one launch per triplet)
        i, j, k = (int(x) for x in mine[len(mine) // 2])
        prof = [ft.profile_triplet(i, j, k, mode, **kw) for _ in range(3)]
        gemm_ms = statistics.median(p[1] for p in prof)
        per_launch = fp64_eq
        peak, peak_src = fp64_peak, "measured (cuBLAS DGEMM 8192^3 in this run; FP64 is not in MEASURED_PEAKS.json)"
        kernel = "dmma_gemm_kernel"
        phase = dict(zip(["l_sum", "d_sum", "energy", "reduce"], prof[1]))
        timing = "profile_triplet: CUDA events around one triplet's launches, after the timed region"
    else:
        # live: CUDA events around every batch's launches inside the timed region
        nb, ntr = max(1, pt["batches"]), max(1, pt["triplets"])
        gemm_ms = pt["contraction_ms"] / nb                 # average contraction launch (one batch)
        fp64_eq = 12.0 * float(v) ** 3 * (v + o)           # l-sum and d-sum terms run in the same launch
        per_launch = fp64_eq * S * (S + 1) / 2 * ntr / nb  # BF16 digit-plane products of one launch
        peak, peak_src = peaks.get("bf16_tflops", 1900.0), "MEASURED_PEAKS.json bf16_tflops (burst), of measured"
        kernel = "oz_pair_kernel"                          # the two-CTA cluster contraction (default path)
        phase = {"contraction_per_triplet": pt["contraction_ms"] / ntr, "energy_per_triplet": pt["energy_ms"] / ntr,
                 "batches": pt["batches"], "triplets_per_batch": ntr / nb}
        timing = "live CUDA events on the launching stream around each batch's contraction launch in the timed region"
    achieved = per_launch / (gemm_ms * 1e-3) / 1e12
    roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": profile_traffic(kernel), "kernel": kernel,
            "per_launch_flops": per_launch, "launch_ms": gemm_ms, "peak_source": peak_src,
            "fp64_equivalent_tflops": (per_launch / (S * (S + 1) / 2) if split else per_launch)
                                      / (gemm_ms * 1e-3) / 1e12,
            "phase_ms": phase, "timing": timing}

    # plain FP64 on the same shape (projected from a few triplets) and |dE| on the CPU sample
    # learned slice count on the same batches (side measurement; the headline is the fixed count)
    learned_line = None
    if mode == "ozaki" and model is not None:
        from exachem_gb300 import learned
        lkw = {"slices": 5, "energy_budget": args.budget, "budget_triplets": int(len(tri_all))}
        ft.triplet_energies(warm[0], "learned", **lkw)
        torch.cuda.synchronize()
        l0, l1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0.record(stream)
        mean_s, esc, prods = [], 0, 0.0
        for b in batches:
            ft.triplet_energies(b, "learned", **lkw)
            m, e, pr = learned.learned_stats(ft, with_products=True)
            mean_s.append(m)
            esc += e
            prods += pr
        l1.record(stream)
        torch.cuda.synchronize()
        l_elapsed = l0.elapsed_time(l1) * 1e-3
        learned_line = {"value": l_elapsed / frac, "unit": UNIT, "budget": args.budget,
                        "acceptance": "3 sqrt(sum sigma_t^2) <= budget x sum |E(T)_t| over the whole call "
                                      "(each batched call takes its sqrt(n_call / n_total) share)",
                        "mean_predicted_slices": float(np.mean(mean_s)), "escalations": int(esc),
                        "digit_plane_products_per_triplet": prods / max(1, timed_trip),
                        "fixed_count_products_per_triplet": S * (S + 1) / 2}

    fp64_proj, dE = None, None
    if rank == 0 and mode != "fp64":
        fb = spread_sample(mine, args.fp64_batch, offset=7)
        ft.triplet_energies(fb[:1], "fp64")
        torch.cuda.synchronize()
        ta = time.perf_counter()
        ft.triplet_energies(fb, "fp64")
        torch.cuda.synchronize()
        fp64_proj = (time.perf_counter() - ta) / len(fb) * len(tri_all) / world
        f4, f5 = ft.triplet_energies(cpu_samp, "fp64")
        s4, s5 = ft.triplet_energies(cpu_samp, mode, **kw)
        dE = {"triplets": cpu_samp.tolist(), "rel_E(T)_vs_fp64": (np.abs(s5 - f5) / np.abs(f5)).tolist(),
              "rel_E[T]_vs_fp64": (np.abs(s4 - f4) / np.abs(f4)).tolist()}
        if learned_line is not None:
            # one call of 4 triplets in learned mode against FP64 (the acceptance test is on a
            # call's total; FP64 takes ~0.85 s per triplet at this size)
            lb = batches[0][:4]
            _, lf5 = ft.triplet_energies(lb, "fp64")
            _, ll5 = ft.triplet_energies(lb, "learned", slices=5, energy_budget=args.budget,
                                         budget_triplets=int(len(tri_all)))
            learned_line["sample_rel_error_of_sum"] = float(abs(ll5.sum() - lf5.sum()) / np.abs(lf5).sum())
            learned_line["sample"] = "4 triplets of the first batch, one call, against the FP64 path"

    # end to end through the C ABI with host (pinned) buffers: upload + one batch + readback
    e2e = None
    if host is not None:
        harr = {k: host[k].numpy() for k in keys}
        h2d = sum(a.nbytes for a in harr.values())
        b1, b2 = batches[0], batches[-1]
        torch.cuda.synchronize()
        ta = time.perf_counter()
        ft.upload(*[harr[k] for k in keys])              # host -> device, repacks, finiteness check
        torch.cuda.synchronize()
        tb = time.perf_counter()
        ft.triplet_energies(b1, mode, **kw)              # first call after an upload: digit planes too
        tc = time.perf_counter()
        ft.triplet_energies(b2, mode, **kw)              # steady state, results read back to the host
        td = time.perf_counter()
        per_trip = (td - tc) / len(b2)
        n_mine = len(tri_all) / world
        e2e_val = (tb - ta) + (tc - tb) + per_trip * (n_mine - len(b1))
        e2e = {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 16 * len(b2),
               "upload_s": tb - ta, "first_batch_s": tc - tb, "steady_per_triplet_s": per_trip,
               "projection": "upload + first batch (slices the operands) + steady per-triplet API time x rest"}
        del host, harr

    # CPU baseline: the oracle's C restatement on this host, on the sample triplet(s)
    cpu = None
    if host_slabs is not None:
        t_cpu, (c4, c5), cores = cpu_baseline_port(host_slabs, cpu_samp)
        g4, g5 = ft.triplet_energies(cpu_samp, "fp64")
        cpu = {"value": t_cpu / len(cpu_samp) * len(tri_all), "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{len(cpu_samp)} triplet(s) {cpu_samp.tolist()} of {len(tri_all)} at o={o} v={v} "
                         f"(oracle C restatement, {cores} OpenMP threads, {t_cpu:.1f} s), projected to the whole call",
               "fp64_gpu_vs_cpu_max_rel": float(np.max(np.abs(g5 - c5) / np.abs(c5)))}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / max(1, len(batches)),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if mode == "fp64" else "bf16 digit planes (exact FP32 levels), float-float recombination",
            "data": "synthetic (seeded generator, built on GPU)",
            "config": {"workload": f"closed-shell (T) o={o} v={v} seed={seed} ragged tiles", "o": o, "v": v,
                       "mode": mode, "slices": S if mode != "fp64" else None, "tile_config": tile,
                       "occ_tiles": occ_tiles, "vir_tiles": vir_tiles, "triplets_total": int(len(tri_all)),
                       "triplets_timed": int(timed_trip), "timed_fraction": frac,
                       "projection": None if frac >= 1 else "value = timed seconds / timed_fraction",
                       "l2": "inputs (75 GB) and per-triplet scratch (3 GB) exceed L2; no flush"},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
            "energy_sample": dE, "partial_energy_timed": {"e_bracket_T": esum4, "e_paren_T": esum5},
            "learned": learned_line,
            "fp64_projected_s": fp64_proj, "speedup_vs_fp64": (fp64_proj / value) if fp64_proj else None,
            "setup": {"generate_s": t_gen, "fp64_dgemm_tflops": fp64_peak},
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
