"""Training data, training and use of the per-triplet slice-count model.

Labels: for the sampled triplets of a system, the digit-plane counts S in 2..smax that a greedy
allocation gives under the LEARNED mode's own acceptance test 3 sum_t sigma_t <= budget
sum_t |E_t| (sigma_t: the library's a-posteriori error estimate of triplet t at its count): all
start at 2 and the triplet with the largest sigma_t moves up one count until the test passes
(label_triplets), against half the budget the
model will run with (a safety margin: an underestimate costs a rerun).  The measured errors against
the library's own FP64 path are kept beside the labels.  Features come from the library
(ccsdt_triplet_features, 12 per triplet).  Training runs on the GPU through ccsdt_mlp_train
(hand-written FP32 forward / backward / Adam kernels).

The allowance scales with the system's own energies: with the synthetic generator triplet
energies range over many decades (1e-6 .. 1e7 Eh), so a fixed absolute budget would be either
unreachable or void.
"""
from __future__ import annotations

import ctypes
import json
from pathlib import Path

import numpy as np

from . import ccsd_t as ct

MODEL_PATH = Path(__file__).resolve().parent / "slice_model.json"
NPARAM = 64 * 12 + 64 + 64 * 64 + 64 + 7 * 64 + 7
_F = ctypes.POINTER(ctypes.c_float)
_I = ctypes.POINTER(ctypes.c_int)


def _lib():
    lib = ct.load_library()
    lib.ccsdt_mlp_grad.argtypes = [_F, _F, _I, ctypes.c_int, _F, _F]
    lib.ccsdt_mlp_train.argtypes = [_F, _I, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                    ctypes.c_uint, ctypes.c_int, _F, _F]
    lib.ccsdt_mlp_predict.argtypes = [_F, _F, ctypes.c_int, _I, _F]
    lib.ccsdt_triplet_features.argtypes = [ctypes.c_void_p, ctypes.c_long, _I, _F]
    lib.ccsdt_set_slice_model.argtypes = [ctypes.c_void_p, _F]
    lib.ccsdt_learned_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_double)]
    for n in ("ccsdt_mlp_grad", "ccsdt_mlp_train", "ccsdt_mlp_predict", "ccsdt_triplet_features",
              "ccsdt_set_slice_model", "ccsdt_learned_stats"):
        getattr(lib, n).restype = ctypes.c_int
    return lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def mlp_grad(params, X, y):
    """GPU gradient of the mean cross-entropy (labels y in 0..6)."""
    p, X, y = _f32(params), _f32(X), np.ascontiguousarray(y, dtype=np.int32)
    g, loss = np.zeros(NPARAM, np.float32), ctypes.c_float()
    st = _lib().ccsdt_mlp_grad(p.ctypes.data_as(_F), X.ctypes.data_as(_F), y.ctypes.data_as(_I), len(y),
                               g.ctypes.data_as(_F), ctypes.byref(loss))
    if st:
        raise ct.CCSDTError(st, "ccsdt_mlp_grad")
    return g, loss.value


def mlp_train(X, y, epochs=300, batch=64, lr=3e-3, seed=0, params=None):
    p = _f32(params) if params is not None else np.zeros(NPARAM, np.float32)
    X, y = _f32(X), np.ascontiguousarray(y, dtype=np.int32)
    loss = ctypes.c_float()
    st = _lib().ccsdt_mlp_train(X.ctypes.data_as(_F), y.ctypes.data_as(_I), len(y), epochs, batch, lr, seed,
                                int(params is None), p.ctypes.data_as(_F), ctypes.byref(loss))
    if st:
        raise ct.CCSDTError(st, "ccsdt_mlp_train")
    return p, loss.value


def mlp_predict(params, X):
    p, X = _f32(params), _f32(X)
    s = np.zeros(len(X), np.int32)
    st = _lib().ccsdt_mlp_predict(p.ctypes.data_as(_F), X.ctypes.data_as(_F), len(X), s.ctypes.data_as(_I), None)
    if st:
        raise ct.CCSDTError(st, "ccsdt_mlp_predict")
    return s


def features(ft: "ct.FusedTriples", tri) -> np.ndarray:
    t = np.ascontiguousarray(np.asarray(tri, dtype=np.int32).reshape(-1, 3))
    f = np.zeros((len(t), 12), np.float32)
    ft._check(_lib().ccsdt_triplet_features(ft.h, len(t), t.ctypes.data_as(_I), f.ctypes.data_as(_F)))
    return f


def set_model(ft: "ct.FusedTriples", params):
    p = _f32(params)
    ft._keep_model = p
    ft._check(_lib().ccsdt_set_slice_model(ft.h, p.ctypes.data_as(_F)))


def learned_stats(ft: "ct.FusedTriples", with_products=False):
    """(mean predicted slice count, escalations[, digit-plane products run]) of the last call."""
    m, f, p = ctypes.c_double(), ctypes.c_long(), ctypes.c_double()
    _lib().ccsdt_learned_stats(ft.h, ctypes.byref(m), ctypes.byref(f), ctypes.byref(p))
    return (m.value, f.value, p.value) if with_products else (m.value, f.value)


def label_triplets(ft, tri, budget=1e-8, smax=7):
    """Slice-count labels of the sampled triplets `tri` of the handle's system: the counts a greedy
    allocation gives under the LEARNED mode's own acceptance test 3 sum_t sigma_t <= budget
    sum_t |E_t(FP64)| (sigma_t: the library's a-posteriori estimate of triplet t's error at its
    count, ccsdt_triplet_error_estimates; the test is linear, so the sample stands for the system
    without any rescaling).  Every triplet starts at 2 planes; while the test fails, the triplet with
    the largest sigma_t moves one count up (it buys the largest cut per extra product, as sigma falls
    by ~2^-7 per plane), up to smax.
    Returns the labels, the measured errors |E_t(S) - E_t(FP64)| / |E_t(FP64)| [S - 2][t] and the
    FP64 energies (the plain kernel is the yardstick)."""
    _, ref = ft.triplet_energies(tri, "fp64")
    allow = budget * np.abs(ref).sum() / 3.0
    sig, errs = [], []
    for S in range(2, smax + 1):
        _, e, est = ft.triplet_error_estimates(tri, S)
        sig.append(est)
        errs.append(np.abs(e - ref) / np.maximum(np.abs(ref), 1e-300))
    sig, errs = np.array(sig), np.array(errs)               # [S-2][t]
    lab = np.full(len(ref), 2)
    cur = sig[0].copy()
    while np.sum(cur) > allow:
        t = int(np.argmax(np.where(lab < smax, cur, -1.0)))
        if lab[t] >= smax or cur[t] <= 0:
            break
        lab[t] += 1
        cur[t] = sig[lab[t] - 2][t]
    return lab, errs, ref


def training_systems(n=20, seed0=100, o_range=(20, 60), v_range=(150, 500), scale_range=(0.5, 3.0)):
    """The training systems: seeds seed0.. with o, v and the T2 scale drawn uniformly from the
    ranges (by default the ones the slice-count model is specified for: o in [20, 60], v in
    [150, 500], T2 x [0.5, 3], seeds 100-119)."""
    rng = np.random.default_rng(12345)
    out = []
    for s in range(seed0, seed0 + n):
        o = int(rng.integers(o_range[0], o_range[1] + 1))
        v = int(rng.integers(v_range[0], v_range[1] + 1))
        sc = float(rng.uniform(*scale_range))
        out.append((o, v, s, sc))
    return out


LABEL_MARGIN = 0.5


def build_training_set(systems, per_system=24, budget=1e-8, smax=7, log=print, margin=LABEL_MARGIN):
    """Features and labels of per_system sampled triplets of each system (inputs built on the GPU,
    bit-identical to the host generator).  The labels are allocated against margin x budget: the
    sample only estimates the system's error budget, and a triplet predicted one count too low
    costs a rerun (the acceptance test escalates it), while one predicted too high costs only the
    difference in digit-plane products."""
    import torch
    from .generator import generate_device
    X, Y, meta = [], [], []
    for (o, v, seed, sc) in systems:
        d = generate_device(o, v, seed, device="cuda", t2_scale=sc)
        ft = ct.FusedTriples(o, v, ts=40)
        ft.upload_dict(d)
        del d
        torch.cuda.empty_cache()
        allt = ct.all_triplets(o)
        allt = allt[allt[:, 0] != allt[:, 2]]
        rng = np.random.default_rng(seed)
        tri = allt[np.sort(rng.choice(len(allt), size=min(per_system, len(allt)), replace=False))]
        lab, errs, _ = label_triplets(ft, tri, budget * margin, smax)
        X.append(features(ft, tri))
        Y.append(lab - 2)
        meta.append({"o": o, "v": v, "seed": seed, "t2_scale": sc, "labels": np.bincount(lab, minlength=smax + 1).tolist()})
        log(f"system o={o} v={v} seed={seed} t2x{sc:.2f}: label histogram {meta[-1]['labels'][2:]}")
        ft.close()
    return np.concatenate(X), np.concatenate(Y).astype(np.int32), meta


def save_model(params, meta, path=MODEL_PATH):
    Path(path).write_text(json.dumps({"params": [float(x) for x in params], "meta": meta}) + "\n")


def load_model(path=MODEL_PATH):
    d = json.loads(Path(path).read_text())
    return np.asarray(d["params"], np.float32), d.get("meta", {})


def main(argv=None):
    """Train the shipped model on the GPU: python -m exachem_gb300.learned [--out PATH] [--per-system N]"""
    import argparse
    import time
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(MODEL_PATH))
    ap.add_argument("--per-system", type=int, default=24)
    ap.add_argument("--smax", type=int, default=6, help="largest label (digit-plane count) considered")
    ap.add_argument("--budget", type=float, default=1e-8, help="the LEARNED mode's acceptance budget")
    a = ap.parse_args(argv)
    t0 = time.time()
    systems = training_systems()
    X, y, meta = build_training_set(systems, per_system=a.per_system, budget=a.budget, smax=a.smax)
    params, loss = mlp_train(X, y, epochs=400, batch=64, lr=3e-3, seed=7)
    acc = float((mlp_predict(params, X) - 2 == y).mean())
    print(f"trained on {len(y)} triplets: loss {loss:.4f}, accuracy {acc:.3f}, {time.time() - t0:.0f} s")
    save_model(params, {"systems": meta, "budget": a.budget, "label_margin": LABEL_MARGIN, "loss": loss,
                        "train_accuracy": acc,
                        "label_histogram": np.bincount(y + 2, minlength=9).tolist(),
                        "per_system": a.per_system, "smax": a.smax, "train_seconds": time.time() - t0}, a.out)


if __name__ == "__main__":
    main()
