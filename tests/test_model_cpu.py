"""CPU checks of the slice-count model's host side: the numpy oracle's gradient against finite
differences (it is the checker of the GPU training kernels), the shipped model file, and the C++
adapter's reader of that file."""
import subprocess

import numpy as np

from conftest import ROOT


def test_mlp_oracle_gradient_matches_finite_differences():
    from oracle import mlp_oracle
    rng = np.random.default_rng(5)
    n = sum(int(np.prod(s)) for _, s in mlp_oracle.SIZES)
    p = rng.normal(0, 0.3, n)
    X = rng.normal(0, 1, (17, mlp_oracle.IN))
    y = rng.integers(0, mlp_oracle.OUT, 17)
    loss, g = mlp_oracle.loss_and_grad(p, X, y)
    idx = rng.choice(n, 40, replace=False)
    h = 1e-6
    for q in idx:
        pp, pm = p.copy(), p.copy()
        pp[q] += h
        pm[q] -= h
        fd = (mlp_oracle.loss_and_grad(pp, X, y)[0] - mlp_oracle.loss_and_grad(pm, X, y)[0]) / (2 * h)
        assert abs(fd - g[q]) <= 1e-6 * max(1.0, abs(fd)), (q, fd, g[q])


def test_shipped_model_file():
    import json
    from oracle import mlp_oracle
    d = json.loads((ROOT / "exachem_gb300" / "slice_model.json").read_text())
    p = np.asarray(d["params"], np.float64)
    n = sum(int(np.prod(s)) for _, s in mlp_oracle.SIZES)
    assert p.shape == (n,) and np.all(np.isfinite(p))
    meta = d["meta"]
    assert meta["budget"] > 0 and 0.5 <= meta["train_accuracy"] <= 1.0
    # the numpy forward pass gives a slice count in 2..8 for plausible features
    X = np.random.default_rng(1).uniform(-1, 1, (32, mlp_oracle.IN))
    P = mlp_oracle.unpack(p)
    z = np.maximum(np.maximum(X @ P["W1"].T + P["b1"], 0) @ P["W2"].T + P["b2"], 0) @ P["W3"].T + P["b3"]
    s = 2 + z.argmax(1)
    assert s.min() >= 2 and s.max() <= 8


def test_adapter_reads_the_model_file(tmp_path):
    exe = tmp_path / "read_model"
    subprocess.run(["g++", "-O2", "-std=c++17", str(ROOT / "tests" / "compat" / "read_model.cpp"), "-o", str(exe),
                    "-I", str(ROOT / "include")], check=True, capture_output=True, text=True)
    path = ROOT / "exachem_gb300" / "slice_model.json"
    out = subprocess.run([str(exe), str(path)], check=True, capture_output=True, text=True).stdout.split()
    from exachem_gb300.learned import load_model
    p, _ = load_model(path)
    w = np.arange(len(p)) % 97 + 1
    assert int(out[0]) == len(p)
    assert abs(float(out[1]) - float(p.astype(np.float64).sum())) <= 1e-6 * max(1.0, abs(float(out[1])))
    assert abs(float(out[2]) - float((p.astype(np.float64) * w).sum())) <= 1e-6 * max(1.0, abs(float(out[2])))


def test_opts_partial_array_storage_names():
    """The Python options map the partial-array storage names onto opts.p_storage (0 auto, 1
    float-float, 2 FP32, 3 FP64) and reject unknown ones."""
    import pytest
    from exachem_gb300.ccsd_t import FusedTriples
    for name, code in (("auto", 0), ("ff", 1), ("f32", 2), ("f64", 3)):
        assert FusedTriples.opts("ozaki", slices=2, p_storage=name).p_storage == code
    assert FusedTriples.opts("ozaki", p_storage=3).p_storage == 3
    with pytest.raises(KeyError):
        FusedTriples.opts("ozaki", p_storage="fp16")
