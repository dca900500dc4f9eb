"""Learned slice count: the GPU training kernels' gradients against a float64 numpy
restatement (and finite differences), training reduces the loss, BF16 inference agrees
with an FP32 forward pass, and the LEARNED mode of the (T) call meets its budget while
spending fewer digit-plane products than the fixed slice count that meets it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(n=96, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.normal(0, 1, (n, 12)).astype(np.float32)
    w = rng.normal(0, 1, 12)
    y = np.clip(np.round(2 + X @ w * 0.7), 0, 6).astype(np.int32)
    return X, y


def test_mlp_gradient_matches_numpy_oracle(built):
    from exachem_gb300 import learned
    from oracle.mlp_oracle import loss_and_grad
    X, y = _data()
    p = np.random.default_rng(3).normal(0, 0.2, learned.NPARAM).astype(np.float32)
    g, loss = learned.mlp_grad(p, X, y)
    l64, g64 = loss_and_grad(p.astype(np.float64), X, y)
    assert abs(loss - l64) <= 1e-5 * abs(l64)
    assert np.abs(g - g64).max() <= 1e-5 * np.abs(g64).max() + 1e-7
    # central finite differences of the float64 loss on a few coordinates
    for idx in (0, 100, 900, 4000, 5440):
        e = np.zeros_like(p, dtype=np.float64)
        e[idx] = 1e-4
        fd = (loss_and_grad(p + e, X, y)[0] - loss_and_grad(p - e, X, y)[0]) / 2e-4
        assert abs(fd - g[idx]) <= 1e-3 * max(1e-3, abs(fd))


def test_mlp_training_reduces_loss_and_bf16_inference(built):
    from exachem_gb300 import learned
    from oracle.mlp_oracle import unpack
    X, y = _data(256, 1)
    p0 = np.zeros(learned.NPARAM, np.float32)
    p, loss = learned.mlp_train(X, y, epochs=200, batch=32, lr=3e-3, seed=1)
    _, loss0 = learned.mlp_grad(p, X, y)
    assert loss < 0.5 * np.log(7) and abs(loss - loss0) <= 1e-5
    s = learned.mlp_predict(p, X)
    P = unpack(p)
    h = np.maximum(np.maximum(X @ P["W1"].T + P["b1"], 0) @ P["W2"].T + P["b2"], 0) @ P["W3"].T + P["b3"]
    agree = (s - 2 == h.argmax(1)).mean()
    assert agree >= 0.95                          # BF16 inference vs FP32 forward
    assert ((s - 2) == y).mean() >= 0.8


def test_learned_mode_meets_budget_and_saves_products(built):
    from exachem_gb300 import ccsd_t as ct, learned
    from exachem_gb300.generator import generate
    # train on three small systems, evaluate on a held-out one
    systems = [(10, 60, 100, 1.0), (12, 70, 101, 2.0), (14, 64, 102, 0.7)]
    X, y, _ = learned.build_training_set(systems, per_system=30, budget=1e-8, smax=6, log=lambda *a: None)
    params, _ = learned.mlp_train(X, y, epochs=300, batch=32, lr=3e-3, seed=5)
    d = generate(11, 66, 103, t2_scale=1.5)
    ft = ct.FusedTriples(11, 66, ts=40)
    ft.upload_dict(d)
    ref = ft.energy("fp64")["e_paren_T"]
    learned.set_model(ft, params)
    r = ft.energy("learned", slices=6, energy_budget=1e-8)
    mean_s, fallbacks = learned.learned_stats(ft)
    assert abs(r["e_paren_T"] - ref) <= 2e-8 * abs(ref)
    # the fixed count that meets the same per-triplet budget everywhere
    tri = ct.all_triplets(11)
    tri = tri[tri[:, 0] != tri[:, 2]]
    lab, _, _ = learned.label_triplets(ft, tri, budget=1e-8, smax=6)
    fixed = int(lab.max())
    cost = lambda S: S * (S + 1) / 2
    pred = learned.mlp_predict(params, learned.features(ft, tri))
    n = len(tri)
    learned_cost = (sum(cost(min(max(s, 2), 6)) for s in pred) + fallbacks * cost(6)) / n
    print(f"fixed S={fixed} ({cost(fixed)} products) vs learned mean S={mean_s:.2f} "
          f"({learned_cost:.2f} products incl. {fallbacks} full-slice fallbacks)")
    assert learned_cost <= cost(fixed) + 1e-9
    assert fallbacks <= 0.25 * n


def test_learned_mode_groups_equal_fixed_count_runs(built):
    """LEARNED runs each predicted count as one batched persistent pass with the results
    scattered back to each triplet's own index: every triplet must equal the same triplet
    run alone at its predicted count (no fallbacks with a budget of 1)."""
    from exachem_gb300 import ccsd_t as ct, learned
    from exachem_gb300.generator import generate
    o, v = 9, 48
    ft = ct.FusedTriples(o, v, ts=24)
    ft.upload_dict(generate(o, v, 77))
    tri = ct.all_triplets(o)
    X = learned.features(ft, tri)
    y = np.random.default_rng(3).integers(0, 4, len(tri)).astype(np.int32)   # counts 2..5
    params, _ = learned.mlp_train(X, y, epochs=300, batch=32, lr=3e-3, seed=2)
    pred = np.clip(learned.mlp_predict(params, X), 2, 5)
    assert len(set(pred.tolist())) >= 2
    learned.set_model(ft, params)
    e4, e5 = ft.triplet_energies(tri, "learned", slices=5, energy_budget=1.0)
    _, fallbacks = learned.learned_stats(ft)
    assert fallbacks == 0
    for S in sorted(set(pred.tolist())):
        sel = pred == S
        f4, f5 = ft.triplet_energies(tri[sel], "ozaki", slices=S)
        np.testing.assert_allclose(e5[sel], f5, rtol=1e-13, atol=0)
        np.testing.assert_allclose(e4[sel], f4, rtol=1e-13, atol=0)
