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
    """LEARNED accepts when 3 sum_t sigma_t <= budget sum |E_t|: the measured error must meet the
    budget, and the digit-plane products it runs (escalations included) must be strictly fewer
    than those of the smallest fixed count that passes the same test.  The budget sits between the
    fixed counts (2 planes miss it, 3 meet it with room to spare on these ~300-triplet systems),
    where a per-triplet choice can gain: triplets with small energies stay at 2 planes."""
    from exachem_gb300 import ccsd_t as ct, learned
    from exachem_gb300.generator import generate
    budget = 1e-6
    systems = [(10, 60, 100, 1.0), (12, 70, 101, 2.0), (14, 64, 102, 0.7)]
    X, y, _ = learned.build_training_set(systems, per_system=30, budget=budget, smax=6, log=lambda *a: None)
    params, _ = learned.mlp_train(X, y, epochs=300, batch=32, lr=3e-3, seed=5)
    d = generate(11, 66, 103, t2_scale=1.5)
    ft = ct.FusedTriples(11, 66, ts=40)
    ft.upload_dict(d)
    ref = ft.energy("fp64")["e_paren_T"]
    tri = ct.all_triplets(11)
    tri = tri[tri[:, 0] != tri[:, 2]]
    _, ref_t = ft.triplet_energies(tri, "fp64")
    allow = budget * np.abs(ref_t).sum()
    learned.set_model(ft, params)
    r = ft.energy("learned", slices=5, energy_budget=budget)
    mean_s, escalations, products = learned.learned_stats(ft, with_products=True)
    assert abs(r["e_paren_T"] - ref) <= allow
    assert r["abs_err_bound"] <= allow * (1 + 1e-12)
    cost = lambda S: S * (S + 1) / 2
    fixed = 5
    for S in (2, 3, 4):
        _, _, est = ft.triplet_error_estimates(tri, S)
        if 3 * np.sum(est) <= allow:
            fixed = S
            break
    n = len(tri)
    print(f"fixed S={fixed} ({cost(fixed)} products) vs learned mean S={mean_s:.2f} "
          f"({products / n:.2f} products incl. {escalations} escalations)")
    # the gain: strictly fewer digit-plane products than the cheapest fixed count that passes
    assert products / n < cost(fixed), (products / n, cost(fixed))


def test_learned_mode_groups_equal_fixed_count_runs(built):
    """LEARNED runs each predicted count as one batched persistent pass with the results
    scattered back to each triplet's own index: every triplet must equal the same triplet
    run alone at its predicted count (no escalations with a budget of 1, i.e. an allowance of
    the mean |E(T)_t| per triplet)."""
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


def test_error_estimate_covers_measured_error(built):
    """The per-triplet estimate sigma_t (ccsdt_triplet_error_estimates) is a standard deviation:
    3 sigma must cover the error measured against the FP64 path for nearly every triplet, and
    sigma must not be uselessly pessimistic."""
    from exachem_gb300 import ccsd_t as ct
    from exachem_gb300.generator import generate
    ratios = []
    for (o, v, seed, sc) in [(10, 64, 301, 1.0), (12, 90, 302, 2.5), (9, 120, 303, 0.6)]:
        ft = ct.FusedTriples(o, v, ts=32)
        ft.upload_dict(generate(o, v, seed, t2_scale=sc))
        tri = ct.all_triplets(o)
        tri = tri[tri[:, 0] != tri[:, 2]]
        _, ref = ft.triplet_energies(tri, "fp64")
        for S in (2, 3, 4):
            _, e5, est = ft.triplet_error_estimates(tri, S)
            err = np.abs(e5 - ref)
            keep = err > 1e-13 * np.abs(ref)          # below that the float-float floor dominates
            ratios.append(est[keep] / err[keep])
        ft.close()
    r = np.concatenate(ratios)
    q = np.quantile(r, [0.01, 0.05, 0.5])
    print(f"sigma / measured error: 1% {q[0]:.2f}, 5% {q[1]:.2f}, median {q[2]:.2f} over {len(r)} cases")
    assert (3 * r >= 1).mean() >= 0.98
    assert q[2] <= 10


def test_batched_call_is_held_to_the_same_relative_budget(built):
    """The acceptance test is linear in the triplets (3 sum_t sigma_t <= budget sum_t |E_t|), so a
    call that is one part of a larger computation is held to exactly the test of the whole:
    budget_triplets changes nothing."""
    from exachem_gb300 import ccsd_t as ct, learned
    from exachem_gb300.generator import generate
    params, _ = learned.load_model()
    ft = ct.FusedTriples(10, 64, ts=32)
    ft.upload_dict(generate(10, 64, 404))
    tri = ct.all_triplets(10)
    learned.set_model(ft, params)
    a4, a5 = ft.triplet_energies(tri, "learned", slices=5, energy_budget=1e-9)
    _, esc_whole, prod_whole = learned.learned_stats(ft, with_products=True)
    b4, b5 = ft.triplet_energies(tri, "learned", slices=5, energy_budget=1e-9, budget_triplets=100 * len(tri))
    _, esc_part, prod_part = learned.learned_stats(ft, with_products=True)
    assert esc_part == esc_whole and prod_part == prod_whole
    assert np.array_equal(a5, b5) and np.array_equal(a4, b4)
