"""The learned warm start end to end on small lattices: converged weights from
the batched engine train the MLP on the device; on held-out (L, T) the weight
iteration from the network's prediction reaches the same flat-histogram
criterion in far fewer iterations than from the zero weight (same seeds,
same options).  The two non-learned arms (the reference's piecewise-linear
form and the full weights, interpolated in T) run beside it and converge."""
import numpy as np
import pytest


@pytest.mark.gpu
def test_warm_start_cuts_iterations(muca):
    from muca_gb300 import warm_start as ws
    rng = np.random.default_rng(1)
    Ts = np.round(np.arange(0.40, 0.801, 0.05), 3)
    train_inst = [(L, 1024, float(T), float(rng.uniform(1.5, 1.99)), 100 + k)
                  for k, (L, T) in enumerate([(L, T) for L in (8, 16) for T in Ts])]
    res, _, W = ws.converge(train_inst)
    assert all(r.converged for r in res)
    x, t = ws.training_set(train_inst, W)
    held = [(16, 1024, 0.53, 1.9, 900), (16, 1024, 0.67, 1.6, 901), (8, 1024, 0.61, 1.7, 902)]
    with muca.MLP(seed=7) as net:
        losses = ws.train(net, x, t, schedule=((3000, 1e-3), (3000, 3e-4)))
        assert losses[-100:].mean() < 1e-3 * losses[:10].mean()
        sources = [(L, T, w) for (L, _, T, _, _), w in zip(train_inst, W)]
        ab = ws.ab_test(net, held, sources=sources)
    rows = ab["instances"]
    assert all(r[k + "_converged"] for r in rows for k in ("zero", "mlp", "pl", "interp"))
    assert ab["iters_ratio"] >= 2.0, ab
    # the surrogate is within a few units of lnW over a range of hundreds
    for r in rows:
        assert r["surrogate_lnw_rms_err"] < 0.05 * r["lnw_range"], r
