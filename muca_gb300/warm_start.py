"""Learned warm start of the weight iteration: produce converged weights with
the batched engine, train the MLP on them, and compare, on held-out (L, T,
Delta), the iterations and device time of the weight iteration from the zero
weight against the same iteration from the network's prediction.

The reference's only alternative to a zero initial weight is an extrapolated
weight file read by its `continuing` path (muca_delta_multigpu.cu:223-235);
the prediction takes that place here.  The iteration itself is unchanged:
same update rule, same schedule, same stop criterion (min/mean >= 0.5), so the
iteration remains the judge of the surrogate's error.

    python -m muca_gb300.warm_start [--L 16,24,32,48] [--chains 1024] ...

prints one JSON object with the training set, the network's training curve
and the per-instance A/B.  The weight over E_Delta = sum s_i^2 does not
depend on Delta (Delta enters only the reweighting), so Delta is an input
the network learns to ignore; it is kept to match the (L, T, Delta, x) input.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

import muca_gb300 as m

# the weight iteration used for the training data and both arms of the A/B
RUN_OPTS = dict(starting_M=1, rule=m.UPDATE_TRIVIAL, nup_schedule=1, flat_minmean=1, max_iter=8000,
                graph_iters=32, starting_sweeps=1, nup_max=1 << 18)


def converge(instances, opts=RUN_OPTS, warm=None, device=0):
    """Runs the weight iteration for instances [(L, nchains, T, Delta, seed)]
    in one batch; warm: optional initial lnW per instance.  Returns (results,
    device seconds, converged weights)."""
    with m.Batch([(L, nc, 1.0 / T, seed) for L, nc, T, _, seed in instances], device=device) as b:
        if warm is not None:
            for i, w in enumerate(warm):
                b.set_weights(i, w)
        res, sec = b.run(**opts)
        return res, sec, [b.get_weights(i) for i in range(len(instances))]


def training_set(instances, weights):
    xs, ts = [], []
    for (L, _, T, D, _), w in zip(instances, weights):
        x, t = m.mlp_features(L, T, D, w)
        xs.append(x)
        ts.append(t)
    return np.concatenate(xs), np.concatenate(ts)


def train(net, x, t, schedule=((10000, 1e-3), (10000, 3e-4), (10000, 1e-4)), batch=4096, seed=3):
    """Adam with a stepwise learning rate; returns the per-step losses."""
    net.set_data(x, t)
    return np.concatenate([net.train(steps, batch=batch, lr=lr, seed=seed + k)
                           for k, (steps, lr) in enumerate(schedule)])


def ab_test(net, held, opts=RUN_OPTS, device=0):
    """Zero weight against the network's weight on the same held-out
    instances (same seeds, same options)."""
    warm = [net.log_weights(L, T, D) for L, _, T, D, _ in held]
    rz, sz, wz = converge(held, opts, None, device)
    rm, sm, _ = converge(held, opts, warm, device)
    rows = []
    for i, (L, nc, T, D, seed) in enumerate(held):
        e = warm[i] - wz[i]
        rows.append({"L": L, "T": T, "delta": D, "chains": nc, "zero_iters": rz[i].iterations,
                     "zero_converged": bool(rz[i].converged), "mlp_iters": rm[i].iterations,
                     "mlp_converged": bool(rm[i].converged),
                     "surrogate_lnw_rms_err": float(np.sqrt(np.mean((e - e.mean()) ** 2))),
                     "lnw_range": float(wz[i].max() - wz[i].min())})
    iz = sum(r["zero_iters"] for r in rows)
    im = sum(r["mlp_iters"] for r in rows)
    return {"instances": rows, "zero_iters_total": iz, "mlp_iters_total": im,
            "iters_ratio": iz / max(1, im), "zero_device_s": sz, "mlp_device_s": sm,
            "time_ratio": sz / sm if sm > 0 else None}


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--L", default="16,24,32,48")
    p.add_argument("--chains", type=int, default=1024)
    p.add_argument("--t-step", type=float, default=0.025)
    p.add_argument("--held-T", default="0.53,0.67")
    p.add_argument("--steps", type=int, default=10000, help="Adam steps per learning-rate stage (3 stages)")
    p.add_argument("--schedule", type=int, default=RUN_OPTS["nup_schedule"])
    p.add_argument("--device", type=int, default=0)
    a = p.parse_args(argv)
    Ls = [int(v) for v in a.L.split(",")]
    Ts = np.round(np.arange(0.40, 0.8 + 1e-9, a.t_step), 4)
    rng = np.random.default_rng(0)
    opts = dict(RUN_OPTS, nup_schedule=a.schedule)
    train_inst = [(L, a.chains, float(T), float(rng.uniform(1.5, 1.99)), 1000 + k)
                  for k, (L, T) in enumerate([(L, T) for L in Ls for T in Ts])]
    t0 = time.time()
    res, sec, W = converge(train_inst, opts, None, a.device)
    ok = [i for i, r in enumerate(res) if r.converged]
    x, t = training_set([train_inst[i] for i in ok], [W[i] for i in ok])
    gen = {"instances": len(train_inst), "converged": len(ok), "device_s": sec, "wall_s": time.time() - t0,
           "iters_median": float(np.median([r.iterations for r in res])), "points": int(x.shape[0])}
    with m.MLP(device=a.device, seed=7) as net:
        t0 = time.time()
        sched = ((a.steps, 1e-3), (a.steps, 3e-4), (a.steps, 1e-4))
        losses = train(net, x, t, schedule=sched)
        fit = {"steps": int(losses.size), "batch": 4096, "lr": [s[1] for s in sched],
               "loss_first": float(losses[:10].mean()), "loss_last": float(losses[-100:].mean()),
               "wall_s": time.time() - t0}
        held = [(L, a.chains, float(T), float(rng.uniform(1.5, 1.99)), 5000 + k)
                for k, (L, T) in enumerate([(L, float(T)) for L in Ls for T in a.held_T.split(",")])]
        ab = ab_test(net, held, opts, a.device)
    out = {"run_opts": {k: v for k, v in opts.items()}, "training_set": gen, "fit": fit, "ab": ab}
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    main()
