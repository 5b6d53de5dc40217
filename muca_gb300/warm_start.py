"""Learned warm start of the weight iteration: produce converged weights with
the batched engine, train the MLP on them, and compare, on held-out (L, T,
Delta), the iterations and device time of the weight iteration from the zero
weight against the same iteration from the network's prediction.

The reference's only alternative to a zero initial weight is an extrapolated
weight file read by its `continuing` path (muca_delta_multigpu.cu:223-235);
the prediction takes that place here.  The iteration itself is unchanged:
same update rule, same schedule, same stop criterion (min/mean >= 0.5), so the
iterations it takes measure the surrogate's error.

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

# the weight iteration of every arm of the A/B: schedule 4 (the CPU
# program's NUPDATES x1.05 per iteration) from 16 sweeps of the instance,
# capped at 2^18 attempts per chain; one schedule for every arm
RUN_OPTS = dict(starting_M=1, rule=m.UPDATE_TRIVIAL, nup_schedule=4, flat_minmean=1, max_iter=20000,
                graph_iters=32, starting_sweeps=16, nup_max=1 << 18)
# the training data: NUPDATES from one sweep, doubling once the width is N
# (capped at 2^18)
DATA_OPTS = dict(RUN_OPTS, nup_schedule=1, starting_sweeps=1)


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


# Knots of the reference's piecewise-linear extrapolation, as fractions of N:
# E_Delta = 0, 0.176 N, 0.888 N and N (muca_delta_multigpu.cu:271-307, code
# commented out there).  Between the knots the reference adds straight lines
# whose heights it fitted by hand for one (L, T).
PL_KNOTS = (0.0, 0.176, 0.888, 1.0)


def _bracket(keys, x):
    """Indices (a, b) of the two entries of the sorted `keys` that bracket x,
    or the two nearest ones when x lies outside; lam = (x - ka) / (kb - ka)."""
    b = int(np.clip(np.searchsorted(keys, x), 1, len(keys) - 1))
    ka, kb = keys[b - 1], keys[b]
    return b - 1, b, ((x - ka) / (kb - ka) if kb != ka else 0.0)


def _at_size(L, T, sources, knots):
    same = sorted(((float(Ts), np.asarray(w, np.float64)) for Ls, Ts, w in sources if Ls == L),
                  key=lambda s: s[0])
    N = L * L
    i = np.arange(N + 1, dtype=np.float64)

    def shape(w):
        if w.size != N + 1:
            raise ValueError(f"weight of L={L} has {w.size} entries, not {N + 1}")
        if knots is None:
            return w
        ik = np.unique(np.rint(np.asarray(knots, np.float64) * N).astype(np.int64))
        return np.interp(i, ik, w[ik])

    if len(same) == 1:
        out = shape(same[0][1])
    else:
        a, b, lam = _bracket(np.array([s[0] for s in same]), T)
        out = (1.0 - lam) * shape(same[a][1]) + lam * shape(same[b][1])
    return out - out.mean()


def interpolated_weight(L, T, sources, knots=None):
    """A non-learned initial lnW for (L, T) from converged weights
    sources [(L, T, lnW)].  Per lattice size, the two sources nearest in
    temperature (bracketing T where they can) are interpolated linearly in T
    (extrapolated outside).  With `knots` (fractions of N) each source is
    first reduced to the straight lines through its values at those E_Delta:
    the form of the reference's extrapolation, with the knot heights taken
    from data instead of fitted by hand.  For a size with no source, the two
    nearest sizes are combined the same way, linearly in L, as lnW/N on the
    common axis E_Delta/N (lnW is extensive).  Returns lnW of mean zero (a
    constant shift leaves the iteration unchanged)."""
    sizes = sorted({int(Ls) for Ls, _, _ in sources})
    if not sizes:
        raise ValueError("no converged weight to interpolate from")
    if L in sizes:
        return _at_size(L, T, sources, knots)
    N = L * L
    x = np.arange(N + 1, dtype=np.float64) / N

    def per_site(Ls):
        w = _at_size(Ls, T, sources, knots)
        Ns = Ls * Ls
        return np.interp(x, np.arange(Ns + 1, dtype=np.float64) / Ns, w / Ns)

    if len(sizes) == 1:
        out = N * per_site(sizes[0])
    else:
        a, b, lam = _bracket(np.array(sizes, np.float64), float(L))
        out = N * ((1.0 - lam) * per_site(sizes[a]) + lam * per_site(sizes[b]))
    return out - out.mean()


def ab_test(net, held, opts=RUN_OPTS, device=0, sources=None, graded=False):
    """The zero weight against the network's weight on the same held-out
    instances (same seeds, same options).  With `sources` ([(L, T, lnW)],
    the converged training weights) two non-learned arms run beside them:
    "pl", the reference's piecewise-linear form (knots PL_KNOTS) with knot
    heights interpolated in T, and "interp", the full converged weights
    interpolated in T.  With `graded`, the zero, network and interp arms run
    once more from graded initial spins ("<arm>_g": the chains' E_Delta
    spread over [0, N] as a converged multicanonical ensemble would hold
    them, MUCA_INIT_GRADED) instead of the reference's initial spins."""
    arms = {"mlp": [net.log_weights(L, T, D) for L, _, T, D, _ in held]}
    if sources is not None:
        arms["pl"] = [interpolated_weight(L, T, sources, PL_KNOTS) for L, _, T, _, _ in held]
        arms["interp"] = [interpolated_weight(L, T, sources) for L, _, T, _, _ in held]
    rz, sz, wz = converge(held, opts, None, device)
    runs = {k: converge(held, opts, w, device) for k, w in arms.items()}
    if graded:
        og = dict(opts, reinit_chains=1, graded_init=1)
        runs["zero_g"] = converge(held, og, None, device)
        arms["zero_g"] = [np.zeros_like(w) for w in wz]
        for k in [k for k in ("mlp", "interp") if k in arms]:
            runs[k + "_g"] = converge(held, og, arms[k], device)
            arms[k + "_g"] = arms[k]
    rows = []
    for i, (L, nc, T, D, seed) in enumerate(held):
        row = {"L": L, "T": T, "delta": D, "chains": nc, "zero_iters": rz[i].iterations,
               "zero_converged": bool(rz[i].converged), "lnw_range": float(wz[i].max() - wz[i].min())}
        for k, (r, _, wf) in runs.items():
            e = arms[k][i] - wz[i]
            f = wf[i] - wz[i]
            row[k + "_iters"] = r[i].iterations
            row[k + "_converged"] = bool(r[i].converged)
            row[k + "_lnw_rms_err"] = float(np.sqrt(np.mean((e - e.mean()) ** 2)))
            # the converged weights against the zero arm's (both shifted to mean zero)
            row[k + "_final_rms_vs_zero"] = float(np.sqrt(np.mean((f - f.mean()) ** 2)))
        row["surrogate_lnw_rms_err"] = row["mlp_lnw_rms_err"]
        rows.append(row)
    iz = sum(r["zero_iters"] for r in rows)
    out = {"instances": rows, "zero_iters_total": iz, "zero_device_s": sz}
    for k, (_, s, _) in runs.items():
        ik = sum(r[k + "_iters"] for r in rows)
        out[k + "_iters_total"] = ik
        out[k + "_device_s"] = s
        out[k + "_iters_ratio"] = iz / max(1, ik)
        out[k + "_time_ratio"] = sz / s if s > 0 else None
    out["iters_ratio"] = out["mlp_iters_ratio"]
    out["time_ratio"] = out["mlp_time_ratio"]
    return out


def final_agreement(arm_w, zero_w):
    """The converged weights of an arm against the zero arm's, both shifted
    to mean zero: rms and max |difference| in lnW, and the rms relative to
    the range of lnW."""
    f = np.asarray(arm_w) - np.asarray(zero_w)
    f = f - f.mean()
    rng_ = float(np.max(zero_w) - np.min(zero_w))
    rms = float(np.sqrt(np.mean(f * f)))
    return {"rms": rms, "max": float(np.max(np.abs(f))), "rms_rel_range": rms / rng_ if rng_ > 0 else None}


def agreement_under(net, held, sources, opts, device=0, arms=("mlp", "interp", "pl")):
    """The arms run to `opts`' stop criterion; each arm's converged weights
    against the zero arm's, beside the statistical floor (the zero weight on
    other seeds against the zero weight)."""
    starts = {"mlp": lambda: [net.log_weights(L, T, D) for L, _, T, D, _ in held],
              "interp": lambda: [interpolated_weight(L, T, sources) for L, _, T, _, _ in held],
              "pl": lambda: [interpolated_weight(L, T, sources, PL_KNOTS) for L, _, T, _, _ in held]}
    arms = {k: starts[k]() for k in arms}
    rz, sz, wz = converge(held, opts, None, device)
    out = {"zero": {"iters_total": sum(r.iterations for r in rz), "device_s": sz,
                    "converged": sum(bool(r.converged) for r in rz)}}
    floor_runs = converge([(L, nc, T, D, seed + 7919) for L, nc, T, D, seed in held], opts, None, device)
    runs = dict(arms)
    per = {k: [] for k in list(arms) + ["zero_reseeded"]}
    for k, w0 in runs.items():
        r, sec, wf = converge(held, opts, w0, device)
        out[k] = {"iters_total": sum(x.iterations for x in r), "device_s": sec,
                  "converged": sum(bool(x.converged) for x in r)}
        per[k] = [final_agreement(wf[i], wz[i]) for i in range(len(held))]
    rf, sf, wff = floor_runs
    out["zero_reseeded"] = {"iters_total": sum(x.iterations for x in rf), "device_s": sf,
                            "converged": sum(bool(x.converged) for x in rf)}
    per["zero_reseeded"] = [final_agreement(wff[i], wz[i]) for i in range(len(held))]
    for k, v in per.items():
        out[k]["final_rms_vs_zero_median"] = float(np.median([a["rms"] for a in v]))
        out[k]["final_rms_vs_zero_max"] = float(np.max([a["rms"] for a in v]))
        out[k]["final_rms_rel_range_max"] = float(np.max([a["rms_rel_range"] for a in v]))
        out[k]["final_maxabs_vs_zero_max"] = float(np.max([a["max"] for a in v]))
        out[k]["per_instance_rms"] = [round(a["rms"], 5) for a in v]
    return out


def agreement_instances(held, Lmax, chains=None):
    """The held-out instances run to the reference criterion: those with
    L <= Lmax, with `chains` chains each (None: their own count)."""
    return [(L, chains or nc, T, D, seed) for L, nc, T, D, seed in held if L <= Lmax]


def held_out_instances(Ls, Ts, rng, chains):
    return [(L, chains, float(T), float(rng.uniform(1.5, 1.99)), 5000 + k)
            for k, (L, T) in enumerate([(L, float(T)) for L in Ls for T in Ts])]


def run_study(Ls=(16, 24, 32, 48, 64, 72, 96, 128), chains=256, t_step=0.025, held_T=(0.43, 0.53, 0.63, 0.73),
              held_L=(), schedule=4, steps=10000, device=0, reference_criterion=True, agreement_Lmax=48,
              graded=False, ab_schedules=(), save=None, load=None, progress=None, held_sizes=None, nup_max=None,
              max_iter=None, starting_sweeps=None, agreement_nup_max=1 << 18, agreement_max_iter=40000,
              agreement_arms=("mlp", "interp", "pl"), agreement_d_kl=1e-4, agreement_chains=None):
    """The study: training data from the batched engine (every (L, T) on the
    grid, a seed per instance, DATA_OPTS), the network trained on the
    device, the A/B on the held-out (L, T, Delta) to min/mean >= 0.5 with one
    NUPDATES schedule for every arm (`schedule`, capped at 2^16), and
    (reference_criterion) the arms run to the reference's criterion
    (width == N and D_KL < 1e-4) on the held-out instances of L <=
    agreement_Lmax, for the agreement of the final weights.  `save` writes
    the training set, converged training weights and network parameters to
    an .npz; `load` reads them back instead of generating and training.
    `progress`: a JSON file rewritten with the results so far after every
    stage.  held_sizes: run the A/B only on the held-out instances of these
    sizes; nup_max / max_iter: the A/B's NUPDATES cap and iteration cap;
    agreement_nup_max / agreement_max_iter / agreement_arms / agreement_d_kl:
    the NUPDATES cap, iteration cap, warm starts and D_KL bound (1e-4 is the
    reference's) of the runs to the reference criterion; agreement_chains:
    their chains per instance (None: `chains`)."""
    t_all = time.time()

    def dump(o):
        if progress:
            with open(progress, "w") as f:
                json.dump(o, f)
    rng = np.random.default_rng(0)
    opts = dict(RUN_OPTS, nup_schedule=schedule)
    if nup_max:
        opts["nup_max"] = nup_max
    if max_iter:
        opts["max_iter"] = max_iter
    if starting_sweeps:
        opts["starting_sweeps"] = starting_sweeps
    out = {"run_opts": dict(opts), "data_opts": dict(DATA_OPTS)}
    with m.MLP(device=device, seed=7) as net:
        if load:
            z = np.load(load, allow_pickle=False)
            net.set_params(z["params"])
            src_meta = z["src_meta"]
            src_w = [z["src_w_%d" % i] for i in range(len(src_meta))]
            sources = [(int(Lm), float(Tm), w) for (Lm, Tm), w in zip(src_meta, src_w)]
            for _ in range(len(Ls) * len(np.arange(0.40, 0.8 + 1e-9, t_step))):
                rng.uniform(1.5, 1.99)  # the same held-out Deltas as the generating run
            out["training_set"] = {"loaded": load, "sources": len(sources)}
        else:
            Ts = np.round(np.arange(0.40, 0.8 + 1e-9, t_step), 4)
            train_inst = [(L, chains, float(T), float(rng.uniform(1.5, 1.99)), 1000 + k)
                          for k, (L, T) in enumerate([(L, T) for L in Ls for T in Ts])]
            t0 = time.time()
            res, sec, W = converge(train_inst, DATA_OPTS, None, device)
            ok = [i for i, r in enumerate(res) if r.converged]
            x, t = training_set([train_inst[i] for i in ok], [W[i] for i in ok])
            out["training_set"] = {"instances": len(train_inst), "sizes": list(Ls), "chains": chains,
                                   "converged": len(ok), "device_s": sec, "wall_s": time.time() - t0,
                                   "iters_median": float(np.median([r.iterations for r in res])),
                                   "iters_max": int(max(r.iterations for r in res)), "points": int(x.shape[0])}
            t0 = time.time()
            sched = ((steps, 1e-3), (steps, 3e-4), (steps, 1e-4))
            losses = train(net, x, t, schedule=sched)
            fit_s = time.time() - t0
            flops = 6.0 * losses.size * 4096 * net.n_params  # forward + two backward products
            out["fit"] = {"steps": int(losses.size), "batch": 4096, "lr": [s_[1] for s_ in sched],
                          "loss_first": float(losses[:10].mean()), "loss_last": float(losses[-100:].mean()),
                          "wall_s": fit_s, "tflops": flops / fit_s / 1e12}
            sources = [(train_inst[i][0], train_inst[i][2], W[i]) for i in ok]
            if save:
                arrs = {"params": net.params(),
                        "src_meta": np.array([(Lm, Tm) for Lm, Tm, _ in sources], np.float64)}
                arrs.update({"src_w_%d" % i: w for i, (_, _, w) in enumerate(sources)})
                np.savez(save, **arrs)
        dump(out)
        held = held_out_instances(list(Ls) + list(held_L), held_T, rng, chains)
        if held_sizes:
            held = [h for h in held if h[0] in held_sizes]
        t0 = time.time()
        ab = ab_test(net, held, opts, device, sources, graded=graded)
        ab["wall_s"] = time.time() - t0
        out["ab"] = ab
        dump(out)
        if reference_criterion:
            sub = agreement_instances(held, agreement_Lmax, agreement_chains)
            ro = dict(opts, flat_minmean=0, max_iter=agreement_max_iter, nup_max=agreement_nup_max,
                      d_kl_max=agreement_d_kl)
            t0 = time.time()
            ag = agreement_under(net, sub, sources, ro, device, agreement_arms)
            ag["wall_s"] = time.time() - t0
            ag["instances"] = [(L, T) for L, _, T, _, _ in sub]
            ag["run_opts"] = ro
            out["agreement_reference_criterion"] = ag
            dump(out)
        # the A/B under other NUPDATES schedules (the same network; every arm alike)
        ab_sched = {}
        for sc in ab_schedules:
            ab_sched[int(sc)] = ab_test(net, held, dict(opts, nup_schedule=int(sc)), device, sources)
            out["ab_schedules"] = ab_sched
            dump(out)
    out["wall_s"] = time.time() - t_all
    return out


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--L", default="16,24,32,48,64,72,96,128")
    p.add_argument("--chains", type=int, default=256)
    p.add_argument("--t-step", type=float, default=0.025)
    p.add_argument("--held-T", default="0.43,0.53,0.63,0.73")
    p.add_argument("--held-L", default="", help="held-out lattice sizes beyond the training ones")
    p.add_argument("--graded", action="store_true", help="also run the arms from graded initial spins")
    p.add_argument("--steps", type=int, default=10000, help="Adam steps per learning-rate stage (3 stages)")
    p.add_argument("--schedule", type=int, default=4, help="NUPDATES schedule of every arm")
    p.add_argument("--agreement-Lmax", type=int, default=48,
                   help="largest L of the held-out instances run to the reference criterion")
    p.add_argument("--save", default=None, help="write the training set's weights and the network to this .npz")
    p.add_argument("--load", default=None, help="read them from this .npz instead of generating and training")
    p.add_argument("--progress", default=None, help="JSON file rewritten with the results so far after every stage")
    p.add_argument("--held-sizes", default="", help="run the A/B only on the held-out instances of these sizes")
    p.add_argument("--nup-max", type=int, default=0, help="NUPDATES cap of the A/B (0: RUN_OPTS')")
    p.add_argument("--max-iter", type=int, default=0, help="iteration cap of the A/B (0: RUN_OPTS')")
    p.add_argument("--starting-sweeps", type=int, default=0,
                   help="initial NUPDATES of the A/B in sweeps of each instance (0: RUN_OPTS')")
    p.add_argument("--ab-schedules", default="",
                   help="NUPDATES schedules to repeat the A/B with (same network), e.g. 0,4")
    p.add_argument("--no-reference-criterion", action="store_true",
                   help="skip the runs to width == N and D_KL < 1e-4")
    p.add_argument("--agreement-nup-max", type=int, default=1 << 18,
                   help="NUPDATES cap of the runs to the reference criterion")
    p.add_argument("--agreement-max-iter", type=int, default=40000,
                   help="iteration cap of the runs to the reference criterion")
    p.add_argument("--agreement-d-kl", type=float, default=1e-4,
                   help="D_KL bound of the runs to the reference criterion (the reference's: 1e-4)")
    p.add_argument("--agreement-chains", type=int, default=0,
                   help="chains per instance of the runs to the reference criterion (0: --chains)")
    p.add_argument("--agreement-arms", default="mlp,interp,pl",
                   help="warm starts run to the reference criterion beside the zero weight and its reseeded floor")
    p.add_argument("--device", type=int, default=0)
    a = p.parse_args(argv)
    out = run_study(Ls=[int(v) for v in a.L.split(",")], chains=a.chains, t_step=a.t_step,
                    held_T=[float(v) for v in a.held_T.split(",")],
                    held_L=[int(v) for v in a.held_L.split(",") if v], schedule=a.schedule, steps=a.steps,
                    device=a.device, reference_criterion=not a.no_reference_criterion,
                    agreement_Lmax=a.agreement_Lmax, graded=a.graded,
                    ab_schedules=[int(v) for v in a.ab_schedules.split(",") if v], save=a.save, load=a.load,
                    progress=a.progress, held_sizes=[int(v) for v in a.held_sizes.split(",") if v],
                    nup_max=a.nup_max or None, max_iter=a.max_iter or None,
                    starting_sweeps=a.starting_sweeps or None, agreement_nup_max=a.agreement_nup_max,
                    agreement_max_iter=a.agreement_max_iter,
                    agreement_arms=[v for v in a.agreement_arms.split(",") if v], agreement_d_kl=a.agreement_d_kl,
                    agreement_chains=a.agreement_chains or None)
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    main()
