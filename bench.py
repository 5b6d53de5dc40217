#!/usr/bin/env python3
"""Benchmark of the multicanonical weight-estimation hot path on GB300.

Metric: spin-flip attempts/ns at L=72, one GB300 against the host CPU.  One
step = one iteration of the reference weight loop
(muca_delta_multigpu.cu:374-477) on the workload of the L=72 configuration:
16384 chains, therm = N = 5184 attempts then nup = N recorded attempts per
chain (2 * 5184 * 16384 = 169.9 M attempts), followed by the FP64 trivial
weight update on the device.  Spins start from the reference initialisation
(muca_delta_multigpu.cu:340-354); all inputs are synthetic (no dataset).

  value  device time of the K timed steps (CUDA events on the engine's
         stream), L2 flushed (256 MiB write) before every timed step;
  e2e    the same steps through the C ABI with host buffers: one
         muca_iterate_host call per step (weights H2D from pinned memory,
         sweep, update, weights + histogram D2H, one synchronisation), timed
         on the host clock around the call, L2 flushed before every step;
  roofline      HBM form: 1.5 algorithmic bytes per attempt (2-bit spins:
                site read + write, 4 neighbour reads) over the sweep kernel's
                event time, against the measured copy bandwidth;
  roofline_int  0.5 Philox4x32-7 blocks per attempt against the measured
                Philox block rate of this GPU (muca_philox_peak);
  roofline_issue  warp instructions per launch (ncu, committed profile)
                over the launch time against 4 per clock per SM: the bound
                that applies (lattice resident in shared memory);
  cpu_baseline  the CPU oracle (the reference algorithm restated in C, one
                chain per thread task, all host threads) on full steps.

Beside the headline the default line carries `flat_run` (iterations and time
to a flat histogram), `config2` (the L=72 configuration as written: runs
from starting_M = 1, the recursion, steps from converged weights, the
reference's own chain count), `batch` (256 uneven instances), `production`
(the L=128 configuration: a converged weight, jackknifed <|M|>, chi and U4
over 10 blocks, the reweighting, and the reference's CPU production
algorithm on the host threads) and `random_site` (the CPU weight program's
algorithm on the device, with the oracle's restatement of it on the host
threads); `--only NAME` prints one of them alone.  `--only warm_start` (the
learned warm start's study, minutes of GPU time) and `--only mlp` (the
network's training throughput) are not part of the default line.

`--impl reference` times the reference's CPU algorithm (the oracle port: the
reference CPU sources cannot be built on the GPU host) on the same workload.
With N > 1 processes (torchrun), every rank runs its own shard as reference
device `rank` (its own seeds), no collective on the data path: weak scaling.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L_DEFAULT, CHAINS_DEFAULT = 72, 16384
METRIC = "spin-flip attempts/ns at L=72 (1 GB300 vs host CPU)"
ALG_BYTES_PER_ATTEMPT = 1.5     # 2-bit spins: read+write of the site, 4 neighbour reads
PHILOX_BLOCKS_PER_ATTEMPT = 0.5  # two Philox4x32 blocks per four attempts


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--L", type=int, default=L_DEFAULT)
    p.add_argument("--chains", type=int, default=CHAINS_DEFAULT)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-ref-gpu", action="store_true")
    p.add_argument("--no-extra", action="store_true", help="skip the flat-run, batch and production lines")
    p.add_argument("--only", choices=["flat_run", "config2", "batch", "production", "random_site", "warm_start",
                                      "mlp"],
                   help="run only this extra line and print it (for profiling a smaller case)")
    p.add_argument("--production-L", type=int, default=128, help="lattice size of --only production")
    p.add_argument("--blocks", type=int, default=10, help="jackknife blocks of --only production")
    p.add_argument("--block-sweeps", type=int, default=100, help="production sweeps per block of --only production")
    p.add_argument("--therm-sweeps", type=int, default=100, help="thermalisation sweeps of --only production")
    p.add_argument("--mlp-steps", type=int, default=2048, help="timed training steps of --only mlp")
    p.add_argument("--state-out", default=None, help="--only production: save the converged weight and lattices")
    p.add_argument("--state-in", default=None, help="--only production: start from a saved state (no weight run)")
    p.add_argument("--kernel", type=int, default=0, help="sweep kernel: 0 auto, 1 generic, 2 windowed, 3 specialised")
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            t = [x.strip() for x in line.split(",")]
            if len(t) < 9:
                continue
            try:
                sm.append(float(t[1]))
                mx.append(float(t[2]))
            except ValueError:
                continue
            for n, v in zip(names, t[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.f.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


def profile_traffic():
    """DRAM bytes per sweep launch from the committed ncu summary, if any."""
    try:
        d = json.load(open(os.path.join(ROOT, "profiles", "sweep_traffic.json")))
        return d
    except (OSError, ValueError):
        return None


def issue_roofline(prof, sweep_s, clk, sms):
    """Instruction issue of the sweep: warp instructions per launch (ncu,
    the committed profile of this workload) over the launch's event time,
    against one warp instruction per clock per SM sub-partition (4 per SM)
    at the SM clock sampled during the timed region."""
    if not prof or not prof.get("warp_instructions_per_launch"):
        return None
    mhz = (clk or {}).get("sm_mhz") or 2070.0
    achieved = prof["warp_instructions_per_launch"] / sweep_s
    peak = 4.0 * sms * mhz * 1e6
    return {"bound": "issue", "achieved": achieved / 1e9, "peak": peak / 1e9, "unit": "G warp instructions/s",
            "frac": achieved / peak, "peak_source": "4 warp instructions/clock/SM at the sampled SM clock",
            "instructions_source": prof.get("source")}


def sweep_floor(local, sweep_s, attempts_per_chain, clk):
    """The weight sweep taken apart (muca_sweep_floor): SM cycles per attempt
    of one warp for the whole window and for each of its parts, beside the
    launch's own cycles per attempt per warp (event time x sampled SM clock /
    attempts per chain; one warp per SM sub-partition, as in the parts)."""
    import muca_gb300 as m
    mhz = (clk or {}).get("sm_mhz") or 2070.0
    out = {"unit": "SM cycles per attempt per warp", "geometry": "one block of 4 warps x 32 chains on one SM, "
           "L=72, lattice, FP32 weights and u32 histogram in shared memory, 4096 windows of 8 attempts per lane"}
    for part, name in enumerate(m.SWEEP_FLOOR_PARTS):
        out[name] = m.sweep_floor(part, local)
    out["kernel"] = sweep_s * mhz * 1e6 / attempts_per_chain
    return out


def cpu_oracle_rate(L, chains, nthreads, min_seconds=12.0, max_reps=200):
    """The reference algorithm on the host: full steps (therm=N, nup=N) of
    `chains` chains with `nthreads` POSIX threads; returns (attempts/ns, sample)."""
    import numpy as np
    from oracle import orc
    N = L * L
    lat = orc.init_lattice(L, chains, orc.scheme_weight(0, 0))
    ej, ed, _ = orc.energies(L, lat)
    w32 = np.zeros(N + 1, np.float32)
    done = 0
    t_total = 0.0
    reps = 0
    while reps < max_reps and (t_total < min_seconds or reps < 1):
        t0 = time.perf_counter()
        orc.weight_sweep(L, lat, ej, ed, w32, reps, 100, N, N, nthreads=nthreads)
        t_total += time.perf_counter() - t0
        done += chains * 2 * N
        reps += 1
    return done / (t_total * 1e9), ("%d step(s) of %d chains x (therm N + nup N) at L=%d, %.1f s wall"
                                    % (reps, chains, L, t_total))


def reference_arm(args, ws, rank):
    if rank != 0:
        return 0
    L, chains = args.L, args.chains
    N = L * L
    nthreads = os.cpu_count() or 1
    import numpy as np
    from oracle import orc
    orc.build()
    lat = orc.init_lattice(L, chains, orc.scheme_weight(0, 0))
    ej, ed, _ = orc.energies(L, lat)
    lnw = np.zeros(N + 1)
    h = np.zeros(N + 1, np.uint64)
    # a bounded sample of the workload per step: all chains when one step
    # takes at most ~2 s on this host, fewer otherwise
    t0 = time.perf_counter()
    sub = min(chains, 1024)
    orc.weight_sweep(L, lat[:sub], ej[:sub], ed[:sub], lnw.astype(np.float32), 0, 100, N, N, nthreads=nthreads)
    per_chain = (time.perf_counter() - t0) / sub
    sample = max(nthreads, min(chains, int(2.0 / max(per_chain, 1e-9))))
    lat, ej, ed = lat[:sample].copy(), ej[:sample].copy(), ed[:sample].copy()
    times = []
    for k in range(args.warmup + args.steps):
        h[:] = 0
        t0 = time.perf_counter()
        orc.weight_sweep(L, lat, ej, ed, lnw.astype(np.float32), k, 100, N, N, nthreads=nthreads, hist=h)
        orc.lib().orc_update_trivial_gpu(h, N, lnw)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
    attempts = sample * 2 * N
    v = attempts * len(times) / (sum(times) * 1e9)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "attempts/ns", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32+f32",
            "data": "synthetic (reference initial spins, zero initial weights)",
            "config": {"workload": "weight-estimation iteration, L=%d, %d chains, therm=N, nup=N, trivial update"
                                   % (L, chains), "L": L, "chains": chains, "chains_timed_per_step": sample},
            "cpu_baseline": {"value": v, "unit": "attempts/ns", "cores": nthreads, "kind": "port",
                             "sample": "%d of %d chains per step (therm N + nup N), %d steps" % (sample, chains,
                                                                                               len(times))},
            "e2e": {"value": v, "unit": "attempts/ns", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def ours_arm(args, ws, rank, local):
    import numpy as np
    import torch
    import muca_gb300 as m
    from muca_gb300 import build as b

    b.build()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist_
        dist_.init_process_group("nccl", device_id=torch.device("cuda", local))
        dist = dist_
    L, chains = args.L, args.chains
    N = L * L
    attempts_per_step = chains * 2 * N
    stream = torch.cuda.Stream()
    eng = m.Engine(L, nchains=chains, device=local, stream=stream.cuda_stream, dev_offset=rank, kernel=args.kernel)
    eng.init_chains(m.INIT_WEIGHT, 0)
    # the initialisation once more under CUDA events (lattices from the
    # reference's Philox scheme, then E_J and E_Delta): outside the timed
    # steps, reported beside them
    i0, i1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    i0.record(stream)
    eng.init_chains(m.INIT_WEIGHT, 0)
    i1.record(stream)
    i1.synchronize()
    init_ms = i0.elapsed_time(i1)
    eng.set_weights(np.zeros(N + 1))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    k = 0
    for _ in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.zero_()
        eng.sweep(k, 100, 1000, N, N)
        eng.update_weights(m.UPDATE_TRIVIAL, wait=False)
        k += 1
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier()
    t_wall0 = time.perf_counter()
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0, e1, e2 = ev[i]
        e0.record(stream)
        eng.sweep(k, 100, 1000, N, N)
        e1.record(stream)
        eng.update_weights(m.UPDATE_TRIVIAL, wait=False)
        e2.record(stream)
        k += 1
    barrier()
    t_wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    sweep_ms = [a.elapsed_time(b_) for a, b_, _ in ev]
    step_ms = [a.elapsed_time(c_) for a, _, c_ in ev]
    t_dev = sum(step_ms) * 1e-3
    # max over ranks
    if dist is not None:
        t = torch.tensor([t_dev, sum(sweep_ms) * 1e-3, t_wall], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_dev, t_sweep, t_wall = (float(x) for x in t.tolist())
    else:
        t_sweep = sum(sweep_ms) * 1e-3
    value = ws * attempts_per_step * args.steps / (t_dev * 1e9)

    # e2e through the C ABI with host buffers (pinned)
    h_w = torch.zeros(N + 1, dtype=torch.float64).pin_memory()
    h_hist = torch.zeros(N + 1, dtype=torch.int64).pin_memory()
    w_np = h_w.numpy()
    hist_np = h_hist.numpy().view(np.uint64)
    barrier()
    t_e2e = 0.0
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()  # L2 flushed before every step, outside the timed call
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        # weights in, sweep, update, weights and histogram out: one C-ABI call that returns after
        # its single synchronisation
        eng.iterate_host(w_np, k, 100, 1000, N, N, m.UPDATE_TRIVIAL, lnw_out=w_np, hist_out=hist_np)
        t_e2e += time.perf_counter() - t0
        k += 1
    barrier()
    if dist is not None:
        t = torch.tensor([t_e2e], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_e2e = float(t.item())
    e2e = ws * attempts_per_step * args.steps / (t_e2e * 1e9)

    out = None
    if rank == 0:
        peaks = measured_peaks()
        hbm_peak = peaks["hbm_gbs"] if peaks else 6800.0
        sweep_avg = t_sweep / args.steps
        att_rate = attempts_per_step / sweep_avg
        prof = profile_traffic()
        philox_peak = m.philox_peak(local, 7)
        out = {
            "metric": METRIC, "value": value, "unit": "attempts/ns", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32+f32",
            "data": "synthetic (reference initial spins, weights start at zero and follow the trivial update)",
            "config": {"workload": "weight-estimation iteration, L=%d (N=%d), %d chains, therm=N + nup=N attempts "
                                   "per chain, FP64 trivial update" % (L, N, chains),
                       "L": L, "chains_per_gpu": chains, "attempts_per_step_per_gpu": attempts_per_step,
                       "l2": "flushed before every timed step (256 MiB write, outside the events)",
                       "parallelism": "dp%d (independent chain shards, reference device = rank)" % ws,
                       "chains_per_block": eng.info.chains_per_block, "blocks": eng.info.blocks,
                       "smem_bytes": eng.info.smem_bytes},
            "e2e": {"value": e2e, "unit": "attempts/ns", "h2d_bytes_per_step": 8 * (N + 1),
                    "d2h_bytes_per_step": 16 * (N + 1) + 4,
                    "path": "muca_iterate_host (weights H2D, sweep, update, weights and histogram D2H, "
                            "one synchronisation) from pinned host buffers"},
            "roofline": {"bound": "hbm", "achieved": ALG_BYTES_PER_ATTEMPT * att_rate / 1e9, "peak": hbm_peak,
                         "unit": "GB/s", "frac": ALG_BYTES_PER_ATTEMPT * att_rate / 1e9 / hbm_peak,
                         "traffic": prof.get("dram_bytes_per_launch") if prof else None,
                         "peak_source": "measured" if peaks else "fallback",
                         "note": "lattice resident in shared memory; HBM is not the bound (see roofline_int)"},
            "roofline_int": {"bound": "int", "achieved": PHILOX_BLOCKS_PER_ATTEMPT * att_rate / 1e9,
                             "peak": philox_peak / 1e9, "unit": "G Philox4x32-7 blocks/s",
                             "frac": PHILOX_BLOCKS_PER_ATTEMPT * att_rate / philox_peak,
                             "peak_source": "measured (muca_philox_peak on this GPU)"},
            "roofline_issue": issue_roofline(prof, sweep_avg, clk, eng.info.sms),
            "sweep_floor": sweep_floor(local, sweep_avg, 2 * N, clk),
            "sweep_ms": 1e3 * sweep_avg, "init_ms": init_ms, "gpu_launches": 4 * args.steps,  # per step: the sweep and the three passes of the update
            "clocks": clk, "wall_s_timed_region": t_wall,
        }
    eng.close()
    if rank == 0 and ws == 1 and not args.no_ref_gpu:
        out["ref_gpu_kernel"] = ref_gpu_kernel_rate(L, chains)
    if rank == 0 and ws == 1 and not args.no_extra:
        for key, fn in (("flat_run", flat_run_metric), ("config2", config2_metric), ("batch", batch_metric),
                        ("production", production_metric), ("random_site", random_site_metric)):
            try:
                out[key] = fn(local)
            except Exception as ex:  # an extra line never fails the bench
                out[key] = {"error": str(ex)[:200]}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        nthreads = os.cpu_count() or 1
        v, sample = cpu_oracle_rate(L, chains, nthreads)
        out["cpu_baseline"] = {"value": v, "unit": "attempts/ns", "cores": nthreads, "kind": "port",
                               "sample": sample}
    if rank == 0:
        print(json.dumps(out))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def flat_run_metric(local):
    """Second metric of the L=72 configuration: weight iterations (and device
    time) until the histogram is flat at min/mean >= 0.5.  The update is the
    reference GPU program's trivial one (lnW -= ln H); the reference's
    weight_recursion, run to the same criterion, does not flatten within
    thousands of iterations from a zero weight."""
    import muca_gb300 as m
    L, nc = 72, 16384
    N = L * L
    with m.Engine(L, nchains=nc, device=local) as e:
        res, _ = e.weight_run(starting_M=N, rule=m.UPDATE_TRIVIAL, nup_schedule=1, flat_minmean=1, max_iter=6000,
                              nup_max=1 << 20, init_scheme=m.INIT_CHAIN_COUNTER, records=1, graph_iters=32)
    return {"metric": "weight iterations to a flat histogram (min/mean >= 0.5) at L=72", "L": L, "chains": nc,
            "iterations": res.iterations, "converged": bool(res.converged),
            "width_reached_iteration": res.width_reached_iter, "device_s": res.total_kernel_s,
            "wall_s": res.wall_s, "update": "trivial (lnW -= ln H for H > 1, then lnW -= lnW[0])",
            "schedule": "NUPDATES = N, doubling once the width is N (cap 2^20)",
            "init": "Philox4x32-10, key 2024, counter = chain id",
            "loop": "32 iterations (clear, sweep, update) per CUDA-graph replay; device_s = CUDA events "
                    "around the replays, wall_s = host clock of the whole run"}


def config2_metric(local, steps=10):
    """The L=72 configuration as written: runs from starting_M = 1 with
    NUPDATES doubling every iteration (cap 2^20), with the trivial update and
    with recursive_update = 1 (the reference's weight_recursion,
    muca_delta_multigpu.cu:833-859), to min/mean >= 0.5; then the headline
    step (sweep therm N + nup N, then the update) timed from the converged
    weights, with each update rule, and each update alone; and the sweep at
    the reference's own chain count (maxThreadsPerSM * SMs).  L2 is flushed
    before every timed step."""
    import numpy as np
    import torch
    import muca_gb300 as m
    L, nc = 72, 16384
    N = L * L
    out = {"L": L, "chains": nc}
    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    runs = {}
    w_conv = None
    plans = (("flat_run_reference_schedule", m.UPDATE_TRIVIAL, 0, 0, 20000,
              "NUPDATES = starting_M = 1 until the width is N, then (NUP + 1) * 1.01 per iteration "
              "(muca_delta_multigpu.cu:379-382)"),
             ("flat_run_doubling", m.UPDATE_TRIVIAL, 2, 1 << 14, 20000,
              "NUPDATES = starting_M = 1 doubling every iteration, capped at 2^14"),
             ("flat_run_recursion", m.UPDATE_RECURSION, 0, 0, 3000,
              "recursive_update = 1 (weight_recursion, muca_delta_multigpu.cu:833-859), reference schedule"))
    for key, rule, sched, cap, max_iter, desc in plans:
        with m.Engine(L, nchains=nc, device=local, stream=stream.cuda_stream) as e:
            res, _ = e.weight_run(starting_M=1, rule=rule, nup_schedule=sched, flat_minmean=1, max_iter=max_iter,
                                  nup_max=cap, records=1, graph_iters=32)
            if key == "flat_run_reference_schedule":
                w_conv = e.get_weights()
            h = e.histogram()
        runs[key] = {"schedule": desc, "iterations": res.iterations, "converged": bool(res.converged),
                     "width_reached_iteration": None if res.width_reached_iter == 0xFFFFFFFF else res.width_reached_iter,
                     "device_s": res.total_kernel_s, "wall_s": res.wall_s,
                     "attempts": int(res.total_run + res.iterations * N * nc),
                     "final_min_over_mean": float(h.min() / max(h.mean(), 1e-300))}
    out.update(runs)
    out["stop"] = "min/mean >= 0.5 (iteration cap as given); therm = N per iteration; 32 iterations per graph"
    # the headline step from the converged weights, each update rule
    steps_out = {}
    with m.Engine(L, nchains=nc, device=local, stream=stream.cuda_stream) as e:
        e.init_chains(m.INIT_WEIGHT, 0)
        for key, rule in (("trivial", m.UPDATE_TRIVIAL), ("recursion", m.UPDATE_RECURSION)):
            e.set_weights(w_conv)
            k = 0
            for _ in range(3):
                e.sweep(k, 100, 1000, N, N)
                e.update_weights(rule, wait=False)
                k += 1
            ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
            for i in range(steps):
                e.set_weights(w_conv)  # every timed step starts from the converged weights
                with torch.cuda.stream(stream):
                    flush.zero_()
                a, b, c = ev[i]
                a.record(stream)
                e.sweep(k, 100, 1000, N, N)
                b.record(stream)
                e.update_weights(rule, wait=False)
                c.record(stream)
                k += 1
            torch.cuda.synchronize()
            step_ms = [x[0].elapsed_time(x[2]) for x in ev]
            upd_ms = [x[1].elapsed_time(x[2]) for x in ev]
            steps_out[key] = {"value": 2 * N * nc * steps / (sum(step_ms) * 1e6), "unit": "attempts/ns",
                              "ms_per_step": sum(step_ms) / steps, "update_us": 1e3 * statistics.median(upd_ms),
                              "update_share": sum(upd_ms) / sum(step_ms)}
    out["steps_from_converged_weights"] = steps_out
    # the sweep at the reference's own chain count
    nd = m.default_chains(local)
    with m.Engine(L, nchains=nd, device=local, stream=stream.cuda_stream) as e:
        e.init_chains(m.INIT_WEIGHT, 0)
        e.set_weights(w_conv)
        e.sweep(0, 100, 1000, N, N)
        best = None
        for k in range(3):
            with torch.cuda.stream(stream):
                flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            e.sweep(k + 1, 100, 1000, N, N)
            b.record(stream)
            b.synchronize()
            t = a.elapsed_time(b)
            best = t if best is None else min(best, t)
        out["reference_default_chains"] = {"chains": nd, "value": nd * 2 * N / (best * 1e6), "unit": "attempts/ns",
                                           "ms": best, "lattice_in_smem": bool(e.info.lattice_in_smem),
                                           "chains_per_block": e.info.chains_per_block,
                                           "timing": "best of 3 sweeps (therm N + nup N), converged weights"}
    return out


def warm_start_metric(local):
    """The learned warm start on the batched configuration's instances:
    converged weights of every (L, T) with L in {16, 24, 32} and T on a grid
    of 0.40..0.80 in steps of 0.05 (1024 chains each) train the MLP on the
    device. Then 12 held-out (L, T, Delta) (T in {0.43, 0.53, 0.63, 0.73})
    run the weight iteration from four starts: the zero weight, the
    network's weight, and two non-learned starts. Every arm uses one
    NUPDATES schedule (x1.05 per iteration from 16 sweeps, capped at 2^18)
    and runs to min/mean >= 0.5; the study reports iterations, device time
    and wall time. The held-out instances at L = 16 (16384 chains each) then
    run to width == N and D_KL < 1e-5, for the agreement of the final
    weights with the zero arm's, beside the zero weight on other seeds. The
    reference's D_KL < 1e-4 resolves lnW only to a few 1e-2. Minutes of GPU
    time: not part of the default line."""
    from muca_gb300 import warm_start as ws
    out = ws.run_study(Ls=(16, 24, 32), chains=1024, t_step=0.05, held_sizes=(16, 24, 32), device=local,
                       agreement_Lmax=16, agreement_chains=16384, agreement_nup_max=1 << 21,
                       agreement_d_kl=1e-5, agreement_max_iter=1000, agreement_arms=("mlp",))
    ab = out["ab"]
    ag = out.get("agreement_reference_criterion", {})
    out["summary"] = {
        "iters_ratio_mlp_vs_zero": ab["mlp_iters_ratio"], "device_time_ratio_mlp_vs_zero": ab["mlp_time_ratio"],
        "iters_ratio_interp_vs_zero": ab["interp_iters_ratio"],
        "device_time_ratio_interp_vs_zero": ab["interp_time_ratio"],
        "iters_ratio_pl_vs_zero": ab["pl_iters_ratio"], "device_time_ratio_pl_vs_zero": ab["pl_time_ratio"],
        "ab_wall_s": ab.get("wall_s"),
        "final_lnw_rms_mlp_vs_zero_max": ag.get("mlp", {}).get("final_rms_vs_zero_max"),
        "final_lnw_rms_reseeded_zero_vs_zero_max": ag.get("zero_reseeded", {}).get("final_rms_vs_zero_max")}
    return out


def mlp_metric(local, steps=2048, batch=4096):
    """Training throughput of the warm-start network on this GPU: `steps`
    Adam steps (minibatch gather, forward, backward, weight gradients,
    update; 32 steps per CUDA graph) at batch 4096 on a synthetic set of the
    warm start's size (663,816 points: every bin of 17 temperatures at each
    L in {16..128}).  FLOPs per step: 6 x parameters x batch (the forward
    product, and the two backward products)."""
    import numpy as np
    import muca_gb300 as m
    rng = np.random.default_rng(0)
    n = 663816
    x = np.stack([rng.choice([16, 24, 32, 48, 64, 72, 96, 128], n) / 128.0, rng.uniform(0.4, 0.8, n),
                  rng.uniform(1.5, 1.99, n), rng.uniform(0.0, 1.0, n)], axis=1).astype(np.float32)
    t = (np.sin(3.0 * x[:, 3]) * x[:, 1] - 0.5 * x[:, 0] * x[:, 3] ** 2).astype(np.float32)
    with m.MLP(device=local, seed=1) as net:
        net.set_data(x, t)
        net.train(64, batch=batch, lr=1e-3, seed=2)  # warm-up: graph capture, scratch
        t0 = time.perf_counter()
        losses = net.train(steps, batch=batch, lr=1e-3, seed=3)
        dt = time.perf_counter() - t0
        flops = 6.0 * net.n_params * batch * steps
    return {"metric": "warm-start network training throughput", "steps": steps, "batch": batch,
            "params": int(net.n_params), "s": dt, "steps_per_s": steps / dt, "tflops": flops / dt / 1e12,
            "unit": "TFLOP/s (FP32, CUDA cores)", "loss_first": float(losses[:8].mean()),
            "loss_last": float(losses[-64:].mean()),
            "timing": "host clock around the train call (graph replays and one synchronisation)"}


def batch_metric(local, iters=32):
    """The batched engine on 256 uneven instances (L in {16..128}, T in
    [0.4, 0.8], 256 chains each, seed = instance id): device throughput of
    `iters` graph-captured iterations at NUPDATES = N per instance."""
    import numpy as np
    import muca_gb300 as m
    Ls = [16, 24, 32, 48, 64, 72, 96, 128]
    inst = []
    for i in range(256):
        r = np.random.default_rng(i)
        inst.append((int(r.choice(Ls)), 256, 1.0 / float(r.uniform(0.4, 0.8)), i))
    with m.Batch(inst, device=local) as b:
        info = b.info()
        res, sec = b.run(starting_sweeps=1, rule=m.UPDATE_TRIVIAL, nup_schedule=0, flat_minmean=1, max_iter=iters,
                         graph_iters=iters)
    att = sum(r.iterations * L * L * nc + r.total_run for r, (L, nc, _, _) in zip(res, inst))
    return {"metric": "batched weight iterations, spin-flip attempts/ns", "value": att / (sec * 1e9),
            "unit": "attempts/ns", "instances": len(inst), "iterations": iters, "attempts": att, "device_s": sec,
            "shape": {"chains_per_block": info.shape.chains_per_block, "lattice_in_smem": info.shape.lattice_in_smem,
                      "hist_in_smem": info.shape.hist_in_smem, "blocks_per_sm": info.shape.blocks_per_sm,
                      "shapes_tried": info.n_tried},
            "graph": "%d iterations (clear, persistent sweep, update) per CUDA graph" % iters}


def random_site_metric(local, L=72, nc=16384):
    """The CPU weight program's random-site algorithm (muca_mag.cpp:312-393:
    random site, three Philox streams, FP64 weights) on the device
    (MUCA_ALGO_RANDOM_SITE), at the headline's L and chain count: one sweep
    of therm = N and nup = N attempts per chain, CUDA events around the
    launch (best of 3 after a warm-up).  host_logf 0 decides with CUDA's
    logf (the reference's mcs2), 1 with the host libm's (bit-exact with the
    CPU program).  Beside it, the oracle's restatement of muca_mag's mcs on
    every chain with all host threads: the reference CPU algorithm."""
    import numpy as np
    import torch
    import muca_gb300 as m
    from concurrent.futures import ThreadPoolExecutor
    from oracle import orc
    N = L * L
    att = nc * 2 * N
    out = {"metric": "random-site sweep attempts/ns at L=%d (the CPU weight program's algorithm)" % L,
           "unit": "attempts/ns", "chains": nc, "attempts_per_chain": 2 * N,
           "timing": "CUDA events around one sweep launch, best of 3 after a warm-up; zero weights"}
    stream = torch.cuda.Stream()
    for hl, key in ((0, "cuda_logf"), (1, "host_logf")):
        with m.Engine(L, nchains=nc, device=local, algorithm=m.ALGO_RANDOM_SITE, host_logf=hl,
                      stream=stream.cuda_stream) as e:
            e.set_weights(np.zeros(N + 1))
            e.init_chains(m.INIT_MUCA_MAG, 0)
            e.sweep(0, 0, 0, N, N)
            best = None
            for k in range(3):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                e.sweep(k + 1, 0, 0, N, N)
                b.record(stream)
                b.synchronize()
                t = a.elapsed_time(b)
                best = t if best is None else min(best, t)
        out[key] = att / (best * 1e6)
        out[key + "_ms"] = best
    # the oracle's muca_mag mcs over every chain, all host threads (ctypes
    # releases the interpreter lock during each call)
    Lb = orc.lib()
    lat = orc.init_lattice(L, nc, orc.scheme_muca_mag(0))
    ej, ed, _ = orc.energies(L, lat)
    lnw = np.zeros(N + 1)
    nthreads = os.cpu_count() or 1

    def chains(lo, hi):
        hc = np.zeros(N + 1, np.uint64)
        e1 = np.zeros(1, np.int32)
        e2 = np.zeros(1, np.int32)
        for c in range(lo, hi):
            e1[0], e2[0] = ej[c], ed[c]
            Lb.orc_muca_mag_mcs(L, c, lat[c], e1, e2, lnw, hc, 1, 0, N, N)

    bounds = np.linspace(0, nc, nthreads + 1).astype(int)
    t0 = time.perf_counter()
    with ThreadPoolExecutor(nthreads) as ex:
        list(ex.map(lambda i: chains(bounds[i], bounds[i + 1]), range(nthreads)))
    dt = time.perf_counter() - t0
    out["cpu"] = {"value": att / (dt * 1e9), "unit": "attempts/ns", "cores": nthreads, "kind": "port",
                  "sample": "all %d chains, one sweep (therm N + nup N), %.1f s wall" % (nc, dt)}
    return out


def converge_weight(L, local, nc=16384, stream=None):
    """A converged weight of the L=72 configuration's kind at size L: the
    trivial update from zero weights, therm = N and NUPDATES = N doubling
    once the width is N (cap 2^20), Philox4x32-10 initial spins (key 2024,
    counter = chain id), until min/mean >= 0.5; 32 iterations per CUDA-graph
    replay.  Returns (weights, the chains' final lattices, summary)."""
    import muca_gb300 as m
    N = L * L
    with m.Engine(L, nchains=nc, device=local, stream=stream) as e:
        res, _ = e.weight_run(starting_M=N, rule=m.UPDATE_TRIVIAL, nup_schedule=1, flat_minmean=1, max_iter=20000,
                              nup_max=1 << 20, init_scheme=m.INIT_CHAIN_COUNTER, records=1, graph_iters=32)
        w = e.get_weights()
        lat = e.get_lattice()
    return w, lat, {"L": L, "chains": nc, "iterations": res.iterations, "converged": bool(res.converged),
                    "width_reached_iteration": res.width_reached_iter, "device_s": res.total_kernel_s,
                    "wall_s": res.wall_s, "lnW_range": float(w.max() - w.min())}


def cpu_produce_rate(L, lnw, nthreads, min_seconds=10.0):
    """The reference CPU production algorithm (produce.cpp mcs, restated and
    pinned in the oracle) with one chain per host thread, as produce_mpi runs
    one chain per rank: production sweeps from the given weight, repeated
    until about min_seconds of wall time; returns (attempts/ns, sample)."""
    import numpy as np
    from concurrent.futures import ThreadPoolExecutor
    from oracle import orc
    Lb = orc.lib()
    N = L * L
    lnw = np.ascontiguousarray(lnw, np.float64)
    lats, st, hists = [], [], []
    for r in range(nthreads):
        lat = orc.init_lattice(L, 1, Lb.orc_scheme_produce_cpu(0), chain0=r).reshape(-1).copy()
        ej, ed, mg = (np.array([v[0]], np.int32) for v in orc.energies(L, lat[None, :]))
        lats.append(lat)
        st.append((ej, ed, mg))
        hists.append(np.zeros((N + 1) * (N + 2) // 2, np.uint64))  # lazily mapped; one per rank

    def run(r, k, sweeps):
        ej, ed, mg = st[r]
        Lb.orc_produce_cpu_mcs(L, r, lats[r], ej, ed, mg, lnw, hists[r], 0, k, 0, sweeps * N)

    done, t_total, k, sweeps = 0, 0.0, 0, 1
    with ThreadPoolExecutor(nthreads) as ex:
        while t_total < min_seconds:
            t0 = time.perf_counter()
            list(ex.map(lambda r: run(r, k, sweeps), range(nthreads)))
            dt = time.perf_counter() - t0
            t_total += dt
            done += nthreads * sweeps * N
            k += 1
            sweeps = max(1, min(64, int(sweeps * 2 if dt < 2.0 else sweeps)))
    return done / (t_total * 1e9), ("%d chains (one per host thread), %d production sweeps each at L=%d from the "
                                    "converged weight, %.1f s wall" % (nthreads, done // (nthreads * N), L, t_total))


def production_metric(local, L=128, with_ref=True, kernel=0, blocks=10, therm_sweeps=100, block_sweeps=100,
                      with_cpu=True, state_in=None, state_out=None):
    """The L=128 production configuration with its shapes and scaled sweep
    counts: a converged L=128 weight (converge_weight), 16384 chains from the
    reference production initialisation, `therm_sweeps` thermalisation
    sweeps, then `blocks` jackknife blocks of `block_sweeps` production
    sweeps each (the JACKS blocks of produce.cpp:201-247; seeds of the
    reference's block loop, produce2_multigpu.cu:324-347), every block's 2D
    (E_Delta, M) histogram reweighted at Delta = 1.96 (produce2_multigpu.cu:
    293-300,498-518) into <|M|>, chi and U4, jackknifed over the blocks.
    The configuration asks for 10^5 thermalisation and 10^7 production sweeps;
    the run scales them by therm_sweeps / 10^5 and blocks * block_sweeps / 10^7.
    So few sweeps move a walker only ~10^3 bins along E_Delta (N + 1 =
    16385 bins), so the chains start from the weight run's final lattices,
    which the converged multicanonical walk has spread over all of E_Delta,
    instead of fresh random spins (E_Delta ~ 2N/3 for every chain): from
    there no block would sample the E_Delta that dominate the reweighting at
    Delta = 1.96, and every Boltzmann factor of the rows it did sample would
    underflow.

    state_out / state_in: save the converged weight and lattices to an .npz
    file, or start from one instead of converging (to profile the
    production sweep alone)."""
    import numpy as np
    import torch
    import muca_gb300 as m
    nc = 16384
    N = L * L
    beta, delta = 2.0, 1.96
    stream = torch.cuda.Stream()
    if state_in:
        st = np.load(state_in)
        w, lat_w, wsum = st["w"], st["lat"], {"from": "saved state", "L": L}
    else:
        w, lat_w, wsum = converge_weight(L, local, nc, stream.cuda_stream)
    if state_out:
        np.savez(state_out, w=w, lat=lat_w)
    per_block = []
    with m.Engine(L, nchains=nc, device=local, mode=m.MODE_PRODUCE, stream=stream.cuda_stream, kernel=kernel) as e:
        e.set_lattice(lat_w)  # the equilibrated multicanonical walkers
        del lat_w
        e.set_weights(w)
        e.weight_shift(beta, delta)  # the reweighting copy only; the sweep keeps w
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        e.sweep(0, 100, 1000, therm_sweeps * N, 0)  # thermalisation: iter 0, seed SEED+1000*GPU+l (l = 0)
        a1.record(stream)
        sweep_ms, obs_ms = [], []
        for jj in range(blocks):
            b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            b0.record(stream)
            e.sweep(jj, 100, 2000, 0, block_sweeps * N)  # block jj: iter jj, seed SEED+2000*GPU+l
            b1.record(stream)
            b1.synchronize()
            t0 = time.perf_counter()
            o = e.observables(beta, delta)  # launch, reweighting kernels, read-back
            obs_ms.append(1e3 * (time.perf_counter() - t0))
            per_block.append((o.m_abs, o.chi, o.u4))
            sweep_ms.append(b0.elapsed_time(b1))
        torch.cuda.synchronize()
        therm_ms = a0.elapsed_time(a1)
        info = e.info
        jk = [e.jackknife(np.array([pb[i] for pb in per_block])) for i in range(3)]
    att = nc * block_sweeps * N * blocks
    bins = (N + 1) * (N + 2) // 2
    out = {"metric": "production sweep attempts/ns at L=%d" % L, "value": att / (sum(sweep_ms) * 1e6),
           "unit": "attempts/ns", "chains": nc, "kernel": info.kernel, "lattice_in_smem": info.lattice_in_smem,
           "weight": wsum,
           "therm": {"sweeps": therm_sweeps, "ms": therm_ms,
                     "value": nc * therm_sweeps * N / (therm_ms * 1e6)},
           "start": "the weight run's final lattices (spread over E_Delta by the converged walk)",
           "blocks": blocks, "block_sweeps": block_sweeps,
           "scale": {"therm": therm_sweeps / 1e5, "production": blocks * block_sweeps / 1e7},
           "observables": {"delta": delta, "beta": beta,
                           "m_abs": {"value": jk[0][0], "jackknife_error": jk[0][1]},
                           "chi": {"value": jk[1][0], "jackknife_error": jk[1][1]},
                           "u4": {"value": jk[2][0], "jackknife_error": jk[2][1]},
                           "per_block": [list(pb) for pb in per_block]},
           "timing": "CUDA events around each block's production launch",
           "reweighting": {"bins": bins, "ms": statistics.median(obs_ms), "GB_per_s": 8 * bins / statistics.median(
               obs_ms) / 1e6, "timing": "host clock per block (launch, two kernels, read-back of 4 sums), median"}}
    ref = None
    try:  # the reference production kernel on the same lattice, weights and step
        if not with_ref:
            raise RuntimeError("not requested")
        from oracle import orc
        orc.build(refgpu=True)
        if orc.refgpu() is not None:
            with m.Engine(L, nchains=nc, device=local, mode=m.MODE_PRODUCE) as e2:
                e2.init_chains(m.INIT_PRODUCE, 0)
                lat0 = e2.get_lattice()
            z = np.zeros(nc, np.int32)
            lat1, _, ej, ed, mg, _ = orc.refgpu_produce(L, lat0, w, z, z, z, 0, 100, N, 0, compute_energies=True)
            _, _, _, _, _, ms = orc.refgpu_produce(L, lat1, w, ej, ed, mg, 1, 100, 0, 4 * N)
            ref = {"value": nc * 4 * N / (ms * 1e6), "ms": ms, "sweeps": 4,
                   "kernel": "produce2_multigpu.cu mcs, compiled for sm_103a, same lattice and converged weights"}
    except Exception as ex:  # noqa: BLE001
        ref = {"unavailable": str(ex)[:200]}
    out["ref_gpu_kernel"] = ref
    if with_cpu:
        nthreads = os.cpu_count() or 1
        v, sample = cpu_produce_rate(L, w, nthreads)
        out["cpu_baseline"] = {"value": v, "unit": "attempts/ns", "cores": nthreads, "kind": "port",
                               "sample": sample}
    return out


def ref_gpu_kernel_rate(L, chains):
    """The reference weight kernel (muca_delta_multigpu.cu:737-829, compiled
    unchanged for sm_103a) on the same step, at the config's chain count and
    at the reference's own default (maxThreadsPerSM * SMs).  Spins come from
    the reference initialisation (our device init, which equals it); the
    reference's own init kernels form E_J and E_Delta."""
    try:
        import numpy as np
        from oracle import orc
        orc.build(refgpu=True)
        if orc.refgpu() is None:
            return {"unavailable": "reference cubins not present"}
        import muca_gb300 as m
        N = L * L
        res = {"unit": "attempts/ns", "step": "therm=N + nup=N attempts per chain, one launch"}
        for label, nw in (("config_chains", chains), ("reference_default_chains", m.default_chains(0))):
            nw = nw // 256 * 256
            with m.Engine(L, nchains=nw) as e:
                e.init_chains(m.INIT_WEIGHT, 0)
                lat = e.get_lattice()
            z = np.zeros(nw, np.int32)
            w32 = np.zeros(N + 1, np.float32)
            lat, _, ej, ed, _ = orc.refgpu_weight(L, lat, w32, z, z, 0, 100, N, 0, compute_energies=True)
            _, _, _, _, ms = orc.refgpu_weight(L, lat, w32, ej, ed, 1, 100, N, N)
            res[label] = {"chains": nw, "value": nw * 2 * N / (ms * 1e6), "ms": ms}
        return res
    except Exception as ex:  # report, never fail the bench on the extra line
        return {"unavailable": str(ex)[:200]}


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return reference_arm(args, ws, rank)
    if args.only:
        import torch
        torch.cuda.set_device(local)
        from muca_gb300 import build as b
        b.build()
        fn = {"flat_run": flat_run_metric, "config2": config2_metric, "batch": batch_metric,
              "random_site": random_site_metric, "warm_start": warm_start_metric,
              "mlp": lambda d: mlp_metric(d, steps=args.mlp_steps),
              "production": lambda d: production_metric(d, args.production_L, with_ref=False, kernel=args.kernel,
                                                        blocks=args.blocks, block_sweeps=args.block_sweeps,
                                                        therm_sweeps=args.therm_sweeps,
                                                        with_cpu=not args.no_cpu_baseline,
                                                        state_in=args.state_in, state_out=args.state_out)}[args.only]
        print(json.dumps(fn(local)))
        return 0
    return ours_arm(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
