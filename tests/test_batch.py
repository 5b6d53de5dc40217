"""Batches of weight runs (muca_batch_*): with beta = 2 every instance equals
a single simulation with the same seeds (muca_params.dev_offset = seed), bit
for bit, for every block shape the autotuner can pick; with another beta it
equals the oracle's weight loop with the FP32 term (float)(-beta*dE).  The
reference loop these follow is muca_delta_multigpu.cu:374-477."""
import ctypes

import numpy as np
import pytest

# uneven sizes, chain counts that divide and do not divide the block shapes
INSTANCES = [(16, 256, 2.0, 0), (24, 96, 2.0, 1), (8, 64, 2.0, 2), (32, 128, 2.0, 3)]
SHAPES = [(32, 0, 0), (64, 1, 0), (128, 0, 1), (256, 1, 1), None]


def _single(muca, L, nc, seed, **kw):
    with muca.Engine(L, nchains=nc, dev_offset=seed) as e:
        r, _ = e.weight_run(starting_M=1, records=1, **kw)
        return r, e.get_weights(), e.histogram()


def test_batch_rejects_bad_instances():
    """Checked before any CUDA call: no GPU needed."""
    from muca_gb300 import build as b
    b.build()
    import muca_gb300 as m
    for bad, msg in (([(12, 64, 2.0, 0)], "multiple of 8"), ([(136, 64, 2.0, 0)], "8..128"),
                     ([(16, 0, 2.0, 0)], "nchains"), ([(16, 64, 0.0, 0)], "beta"),
                     ([(16, 64, float("nan"), 0)], "beta"), ([], "instances")):
        with pytest.raises(m.MucaError, match=msg):
            m.Batch(bad)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "autotune" if s is None else "cpb%d_lat%d_hist%d" % s)
def test_batch_equals_single_simulations(muca, shape):
    kw = dict(flat_minmean=1, max_iter=60)
    with muca.Batch(INSTANCES, shape=shape) as b:
        res, sec = b.run(starting_M=1, graph_iters=8, **kw)
        ws = [b.get_weights(i) for i in range(len(INSTANCES))]
        hs = [b.histogram(i) for i in range(len(INSTANCES))]
        info = b.info()
    assert sec > 0
    if shape is not None:
        assert (info.shape.chains_per_block, info.shape.lattice_in_smem, info.shape.hist_in_smem) == shape
    for i, (L, nc, beta, seed) in enumerate(INSTANCES):
        r, w, h = _single(muca, L, nc, seed, **kw)
        assert (res[i].iterations, res[i].converged) == (r.iterations, r.converged), i
        assert res[i].total_run == r.total_run, i
        np.testing.assert_array_equal(ws[i], w, err_msg="instance %d" % i)
        np.testing.assert_array_equal(hs[i], h, err_msg="instance %d" % i)


# lattice placement 2: in shared memory for the instances whose block fits
# (L = 16 and 72 here), in global memory for the rest (L = 128)
MIXED = [(128, 64, 2.0, 5), (16, 256, 2.0, 0), (72, 128, 2.0, 6)]


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(128, 2, 1), (64, 2, 0)], ids=lambda s: "cpb%d_lat%d_hist%d" % s)
def test_batch_lattice_where_it_fits_equals_single_simulations(muca, shape):
    kw = dict(flat_minmean=1, max_iter=12)
    with muca.Batch(MIXED, shape=shape) as b:
        res, _ = b.run(starting_M=1, graph_iters=4, **kw)
        ws = [b.get_weights(i) for i in range(len(MIXED))]
        hs = [b.histogram(i) for i in range(len(MIXED))]
        info = b.info()
    assert (info.shape.chains_per_block, info.shape.lattice_in_smem, info.shape.hist_in_smem) == shape
    for i, (L, nc, beta, seed) in enumerate(MIXED):
        r, w, h = _single(muca, L, nc, seed, **kw)
        assert (res[i].iterations, res[i].total_run) == (r.iterations, r.total_run), i
        np.testing.assert_array_equal(ws[i], w, err_msg="instance %d" % i)
        np.testing.assert_array_equal(hs[i], h, err_msg="instance %d" % i)


@pytest.mark.gpu
def test_batch_graded_init_equals_single_simulations(muca):
    """graded_init = 1 with reinit_chains: instance i starts from the
    MUCA_INIT_GRADED spins of a single context with dev_offset = seed."""
    kw = dict(flat_minmean=1, max_iter=20)
    inst = INSTANCES[:3]
    with muca.Batch(inst) as b:
        res, _ = b.run(starting_M=1, graph_iters=4, reinit_chains=1, graded_init=1, **kw)
        ws = [b.get_weights(i) for i in range(len(inst))]
        hs = [b.histogram(i) for i in range(len(inst))]
    for i, (L, nc, beta, seed) in enumerate(inst):
        with muca.Engine(L, nchains=nc, dev_offset=seed) as e:
            r, _ = e.weight_run(starting_M=1, records=1, init_scheme=muca.INIT_GRADED, **kw)
            w, h = e.get_weights(), e.histogram()
        assert (res[i].iterations, res[i].total_run) == (r.iterations, r.total_run), i
        np.testing.assert_array_equal(ws[i], w, err_msg="instance %d" % i)
        np.testing.assert_array_equal(hs[i], h, err_msg="instance %d" % i)


@pytest.mark.gpu
@pytest.mark.parametrize("sched", [0, 3, 4, 5])
def test_batch_schedules_equal_single_simulations(muca, sched):
    kw = dict(nup_schedule=sched, flat_minmean=1, max_iter=25, nup_max=1 << 14)
    inst = INSTANCES[:3]
    with muca.Batch(inst) as b:
        res, _ = b.run(starting_M=1, graph_iters=4, **kw)
        ws = [b.get_weights(i) for i in range(len(inst))]
    for i, (L, nc, beta, seed) in enumerate(inst):
        r, w, _ = _single(muca, L, nc, seed, **kw)
        assert (res[i].iterations, res[i].total_run) == (r.iterations, r.total_run), i
        np.testing.assert_array_equal(ws[i], w, err_msg="instance %d" % i)


@pytest.mark.gpu
def test_batch_recursion_doubling_equals_single_simulations(muca):
    kw = dict(rule=muca.UPDATE_RECURSION, nup_schedule=1, flat_minmean=1, max_iter=40)
    inst = INSTANCES[:3]
    with muca.Batch(inst) as b:
        res, _ = b.run(starting_M=1, graph_iters=5, **kw)
        ws = [b.get_weights(i) for i in range(len(inst))]
    for i, (L, nc, beta, seed) in enumerate(inst):
        r, w, _ = _single(muca, L, nc, seed, **kw)
        assert (res[i].iterations, res[i].converged) == (r.iterations, r.converged), i
        np.testing.assert_array_equal(ws[i], w, err_msg="instance %d" % i)


@pytest.mark.gpu
def test_batch_other_beta_vs_oracle(muca, orc):
    inst = [(8, 64, 1.6, 5), (16, 32, 2.5, 6), (8, 32, 0.7, 7)]
    max_iter = 40
    with muca.Batch(inst) as b:
        res, _ = b.run(starting_M=1, flat_minmean=1, max_iter=max_iter)
        ws = [b.get_weights(i) for i in range(len(inst))]
    Lb = orc.lib()
    try:
        for i, (L, nc, beta, seed) in enumerate(inst):
            N = L * L
            Lb.orc_set_beta(beta)
            o = orc.WeightOpts(L=L, nchains=nc, jack=0, gpu=seed, starting_M=1, recursive=0, hold_until_full=0,
                               flat_minmean=1, max_iter=max_iter, rounds=7, nthreads=8, width_start=0)
            lat = orc.init_lattice(L, nc, orc.scheme_weight(0, seed)).reshape(-1).copy()
            ej, ed, _ = orc.energies(L, lat.reshape(nc, N))
            lnw = np.zeros(N + 1)
            pacc = np.zeros(N + 1)
            rec = np.zeros(5 * max_iter)
            conv = ctypes.c_int()
            it = Lb.orc_weight_run(ctypes.byref(o), lat, ej, ed, lnw, pacc, rec, max_iter, ctypes.byref(conv))
            assert (res[i].iterations, res[i].converged) == (it, conv.value), i
            np.testing.assert_allclose(ws[i], lnw, rtol=1e-12, atol=1e-9, err_msg="instance %d" % i)
    finally:
        Lb.orc_set_beta(0.0)


@pytest.mark.gpu
def test_batch_warm_start_and_rerun(muca):
    """set_weights is the warm start of the next run; a rerun with fresh
    chains and the same warm start repeats the result."""
    L, nc, seed = 16, 128, 4
    rng = np.random.default_rng(3)
    w0 = np.cumsum(rng.normal(-0.3, 0.2, L * L + 1))
    kw = dict(flat_minmean=1, max_iter=50)
    with muca.Engine(L, nchains=nc, dev_offset=seed) as e:
        e.set_weights(w0)
        r, _ = e.weight_run(starting_M=1, records=1, **kw)
        w = e.get_weights()
    with muca.Batch([(L, nc, 2.0, seed), (8, 64, 2.0, 9)]) as b:
        out = []
        for _ in range(2):
            b.set_weights(0, w0)
            b.set_weights(1, np.zeros(65))
            res, _ = b.run(starting_M=1, reinit_chains=1, **kw)
            out.append((res[0].iterations, b.get_weights(0)))
    for its, wb in out:
        assert its == r.iterations
        np.testing.assert_array_equal(wb, w)


@pytest.mark.gpu
def test_batch_autotuner_table(muca):
    with muca.Batch(INSTANCES) as b:
        info = b.info()
    tried = [info.tried[k] for k in range(info.n_tried)]
    assert len(tried) >= 4
    assert info.shape.ms == min(t.ms for t in tried)
    assert info.grid % 152 == 0 or info.grid > 0
    assert info.n_items == sum((nc + info.shape.chains_per_block - 1) // info.shape.chains_per_block
                               for _, nc, _, _ in INSTANCES)
