"""Bit-exact parity of the sweeps whose lattice stays in global memory.

The planner keeps a block's lattice in shared memory whenever that fits in
as few waves of blocks as global placement; otherwise (L = 128 in every
mode, production's FP64 table at large L, or more chains than one wave of
shared-memory blocks holds) the kernels read and write the packed lattice in
global memory through L1/L2.  That is the path of the L = 128 production
configuration and of the largest batch instances.  Every test here asserts
`lattice_in_smem == 0` and compares lattices, E_J, E_Delta, M and
histograms bit for bit with the oracle (the reference kernels restated on
the CPU) and with the reference's own kernels compiled for this GPU
(muca_delta_multigpu.cu:737-829, produce2_multigpu.cu:401-496).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 100


def _random_walk_weights(N, rng, sigma=1.5):
    # differences straddling the Metropolis threshold
    return np.cumsum(rng.normal(0.0, sigma, N + 1)) * 0.5


def _muca_like_weights(N, rng):
    # the shape of a converged multicanonical weight over E_Delta: a steady
    # drift of lnW over [0, N] (range ~ 10^4 at L = 128) with small noise
    w = np.cumsum(rng.normal(-0.6, 0.3, N + 1))
    return w - w[0]


def _i32(a):
    return np.ascontiguousarray(a, np.int32).copy()


def _run_produce(muca, L, nch, kernel, lnw, therm, nup, it=5):
    with muca.Engine(L, nchains=nch, mode=muca.MODE_PRODUCE, kernel=kernel) as e:
        assert e.info.lattice_in_smem == 0, "expected the lattice in global memory"
        e.set_weights(lnw)
        e.init_chains(muca.INIT_PRODUCE, 0)
        lat0 = e.get_lattice()
        ej0, ed0, mg0 = e.chain_state()
        e.sweep(it, SEED, 2000, therm, nup)
        lat1 = e.get_lattice()
        ej1, ed1, mg1 = e.chain_state()
        h = e.histogram()
        used = e.info.kernel
    return used, (lat0, ej0, ed0, mg0), (lat1, ej1, ed1, mg1), h


# (L, chains, kernel): 0 = the planner's choice (the windowed kernel behind
# the row ring for production with a global lattice), 1 generic, 2 windowed,
# 3 specialised;
# 100 chains leave padding lanes in the last warp
PRODUCE_CASES = [(128, 128, 0), (128, 64, 1), (128, 64, 2), (128, 100, 3)]


@pytest.mark.parametrize("L,nch,kernel", PRODUCE_CASES)
@pytest.mark.parametrize("weights", ["random_walk", "muca_like"])
def test_produce_global_lattice_vs_oracle(muca, orc, L, nch, kernel, weights):
    N = L * L
    rng = np.random.default_rng(L + nch + kernel)
    lnw = _random_walk_weights(N, rng) if weights == "random_walk" else _muca_like_weights(N, rng)
    therm, nup = N, 3000 + 7
    used, (lat0, ej0, ed0, mg0), (lat1, ej1, ed1, mg1), h = _run_produce(muca, L, nch, kernel, lnw, therm, nup)
    if kernel == 0:
        assert used == 2, "the planner's production kernel with a global lattice is the windowed one"
    oej, oed, omg = _i32(ej0), _i32(ed0), _i32(mg0)
    olat, oh = orc.produce_sweep(L, lat0.copy(), oej, oed, omg, lnw, 5, SEED, therm, nup, nthreads=8)
    np.testing.assert_array_equal(lat1, olat)
    np.testing.assert_array_equal(ed1, oed)
    np.testing.assert_array_equal(ej1, oej)
    np.testing.assert_array_equal(mg1, omg)
    assert np.array_equal(h, oh), "2D histogram differs from the oracle (%d bins)" % int((h != oh).sum())
    assert int(h.sum()) == nch * nup


@pytest.mark.parametrize("kernel", [0, 1, 2, 3])
def test_produce_global_lattice_vs_reference_kernel(muca, orc, refgpu, kernel):
    L, nch = 128, 256
    N = L * L
    rng = np.random.default_rng(40 + kernel)
    lnw = _muca_like_weights(N, rng)
    therm, nup = N, 2000 + 3
    _, (lat0, ej0, ed0, mg0), (lat1, ej1, ed1, mg1), h = _run_produce(muca, L, nch, kernel, lnw, therm, nup, it=2)
    rl, rh, rej, red, rmg, _ = orc.refgpu_produce(L, lat0, lnw, ej0, ed0, mg0, 2, SEED, therm, nup)
    np.testing.assert_array_equal(lat1, rl)
    np.testing.assert_array_equal(ed1, red)
    np.testing.assert_array_equal(ej1, rej)
    np.testing.assert_array_equal(mg1, rmg)
    assert np.array_equal(h, rh), "2D histogram differs from the reference kernel"


@pytest.mark.parametrize("kernel", [1, 2, 3])
def test_weight_global_lattice_L128_vs_oracle(muca, orc, kernel):
    L, nch = 128, 64
    N = L * L
    rng = np.random.default_rng(128 + kernel)
    lnw = _random_walk_weights(N, rng)
    therm, nup = N, N + 2000 + 5
    with muca.Engine(L, nchains=nch, kernel=kernel) as e:
        assert e.info.lattice_in_smem == 0
        e.set_weights(lnw)
        e.init_chains(muca.INIT_WEIGHT, 1)
        lat0 = e.get_lattice()
        ej0, ed0, _ = e.chain_state()
        e.sweep(4, SEED, 1000, therm, nup)
        lat1 = e.get_lattice()
        ej1, ed1, _ = e.chain_state()
        h = e.histogram()
    oej, oed = _i32(ej0), _i32(ed0)
    olat, oh = orc.weight_sweep(L, lat0.copy(), oej, oed, lnw.astype(np.float32), 4, SEED, therm, nup, nthreads=8)
    np.testing.assert_array_equal(lat1, olat.reshape(nch, N))
    np.testing.assert_array_equal(ed1, oed)
    np.testing.assert_array_equal(ej1, oej)
    np.testing.assert_array_equal(h, oh)


@pytest.mark.parametrize("kernel", [1, 2, 3])
def test_weight_global_lattice_L128_vs_reference_kernel(muca, orc, refgpu, kernel):
    L, nch = 128, 256
    N = L * L
    rng = np.random.default_rng(7 * kernel)
    lnw = _random_walk_weights(N, rng)
    w32 = lnw.astype(np.float32)
    therm, nup = N, 3001
    with muca.Engine(L, nchains=nch, kernel=kernel) as e:
        assert e.info.lattice_in_smem == 0
        e.set_weights(lnw)
        e.init_chains(muca.INIT_WEIGHT, 0)
        lat0 = e.get_lattice()
        ej0, ed0, _ = e.chain_state()
        e.sweep(3, SEED, 1000, therm, nup)
        lat1 = e.get_lattice()
        ej1, ed1, _ = e.chain_state()
        h = e.histogram()
    rl, rh, rej, red, _ = orc.refgpu_weight(L, lat0, w32, ej0, ed0, 3, SEED, therm, nup)
    np.testing.assert_array_equal(lat1, rl)
    np.testing.assert_array_equal(ed1, red)
    np.testing.assert_array_equal(ej1, rej)
    np.testing.assert_array_equal(h, rh)


@pytest.mark.parametrize("L,nch,mode,kernel", [(96, 19456, "weight", 2), (96, 19456, "weight", 3),
                                                (72, 19456, "produce", 3)])
def test_many_chains_push_the_lattice_to_global_memory(muca, orc, L, nch, mode, kernel):
    """More chains than one wave of shared-memory blocks holds: the planner
    keeps the lattice in global memory (one wave of 128-chain blocks).  Every
    chain's final energies agree with its lattice, the histogram holds
    chains * nup entries, and three chain ranges (first block, a middle
    block boundary, last block) match the oracle bit for bit."""
    N = L * L
    produce = mode == "produce"
    rng = np.random.default_rng(L * 3 + kernel)
    lnw = _random_walk_weights(N, rng, sigma=0.8)
    therm, nup = N, N + 8
    with muca.Engine(L, nchains=nch, kernel=kernel, mode=muca.MODE_PRODUCE if produce else muca.MODE_WEIGHT) as e:
        assert e.info.lattice_in_smem == 0 and e.info.kernel == kernel
        cpb = e.info.chains_per_block
        e.set_weights(lnw)
        e.init_chains(muca.INIT_PRODUCE if produce else muca.INIT_WEIGHT, 0)
        lat0 = e.get_lattice()
        ej0, ed0, mg0 = e.chain_state()
        e.sweep(6, SEED, 2000 if produce else 1000, therm, nup)
        lat1 = e.get_lattice()
        ej1, ed1, mg1 = e.chain_state()
        h = e.histogram()
    assert int(h.sum()) == nch * nup
    oj, od, om = orc.energies(L, lat1)
    np.testing.assert_array_equal(ej1, oj)
    np.testing.assert_array_equal(ed1, od)
    mid = (nch // cpb // 2) * cpb
    for lo, hi in ((0, 40), (mid - 20, mid + 20), (nch - 40, nch)):
        a = lat0[lo:hi].copy()
        ej, ed, mg = _i32(ej0[lo:hi]), _i32(ed0[lo:hi]), _i32(mg0[lo:hi])
        if produce:
            orc.produce_sweep(L, a, ej, ed, mg, lnw, 6, SEED, therm, nup, chain0=lo, nthreads=8)
            np.testing.assert_array_equal(mg1[lo:hi], mg)
        else:
            orc.weight_sweep(L, a, ej, ed, lnw.astype(np.float32), 6, SEED, therm, nup, chain0=lo, nthreads=8)
        np.testing.assert_array_equal(lat1[lo:hi], a.reshape(hi - lo, N))
        np.testing.assert_array_equal(ed1[lo:hi], ed)
        np.testing.assert_array_equal(ej1[lo:hi], ej)
