"""Failure detection without faulting the GPU.

The reference's only checks are cudaGetLastError after each launch
(muca_delta_multigpu.cu:417-421) and an uncapped loop (:374).  Here every
device-side wait (the mbarrier waits of the warp-specialised sweep) is
bounded per wait; a launch whose wait runs out ends normally, sets the
context's error word, and the next synchronising call returns
MUCA_ERR_TIMEOUT.  The test makes a wait run out by a flag that nothing sets:
the test hook keeps the producer warps from ever signalling a filled slot,
with a short wait limit.  Nothing traps, faults or hangs; afterwards the
same context runs a normal sweep that matches the oracle bit for bit, and is
destroyed cleanly.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TIMEOUT = 3  # MUCA_ERR_TIMEOUT


@pytest.mark.parametrize("mode", ["weight", "produce"])
def test_bounded_wait_runs_out_and_context_stays_usable(muca, orc, mode):
    L, nch = 16, 64
    N = L * L
    produce = mode == "produce"
    rng = np.random.default_rng(2)
    lnw = np.cumsum(rng.normal(0.0, 1.0, N + 1)) * 0.5
    with muca.Engine(L, nchains=nch, kernel=muca.KERNEL_SPECIALIZED,
                     mode=muca.MODE_PRODUCE if produce else muca.MODE_WEIGHT) as e:
        e.set_weights(lnw)
        e.init_chains(muca.INIT_PRODUCE if produce else muca.INIT_WEIGHT, 0)
        e.set_wait_limit(1 << 20)  # about 0.5 ms without progress
        e.set_test_hooks(muca.HOOK_SILENT_PRODUCER)
        e.sweep(0, 100, 1000, N, N)
        with pytest.raises(muca.MucaError) as ex:
            e.histogram()
        assert ex.value.status == TIMEOUT
        assert "gave up" in str(ex.value)
        # the error word was cleared by that report: the context is usable again
        e.set_test_hooks(0)
        e.set_wait_limit(0)
        e.init_chains(muca.INIT_PRODUCE if produce else muca.INIT_WEIGHT, 0)
        lat0 = e.get_lattice()
        ej0, ed0, mg0 = e.chain_state()
        e.sweep(1, 100, 2000 if produce else 1000, N, 300)
        lat1 = e.get_lattice()
        h = e.histogram()
    ej, ed, mg = (np.ascontiguousarray(x, np.int32).copy() for x in (ej0, ed0, mg0))
    if produce:
        olat, oh = orc.produce_sweep(L, lat0.copy(), ej, ed, mg, lnw, 1, 100, N, 300, nthreads=4)
    else:
        olat, oh = orc.weight_sweep(L, lat0.copy(), ej, ed, lnw.astype(np.float32), 1, 100, N, 300, nthreads=4)
    np.testing.assert_array_equal(lat1, olat.reshape(nch, N))
    np.testing.assert_array_equal(h, oh)


def test_wait_bound_is_per_wait_not_per_launch(muca, orc):
    """A launch that runs far longer than the wait limit but keeps making
    progress completes: the bound measures a wait, not the launch."""
    import torch
    L, nch = 64, 4096
    N = L * L
    s = torch.cuda.Stream()
    with muca.Engine(L, nchains=nch, kernel=muca.KERNEL_SPECIALIZED, stream=s.cuda_stream) as e:
        e.init_chains(muca.INIT_WEIGHT, 0)
        e.set_wait_limit(1 << 20)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        e.sweep(0, 100, 1000, N, 100 * N)
        b.record(s)
        h = e.histogram()  # raises on a timeout
        b.synchronize()
        ms = a.elapsed_time(b)
    assert int(h.sum()) == nch * 100 * N
    # the launch took many times the limit (2^20 cycles is about 0.5 ms)
    assert ms > 5.0, ms


def test_wait_limit_and_hooks_are_checked(muca):
    with muca.Engine(16, nchains=32) as e:
        with pytest.raises(muca.MucaError):
            e.set_wait_limit(1 << 41)
        with pytest.raises(muca.MucaError):
            e.set_test_hooks(4)
