"""The windowed weight sweep's shared u32 histogram bins are flushed into
the u64 device histogram between rows whenever a launch could otherwise put
2^32 entries into one bin.  MUCA_HOOK_FLUSH_ROWS makes every recorded row
take that path; lattices, energies and histograms must still equal the
oracle's (the reference kernel mcs, muca_delta_multigpu.cu:737-829) bit for
bit, with the lattice in shared memory and behind the row ring, and with
therm and nup not multiples of a row so that the step-by-step tail runs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("L,nch", [(24, 256), (72, 128), (128, 64)])
def test_flushing_shared_bins_between_rows_changes_nothing(muca, orc, L, nch):
    N = L * L
    rng = np.random.default_rng(L)
    lnw = np.cumsum(rng.normal(0.0, 1.2, N + 1)) * 0.5
    therm, nup = N + 37, 3 * N + 11
    with muca.Engine(L, nchains=nch, kernel=muca.KERNEL_WINDOWED) as e:
        assert e.info.kernel == muca.KERNEL_WINDOWED
        e.set_weights(lnw)
        e.init_chains(muca.INIT_WEIGHT, 0)
        lat0 = e.get_lattice()
        ej0, ed0, _ = e.chain_state()
        e.set_test_hooks(muca.HOOK_FLUSH_ROWS)
        e.sweep(2, 100, 1000, therm, nup)
        lat1 = e.get_lattice()
        ej1, ed1, _ = e.chain_state()
        h = e.histogram()
        e.set_test_hooks(0)
    ej, ed = (np.ascontiguousarray(x, np.int32).copy() for x in (ej0, ed0))
    olat, oh = orc.weight_sweep(L, lat0.copy(), ej, ed, lnw.astype(np.float32), 2, 100, therm, nup, nthreads=8)
    np.testing.assert_array_equal(lat1, olat.reshape(nch, N))
    np.testing.assert_array_equal(ej1, ej)
    np.testing.assert_array_equal(ed1, ed)
    np.testing.assert_array_equal(h, oh)
    assert int(h.sum()) == nch * nup
