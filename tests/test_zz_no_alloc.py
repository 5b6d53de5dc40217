"""muca_observables_noalloc: the reweighting sums over caller-owned device
buffers, with a static scratch array instead of any allocation.  Checked
against muca_compute_observables (the context path, same kernels) and
against the oracle's restatement of the reference's observables
(produce2_multigpu.cu:498-518) on two calls in a row, and the device's free
memory is checked to stay the same across warm calls.  This file is
collected last, so that in a full run the first call of the no-allocation
path comes after the other tests' use of the library."""
import numpy as np
import pytest


def _inputs(L, seed):
    N = L * L
    rng = np.random.default_rng(seed)
    hs = (N + 1) * (N + 2) // 2
    h = rng.integers(0, 10000, hs).astype(np.uint64)
    h[rng.random(hs) < 0.4] = 0
    lnw = np.cumsum(rng.normal(-1.0, 0.5, N + 1))
    return h, lnw


def _context_sums(muca, L, h, lnw, beta, delta):
    """{sum, m1, m2, m4} through the context path, and the shifted weights it used."""
    with muca.Engine(L, nchains=64, mode=muca.MODE_PRODUCE) as e:
        e.set_weights(lnw)
        e.set_histogram(h)
        e.weight_shift(beta, delta)
        w = e.reweighting_weights()
        ob = e.observables(beta, delta)
    return np.array([ob.sum, ob.m1, ob.m2, ob.m4]), w


def test_noalloc_rejects_bad_arguments():
    """Rejected before any CUDA call: no GPU needed."""
    from muca_gb300 import build as b
    b.build()
    import muca_gb300 as m
    fake = 0x1000  # never dereferenced: the checks come first
    for L in (0, 1, 129, 4096):
        with pytest.raises(m.MucaError, match="outside 2..128"):
            m.observables_noalloc(0, fake, fake, L, 2.0, 1.9, fake)
    with pytest.raises(m.MucaError, match="NULL device pointer"):
        m.observables_noalloc(0, 0, fake, 8, 2.0, 1.9, fake)
    with pytest.raises(m.MucaError, match="NULL device pointer"):
        m.observables_noalloc(0, fake, fake, 8, 2.0, 1.9, 0)


@pytest.mark.gpu
@pytest.mark.parametrize("L", [8, 16, 64])
def test_noalloc_matches_context_path_two_calls(muca, orc, L):
    import torch
    beta = 2.0
    cases = [(_inputs(L, 3 * L), 1.5), (_inputs(L, 3 * L + 1), 1.99)]
    expected, dev = [], []
    for (h, lnw), delta in cases:
        sums, w = _context_sums(muca, L, h, lnw, beta, delta)
        expected.append(sums)
        dev.append((torch.from_numpy(h.view(np.int64)).cuda(), torch.from_numpy(w).cuda()))
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    # outputs start as NaN: the call must write every entry
    outs = [torch.full((4,), float("nan"), dtype=torch.float64, device="cuda") for _ in cases]
    # two calls in a row on one stream, no host synchronisation between them
    for ((hd, wd), (_, delta)), out in zip(zip(dev, cases), outs):
        muca.observables_noalloc(0, hd.data_ptr(), wd.data_ptr(), L, beta, delta, out.data_ptr(), stream)
    torch.cuda.synchronize()
    for out, exp in zip(outs, expected):
        np.testing.assert_allclose(out.cpu().numpy(), exp, rtol=1e-13, atol=0)
    # the oracle (the reference's long-double sums) on the same shifted weights
    N = L * L
    for ((h, _), delta), (_, wd), out in zip(cases, dev, outs):
        bz = np.zeros(N + 1)
        orc.lib().orc_boltz(beta, delta, N, wd.cpu().numpy().copy(), bz, 0)
        o = orc.observables(beta, N, h, bz)
        np.testing.assert_allclose(out.cpu().numpy(), o[3:], rtol=1e-12, atol=0)
    # the same input again gives the same sums (no state carried between calls)
    (hd, wd), (_, delta) = dev[0], cases[0]
    again = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
    muca.observables_noalloc(0, hd.data_ptr(), wd.data_ptr(), L, beta, delta, again.data_ptr(), stream)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(again.cpu().numpy(), outs[0].cpu().numpy())


@pytest.mark.gpu
def test_noalloc_leaves_free_memory_unchanged(muca):
    """The defining property: after a first call (which may load the module
    and looks up the scratch address) further calls change the device's free
    memory (cudaMemGetInfo) by nothing, and leave the current device alone."""
    import torch
    L, beta = 32, 2.0
    h, lnw = _inputs(L, 11)
    hd = torch.from_numpy(h.view(np.int64)).cuda()
    wd = torch.from_numpy(lnw).cuda()
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    muca.observables_noalloc(0, hd.data_ptr(), wd.data_ptr(), L, beta, 1.9, out.data_ptr(), stream)
    torch.cuda.synchronize()
    first = out.cpu().numpy().copy()
    free0, _ = torch.cuda.mem_get_info()
    for k in range(3):
        muca.observables_noalloc(0, hd.data_ptr(), wd.data_ptr(), L, beta, 1.9, out.data_ptr(), stream)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, "free device memory moved by %d bytes" % (free0 - free1)
    assert torch.cuda.current_device() == 0
    np.testing.assert_array_equal(out.cpu().numpy(), first)
