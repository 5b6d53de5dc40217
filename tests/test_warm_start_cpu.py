"""The non-learned warm starts of the A/B, on the host: the full-weight and
the piecewise-linear (reference knots) interpolation in temperature."""
import numpy as np
import pytest

from muca_gb300 import warm_start as ws


def _sources(L):
    N = L * L
    i = np.arange(N + 1) / N
    return [(L, 0.4, 50 * np.sin(3 * i) + 7.0), (L, 0.6, 80 * i * i - 3.0), (L, 0.8, 20 * i)]


def test_interp_reproduces_a_source():
    L = 6
    src = _sources(L)
    for _, T, w in src:
        out = ws.interpolated_weight(L, T, src)
        np.testing.assert_allclose(out, w - w.mean(), atol=1e-12)
        assert abs(out.mean()) < 1e-12


def test_interp_is_linear_in_T_between_the_bracket():
    L = 5
    src = _sources(L)
    a, b = src[0][2], src[1][2]
    out = ws.interpolated_weight(L, 0.45, src)
    ref = 0.75 * a + 0.25 * b
    np.testing.assert_allclose(out, ref - ref.mean(), atol=1e-12)
    # outside the range: the two nearest, extended linearly
    out = ws.interpolated_weight(L, 0.9, src)
    ref = -0.5 * src[1][2] + 1.5 * src[2][2]
    np.testing.assert_allclose(out, ref - ref.mean(), atol=1e-12)


def test_pl_is_straight_between_the_reference_knots():
    L = 10
    N = L * L
    src = _sources(L)
    w = src[0][2]
    out = ws.interpolated_weight(L, 0.4, src, ws.PL_KNOTS)
    ik = np.rint(np.array(ws.PL_KNOTS) * N).astype(int)
    assert list(ik) == [0, 18, 89, 100]
    shift = (out - w)[0]
    np.testing.assert_allclose(out[ik], w[ik] + shift, atol=1e-12)
    for a, b in zip(ik[:-1], ik[1:]):
        seg = out[a:b + 1]
        np.testing.assert_allclose(np.diff(seg, 2), 0, atol=1e-9)


def test_interp_across_sizes_is_extensive():
    # lnW_L(i) = N g_T(i/N) with g linear in x: the per-site weights of the
    # sizes 4 and 8 are interpolated exactly, linearly in L and T
    def src(L, T):
        N = L * L
        x = np.arange(N + 1) / N
        return (L, T, N * ((3.0 + 10 * T) * x + 0.1 * L))
    sources = [src(L, T) for L in (4, 8) for T in (0.4, 0.6)]
    L, T = 6, 0.5
    N = L * L
    x = np.arange(N + 1) / N
    ref = N * ((3.0 + 10 * T) * x)
    out = ws.interpolated_weight(L, T, sources)
    np.testing.assert_allclose(out, ref - ref.mean(), atol=1e-9)
    # a single size is only rescaled
    out = ws.interpolated_weight(L, T, sources[:2])
    np.testing.assert_allclose(out, ref - ref.mean(), atol=1e-9)


def test_interp_input_checks():
    with pytest.raises(ValueError):
        ws.interpolated_weight(7, 0.5, [])
    with pytest.raises(ValueError):
        ws.interpolated_weight(6, 0.5, [(6, 0.5, np.zeros(10))])


def test_final_agreement_ignores_the_additive_constant():
    rng = np.random.default_rng(0)
    w = np.cumsum(rng.normal(0, 1, 101))
    a = ws.final_agreement(w + 3.25, w)
    assert a["rms"] < 1e-12 and a["max"] < 1e-12
    d = np.zeros(101)
    d[50] = 0.101
    a = ws.final_agreement(w + d, w)
    f = d - d.mean()
    assert abs(a["rms"] - np.sqrt(np.mean(f * f))) < 1e-15
    assert abs(a["max"] - abs(f).max()) < 1e-15
    assert abs(a["rms_rel_range"] - a["rms"] / (w.max() - w.min())) < 1e-15


def test_agreement_instances_take_their_own_chain_count():
    held = [(16, 1024, 0.43, 1.7, 5000), (24, 1024, 0.53, 1.8, 5001), (16, 1024, 0.63, 1.9, 5002)]
    assert ws.agreement_instances(held, 16) == [held[0], held[2]]
    assert ws.agreement_instances(held, 16, 16384) == [(16, 16384, 0.43, 1.7, 5000), (16, 16384, 0.63, 1.9, 5002)]
    assert ws.agreement_instances(held, 8) == []


def test_agreement_under_runs_the_floor_on_other_seeds(monkeypatch):
    """The zero arm, the requested warm starts and the zero weight on seeds
    + 7919 (the statistical floor), each compared with the zero arm."""
    calls = []

    class R:
        def __init__(self, it):
            self.iterations, self.converged = it, 1

    def fake_converge(inst, opts, warm=None, device=0):
        calls.append(([i[4] for i in inst], None if warm is None else [float(w[0]) for w in warm]))
        off = 0.0 if warm is None else 0.01
        off += 0.005 if inst[0][4] > 6000 else 0.0
        return [R(10) for _ in inst], 0.5, [np.linspace(0, 1, 17) + off * np.linspace(-1, 1, 17) for _ in inst]

    class Net:
        def log_weights(self, L, T, D):
            return np.full(L * L + 1, 2.0)

    monkeypatch.setattr(ws, "converge", fake_converge)
    held = [(4, 8, 0.5, 1.9, 100), (4, 8, 0.6, 1.9, 101)]
    out = ws.agreement_under(Net(), held, [], {"flat_minmean": 0}, arms=("mlp",))
    assert set(out) == {"zero", "mlp", "zero_reseeded"}
    seeds = [c[0] for c in calls]
    assert seeds == [[100, 101], [100 + 7919, 101 + 7919], [100, 101]]
    assert calls[2][1] == [2.0, 2.0]  # the network's start
    ramp = np.linspace(-1, 1, 17)
    rms = lambda c: float(np.sqrt(np.mean((c * ramp) ** 2)))
    assert abs(out["mlp"]["final_rms_vs_zero_max"] - rms(0.01)) < 1e-12
    assert abs(out["zero_reseeded"]["final_rms_vs_zero_max"] - rms(0.005)) < 1e-12
    assert out["zero"]["iters_total"] == 20 and out["mlp"]["converged"] == 2
