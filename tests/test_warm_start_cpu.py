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
