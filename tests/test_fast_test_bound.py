"""The error bound behind the production scan's FP32 fast test, checked in
numpy's IEEE arithmetic (CPU only).

The production sweep (sweep_core.cuh: prologue<..., DT> and scan_window)
stages T[E] = {(float)(w[E-1] - w[E]), (float)(w[E+1] - w[E])} from the FP64
weights, forms fast = fl32(f2 + dl) with dl the entry of dDel (0 for
dDel = 0), and decides with g = fl32(l - fast), where the reference forms
diff = fl64(fl64(f2 + w[E+dDel]) - w[E]) (produce2_multigpu.cu:474) and
accepts on  diff >= 0 || logf(u) < diff.  The kernel takes

    tol = 2 (2^-24 (2 md + 16) + 2^-53 (max|w| + 32 + 2 md))   (times 1.0001)

with md = max|T|, claims |fast - diff| <= tol / 2, and replays a window
whenever |g| <= tol + eps (eps covers __logf against logf).  These tests
check the claim and the sign rule it implies on random and adversarial
weights, with l the exact float logf of every attempt's uniform.
"""
import numpy as np
import pytest

F2 = np.arange(-16, 17, 2, dtype=np.float32)  # -2 dE for dE in [-8, 8]


def _tol(w):
    d = np.diff(w)
    md = float(np.max(np.abs(d.astype(np.float32)))) if d.size else 0.0
    mw = float(np.max(np.abs(w)))
    m = md * 1.0001
    return np.float32((2.0 * 2.0 ** -24 * (2.0 * m + 16.0) + 2.0 * 2.0 ** -53 * (mw + 32.0 + 2.0 * m)) * 1.0001)


def _cases(w):
    """every (E, dDel, f2): dl, fast (FP32 as the kernel) and diff (FP64 as the reference)"""
    N = w.size - 1
    E = np.arange(N + 1)
    out = []
    for dd in (-1, 0, 1):
        ok = (E + dd >= 0) & (E + dd <= N)
        e = E[ok]
        dl = np.zeros(e.size, np.float32) if dd == 0 else (w[e + dd] - w[e]).astype(np.float32)
        for f2 in F2:
            fast = (np.float32(f2) + dl).astype(np.float32)          # one FP32 addition, round to nearest
            diff = (np.float64(f2) + w[e + dd]) - w[e]                # the reference's FP64 difference
            out.append((fast, diff))
    fast = np.concatenate([a for a, _ in out])
    diff = np.concatenate([b for _, b in out])
    return fast, diff


def _weights():
    rng = np.random.default_rng(17)
    N = 4096
    walk = np.cumsum(rng.normal(0.0, 1.5, N + 1)) * 0.5
    return {
        "zero": np.zeros(N + 1),
        "walk": walk,
        "walk_offset_1e4": walk + 1.0e4,
        "steep": np.cumsum(rng.normal(0.0, 40.0, N + 1)),
        "near_f2": np.cumsum(rng.choice([-16.0, -8.0, 8.0, 16.0], N + 1) + rng.normal(0.0, 1e-6, N + 1)),
        "large": rng.uniform(-1e5, 1e5, N + 1),
    }


@pytest.mark.parametrize("name", list(_weights().keys()))
def test_fast_difference_within_half_tol(name):
    w = _weights()[name]
    tol = _tol(w)
    fast, diff = _cases(w)
    err = np.abs(fast.astype(np.float64) - diff)
    assert np.all(err <= tol / 2), (name, float(err.max()), float(tol))


@pytest.mark.parametrize("name", list(_weights().keys()))
def test_band_outside_tol_keeps_the_reference_decision(name):
    """Outside the band, g = fl32(l - fast) < 0 is the reference's decision
    diff >= 0 || l < diff (l = the exact float logf, always < 0)."""
    w = _weights()[name]
    tol = _tol(w)
    fast, diff = _cases(w)
    rng = np.random.default_rng(5)
    k = rng.integers(0, 1 << 23, fast.size)
    u = ((2 * k + 1) * 2.0 ** -24).astype(np.float32)      # u01fixedpt<float>: (1 | (r >> 8)) 2^-24
    l = np.log(u.astype(np.float64)).astype(np.float32)     # a float logf (exact rounding stands in for CUDA's)
    # half the attempts with l placed right at the threshold, where the band matters
    near = rng.random(fast.size) < 0.5
    l = np.where(near & (fast < 0), (fast + np.float32(rng.normal(0.0, 4.0, fast.size)) * tol).astype(np.float32), l)
    l = np.minimum(l, np.float32(-2.0 ** -24))               # logf(u) < 0 for every u
    g = (l - fast).astype(np.float32)
    outside = np.abs(g) > tol
    ref = (diff >= 0) | (l.astype(np.float64) < diff)
    assert outside.sum() > 0.4 * fast.size
    np.testing.assert_array_equal((g < 0)[outside], ref[outside])
