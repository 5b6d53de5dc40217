"""The weight sweep taken apart (muca_sweep_floor): the per-warp cycle
counts of its parts are finite and ordered as their work is nested.  The
bare chain of decisions is part of the scan, and the scan (with its store
and histogram entries) is part of the whole window, as are the draws and
the decode."""
import math

import pytest

pytestmark = pytest.mark.gpu


def test_parts_are_ordered(muca):
    c = [muca.sweep_floor(p, windows=2048) for p in range(7)]
    whole, decode, scan, chain, draws, fadd, lds = c
    print("cycles per attempt per warp: whole %.1f, draws+decode %.1f, scan+store+hist %.1f, chain %.1f, "
          "draws %.1f; latency: FP32 add %.1f, shared load %.1f" % tuple(c))
    assert all(math.isfinite(x) and x > 0 for x in c)
    assert chain <= scan * 1.05
    assert scan < whole and decode < whole and draws < decode
    # a dependent add takes a few cycles, a shared-memory load tens
    assert 1.0 < fadd < lds < 200.0
