"""Shared test set-up.

Markers: `gpu` marks tests that need a CUDA device (run with -m gpu on a
GB300); everything else runs on a CPU-only machine.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def orc():
    from oracle import orc as o
    o.build()
    return o


@pytest.fixture(autouse=True)
def _device_acceptance_logf(request):
    """GPU tests compare with what the reference kernels compute on the device,
    whose acceptance test uses CUDA's logf; the oracle takes the device's logf
    values for them (libm's logf differs by one ulp for some u).  CPU tests
    keep libm's, as the reference's CPU programs do."""
    if request.node.get_closest_marker("gpu") is None:
        yield
        return
    from oracle import orc as o
    o.build(refgpu=True)
    o.use_device_logf(True)
    yield
    o.use_device_logf(False)


@pytest.fixture(scope="session")
def muca():
    """The engine, built for sm_103a; GPU tests only."""
    from muca_gb300 import build as b
    b.build()
    import muca_gb300
    muca_gb300.lib()
    return muca_gb300


@pytest.fixture(scope="session")
def refgpu(orc):
    """Launcher of the reference kernels (cubins compiled from the reference
    sources).  Where the cubins are missing the tests that need them skip,
    unless MUCA_REQUIRE_REF_KERNELS=1 says they must be there: then they fail."""
    try:
        orc.build(refgpu=True)
        launcher = orc.refgpu()
    except Exception as ex:  # noqa: BLE001
        launcher, why = None, str(ex)
    else:
        why = "reference cubins not present in this checkout"
    if launcher is None:
        if os.environ.get("MUCA_REQUIRE_REF_KERNELS") == "1":
            pytest.fail("reference kernels required (MUCA_REQUIRE_REF_KERNELS=1): " + why)
        pytest.skip(why)
    return launcher
