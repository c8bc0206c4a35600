import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "bluetangle.jl_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the engine's kernels)")
    # the C-ABI library must exist for the ABI/host tests; build it when missing
    lib = os.path.join(PKG, "libbtgpu.so")
    if not os.path.exists(lib):
        sys.path.insert(0, PKG)
        import build as _b
        _b.build()


@pytest.fixture(scope="session")
def ctx():
    import bluetangle_gpu as bt
    try:
        c = bt.Context(0, seed=12345)
    except bt.BTError as e:
        if e.code == -4:  # BT_ERR_DEVICE: no CUDA device in this machine
            pytest.skip("no CUDA device")
        raise
    bt.Context._default = c
    yield c
    c.close()


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def kref():
    import kron_ref
    return kron_ref
