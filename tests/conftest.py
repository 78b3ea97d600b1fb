import pathlib
import sys

import pytest

REPO = pathlib.Path(__file__).resolve().parent.parent
for p in (REPO, REPO / "phys-engine_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = REPO / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls the engine through its C ABI")


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    cache = {}

    def load(name):
        if name not in cache:
            cache[name] = dict(np.load(GOLDEN / f"{name}.npz", allow_pickle=False))
        return cache[name]

    return load


@pytest.fixture(scope="session")
def gpu():
    """The CUDA engine; fails loudly if it is missing (no CPU fallback)."""
    from phys_gb300 import engine

    lib = engine.lib()
    if lib.pe_device_count() < 1:
        pytest.fail("no CUDA device visible to the engine")
    return engine
