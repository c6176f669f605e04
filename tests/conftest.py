import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), os.pardir))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built CUDA library")


@pytest.fixture(scope="session")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def ft():
    """The CUDA library, initialised on cuda:0 (GPU tests only)."""
    import libftcrypto_gb300 as lib
    lib.build()
    code = lib.api.lib().ft_crypto_init()
    if code:
        pytest.fail(f"ft_crypto_init failed: {lib.error_str(code)} — GPU tests need an sm_103 device")
    return lib


def hx(s: str) -> np.ndarray:
    return np.frombuffer(bytes.fromhex(s), dtype=np.uint8).copy()


def hxs(items) -> np.ndarray:
    return np.stack([hx(s) for s in items])
