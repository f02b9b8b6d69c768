"""Test configuration: the ``gpu`` marker and shared fixtures.

``-m "not gpu"`` runs on any host (oracle vs golden vectors, host graph code,
C-ABI exports).  ``-m gpu`` needs a GB300 and the built libbitruss.so; those
tests call the engine through its C ABI and compare with the oracle.
"""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = ["aw", "er_config1", "er_small0", "er_small1", "er_small2", "er_small3",
                "er_small4", "cl5k", "cl20k", "sparse"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built CUDA library")


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build(ref=False)
    return O


@pytest.fixture(scope="session")
def engine():
    import gpu_bitruss_gb300 as bt
    if not os.path.exists(bt.LIB_PATH):
        bt.build()
    bt.load()
    return bt


@pytest.fixture(scope="session")
def gpu_ctx(engine):
    """One device context for the GPU tests (fails loudly without a GB300)."""
    ctx = engine.Context(0)
    yield ctx
    ctx.close()
