import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C-ABI library)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on CPU")


@pytest.fixture(scope="session")
def oracle():
    from oracle.pyoracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    """The reference's own CPU backend (oracle/_ref), or skip when it cannot be built."""
    from oracle import pyoracle
    try:
        path = pyoracle.build_reference()
    except Exception as exc:  # pragma: no cover - depends on the machine
        pytest.skip(f"reference CPU backend unavailable: {exc}")
    if not path:
        pytest.skip("reference CPU backend unavailable (no reference tree, no generated source)")
    return pyoracle.Reference(path)


@pytest.fixture(scope="session")
def golden_scene(oracle):
    """Loader for the validation scenes shipped with the reference."""
    def load(name):
        path = os.path.join(GOLDEN, f"{name}.obj")
        v, m, leaf, bmin, bmax = oracle.load_tree_with_soil(path)
        data = np.load(os.path.join(GOLDEN, f"{name}_vulkan.npz"))
        return dict(path=path, vertices=v, materials=m, leaf=leaf, bmin=bmin, bmax=bmax,
                    golden=data)
    return load


@pytest.fixture(scope="session")
def lib():
    """The CUDA library through its C-ABI (loads without a GPU)."""
    from streamsim_gb300 import facetcu
    return facetcu.load()
