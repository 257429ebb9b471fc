import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")
    config.addinivalue_line("markers", "slow: long-running CPU case")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle, build_oracle

    build_oracle()
    return Oracle()


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    return np.load(os.path.join(ROOT, "tests", "golden", "reference_golden.npz"))


@pytest.fixture(scope="session")
def reference():
    """The compiled reference (only where its sources exist)."""
    from oracle.oracle import REF_SO, Reference, build_oracle

    if not os.path.exists(REF_SO):
        from oracle.oracle import reference_sources_present

        if not reference_sources_present():
            pytest.skip("reference sources not present on this host")
        build_oracle(ref=True)
    return Reference()
