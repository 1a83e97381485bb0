"""Shared test set-up: import paths, the `gpu` marker, checker builds."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("oracle", "recon-scanner_gb300", "tests"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.build_oracle(ref=False)
    return oracle.load("oracle")


@pytest.fixture(scope="session")
def ref_lib():
    import oracle

    if oracle.reference_tree() is None and not os.path.exists(oracle.REF_SO):
        pytest.skip("reference tree not present on this host")
    oracle.build_oracle(ref=True)
    return oracle.load("reference")
