"""pytest configuration: the `gpu` marker and import paths.

Tests marked `gpu` need a CUDA device (sm_103); everything else runs on CPU.
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "skylens-stream-rs_gb300"), os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def matcher():
    import skylens_match as sm
    m = sm.Matcher()
    yield m
    m.close()
