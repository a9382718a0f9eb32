import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_collection_modifyitems(config, items):
    # Tests marked gpu are selected with -m gpu; when run without a GPU they
    # fail loudly rather than skip, so a silent CPU pass is impossible.
    pass


@pytest.fixture(scope="session")
def golden_cases():
    from tests.golden_io import load_all
    return load_all()
