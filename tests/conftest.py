"""Shared pytest set-up: the ``gpu`` marker, import paths and the oracle build."""

import pathlib
import sys

import pytest

REPO = pathlib.Path(__file__).resolve().parent.parent
for p in (REPO, REPO / "hoomd-blue_gb300", REPO / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")


@pytest.fixture(scope="session", autouse=True)
def _oracle_built():
    from oracle import build
    build.build_oracle()
    yield
