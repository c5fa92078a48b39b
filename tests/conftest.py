import os
import pathlib
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))
os.environ.setdefault("ORACLE_QUIET", "1")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def golden():
    path = ROOT / "tests" / "golden" / "golden.npz"
    return dict(np.load(path, allow_pickle=False))


_MATS = {}


@pytest.fixture(scope="session")
def mats():
    from cases import MATRICES

    class _M:
        def __getitem__(self, name):
            if name not in _MATS:
                _MATS[name] = MATRICES[name]()
            return _MATS[name]

    return _M()
