"""Shared pytest setup: the ``gpu`` marker and the golden-case fixtures."""
import gzip
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = ["nma_amoeba", "nma_amoeba_cut", "nma_wang", "nma_wang_cut", "1crn_amoeba",
                "1crn_wang", "1ao6cut_wang", "1ubq_amoeba", "1ubq_wang"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU case")


@pytest.fixture(scope="session")
def golden():
    return np.load(os.path.join(GOLDEN_DIR, "golden.npz"))


@pytest.fixture(scope="session")
def golden_mmp(tmp_path_factory):
    """Decompress every golden .mmp input once; returns {case: path}."""
    d = tmp_path_factory.mktemp("golden_mmp")
    out = {}
    for name in GOLDEN_CASES:
        p = d / (name + ".mmp")
        with gzip.open(os.path.join(GOLDEN_DIR, name + ".mmp.gz"), "rb") as f:
            p.write_bytes(f.read())
        out[name] = str(p)
    return out
