import gzip
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")
if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)   # config_fixtures: the oracle fixtures of the benchmark configurations


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on CPU")


def golden_vhr_text(name: str) -> str:
    with gzip.open(os.path.join(GOLDEN, name + ".gz"), "rt") as f:
        return f.read()
