import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")


GOLDEN = os.path.join(HERE, "golden")


def golden_files(prefix=""):
    return sorted(os.path.join(GOLDEN, f) for f in os.listdir(GOLDEN)
                  if f.endswith(".npz") and f.startswith(prefix))
