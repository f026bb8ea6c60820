import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

DATA = os.path.join(ROOT, "tests", "data")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built engine library")


@pytest.fixture(scope="session")
def data_dir():
    return DATA


def inp(name):
    return os.path.join(DATA, name + ".inp")


def golden_overrides(fx):
    """The .inp lines a golden fixture's run adds to its case: a restart from
    frame `frame` of a reference-written trajectory under golden/outputs."""
    if "restart" not in fx:
        return ""
    trj, frame = fx["restart"]
    return "restart_traj_file=%s\nrestart_step=%d\n" % (os.path.join(GOLDEN, "outputs", trj), frame)
