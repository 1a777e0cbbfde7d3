"""Shared fixtures: potentials and structures from tests/golden, the oracle."""
import gzip
import json
import os
import shutil
import sys

import numpy as np
import pytest

TESTS = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(TESTS)
GOLDEN = os.path.join(TESTS, "golden")
sys.path.insert(0, os.path.join(REPO, "lammps-mlip-package_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def potdir(tmp_path_factory):
    """Decompressed regression potentials: {name: path}."""
    d = tmp_path_factory.mktemp("pots")
    out = {}
    for name in ["gtinv-197", "gtinv-820", "gtinv-434", "pair-60", "pair-17"]:
        p = d / (name + ".mlip")
        with gzip.open(os.path.join(GOLDEN, name + ".mlip.gz"), "rb") as fi, open(p, "wb") as fo:
            shutil.copyfileobj(fi, fo)
        out[name] = str(p)
    return out


def structure(name):
    from mlipg.structures import read_lammps_data
    return read_lammps_data(os.path.join(GOLDEN, name))
