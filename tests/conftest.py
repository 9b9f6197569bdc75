"""Shared fixtures.  The CUDA library (libsffg.so) and the CPU oracle are
built in-tree on first use; tests that need a GPU carry @pytest.mark.gpu."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def lib():
    from nabc_gb300 import _build, sff
    _build.build()
    L = sff.lib()
    # the reference's informational lines ("Reading parm file", "ff:") go to
    # nabout; keep them out of the test report
    sff.set_output(os.devnull)
    return L


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def checks():
    with open(os.path.join(GOLDEN, "checks.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def refrun():
    return dict(np.load(os.path.join(GOLDEN, "refrun.npz")))


def golden_path(name):
    for sub in ("ref", "synth"):
        p = os.path.join(GOLDEN, sub, name)
        if os.path.exists(p):
            return p
    raise FileNotFoundError(name)


def load_case(case):
    """(prm, x) for a case of checks.json through the library's rdparm and
    the reference's coordinate readers (PDB columns or restart file)."""
    from nabc_gb300 import sff
    prm = sff.rdparm(golden_path(case["prmtop"]))
    n = sff.natom(prm)
    cpath = golden_path(case["coords"])
    if cpath.endswith(".pdb"):
        x = sff.read_pdb_coords(cpath, n)
    else:
        x, _ = sff.getxv(cpath, n)
    return prm, x
