import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "sph-exa-nnet_gb300")
for p in (os.path.join(PKG, "data"), PKG, os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def helm_table():
    import gen_helm_table
    return np.stack([gen_helm_table.tables()[n] for n in gen_helm_table.NAMES]).reshape(-1)


@pytest.fixture(scope="session")
def port(helm_table):
    import importlib.util
    spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(REPO, "oracle", "build.py"))
    ob = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ob)
    ob.build_oracle()
    from oracle import Oracle
    o = Oracle("port")
    o.load_helmholtz(helm_table)
    return o


@pytest.fixture(scope="session")
def ref(helm_table):
    from oracle import Oracle
    try:
        o = Oracle("ref")
    except FileNotFoundError:
        pytest.skip("reference build (oracle/_ref) not present on this machine")
    o.load_helmholtz(helm_table)
    return o


def golden(name):
    return np.load(os.path.join(GOLDEN, name))
