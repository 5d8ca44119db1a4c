import gzip
import os
import shutil
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def extract_case(case, dest):
    """Unpack tests/golden/<case>/*.gz into dest; returns dest."""
    src = os.path.join(GOLDEN, case)
    os.makedirs(dest, exist_ok=True)
    for f in os.listdir(src):
        if f.endswith(".gz"):
            with gzip.open(os.path.join(src, f), "rb") as a, open(os.path.join(dest, f[:-3]), "wb") as b:
                shutil.copyfileobj(a, b)
    return dest


CONF = {
    "512_particles": "512_particles_bruteforce_LawDefault_noPeriodicity.conf",
    "518_poly": "518_poly_bruteforce_default_noperiod.conf",
    "50_prismes_gravity": "50_prismes_gravity.conf",
}


@pytest.fixture(scope="session")
def golden_dir(tmp_path_factory):
    base = tmp_path_factory.mktemp("golden")
    for case in CONF:
        extract_case(case, str(base / case))
    return base


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    from rockable_gb300 import build_ext
    build_ext.build()
    from rockable_gb300 import abi
    return abi
