import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "simple-ts_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, ORACLE, GOLDEN):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def oracle_built():
    from build_oracle import build_oracle
    build_oracle()
    return True


@pytest.fixture(scope="session")
def lib_built():
    import build as stsbuild
    stsbuild.build()
    import sts
    return sts.load()


@pytest.fixture(scope="session")
def golden_records():
    import json
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return {r["name"]: r for r in json.load(f)}


def golden_case(name):
    """Rebuilds the case a golden record was made from (same builders as make_golden.py)."""
    import sts_cases as sc
    import make_golden
    for n, case, fixed in make_golden.cases():
        if n == name:
            return case, fixed
    if name == "shipped_example_5steps":
        return sc.shipped_example(5), True
    raise KeyError(name)
