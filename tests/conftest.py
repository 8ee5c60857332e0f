import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "sgm-bench_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on the GPU box)")


@pytest.fixture(scope="session")
def engine():
    import sgmgb
    eng = sgmgb.Engine(0)
    yield eng
    eng.close()


@pytest.fixture(scope="session")
def ref_fixtures():
    import json
    with open(os.path.join(GOLDEN_DIR, "reference_scenes.json")) as f:
        return json.load(f)
