import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 and the built CUDA library")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def engine():
    """The built GB300 engine library (fails loudly if it is missing or no GB300 is present)."""
    import lf_dem_gb300 as E
    from lf_dem_gb300 import build as B
    B.build()
    E.load()
    rc, name, cc, nsm = E.device_info(0)
    if rc != E.LFG_OK:
        pytest.fail(f"no usable sm_103 device: rc={rc} name={name} cc={cc}")
    return E
