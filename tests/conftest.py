import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA path)")


@pytest.fixture(scope="session")
def built():
    import __graft_entry__
    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def driver(built):
    from kazan_gb300 import vk
    return vk.Driver()


@pytest.fixture(scope="session")
def renderer(driver):
    from kazan_gb300 import render
    r = render.Renderer(driver)
    yield r
    r.close()
