import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "r-scape_gb300")
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def covgpu():
    build = _load("rscape_gb300_build", os.path.join(PKG, "build.py"))
    build.build()
    return _load("covgpu", os.path.join(PKG, "covgpu.py"))


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O
