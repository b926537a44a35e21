"""Test configuration: registers the `gpu` marker, loads the package
(directory polgraw-allsky_gb300, import name polgraw_gb300) and puts the
oracle binding and the golden helpers on sys.path."""
from __future__ import annotations

import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def load_package():
    name = "polgraw_gb300"
    if name in sys.modules:
        return sys.modules[name]
    d = os.path.join(ROOT, "polgraw-allsky_gb300")
    spec = importlib.util.spec_from_file_location(name, os.path.join(d, "__init__.py"),
                                                  submodule_search_locations=[d])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


load_package()
for p in (os.path.join(ROOT, "oracle"), GOLDEN, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def lib():
    from polgraw_gb300 import build, lib as L
    build.build()
    return L.load()


@pytest.fixture(scope="session")
def gpu_ok(lib):
    if lib.pa_device_count() < 1:
        pytest.fail("no CUDA device visible: GPU tests must run on a GPU host")
    return True
