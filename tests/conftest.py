"""Shared fixtures.  Tests marked `gpu` need a CUDA GPU and the built
libgprt.so; every other test runs on the CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "go-progressive-raytracer_gb300")
for p in (PKG, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def _build_module(path, name):
    import importlib.util
    spec = importlib.util.spec_from_file_location(name, path)
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.fixture(scope="session")
def oracle():
    """The oracle client with its library built."""
    _build_module(os.path.join(ROOT, "oracle", "build.py"), "oracle_build").build()
    from oracle import client
    client.load()
    return client


@pytest.fixture(scope="session")
def gprt_lib():
    """The product library, built in-tree."""
    _build_module(os.path.join(PKG, "build.py"), "gprt_build").build()
    import gprt
    return gprt.capi.load()


@pytest.fixture(scope="session")
def ctx(gprt_lib):
    import gprt
    c = gprt.Context(0)
    yield c
    c.close()
