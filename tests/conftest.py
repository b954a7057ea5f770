"""pytest configuration: the `gpu` marker and import paths.

Tests marked `gpu` need a GB300 and the built library; everything else runs
on CPU (oracle known-answer tests, host logic, ABI symbol checks).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "rust-softrender_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")
    config.addinivalue_line("markers", "recent: GPU tests not yet run on a GPU; they run after all others")


def pytest_collection_modifyitems(config, items):
    # stable: tests marked `recent` move towards the end, in their collected
    # order, so that a failure among them under -x stops none of the others;
    # the allocation-free entry point's file (test_zz_no_alloc.py) stays last
    def rank(it):
        if os.path.basename(str(it.fspath)) == "test_zz_no_alloc.py":
            return 2
        return 1 if it.get_closest_marker("recent") else 0
    items.sort(key=rank)


def _load(name, path):
    import importlib.util
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def built_lib():
    return _load("sr_pkg_build", os.path.join(ROOT, "rust-softrender_gb300", "build.py")).build()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.lib()
    return oracle
