"""Shared test set-up: the gpu marker, and loaders for the oracle and the package.

The package directory is ``gbgperiodicfields.jl_gb300`` (its name holds a dot), so it
is loaded by path and registered as the importable module ``gbgperiodicfields_gb300``.
"""
import importlib.util
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_package():
    name = "gbgperiodicfields_gb300"
    if name in sys.modules:
        return sys.modules[name]
    pkg_dir = ROOT / "gbgperiodicfields.jl_gb300"
    spec = importlib.util.spec_from_file_location(
        name, pkg_dir / "__init__.py", submodule_search_locations=[str(pkg_dir)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def gbg():
    return load_package()


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    o.build()
    return o
