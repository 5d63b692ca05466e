"""Shared pytest setup.

* registers the ``gpu`` marker (tests that need a GB300 and the CUDA library);
* makes the oracle (``oracle/oracle.py``) and the package in ``fluid-sim_gb300/``
  importable without installation.
"""
from __future__ import annotations

import importlib.util
import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libfluidcuda.so")


def load_package():
    """Import ``fluid-sim_gb300/`` as the module ``fluid_sim_gb300``."""
    name = "fluid_sim_gb300"
    if name in sys.modules:
        return sys.modules[name]
    pkg_dir = ROOT / "fluid-sim_gb300"
    spec = importlib.util.spec_from_file_location(name, pkg_dir / "__init__.py",
                                                  submodule_search_locations=[str(pkg_dir)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def golden():
    return json.loads((ROOT / "tests" / "golden" / "reference_results.json").read_text())


@pytest.fixture(scope="session")
def O():
    import oracle

    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def fs():
    return load_package()
