"""Shared fixtures: registers the ``gpu`` marker and imports the package directory
``fairsim-vigor_gb300/`` under the module name ``fairsim_vigor_gb300``."""
import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def load_package():
    name = "fairsim_vigor_gb300"
    if name in sys.modules:
        return sys.modules[name]
    pkg_dir = os.path.join(ROOT, "fairsim-vigor_gb300")
    spec = importlib.util.spec_from_file_location(
        name, os.path.join(pkg_dir, "__init__.py"), submodule_search_locations=[pkg_dir])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def fs():
    return load_package()


@pytest.fixture(scope="session")
def oracle():
    from oracle import refcpu
    refcpu.build()
    refcpu.set_threads(min(8, os.cpu_count() or 1))
    return refcpu


def rel_l2(a, b):
    import numpy as np
    a = np.asarray(a, dtype=np.float64) if not np.iscomplexobj(a) else np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.float64) if not np.iscomplexobj(b) else np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.fixture(scope="session")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
