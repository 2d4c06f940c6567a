import importlib.util
import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__ as ge  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def pkg():
    return ge.load()


@pytest.fixture(scope="session")
def oracle(pkg):
    return ge.load_oracle().Oracle(pkg)


@pytest.fixture(scope="session")
def symref():
    spec = importlib.util.spec_from_file_location("cedar_symref", ROOT / "oracle" / "symbolic_ref.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def gpu(pkg):
    """The loaded CUDA library on a machine with a GPU (fails loudly otherwise)."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without CUDA")
    return pkg.load_library()
