import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Native library and oracle, built once per session."""
    from iactrace_gb300 import _build
    import oracle.oracle as O
    _build.build()
    O.build()
    from iactrace_gb300 import _native
    return _native.load()


@pytest.fixture(scope="session")
def cuda(built):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch.device("cuda", 0)


@pytest.fixture(scope="session")
def reference_checkout():
    """A checkout of GerritRo/iactrace for tests that read its data files
    (the HESS YAML configurations): the directory named by
    IACTRACE_REFERENCE, else a `reference` directory beside this
    repository; skipped when neither holds the reference."""
    for cand in (os.environ.get("IACTRACE_REFERENCE", ""), os.path.join(os.path.dirname(ROOT), "reference")):
        if cand and os.path.isfile(os.path.join(cand, "iactrace", "__init__.py")):
            return cand
    pytest.skip("no checkout of the reference (set IACTRACE_REFERENCE)")
