import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as entry  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the C-ABI on the device)")


_built = False


def _ensure_built():
    global _built
    if not _built:
        entry.build()
        _built = True


@pytest.fixture(scope="session")
def llf():
    _ensure_built()
    return entry.load_package()


@pytest.fixture(scope="session")
def orc():
    _ensure_built()
    return entry.load_oracle()


# A checkout of the reference (read only), for the tests that read its files
# directly; they skip when LLF_REFERENCE_DIR is unset or missing.  Everything
# the other tests need from it is committed under tests/golden/.
REFERENCE = os.environ.get("LLF_REFERENCE_DIR", "")
