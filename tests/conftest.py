import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "parallel-dmd-for-biomolecules_gb300")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

# the reference's parallel-dmd-PRIME20 directory, when present (tests that
# read its files directly skip without it)
REFERENCE = os.environ.get("DMD_REFERENCE_DIR", "")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and runs the engine")


@pytest.fixture(scope="session")
def built():
    import __graft_entry__ as g

    g.build()
    return True


def has_reference() -> bool:
    return os.path.isdir(REFERENCE)


@pytest.fixture(autouse=True)
def _checked_build_bounds(request):
    """In the checked build (DMD_CHECKED=1), every GPU test must also leave
    no out-of-range device index behind."""
    yield
    if os.environ.get("DMD_CHECKED", "") != "1" or request.node.get_closest_marker("gpu") is None:
        return
    import ctypes as C
    from dmdgb import abi
    rec = C.c_longlong()
    rc = abi.load_engine().dmd_debug_bounds(C.byref(rec))
    assert rc == 0, (f"out-of-range device index: site {(rec.value >> 40) & 0x3fffff}, "
                     f"extent {(rec.value >> 20) & 0xfffff}, index {rec.value & 0xfffff}")
