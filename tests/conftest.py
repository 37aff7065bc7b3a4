import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden32():
    import numpy as np
    return dict(np.load(ROOT / "tests" / "golden" / "golden_box32.npz"))


@pytest.fixture(scope="session")
def golden64():
    import numpy as np
    return dict(np.load(ROOT / "tests" / "golden" / "golden_box64.npz"))


@pytest.fixture(scope="session")
def golden128():
    import numpy as np
    return dict(np.load(ROOT / "tests" / "golden" / "golden_box128.npz"))


@pytest.fixture(scope="session")
def box128_case(golden128):
    """The box-128 fixture's job regenerated from its seed (images checked
    against the stored checksums) and the FP64 oracle's evaluation of its
    candidate (about 25 s on the CPU; shared by the tests of a session)."""
    from tests.helpers import box128_case as make
    return make(golden128)


@pytest.fixture(scope="session")
def native_lib():
    """The built library (built here if needed; nvcc cross-compiles)."""
    import __graft_entry__ as g
    g.build()
    from gisapr_gb300 import _native
    return _native.load()
