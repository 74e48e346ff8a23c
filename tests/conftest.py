import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

# the reference checkout: LAVAFRAME_REFERENCE, else a `reference` directory beside this repository
REFERENCE = Path(os.environ.get("LAVAFRAME_REFERENCE", ROOT.parent / "reference"))
REF_REF = ROOT / "oracle" / "_ref"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def native_libs():
    from lavaframe_gb300 import build

    build.build_core()
    build.build_oracle()
    return True


@pytest.fixture(scope="session")
def ctx():
    import lavaframe_gb300 as lf

    c = lf.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def ref_host():
    """The reference's own host code (compiled from a reference checkout into oracle/_ref)."""
    lib = REF_REF / "libref_host.so"
    if not lib.exists():
        from lavaframe_gb300 import build

        try:
            build.build_reference()
        except Exception as e:  # pragma: no cover
            pytest.skip(f"reference build failed: {e}")
    if not lib.exists():
        pytest.skip("no reference checkout on this host")
    from tests import refhost

    return refhost.RefHost(lib)
