import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native():
    """Build (incrementally) every native library the tests use."""
    from heavyrt_gb300 import native_build

    return native_build.build_all()


@pytest.fixture(scope="session")
def host_libs():
    """Only the host-side libraries (oracle, generators, reference checker)."""
    from heavyrt_gb300 import native_build

    return {"workload": native_build.build_workload(), "oracle": native_build.build_oracle(),
            "reference": native_build.build_reference()}


def golden_cases():
    return sorted(p.stem.replace("golden_", "") for p in GOLDEN.glob("golden_*.npz"))
