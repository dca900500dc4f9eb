import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on a GB300)")


@pytest.fixture(scope="session")
def built():
    """Builds the CUDA library (nvcc cross-compiles without a GPU) and the CPU oracle."""
    from exachem_gb300.build import build_library
    import oracle
    build_library()
    oracle.build_port()
    return True


@pytest.fixture(scope="session")
def golden():
    return json.loads((ROOT / "tests" / "golden" / "reference_energies.json").read_text())


def rel_close(got, want, rtol, atol=1e-18):
    return abs(got - want) <= rtol * abs(want) + atol
