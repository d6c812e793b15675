import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) and the built engine library")


@pytest.fixture(scope="session", autouse=True)
def _built_checkers():
    """The oracle port is test infrastructure; build it once per session (fast, plain C)."""
    import subprocess
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    yield
