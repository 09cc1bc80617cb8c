import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT / "chmy.jl_gb300", ROOT / "tests", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libchmy_gb300.so")


@pytest.fixture(scope="session")
def arch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from chmy_gb300 import Arch, GB300Backend

    a = Arch(GB300Backend(), device_id=1)
    yield a
    a.close()
