import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "light-field-remote-vision_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


def _built() -> None:
    lib = ROOT / "light-field-remote-vision_gb300" / "liblfrv.so"
    orc = ROOT / "oracle" / "liblfrv_oracle.so"
    if not lib.exists() or not orc.exists():
        sys.path.insert(0, str(ROOT))
        import __graft_entry__

        __graft_entry__.build()


_built()


@pytest.fixture(scope="session")
def ctx():
    import lfrv

    c = lfrv.Context(0)
    yield c
    c.close()
