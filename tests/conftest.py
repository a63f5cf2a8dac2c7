import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libsisgpu.so")


@pytest.fixture(scope="session")
def sis_ff():
    from sis_gb300.inputs import read_ff

    return read_ff(ROOT / "sis_gb300" / "data" / "sis.ff")


@pytest.fixture(scope="session")
def nn_ff():
    from sis_gb300.inputs import read_ff

    return read_ff(ROOT / "sis_gb300" / "data" / "sis_dih_ReB_NN.ff", bp_model=5)
