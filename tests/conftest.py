import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")


@pytest.fixture(scope="session")
def golden():
    return json.loads((ROOT / "tests" / "golden" / "reference_vectors.json").read_text())


@pytest.fixture(scope="session")
def stntt_lib():
    import stntt_gb300 as st
    from stntt_gb300 import _build

    _build.build()
    return st.lib()


@pytest.fixture(scope="session")
def ctx(stntt_lib):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import stntt_gb300 as st

    c = st.Context(0)
    yield c
    torch.cuda.synchronize()
    c.close()
