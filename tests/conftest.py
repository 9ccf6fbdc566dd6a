import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libmczi_gpu.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle_ref
    oracle_ref.load()
    return oracle_ref


@pytest.fixture(scope="session")
def golden():
    import json
    return json.loads((ROOT / "tests" / "golden" / "reference_vectors.json").read_text())


@pytest.fixture(scope="session")
def gpu_ctx():
    from mczi_gb300 import build
    build.build_gpu_lib()
    from mczi_gb300.mc import Context
    ctx = Context(0)
    yield ctx
    ctx.close()
