import json
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (HERE, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the sm_103a library")
    config.addinivalue_line("markers", "slow: long CPU oracle runs at full configuration size")


@pytest.fixture(scope="session")
def golden():
    return json.load(open(os.path.join(HERE, "golden", "golden.json")))


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads libsofren2_gb300.so; fails loudly without a GPU."""
    import torch  # noqa: F401  (only to learn whether CUDA is visible)
    from sofren2_gb300 import build, runtime
    if not torch.cuda.is_available():
        pytest.fail("a CUDA device is required for -m gpu tests")
    build.build_library()
    return runtime.load_library()


@pytest.fixture(scope="session")
def renderer(gpu_lib):
    from sofren2_gb300 import runtime
    r = runtime.Renderer(640, 360, 1)
    yield r
    r.close()
