import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    # the Kuf autotuner's cache stays inside the test session
    import tempfile
    os.environ.setdefault("FPP_TUNE_CACHE",
                          os.path.join(tempfile.mkdtemp(prefix="fpp_tune_"), "tiles.txt"))


@pytest.fixture(scope="session")
def gpu_lib():
    """The built library, on a machine with a GPU."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    from flare_pp_gb300 import _lib
    return _lib.lib()
