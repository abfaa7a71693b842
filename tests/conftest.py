import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the ctgpu kernels)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def ctlib():
    """The ctgpu shared library, built in-tree if it is missing."""
    from scico_gb300 import _lib, build

    if not _lib.LIB_PATH.exists():
        build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def cuda(ctlib):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch.device("cuda", 0)


@pytest.fixture(autouse=True)
def _device_check_words(request):
    """After every GPU test: the projectors' device error words must be 0
    (a device check that fired and was not read by the test itself means
    work was skipped silently)."""
    yield
    if request.node.get_closest_marker("gpu") is None:
        return
    import torch

    if not torch.cuda.is_available():
        return
    from scico_gb300 import _lib

    lib = _lib.load()
    torch.cuda.synchronize()
    w2, w3 = lib.ct_proj2d_errflag(), lib.ct_proj3d_errflag()
    assert w2 == 0 and w3 == 0, f"device check words left set: proj2d {w2:#x}, proj3d {w3:#x}"
